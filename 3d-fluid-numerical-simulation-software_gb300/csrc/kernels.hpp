// Host-side declarations of the kernel launchers (one translation unit per stage).
#pragma once
#include <vector>
#include "gbt_common.cuh"

namespace gbt {

// launch geometry of one level of a batch: grid.y enumerates solves, grid.x covers the largest
// solve's box (blocks past a smaller solve's end return at once)
struct LaunchCtx {
    Batch batch;
    cudaStream_t stream;
    int maxIM = 0, maxJM = 0, maxKM = 0;     // maxima over the solves of this level
    long long pool_n = 0;                     // elements of one field pool of this level
    // optional stage profiler: called before (begin = 1) and after (begin = 0) a group of
    // launches with the group's name, the number of kernel launches in it and the grid level
    void (*hook)(void *user, const char *stage, int begin, int launches, int level) = nullptr;
    void *hook_user = nullptr;
    int level = 0;                            // grid level of these launches (1 = fine)
    const void *face_tma = nullptr;           // tables of the TMA-staged face stage (mixed form), or null
    const void *face_tma_host = nullptr;      // their header, on the host
    void mark(const char *stage, int begin, int launches = 1) const { if (hook) hook(hook_user, stage, begin, launches, level); }
    dim3 grid_n(long long n, int bs) const { return dim3((unsigned)((n + bs - 1) / bs), batch.nsolve); }
    dim3 grid_cells(int bs) const { return grid_n((long long)(maxIM - 1) * (maxJM - 1) * (maxKM - 1), bs); }
    dim3 grid_faces(int f, int bs) const
    {
        return grid_n((long long)(maxIM - 1 + (f == 0)) * (maxJM - 1 + (f == 1)) * (maxKM - 1 + (f == 2)), bs);
    }
    dim3 grid_plane(int bs) const { return grid_n((long long)(maxIM - 1) * (maxJM - 1), bs); }
};

// boundary patches in device form; every record names its solve
struct DevInOut { int solve, face, is, ie, js, je, ks, ke; };
struct DevWall { int solve, face, rotate, is, ie, js, je, ks, ke; };
// mixing plane: k+ face of slot s1 (rows is..ie, pitch range js1..je1) against the k- face of slot s2
struct DevMix { int s1, s2, is, ie, js1, je1, js2, je2; };
constexpr int kMixVals = 14;                    // per row: both sides' averaged d, u, v, w, p, c; the SA value
struct BcTables {
    const DevInOut *inlet = nullptr; int n_inlet = 0, max_inlet = 0;     // max cells of a patch
    const DevInOut *outlet = nullptr; int n_outlet = 0;
    const DevWall *wall = nullptr; int n_wall = 0, max_wall = 0;
    // walls grouped by their position in each solve's list (the reference applies them in order)
    int n_wall_slot = 0;
    int wall_slot_off[65] = {0};                  // first record of slot q; slot q has off[q+1]-off[q]
    int wall_slot_lines[64] = {0};                // most wall-normal lines of a patch in slot q
    // periodic exchange as a gather list: dst <- rotate(src, sign * delta_th of the solve)
    const long long *per_dst = nullptr, *per_src = nullptr;
    const int *per_meta = nullptr;                // solve * 4 + (sign + 1)
    const double *per_trig = nullptr;             // per solve: cos, sin of +delta_th, then of -delta_th
    long long n_per = 0;
    int max_outlet_im = 0, max_outlet_jm = 0;
    double *outlet_cu = nullptr;                  // per outlet patch: mass-weighted swirl of each radial row
    double *integ_part = nullptr;                 // per solve and section: kIntegralBlocks partial sums of 3
    // Baldwin-Lomax wall distances (fine level): record w holds, for point n0 = 1..N-1 of each of
    // its wall-normal lines t, the distance of cell n0 from the line's wall-face centre at
    // wall_dist[wall_dist_off[w] + (n0 - 1) * lines(w) + t], in the working precision
    void *wall_dist = nullptr;
    const long long *wall_dist_off = nullptr;
    const DevInOut *inlet_first = nullptr, *outlet_first = nullptr;   // per solve: Inlet[1], Outlet[1]
    // mixing planes (applied after every other boundary) and their per-row averages
    const DevMix *mix = nullptr;
    int n_mix = 0, max_mix_rows = 0, max_mix_j = 0;
    double *mix_avg = nullptr;
    // Spalart-Allmaras: ghost cells of the variable filled by interfaces and periodic pairs
    const long long *sa_dst = nullptr, *sa_src = nullptr;
    long long n_sa_gather = 0;
};

constexpr int kIntegralBlocks = 16;             // blocks per inlet/outlet section in the integrals

// Cells of every i+j+k hyperplane of every solve, in "plane order": q runs over the planes of
// solve 0, then those of solve 1, ...; inside a plane by i, then j. start[s*stride + plane] ..
// start[s*stride + plane + 1] are the q of one plane of solve s; max_count[plane] is the largest
// plane over the solves.
struct PlaneTables {
    const int *start = nullptr;
    int stride = 0, max_plane = 0;
    long long nq = 0;
    int cpw = 10, wpb = 1;                        // sweep block shape: cells per warp, warps per block (autotuned)
    // row starts for the tiled scatter of dQ: the plane-order index of interior cell
    // (i, j, k) of solve s is rq[rq_off[s] + (i + j + k) * (IM - 1) + i - 1] + j
    const int *rq = nullptr;
    const long long *rq_off = nullptr;
    std::vector<int> max_count;
};

// Everything the LU-SGS sweeps read, copied into plane order so that the cells of one plane and
// their neighbours in the previous plane are dense in memory (in the k-contiguous box they are
// scattered, one sector per value). Geometry is copied once; the flow inputs before every forward
// sweep; dQ lives here during the sweeps and is scattered back to the box afterwards.
template <typename T>
struct SweepData {
    const long long *cell = nullptr;               // q -> box index (including the solve's base)
    const int *nb[2][3] = {};                      // [0] lower (forward), [1] upper (backward) neighbour q, or -1
    T *gn[3][3] = {}, *gs[3] = {}, *gve[3] = {}, *gvol = nullptr;   // per direction: mean normal, |S|, entrainment
    T *cv[NQ] = {}, *pp = nullptr, *lamc[3] = {}, *lamv[3] = {}, *dt = nullptr, *res[NQ] = {};
    T *dq[NQ] = {};
    // Spalart-Allmaras sweep (null without it), per cell as a neighbour in direction d: normal
    // velocity with the mean flow's dQ added, old variable times old normal velocity, mean |S|,
    // relax * lambda_c, lambda_v; per cell: old variable, diagonal, residual, update
    T *sa_vn[3] = {}, *sa_eb[3] = {}, *sa_s[3] = {}, *sa_rl[3] = {}, *sa_lv[3] = {};
    T *sa_ev0 = nullptr, *sa_alpha = nullptr, *sa_res = nullptr, *sa_dq = nullptr;
};

void launch_geometry(const LaunchCtx &ctx, const Geo &G, double *totalvol);
// the periodic rotation's cosines and sines per solve (BcTables::per_trig), once at create
void launch_periodic_trig(const LaunchCtx &ctx, double *trig);

template <typename T>
void launch_boundary(const LaunchCtx &ctx, const Phys &P, const Geo &G, Flow<T> F, const BcTables &bc);

// residual stages; level = 1 for the fine mesh (turbulence model only there)
// the mixed form's face stage with tiles staged in shared memory by TMA (csrc/face_tma.cu)
bool face_tma_eligible(const std::vector<Lvl> &lv);
void *build_face_tma(const std::vector<Lvl> &lv, const GeoW<float> &G, const Flow<float> &W, size_t *bytes,
                     unsigned char host_header[64]);
void launch_face_tma(const LaunchCtx &ctx, const Phys &P, const PhysW<float> &PC, const GeoW<float> &GW, Flow<float> W,
                     const DevWall *walls);

template <typename T>
void launch_resflux(const LaunchCtx &ctx, const Phys &P, const PhysW<T> &PC, const Geo &G, const GeoW<T> &GW, Flow<T> F,
                    const BcTables &bc, int level, T *scratch_dtmin);

// the mean-flow sweeps; with the Spalart-Allmaras variable present (F.ev), its scalar sweep of each
// direction follows the mean-flow sweep of that direction
template <typename T>
void launch_lusgs_sweeps(const LaunchCtx &ctx, const PhysW<T> &P, const Geo &G, Flow<T> F, const PlaneTables &pt,
                         const SweepData<T> &S);

// fastest block shape of the sweep kernels for this level, as cells_per_warp * 16 + warps_per_block
// (times the plane chains on benign inputs in the plane-order scratch; synchronises the stream)
// whether (cells per warp, warps per block) is one of the compiled sweep shapes
bool sweep_shape_known(int cpw, int wpb);
template <typename T>
int tune_sweep_cpw(const LaunchCtx &ctx, const PhysW<T> &P, const PlaneTables &pt, const SweepData<T> &S);

// Baldwin-Lomax wall distances of every wall line point (fine level, once; see BcTables)
template <typename T>
void launch_wall_distances(const LaunchCtx &ctx, const Geo &G, const BcTables &bc);

// FP32 copies of the geometry the working-precision kernels read (mixed form; once per level)
void launch_geometry_working(const LaunchCtx &ctx, const Geo &G, const GeoW<float> &GW);

// plane-order copy of the sweep's geometry (once per level, after the geometry kernels)
template <typename T>
void launch_sweep_geometry(const LaunchCtx &ctx, const Geo &G, const PlaneTables &pt, const SweepData<T> &S);

template <typename T>
void launch_update(const LaunchCtx &ctx, const Phys &P, const Geo &G, Flow<T> F, int level,
                   int *bad_list, int bad_cap, int *bad_count);

template <typename T>
void launch_res_norm(const LaunchCtx &ctx, const Geo &G, Flow<T> F, const double *totalvol, double *partials,
                     int nblk);

// residual norm with scratch in a static device array; copies the norms to host_out if given
template <typename T>
void launch_res_norm_static(const LaunchCtx &ctx, const Geo &G, Flow<T> F, const double *totalvol, int ncase, double *host_out);

template <typename T>
void launch_integrals(const LaunchCtx &ctx, const Phys &P, const Geo &G, Flow<T> F, const BcTables &bc);

template <typename T>
void launch_primitive(const LaunchCtx &ctx, const Phys &P, Flow<T> F);

template <typename T>
void launch_limiter(const LaunchCtx &ctx, const Phys &P, Flow<T> F, int level, int *bad_list, int bad_cap,
                    int *bad_count);

// multigrid transfer between fine (f) and coarse (c) levels
template <typename T>
void launch_restrict(const LaunchCtx &cf, const LaunchCtx &cc, const Geo &Gf, const Geo &Gc, Flow<T> Ff, Flow<T> Fc);
template <typename T>
void launch_forcing(const LaunchCtx &cc, Flow<T> Fc);
template <typename T>
void launch_delta(const LaunchCtx &cc, Flow<T> Fc);
template <typename T>
void launch_forcing_keep(const LaunchCtx &cc, Flow<T> Fc);
template <typename T>
void launch_add_forcing(const LaunchCtx &cc, Flow<T> Fc);
template <typename T>
void launch_corner(const LaunchCtx &cc, Flow<T> Fc);
template <typename T>
void launch_interpolate(const LaunchCtx &cf, const LaunchCtx &cc, Flow<T> Ff, Flow<T> Fc, int init_from_coarse);

// per-solve scalar stages
void launch_cfl_ramp(const LaunchCtx &ctx, int iter);

// Spalart-Allmaras (sa.cu)
void launch_sa_wall_distance(const LaunchCtx &ctx, const Geo &G, const long long *face_p, const int *face_f, long long n,
                             double *scratch_xyz, const long long *case_off, double *dwall);
void launch_sa_init(const LaunchCtx &ctx, double *ev, double ev_ratio);
template <typename T>
void launch_sa_boundary(const LaunchCtx &ctx, const Phys &P, Flow<T> W, const BcTables &bc);
template <typename T>
void launch_sa_model(const LaunchCtx &ctx, const Phys &P, const GeoW<T> &GW, Flow<T> W);
template <typename T>
void launch_sa_sweep(const LaunchCtx &ctx, const PhysW<T> &PC, const Geo &G, Flow<T> W, const PlaneTables &pt,
                     const SweepData<T> &S, int dir);
template <typename T>
void launch_sa_update(const LaunchCtx &ctx, const Phys &P, Flow<T> W, int *bad_list, int bad_cap, int *bad_count);
template <typename T>
void launch_sa_limit(const LaunchCtx &ctx, Flow<T> W, int *bad_list, int bad_cap, int *bad_count);

}  // namespace gbt
