// Solver orchestration: memory layout of a batch, boundary tables, geometry set-up and the
// reference's iteration sequence (source/Solver.cpp:47-140, source/LU_SGS_Marching.cpp:10-291,
// source/ComputeAllBlockVars.cpp:223-255) as kernel launches on one stream, replayed through
// CUDA graphs.
#include "solver.hpp"
#include "restart_io.hpp"
#include <cmath>
#include <cstring>
#include <cstdio>
#include <cstdlib>
#include <array>
#include <atomic>
#include <chrono>
#include <exception>
#include <thread>
#include <map>
#include <array>
#include <stdexcept>
#include <algorithm>

namespace gbt {

void check_cuda(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(x) check_cuda((x), #x)

NonDim nondimensionalise(const CaseSpec &c)
{
    NonDim n;
    const float PIf = 3.1415926535897932f;
    n.temp_ref = c.Ttin;
    n.vel_ref = std::sqrt(c.Gamma * c.Rgas * n.temp_ref);
    n.mue_ref = 1.716e-5f * std::pow(n.temp_ref / 288.15f, 3.0f / 2.0f) * (288.15f + 110.4f) / (n.temp_ref + 110.4f);
    n.dens_ref = c.Ptin / c.Rgas / n.temp_ref;
    n.re_ref = n.dens_ref * n.vel_ref * c.Len_ref / n.mue_ref;
    double ma_ref = 1.0f;
    n.pout = c.Pout / (n.dens_ref * n.vel_ref * n.vel_ref);
    n.ttin = 1.0f;
    n.ptin = 1.0f / c.Gamma;
    n.rgas = 1.0f / (ma_ref * ma_ref * c.Gamma);
    n.w_rot = (2.0f * PIf * c.rpm / 60.0f) / (n.vel_ref / c.Len_ref);
    n.delta_th = (double)(2.0f * PIf / (float)c.nblade);
    return n;
}

// ----------------------------------------------------------------------------------------
// one mesh level of the whole batch
// ----------------------------------------------------------------------------------------
template <typename T>
struct Level {
    int id = 1;
    std::vector<Lvl> lv;                  // per solve
    std::vector<SolveConst> sc;
    Lvl *lv_d = nullptr;
    SolveConst *sc_d = nullptr;
    long long pool_n = 0;
    int maxIM = 0, maxJM = 0, maxKM = 0, max_plane = 0;
    DevBuf geo_mem, flow_d_mem, flow_t_mem, int_mem, tab_mem, meta_mem;
    Geo G{};
    GeoW<T> GW{};                         // working-precision geometry (aliases in FP64, FP32 copies in mixed)
    DevBuf geow_mem;
    DevBuf tma_mem;                       // tables of the TMA-staged face stage (mixed form)
    unsigned char tma_host[64] = {};      // their header
    DevBuf fd_mem;                        // JST face dissipation
    DevBuf sa_mem, sa_tab_mem;            // Spalart-Allmaras fields; its tables
    DevBuf wdist_mem;                     // Baldwin-Lomax wall distances (fine level)
    Flow<T> W{};
    double *totalvol = nullptr, *blockvol = nullptr;
    BcTables bc;
    PlaneTables planes;
    SweepData<T> sweep;
    DevBuf plane_mem;
    std::vector<DevWall> walls_h;
    bool use_force = false;
    LaunchCtx ctx(const Batch &B, cudaStream_t s) const
    {
        LaunchCtx c;
        c.batch = B;
        c.batch.lv = lv_d;
        c.batch.sc = sc_d;
        c.stream = s;
        c.maxIM = maxIM; c.maxJM = maxJM; c.maxKM = maxKM;
        c.pool_n = pool_n;
        c.face_tma = tma_mem.p;
        c.face_tma_host = tma_host;
        return c;
    }
};

// level boxes of one case: level 2 re-indexes the patches of level 1 (source/UserInput.cpp:449-796)
static int ci(int s0, int e0, bool first) { return first ? (s0 + 1) / 2 : (s0 == e0 ? (e0 + 1) / 2 : e0 / 2); }
static void coarse_patch(int &s, int &e) { int a = s, b = e; s = ci(a, b, true); e = ci(a, b, false); }

struct LevelCase {
    int IM, JM, KM;
    std::vector<PatchIO> in, out;
    std::vector<WallIO> walls;
    std::vector<double> x, y, z;          // nodes, ((k-1)*JM + (j-1))*IM + (i-1)
};

// a periodic pair or block interface on a level (each coarser level re-indexes the previous one's)
static PeriodicIO level_pair(PeriodicIO p, int level)
{
    for (int l = 2; l <= level; l++)
        for (int d = 0; d < 3; d++) { coarse_patch(p.r1[2 * d], p.r1[2 * d + 1]); coarse_patch(p.r2[2 * d], p.r2[2 * d + 1]); }
    return p;
}
static PatchIO level_patch(PatchIO p, int level)
{
    for (int l = 2; l <= level; l++) { coarse_patch(p.is, p.ie); coarse_patch(p.js, p.je); coarse_patch(p.ks, p.ke); }
    return p;
}

// every second node and the re-indexed patches of a level
static LevelCase coarsen(const LevelCase &c)
{
    LevelCase L;
    L.IM = (c.IM + 1) / 2; L.JM = (c.JM + 1) / 2; L.KM = (c.KM + 1) / 2;
    size_t n = (size_t)L.IM * L.JM * L.KM;
    L.x.resize(n); L.y.resize(n); L.z.resize(n);
    for (int k = 1; k <= L.KM; k++)
        for (int j = 1; j <= L.JM; j++)
            for (int i = 1; i <= L.IM; i++) {
                size_t q = ((size_t)(k - 1) * L.JM + (j - 1)) * L.IM + (i - 1);
                size_t f = ((size_t)(2 * k - 2) * c.JM + (2 * j - 2)) * c.IM + (2 * i - 2);
                L.x[q] = c.x[f]; L.y[q] = c.y[f]; L.z[q] = c.z[f];
            }
    for (auto p : c.in) { coarse_patch(p.is, p.ie); coarse_patch(p.js, p.je); coarse_patch(p.ks, p.ke); L.in.push_back(p); }
    for (auto p : c.out) { coarse_patch(p.is, p.ie); coarse_patch(p.js, p.je); coarse_patch(p.ks, p.ke); L.out.push_back(p); }
    for (auto w : c.walls) { coarse_patch(w.is, w.ie); coarse_patch(w.js, w.je); coarse_patch(w.ks, w.ke); L.walls.push_back(w); }
    return L;
}

static LevelCase level_case(const CaseSpec &c, int level)
{
    if (level > 1) return coarsen(level_case(c, level - 1));
    LevelCase L;
    L.IM = c.IM; L.JM = c.JM; L.KM = c.KM;
    L.in = c.inlets; L.out = c.outlets; L.walls = c.walls;
    L.x = c.x; L.y = c.y; L.z = c.z;
    return L;
}

// whether a block and all its patches coarsen a second time: node counts with (N-1) a multiple of
// 4 and (N-1)/4 > 2, and every patch range odd-aligned on the second level as well (the
// reference's own check allows at most two levels: source/UserInput.cpp:799-1068)
static bool coarsens_twice(const CaseSpec &c)
{
    auto dim_ok = [](int N) { return (N - 1) % 4 == 0 && (N - 1) / 4 > 2; };
    if (!dim_ok(c.IM) || !dim_ok(c.JM) || !dim_ok(c.KM)) return false;
    auto rng_ok = [](int s, int e) {
        if (s != e) e = e + 1;
        return (s - 1) % 4 == 0 && (e - 1) % 4 == 0;
    };
    auto patch_ok = [&](int is, int ie, int js, int je, int ks, int ke) { return rng_ok(is, ie) && rng_ok(js, je) && rng_ok(ks, ke); };
    for (auto &p : c.inlets) if (!patch_ok(p.is, p.ie, p.js, p.je, p.ks, p.ke)) return false;
    for (auto &p : c.outlets) if (!patch_ok(p.is, p.ie, p.js, p.je, p.ks, p.ke)) return false;
    for (auto &w : c.walls) if (!patch_ok(w.is, w.ie, w.js, w.je, w.ks, w.ke)) return false;
    for (const auto *lst : {&c.periodics, &c.interiors, &c.mixing})
        for (auto &p : *lst)
            if (!patch_ok(p.r1[0], p.r1[1], p.r1[2], p.r1[3], p.r1[4], p.r1[5]) ||
                !patch_ok(p.r2[0], p.r2[1], p.r2[2], p.r2[3], p.r2[4], p.r2[5]))
                return false;
    return true;
}

// Face-local traversal of a periodic patch in the order of the reference's shadow buffers
// (source/ShadowOutIn.cpp:15-164, 324-497): returns, for every (l, m), the interior cell read at
// layer nd and the ghost / reconstruction cell written at layer nd.
struct PatchCell { int l, m; int ri, rj, rk; int gi, gj, gk; };
static std::vector<PatchCell> patch_walk(int fc, int nd, const int *r, int IM, int JM, int KM, int &lmax, int &mmax)
{
    std::vector<PatchCell> v;
    int is = r[0], ie = r[1], js = r[2], je = r[3], ks = r[4], ke = r[5];
    auto rng = [](int s, int e) { std::vector<int> a; int x = s; do { a.push_back(x); x++; } while (x <= e); return a; };
    switch (fc) {
    case 1: lmax = std::abs(ke - ks) + 1; mmax = std::abs(je - js) + 1;
        { int l = 1; for (int k : rng(ks, ke)) { int m = 1; for (int j : rng(js, je)) { v.push_back({l, m, nd, j, k, -nd, j, k}); m++; } l++; } } break;
    case 2: lmax = std::abs(je - js) + 1; mmax = std::abs(ke - ks) + 1;
        { int l = 1; for (int j : rng(js, je)) { int m = 1; for (int k : rng(ks, ke)) { v.push_back({l, m, IM - nd, j, k, IM + nd, j, k}); m++; } l++; } } break;
    case 3: lmax = std::abs(ie - is) + 1; mmax = std::abs(ke - ks) + 1;
        { int l = 1; for (int i : rng(is, ie)) { int m = 1; for (int k : rng(ks, ke)) { v.push_back({l, m, i, nd, k, i, -nd, k}); m++; } l++; } } break;
    case 4: lmax = std::abs(ke - ks) + 1; mmax = std::abs(ie - is) + 1;
        { int l = 1; for (int k : rng(ks, ke)) { int m = 1; for (int i : rng(is, ie)) { v.push_back({l, m, i, JM - nd, k, i, JM + nd, k}); m++; } l++; } } break;
    case 5: lmax = std::abs(je - js) + 1; mmax = std::abs(ie - is) + 1;
        { int l = 1; for (int j : rng(js, je)) { int m = 1; for (int i : rng(is, ie)) { v.push_back({l, m, i, j, nd, i, j, -nd}); m++; } l++; } } break;
    case 6: lmax = std::abs(ie - is) + 1; mmax = std::abs(je - js) + 1;
        { int l = 1; for (int i : rng(is, ie)) { int m = 1; for (int j : rng(js, je)) { v.push_back({l, m, i, j, KM - nd, i, j, KM + nd}); m++; } l++; } } break;
    default: throw std::runtime_error("bad periodic face type");
    }
    return v;
}
// (l1, m1) of the sending face -> (l2, m2) of the receiving face (source/ShadowOutIn.cpp:167-321)
static void trans(int ori, int l1, int m1, int L1, int M1, int &l2, int &m2)
{
    switch (ori) {
    case 1: l2 = l1; m2 = M1 + 1 - m1; break;
    case 2: l2 = m1; m2 = l1; break;
    case 3: l2 = L1 + 1 - l1; m2 = m1; break;
    case 4: l2 = M1 + 1 - m1; m2 = L1 + 1 - l1; break;
    default: throw std::runtime_error("bad periodic orientation");
    }
}

// interior cells of a level set to the uniform start of their solve (source/Initialization.cpp:17-76):
// five conserved values per slot in init
__global__ void k_fill_uniform(Batch B, double *cv0, double *cv1, double *cv2, double *cv3, double *cv4,
                               const double *init)
{
    const Lvl L = B.lv[blockIdx.y];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
    const double *c = init + 5 * blockIdx.y;
    cv0[p] = c[0]; cv1[p] = c[1]; cv2[p] = c[2]; cv3[p] = c[3]; cv4[p] = c[4];
}

// the uniform start of one slot (init_q) on its level's interior cells
__global__ void k_fill_uniform_slot(Batch B, int slot, double *cv0, double *cv1, double *cv2, double *cv3, double *cv4,
                                    const double *init)
{
    const Lvl L = B.lv[slot];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
    const double *c = init + 5 * slot;
    cv0[p] = c[0]; cv1[p] = c[1]; cv2[p] = c[2]; cv3[p] = c[3]; cv4[p] = c[4];
}

// per slot, kAbsResBlocks partial sums of |R_rho| over the interior cells (fixed order)
constexpr int kAbsResBlocks = 64;
template <typename T>
__global__ void __launch_bounds__(256) k_abs_res_partial(Batch B, const T *res0, double *part)
{
    const Lvl L = B.lv[blockIdx.y];
    const long long n = (long long)(L.IM - 1) * (L.JM - 1) * (L.KM - 1);
    double a = 0.0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(t % (L.KM - 1)) + 1;
        const long long r = t / (L.KM - 1);
        const int j = (int)(r % (L.JM - 1)) + 1, i = (int)(r / (L.JM - 1)) + 1;
        a += fabs((double)res0[ix(L, i, j, k)]);
    }
    __shared__ double sh[256];
    sh[threadIdx.x] = a;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = sh[0];
}

// volume of a case: its blocks' volumes summed in block order (source/ComputeAllBlockVars.cpp:32)
__global__ void k_case_volume(Batch B, const double *blockvol, double *casevol)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B.nsolve) return;
    const SolveConst &c = B.sc[s];
    double v = 0.0;
    for (int b = 0; b < c.nblk; b++) v = v + blockvol[c.lead + b];
    casevol[s] = v;
}

// start of a driver iteration: iteration counter and CFL ramp (source/Solver.cpp:49-60)
// imposed mass flow after the iteration's output (source/Structured_FV3D.cpp:186-193 with
// CSolver::MassFlowImposed, source/Solver.cpp:142-145): once the density residual is below the
// gate and every iter_mass_imp iterations, p_out += relax * p_out * (m_out - m_imposed) / m_imposed
__global__ void k_mass_control(Batch B)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B.nsolve) return;
    const SolveConst &c = B.sc[s];
    SolveState &st = B.st[s];
    if (!c.mass_imposed) return;
    if (st.res[0] <= c.resc_mass_imp && st.iter % c.iter_mass_imp == 0)
        st.pout = st.pout + c.relax_press * st.pout * (st.m_out - c.m_imposed) / c.m_imposed;
}

__global__ void k_iter_begin(Batch B)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B.nsolve) return;
    SolveState &st = B.st[s];
    st.iter += 1;
    if (st.iter > 1) {
        if (st.res[0] <= st.cfl_res) {
            st.cfl = st.cfl * (double)1.2f;
            st.cfl_res = st.cfl_res / (double)10.0f;
        }
        if (st.cfl > (double)10.0f) st.cfl = (double)10.0f;
    }
}

// set-up phase times on stderr when GBTURBO_TIMING is set (the stream is synchronised at each mark
// then, so that device work is charged to its phase)
struct PhaseTimer {
    bool on = std::getenv("GBTURBO_TIMING") != nullptr;
    std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
    void mark(const char *what, cudaStream_t st)
    {
        if (!on) return;
        if (st) cudaStreamSynchronize(st);
        const auto n = std::chrono::steady_clock::now();
        std::fprintf(stderr, "[gbturbo set-up] %-28s %8.1f ms\n", what, std::chrono::duration<double, std::milli>(n - t).count());
        t = n;
    }
};

template <typename T>
class SolverT : public SolverBase {
public:
    Level<T> lev[4];                      // levels 1..ng (ng <= 3)
    DevBuf st_mem, scratch_mem;
    PhysW<T> PC{};                        // physical constants in the working precision
    NonDim nd_ref{};                      // reference scales of the batch (shared gas and inlet options)
    bool reuse = false;                   // the cases start from a restart file (config "use previous solution")
    bool any_mass = false;                // some case imposes its mass flow through the back pressure
    SolveState *st_d = nullptr;
    int *bad_list = nullptr, *bad_count = nullptr;
    const int bad_cap = 4096;
    double *norm_part = nullptr;
    double *init_q = nullptr;             // uniform start: five conserved values per slot
    const int norm_blk = 304;            // two blocks per SM: the FP64 divisions spread over all SMs
    T *dtmin = nullptr;
    cudaGraphExec_t graphs[3] = {nullptr, nullptr, nullptr};
    int phase_runs[3] = {0, 0, 0};        // iterations run in each driver phase (graphs: see iterate)

    // ---- stage profiler
    struct ProfRec { std::string stage; cudaEvent_t a, b; int launches, level; };
    bool profiling = false;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    std::vector<ProfRec> prof;
    std::vector<std::pair<std::string, cudaEvent_t>> open_marks;
    cudaEvent_t next_event()
    {
        if (ev_used == ev_pool.size()) {
            cudaEvent_t e;
            CK(cudaEventCreate(&e));
            ev_pool.push_back(e);
        }
        return ev_pool[ev_used++];
    }
    static void hook_fn(void *user, const char *stage, int begin, int launches, int level)
    {
        SolverT *self = (SolverT *)user;
        cudaEvent_t e = self->next_event();
        CK(cudaEventRecord(e, self->stream));
        if (begin) self->open_marks.push_back({stage, e});
        else {
            for (size_t q = self->open_marks.size(); q-- > 0;)
                if (self->open_marks[q].first == stage) {
                    self->prof.push_back({stage, self->open_marks[q].second, e, launches, level});
                    self->open_marks.erase(self->open_marks.begin() + q);
                    break;
                }
        }
    }
    void profile_begin() override
    {
        CK(cudaStreamSynchronize(stream));
        profiling = true;
        ev_used = 0;
        prof.clear();
        open_marks.clear();
    }
    std::string profile_end() override
    {
        CK(cudaStreamSynchronize(stream));
        profiling = false;
        std::vector<std::string> order;
        std::map<std::string, std::pair<double, long long>> tot;
        // evaluations of the stage (bracketed groups of launches) on levels 1..3 (0: not level-bound)
        std::map<std::string, std::array<long long, 4>> per_level;
        for (auto &r : prof) {
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, r.a, r.b));
            if (!tot.count(r.stage)) { order.push_back(r.stage); per_level[r.stage] = {0, 0, 0, 0}; }
            tot[r.stage].first += ms;
            tot[r.stage].second += r.launches;
            per_level[r.stage][(r.level >= 0 && r.level <= 3) ? r.level : 0] += 1;
        }
        std::string out;
        char buf[320];
        for (auto &n : order) {
            const auto &pl = per_level[n];
            snprintf(buf, sizeof buf, "%s:%.6f:%lld:%lld,%lld,%lld;", n.c_str(), tot[n].first, tot[n].second, pl[1], pl[2],
                     pl[3]);
            out += buf;
        }
        return out;
    }
    struct Mark {
        const SolverT *s; const char *n; int l;
        Mark(const SolverT *s_, const char *n_, int l_ = 1) : s(s_), n(n_), l(l_) { if (s->profiling) hook_fn((void *)s, n, 1, l, 0); }
        ~Mark() { if (s->profiling) hook_fn((void *)s, n, 0, l, 0); }
    };

    Batch batch(int l) const
    {
        Batch B;
        B.lv = lev[l].lv_d; B.sc = lev[l].sc_d; B.st = st_d; B.nsolve = nsolve;
        return B;
    }
    LaunchCtx ctx(int l) const
    {
        LaunchCtx c = lev[l].ctx(batch(l), stream);
        if (profiling) { c.hook = &SolverT::hook_fn; c.hook_user = (void *)this; }
        c.level = l;
        return c;
    }

    PhaseTimer timer;
    explicit SolverT(const std::vector<std::string> &dirs, int prec, int max_levels)
    {
        precision = prec;
        ncase = (int)dirs.size();
        if (ncase < 1) throw std::runtime_error("no case directories given");
        // the case files of a batch are parsed in parallel host threads (text grids of large
        // batches run to gigabytes)
        {
            std::vector<std::vector<CaseSpec>> per_case(ncase);
            std::vector<std::exception_ptr> errs(ncase);
            std::atomic<int> next{0};
            const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
            const unsigned nt = std::min<unsigned>((unsigned)ncase, hw);
            const int per = (int)std::max(1u, std::min(16u, hw / nt));     // parse threads of each case's grid
            std::vector<std::thread> pool;
            for (unsigned t = 0; t < nt; t++)
                pool.emplace_back([&] {
                    for (int i = next++; i < ncase; i = next++) {
                        try { per_case[i] = read_case(dirs[i], per); } catch (...) { errs[i] = std::current_exception(); }
                    }
                });
            for (auto &t : pool) t.join();
            for (auto &e : errs) if (e) std::rethrow_exception(e);
            // one slot per block, the blocks of a case consecutive
            for (int c = 0; c < ncase; c++) {
                case_first.push_back((int)cases.size());
                case_nblk.push_back((int)per_case[c].size());
                for (auto &b : per_case[c]) cases.push_back(std::move(b));
            }
        }
        nsolve = (int)cases.size();
        timer.mark("read case files", nullptr);
        const CaseSpec &c0 = cases[0];
        for (auto &c : cases) {
            if (c.ng != c0.ng || c.coarse_iter != c0.coarse_iter || c.scheme != c0.scheme || c.recon != c0.recon ||
                c.recon_var != c0.recon_var || c.turb != c0.turb || c.equation_ns != c0.equation_ns ||
                c.limiter != c0.limiter || c.global_dt != c0.global_dt || c.Gamma != c0.Gamma || c.Rgas != c0.Rgas ||
                c.k2 != c0.k2 || c.k4 != c0.k4 ||
                c.restart != c0.restart ||
                c.Pr_lam != c0.Pr_lam || c.Pr_tur != c0.Pr_tur || c.Ptin != c0.Ptin || c.Ttin != c0.Ttin ||
                c.Len_ref != c0.Len_ref || c.relax != c0.relax || c.C_timestep != c0.C_timestep ||
                std::memcmp(c.inlet_dir, c0.inlet_dir, sizeof c.inlet_dir) != 0)
                throw std::runtime_error("the cases of one batch must share numerics, gas and inlet options (only grid, back pressure, speed and blade count may differ)");
        }
        ng = c0.ng;
        if (max_levels == 3 && ng == 2) {
            // the three-level V-cycle extension (the reference stops at two levels)
            for (auto &c : cases)
                if (!coarsens_twice(c))
                    throw std::runtime_error("three grid levels need node counts N with (N-1) a multiple of 4 and "
                                             "(N-1)/4 > 2 and patch ranges that stay odd-aligned on the second level");
            ng = 3;
        } else if (max_levels != 2) {
            if (max_levels != 3) throw std::runtime_error("grid levels must be 2 (the reference's maximum) or 3");
            throw std::runtime_error("three grid levels need a multigrid case (config \"use multigrid\" Y)");
        }
        coarse_iter = c0.coarse_iter;
        reuse = c0.restart;
        for (auto &c : cases) any_mass = any_mass || c.mass_imposed;
        NonDim nd0 = nondimensionalise(c0);
        nd_ref = nd0;
        P.gamma = c0.Gamma; P.rgas = nd0.rgas; P.pr_lam = c0.Pr_lam; P.pr_tur = c0.Pr_tur; P.re_ref = nd0.re_ref;
        P.ptin = nd0.ptin; P.ttin = nd0.ttin; P.dens_ref = nd0.dens_ref; P.vel_ref = nd0.vel_ref; P.temp_ref = nd0.temp_ref;
        for (int d = 0; d < 3; d++) P.inlet_dir[d] = c0.inlet_dir[d];
        P.inlet_vnm = std::sqrt(c0.inlet_dir[0] * c0.inlet_dir[0] + c0.inlet_dir[1] * c0.inlet_dir[1] + c0.inlet_dir[2] * c0.inlet_dir[2]);
        P.c_timestep = c0.C_timestep; P.relax = c0.relax;
        P.suth_c1 = (double)(1.0f + 110.4f / 288.15f);
        P.suth_c2 = (double)(110.4f / 288.15f);
        P.equation_ns = c0.equation_ns; P.turb_bl = c0.turb == 100; P.recon_var = c0.recon_var; P.recon = c0.recon;
        P.scheme = c0.scheme; P.limiter = c0.limiter; P.global_dt = c0.global_dt;
        P.k2 = c0.k2; P.k4 = c0.k4;
        P.turb_sa = c0.turb == 200;
        P.ev_ratio = c0.ev_ratio;
        // dummy layers: three for no reconstruction and for JST (source/UserInput.cpp:131-163)
        P.ndummy = (c0.recon == 0 || c0.scheme == 100) ? 3 : 2;
        PC = phys_working<T>(P);

        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        // per-solve state
        st_mem.bytes = sizeof(SolveState) * nsolve;
        CK(cudaMalloc(&st_mem.p, st_mem.bytes));
        st_d = (SolveState *)st_mem.p;
        std::vector<SolveState> st(nsolve);
        for (int s = 0; s < nsolve; s++) {
            std::memset(&st[s], 0, sizeof(SolveState));
            st[s].cfl = cases[s].CFL;
            st[s].cfl_res = (double)1.0E-3f;
            st[s].pout = nondimensionalise(cases[s]).pout;
        }
        CK(cudaMemcpy(st_d, st.data(), st_mem.bytes, cudaMemcpyHostToDevice));
        // scratch: limiter lists, norm partials, global-dt minima
        size_t sb = sizeof(int) * (size_t)nsolve * (bad_cap + 1) + sizeof(double) * (size_t)nsolve * (norm_blk + 1) * 5 +
                    sizeof(T) * nsolve + 256;
        scratch_mem.bytes = sb;
        CK(cudaMalloc(&scratch_mem.p, sb));
        char *q = (char *)scratch_mem.p;
        norm_part = (double *)q; q += sizeof(double) * (size_t)nsolve * norm_blk * 5;
        init_q = (double *)q; q += sizeof(double) * (size_t)nsolve * 5;
        bad_list = (int *)q; q += sizeof(int) * (size_t)nsolve * bad_cap;
        bad_count = (int *)q; q += sizeof(int) * nsolve;
        dtmin = (T *)(((uintptr_t)q + 15) & ~(uintptr_t)15);
        timer.mark("solve state and scratch", stream);
        for (int l = 1; l <= ng; l++) build_level(l);
    }

    ~SolverT() override
    {
        for (auto &g : graphs) if (g) cudaGraphExecDestroy(g);
        for (auto &e : ev_pool) cudaEventDestroy(e);
        if (stream) { cudaStreamSynchronize(stream); cudaStreamDestroy(stream); }
    }

    void build_level(int l)
    {
        Level<T> &Lv = lev[l];
        Lv.id = l;
        std::vector<LevelCase> lc;
        long long base = 0;
        for (int s = 0; s < nsolve; s++) {
            lc.push_back(level_case(cases[s], l));
            const LevelCase &c = lc.back();
            Lvl v;
            v.IM = c.IM; v.JM = c.JM; v.KM = c.KM;
            v.NJ = c.JM + 1 + 2 * PAD; v.NK = c.KM + 1 + 2 * PAD;
            v.base = base;
            base += box_size(c.IM, c.JM, c.KM);
            Lv.lv.push_back(v);
            NonDim nd = nondimensionalise(cases[s]);
            SolveConst sc;
            sc.w_rot = nd.w_rot; sc.delta_th = nd.delta_th; sc.pout = nd.pout; sc.nblade = cases[s].nblade;
            sc.m_imposed = cases[s].m_imposed; sc.relax_press = cases[s].relax_press; sc.resc_mass_imp = cases[s].resc_mass_imp;
            sc.iter_mass_imp = cases[s].iter_mass_imp; sc.mass_imposed = cases[s].mass_imposed ? 1 : 0;
            sc.lead = s - (cases[s].block - 1);
            sc.nblk = cases[s].nblock;
            sc.cix = (int)(std::upper_bound(case_first.begin(), case_first.end(), s) - case_first.begin()) - 1;
            Lv.sc.push_back(sc);
            Lv.maxIM = std::max(Lv.maxIM, c.IM); Lv.maxJM = std::max(Lv.maxJM, c.JM); Lv.maxKM = std::max(Lv.maxKM, c.KM);
            Lv.max_plane = std::max(Lv.max_plane, c.IM + c.JM + c.KM - 3);
        }
        Lv.pool_n = base;
        // the face kernels index a level's pools with 32-bit offsets
        if (base >= (long long)INT32_MAX) throw std::runtime_error("batch too large: a level's pool exceeds 2^31 cells");
        const size_t N = (size_t)base;
        timer.mark("level boxes", nullptr);
        // device descriptors
        CK(cudaMalloc(&Lv.meta_mem.p, sizeof(Lvl) * nsolve + sizeof(SolveConst) * nsolve + 16));
        Lv.lv_d = (Lvl *)Lv.meta_mem.p;
        Lv.sc_d = (SolveConst *)((char *)Lv.meta_mem.p + ((sizeof(Lvl) * nsolve + 15) & ~(size_t)15));
        CK(cudaMemcpy(Lv.lv_d, Lv.lv.data(), sizeof(Lvl) * nsolve, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(Lv.sc_d, Lv.sc.data(), sizeof(SolveConst) * nsolve, cudaMemcpyHostToDevice));
        // geometry pools (FP64)
        const int NGEO = 124;
        Lv.geo_mem.bytes = sizeof(double) * N * NGEO + sizeof(double) * 2 * nsolve;
        CK(cudaMalloc(&Lv.geo_mem.p, Lv.geo_mem.bytes));
        CK(cudaMemset(Lv.geo_mem.p, 0, Lv.geo_mem.bytes));
        double *g = (double *)Lv.geo_mem.p;
        auto take = [&]() { double *r = g; g += N; return r; };
        Geo &G = Lv.G;
        G.x = take(); G.y = take(); G.z = take();
        for (int f = 0; f < 3; f++) {
            for (int c = 0; c < 3; c++) { G.S[f][c] = take(); G.c[f][c] = take(); G.nrm[f][c] = take(); G.t1[f][c] = take(); G.t2[f][c] = take(); }
            G.s[f] = take(); G.r[f] = take(); G.th[f] = take(); G.qe[f] = take();
            for (int c = 0; c < 9; c++) G.m[f][c] = take();
            for (int c = 0; c < 3; c++) { G.sb[f][c] = take(); G.cn[f][c] = take(); }
            G.cs[f] = take(); G.cve[f] = take();
        }
        G.vol = take();
        for (int c = 0; c < 3; c++) G.cc[c] = take();
        for (int c = 0; c < 9; c++) G.cm[c] = take();
        Lv.blockvol = g;                   // per slot: the block's volume
        Lv.totalvol = g + nsolve;          // per slot: the volume of its whole case (CMesh::TotalVol)
        // flow pools
        Lv.flow_d_mem.bytes = sizeof(double) * N * 15;
        CK(cudaMalloc(&Lv.flow_d_mem.p, Lv.flow_d_mem.bytes));
        CK(cudaMemset(Lv.flow_d_mem.p, 0, Lv.flow_d_mem.bytes));
        double *d = (double *)Lv.flow_d_mem.p;
        Flow<T> &W = Lv.W;
        for (int c = 0; c < NQ; c++) { W.cv[c] = d; d += N; W.cvold[c] = d; d += N; W.cv2h[c] = d; d += N; }
        Lv.flow_t_mem.bytes = sizeof(T) * N * 66;
        CK(cudaMalloc(&Lv.flow_t_mem.p, Lv.flow_t_mem.bytes));
        CK(cudaMemset(Lv.flow_t_mem.p, 0, Lv.flow_t_mem.bytes));
        T *t = (T *)Lv.flow_t_mem.p;
        auto tk = [&]() { T *r = t; t += N; return r; };
        for (int c = 0; c < NPV; c++) W.pv[c] = tk();
        W.mut = tk(); W.omega = tk(); W.dt = tk(); W.mul = tk();
        for (int f = 0; f < 3; f++) { W.lamc[f] = tk(); W.lamv[f] = tk(); for (int c = 0; c < NQ; c++) { W.Ff[f][c] = tk(); W.Vf[f][c] = tk(); } }
        for (int c = 0; c < NQ; c++) { W.res[c] = tk(); W.dq[c] = tk(); W.res2h[c] = tk(); W.dq2h[c] = tk(); }
        if (P.turb_sa && l == 1) {
            // Spalart-Allmaras variable, its copy, residual, update, face fluxes and wall distance
            Lv.sa_mem.bytes = sizeof(double) * N * 3 + sizeof(T) * N * 11;
            CK(cudaMalloc(&Lv.sa_mem.p, Lv.sa_mem.bytes));
            CK(cudaMemset(Lv.sa_mem.p, 0, Lv.sa_mem.bytes));
            double *sd = (double *)Lv.sa_mem.p;
            W.ev = sd; W.evg = sd + N; W.dwall = sd + 2 * N;
            T *st = (T *)(sd + 3 * N);
            W.res_ev = st; W.dq_ev = st + N;
            for (int f = 0; f < 3; f++) { W.Fct[f] = st + (2 + f) * N; W.Fvt[f] = st + (5 + f) * N; W.Fv1t[f] = st + (8 + f) * N; }
        }
        if (P.scheme == 100) {
            // face dissipation of JST (source/SpaceDiscr.cpp:611-640)
            Lv.fd_mem.bytes = sizeof(T) * N * 21;
            CK(cudaMalloc(&Lv.fd_mem.p, Lv.fd_mem.bytes));
            CK(cudaMemset(Lv.fd_mem.p, 0, Lv.fd_mem.bytes));
            T *fd = (T *)Lv.fd_mem.p;
            for (int f = 0; f < 3; f++) for (int c = 0; c < NQ; c++) { W.Fd[f][c] = fd; fd += N; }
            for (int f = 0; f < 3; f++) { W.jsens[f] = fd; fd += N; W.jva[f] = fd; fd += N; }
        } else {
            for (int f = 0; f < 3; f++) for (int c = 0; c < NQ; c++) W.Fd[f][c] = nullptr;
        }
        Lv.int_mem.bytes = sizeof(unsigned long long) * N + sizeof(int) * N * 3;
        CK(cudaMalloc(&Lv.int_mem.p, Lv.int_mem.bytes));
        CK(cudaMemset(Lv.int_mem.p, 0, Lv.int_mem.bytes));
        W.blmin = (unsigned long long *)Lv.int_mem.p;
        int *ip = (int *)(W.blmin + N);
        int *wallf[3] = {ip, ip + N, ip + 2 * N};
        for (int f = 0; f < 3; f++) W.wallf[f] = wallf[f];
        // nodes
        {
            std::vector<double> hx(N, 0.0), hy(N, 0.0), hz(N, 0.0);
            for (int s = 0; s < nsolve; s++) {
                const LevelCase &c = lc[s];
                const Lvl &v = Lv.lv[s];
                for (int k = 1; k <= c.KM; k++)
                    for (int j = 1; j <= c.JM; j++)
                        for (int i = 1; i <= c.IM; i++) {
                            size_t q = ((size_t)(k - 1) * c.JM + (j - 1)) * c.IM + (i - 1);
                            long long p = ix(v, i, j, k);
                            hx[p] = c.x[q]; hy[p] = c.y[q]; hz[p] = c.z[q];
                        }
            }
            CK(cudaMemcpy(G.x, hx.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
            CK(cudaMemcpy(G.y, hy.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
            CK(cudaMemcpy(G.z, hz.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
            build_tables(l, lc, hx, hy);
        }
        timer.mark("pools, nodes, patch tables", stream);
        build_planes(l);
        timer.mark("hyperplane tables", stream);
        launch_geometry(ctx(l), G, Lv.blockvol);
        k_case_volume<<<(nsolve + 127) / 128, 128, 0, stream>>>(batch(l), Lv.blockvol, Lv.totalvol);
        if (Lv.W.ev) build_sa_wall_distance(l);
        timer.mark("geometry", stream);
        build_geometry_working(l);
        build_wall_distances(l);
        launch_sweep_geometry<T>(ctx(l), G, Lv.planes, Lv.sweep);
        timer.mark("working geometry, wall lines", stream);
        {
            // block shape of the sweep kernels: GBTURBO_SWEEP_SHAPE="cpw,wpb" pins it; batches of
            // four or more solves time the candidates; smaller ones, where the candidates are within
            // run-to-run noise of each other, take ten cells per one-warp block
            int cpw = 10, wpb = 1;
            const char *pin = std::getenv("GBTURBO_SWEEP_SHAPE");
            if (pin && std::sscanf(pin, "%d,%d", &cpw, &wpb) == 2 && sweep_shape_known(cpw, wpb)) {
            } else if (nsolve >= 4) {
                const int v = tune_sweep_cpw<T>(ctx(l), PC, Lv.planes, Lv.sweep);
                cpw = v / 16;
                wpb = v % 16;
            } else {
                cpw = 10;
                wpb = 1;
            }
            Lv.planes.cpw = cpw;
            Lv.planes.wpb = wpb;
        }
        CK(cudaStreamSynchronize(stream));
        timer.mark("sweep shape", stream);
        CK(cudaGetLastError());
    }

    // Spalart-Allmaras wall distances (CMesh::WallDistanceSA, source/WallDistanceSA.cpp:6-160): every
    // wall face of every block of a case, once
    void build_sa_wall_distance(int l)
    {
        Level<T> &Lv = lev[l];
        std::vector<long long> fp, off(1, 0);
        std::vector<int> ff;
        for (int c = 0; c < ncase; c++) {
            for (int b = 0; b < case_nblk[c]; b++) {
                const int s = case_first[c] + b;
                const Lvl &v = Lv.lv[s];
                for (const WallIO &w : cases[s].walls) {
                    const int f = (w.face - 1) / 2;
                    const bool hi = w.face % 2 == 0;
                    int i0 = w.is, i1 = w.ie, j0 = w.js, j1 = w.je, k0 = w.ks, k1 = w.ke;
                    if (f == 0) i0 = i1 = hi ? v.IM : 1;
                    if (f == 1) j0 = j1 = hi ? v.JM : 1;
                    if (f == 2) k0 = k1 = hi ? v.KM : 1;
                    for (int i = i0; i <= i1; i++)
                        for (int j = j0; j <= j1; j++)
                            for (int k = k0; k <= k1; k++) { fp.push_back(ix(v, i, j, k)); ff.push_back(f); }
                }
            }
            off.push_back((long long)fp.size());
        }
        const long long n = (long long)fp.size();
        auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
        Lv.sa_tab_mem.bytes = al(sizeof(long long) * n) + al(sizeof(int) * n) + al(sizeof(long long) * off.size()) + al(sizeof(double) * 3 * n) + 256;
        CK(cudaMalloc(&Lv.sa_tab_mem.p, Lv.sa_tab_mem.bytes));
        char *q = (char *)Lv.sa_tab_mem.p;
        long long *dp = (long long *)q; q += al(sizeof(long long) * n);
        int *df = (int *)q; q += al(sizeof(int) * n);
        long long *doff = (long long *)q; q += al(sizeof(long long) * off.size());
        double *xyz = (double *)q;
        if (n) {
            CK(cudaMemcpy(dp, fp.data(), sizeof(long long) * n, cudaMemcpyHostToDevice));
            CK(cudaMemcpy(df, ff.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
        }
        CK(cudaMemcpy(doff, off.data(), sizeof(long long) * off.size(), cudaMemcpyHostToDevice));
        launch_sa_wall_distance(ctx(l), Lv.G, dp, df, n, xyz, doff, Lv.W.dwall);
        CK(cudaStreamSynchronize(stream));
    }

    // Baldwin-Lomax wall distances of the fine level (constant geometry, computed once)
    void build_wall_distances(int l)
    {
        Level<T> &Lv = lev[l];
        BcTables &bc = Lv.bc;
        if (l != 1 || !P.turb_bl || bc.n_wall == 0) return;
        std::vector<long long> off(bc.n_wall);
        long long tot = 0;
        for (int w = 0; w < bc.n_wall; w++) {
            const DevWall &wl = Lv.walls_h[w];
            const Lvl &v = Lv.lv[wl.solve];
            const int dirn = (wl.face - 1) / 2;
            const long long lines = (long long)(wl.ie - wl.is + 1) * (wl.je - wl.js + 1) * (wl.ke - wl.ks + 1);
            const int N = dirn == 0 ? v.IM : (dirn == 1 ? v.JM : v.KM);
            off[w] = tot;
            tot += lines * (N - 1);
        }
        const size_t ob = (sizeof(long long) * off.size() + 255) & ~(size_t)255;
        Lv.wdist_mem.bytes = ob + sizeof(T) * (size_t)tot;
        CK(cudaMalloc(&Lv.wdist_mem.p, Lv.wdist_mem.bytes));
        CK(cudaMemcpy(Lv.wdist_mem.p, off.data(), sizeof(long long) * off.size(), cudaMemcpyHostToDevice));
        bc.wall_dist_off = (const long long *)Lv.wdist_mem.p;
        bc.wall_dist = (char *)Lv.wdist_mem.p + ob;
        launch_wall_distances<T>(ctx(l), Lv.G, bc);
    }

    // geometry in the working precision: aliases of the FP64 arrays in the FP64 form, FP32 copies
    // (made on the device, once) in the mixed form
    void build_geometry_working(int l)
    {
        Level<T> &Lv = lev[l];
        const Geo &G = Lv.G;
        GeoW<T> &W = Lv.GW;
        if constexpr (sizeof(T) == 8) {
            for (int f = 0; f < 3; f++) {
                for (int c = 0; c < 3; c++) {
                    W.S[f][c] = G.S[f][c]; W.nrm[f][c] = G.nrm[f][c]; W.t1[f][c] = G.t1[f][c]; W.t2[f][c] = G.t2[f][c];
                    W.sb[f][c] = G.sb[f][c];
                }
                for (int c = 0; c < 2; c++) W.c[f][c] = G.c[f][c];
                W.s[f] = G.s[f];
                W.qe[f] = G.qe[f];
                for (int c = 0; c < 9; c++) W.m[f][c] = G.m[f][c];
            }
            W.vol = G.vol;
            for (int c = 0; c < 2; c++) W.cc[c] = G.cc[c];
            for (int c = 0; c < 9; c++) W.cm[c] = G.cm[c];
        } else {
            const long long N = Lv.pool_n;
            const int NW = 3 * (5 * 3 + 2 + 1 + 1 + 9) + 1 + 2 + 9;
            Lv.geow_mem.bytes = sizeof(T) * (size_t)N * NW;
            CK(cudaMalloc(&Lv.geow_mem.p, Lv.geow_mem.bytes));
            T *g = (T *)Lv.geow_mem.p;
            auto take = [&]() { T *r = g; g += N; return r; };
            for (int f = 0; f < 3; f++) {
                for (int c = 0; c < 3; c++) {
                    W.S[f][c] = take(); W.nrm[f][c] = take(); W.t1[f][c] = take(); W.t2[f][c] = take(); W.sb[f][c] = take();
                }
                for (int c = 0; c < 2; c++) W.c[f][c] = take();
                W.s[f] = take();
                W.qe[f] = take();
                for (int c = 0; c < 9; c++) W.m[f][c] = take();
            }
            W.vol = take();
            for (int c = 0; c < 2; c++) W.cc[c] = take();
            for (int c = 0; c < 9; c++) W.cm[c] = take();
            launch_geometry_working(ctx(l), G, W);
            if constexpr (sizeof(T) == 4) {
                // the face stage's tiles staged by TMA where every box row is 16-byte aligned
                if (face_tma_eligible(Lv.lv)) Lv.tma_mem.p = build_face_tma(Lv.lv, W, Lv.W, &Lv.tma_mem.bytes, Lv.tma_host);
            }
        }
    }

    // cells of the LU-SGS hyperplanes (source/LU_SGS_Marching.cpp:62-74) in plane order, with the
    // plane-order neighbour tables and the plane-order copies of the sweep's inputs
    void build_planes(int l)
    {
        Level<T> &Lv = lev[l];
        PlaneTables &pt = Lv.planes;
        pt.max_plane = Lv.max_plane;
        pt.stride = Lv.max_plane + 2;
        pt.max_count.assign(pt.stride, 0);
        std::vector<long long> cell;
        std::vector<int> start((size_t)nsolve * pt.stride + 1, 0);
        std::vector<int> nbq[2][3];
        std::vector<int> rq;                       // row starts of the transpositions (PlaneTables::rq)
        std::vector<long long> rq_off(nsolve);
        for (int s = 0; s < nsolve; s++) {
            const Lvl &v = Lv.lv[s];
            const int nI = v.IM - 1, nJ = v.JM - 1, nK = v.KM - 1;
            rq_off[s] = (long long)rq.size();
            rq.resize(rq.size() + (size_t)pt.stride * nI, 0);
            // q of interior cell (i,j,k) of this solve
            std::vector<int> qof((size_t)nI * nJ * nK, -1);
            auto at = [&](int i, int j, int k) -> int & { return qof[((size_t)(i - 1) * nJ + (j - 1)) * nK + (k - 1)]; };
            for (int pl = 0; pl < pt.stride; pl++) {
                start[(size_t)s * pt.stride + pl] = (int)cell.size();
                int c = 0;
                if (pl >= 3)
                    for (int i = 1; i <= nI; i++) {
                        bool first = true;
                        for (int j = 1; j <= nJ; j++) {
                            const int k = pl - i - j;
                            if (k < 1 || k > nK) continue;
                            if (first) { rq[(size_t)rq_off[s] + (size_t)pl * nI + (i - 1)] = (int)cell.size() - j; first = false; }
                            at(i, j, k) = (int)cell.size();
                            cell.push_back(ix(v, i, j, k));
                            c++;
                        }
                    }
                pt.max_count[pl] = std::max(pt.max_count[pl], c);
            }
            if (cell.size() > (size_t)0x7fffffff) throw std::runtime_error("batch too large for the plane tables");
            for (int dir = 0; dir < 2; dir++)
                for (int d = 0; d < 3; d++) nbq[dir][d].resize(cell.size(), -1);
            for (int i = 1; i <= nI; i++)
                for (int j = 1; j <= nJ; j++)
                    for (int k = 1; k <= nK; k++) {
                        const int q = at(i, j, k);
                        if (i > 1) nbq[0][0][q] = at(i - 1, j, k);
                        if (j > 1) nbq[0][1][q] = at(i, j - 1, k);
                        if (k > 1) nbq[0][2][q] = at(i, j, k - 1);
                        if (i < nI) nbq[1][0][q] = at(i + 1, j, k);
                        if (j < nJ) nbq[1][1][q] = at(i, j + 1, k);
                        if (k < nK) nbq[1][2][q] = at(i, j, k + 1);
                    }
        }
        start[(size_t)nsolve * pt.stride] = (int)cell.size();
        // start[s*stride + pl + 1] must be the end of plane pl: the last slot of each solve row
        // (pl = stride-1) is empty, so the next row's first entry closes it
        const size_t nq = cell.size();
        pt.nq = (long long)nq;
        auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
        const bool sa = P.turb_sa && l == 1;
        const size_t n_t = 16 + 18 + NQ + (sa ? 19 : 0);   // geometry, flow inputs, dQ (and the SA sweep's)
        Lv.plane_mem.bytes = al(sizeof(int) * start.size()) + al(sizeof(long long) * nq) + 6 * al(sizeof(int) * nq) +
                             al(sizeof(int) * rq.size()) + al(sizeof(long long) * rq_off.size()) + n_t * al(sizeof(T) * nq) + 256;
        CK(cudaMalloc(&Lv.plane_mem.p, Lv.plane_mem.bytes));
        char *q = (char *)Lv.plane_mem.p;
        auto take = [&](size_t b) { char *r = q; q += al(b); return r; };
        int *dstart = (int *)take(sizeof(int) * start.size());
        CK(cudaMemcpy(dstart, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice));
        pt.start = dstart;
        int *drq = (int *)take(sizeof(int) * rq.size());
        CK(cudaMemcpy(drq, rq.data(), sizeof(int) * rq.size(), cudaMemcpyHostToDevice));
        long long *drq_off = (long long *)take(sizeof(long long) * rq_off.size());
        CK(cudaMemcpy(drq_off, rq_off.data(), sizeof(long long) * rq_off.size(), cudaMemcpyHostToDevice));
        pt.rq = drq;
        pt.rq_off = drq_off;
        SweepData<T> &S = Lv.sweep;
        long long *dcell = (long long *)take(sizeof(long long) * nq);
        CK(cudaMemcpy(dcell, cell.data(), sizeof(long long) * nq, cudaMemcpyHostToDevice));
        S.cell = dcell;
        for (int dir = 0; dir < 2; dir++)
            for (int d = 0; d < 3; d++) {
                int *t = (int *)take(sizeof(int) * nq);
                CK(cudaMemcpy(t, nbq[dir][d].data(), sizeof(int) * nq, cudaMemcpyHostToDevice));
                S.nb[dir][d] = t;
            }
        auto arr = [&]() { return (T *)take(sizeof(T) * nq); };
        for (int d = 0; d < 3; d++) {
            for (int c = 0; c < 3; c++) S.gn[d][c] = arr();
            S.gs[d] = arr();
            S.gve[d] = arr();
        }
        S.gvol = arr();
        for (int c = 0; c < NQ; c++) S.cv[c] = arr();
        S.pp = arr();
        for (int d = 0; d < 3; d++) { S.lamc[d] = arr(); S.lamv[d] = arr(); }
        S.dt = arr();
        for (int c = 0; c < NQ; c++) S.res[c] = arr();
        for (int c = 0; c < NQ; c++) S.dq[c] = arr();
        if (sa) {
            for (int d = 0; d < 3; d++) { S.sa_vn[d] = arr(); S.sa_eb[d] = arr(); S.sa_s[d] = arr(); S.sa_rl[d] = arr(); S.sa_lv[d] = arr(); }
            S.sa_ev0 = arr(); S.sa_alpha = arr(); S.sa_res = arr(); S.sa_dq = arr();
        }
    }

    void build_tables(int l, const std::vector<LevelCase> &lc, const std::vector<double> &hx, const std::vector<double> &hy)
    {
        Level<T> &Lv = lev[l];
        BcTables &bc = Lv.bc;
        std::vector<DevInOut> inl, outl, inl1, outl1;
        std::vector<DevWall> walls;
        std::vector<long long> pdst, psrc, sa_dst_h, sa_src_h;
        std::vector<int> pmeta;
        std::vector<int> wallf[3];
        for (int f = 0; f < 3; f++) wallf[f].assign((size_t)Lv.pool_n, 0);
        size_t max_walls = 0;
        for (auto &c : lc) max_walls = std::max(max_walls, c.walls.size());
        if (max_walls > 64) throw std::runtime_error("at most 64 wall patches per case");
        for (int s = 0; s < nsolve; s++) {
            const LevelCase &c = lc[s];
            for (auto &p : c.in) {
                inl.push_back({s, p.face, p.is, p.ie, p.js, p.je, p.ks, p.ke});
                bc.max_inlet = std::max(bc.max_inlet, (p.ie - p.is + 1) * (p.je - p.js + 1));
            }
            for (auto &p : c.out) outl.push_back({s, p.face, p.is, p.ie, p.js, p.je, p.ks, p.ke});
            bc.max_outlet_im = std::max(bc.max_outlet_im, c.IM);
            bc.max_outlet_jm = std::max(bc.max_outlet_jm, c.JM);
            // the sections the case reports (its Inlet[1] and Outlet[1]), on the slot of their block
            const CaseSpec &cs = cases[s];
            const int lead = s - (cs.block - 1);
            const PatchIO fi = level_patch(cs.first_inlet, l), fo = level_patch(cs.first_outlet, l);
            inl1.push_back({lead + fi.block - 1, fi.face, fi.is, fi.ie, fi.js, fi.je, fi.ks, fi.ke});
            outl1.push_back({lead + fo.block - 1, fo.face, fo.is, fo.ie, fo.js, fo.je, fo.ks, fo.ke});
        }
        for (int c = 0; c < ncase; c++) {
            int nout = 0;
            for (int b = 0; b < case_nblk[c]; b++) nout += (int)lc[case_first[c] + b].out.size();
            if (nout != 1) throw std::runtime_error("exactly one axial outlet per case is supported");
        }
        // walls ordered by their position in each case's list, then by solve
        bc.n_wall_slot = (int)max_walls;
        for (size_t q = 0; q < max_walls; q++) {
            bc.wall_slot_off[q] = (int)walls.size();
            int lines = 0;
            for (int s = 0; s < nsolve; s++) {
                if (q >= lc[s].walls.size()) continue;
                const WallIO &w = lc[s].walls[q];
                walls.push_back({s, w.face, w.rotate, w.is, w.ie, w.js, w.je, w.ks, w.ke});
                int nf = (w.ie - w.is + 1) * (w.je - w.js + 1) * (w.ke - w.ks + 1);
                bc.max_wall = std::max(bc.max_wall, nf);
                lines = std::max(lines, nf);
            }
            bc.wall_slot_lines[q] = lines;
        }
        bc.wall_slot_off[max_walls] = (int)walls.size();
        // per-face wall marks in patch order (a later patch overwrites an earlier one's face)
        for (int s = 0; s < nsolve; s++) {
            for (size_t q = 0; q < lc[s].walls.size(); q++) {
                int rec = -1;
                for (int r = bc.wall_slot_off[q]; r < bc.wall_slot_off[q + 1]; r++)
                    if (walls[r].solve == s) rec = r;
                const WallIO &w = lc[s].walls[q];
                int f = (w.face - 1) / 2;
                for (int i = w.is; i <= w.ie; i++)
                    for (int j = w.js; j <= w.je; j++)
                        for (int k = w.ks; k <= w.ke; k++) wallf[f][ix(Lv.lv[s], i, j, k)] = rec + 1;
            }
        }
        // ghost exchange of block interfaces and periodic pairs as one gather list, in the
        // reference's order (all interfaces, then all periodic pairs, each in file order;
        // source/BoundaryCondition.cpp:46-58); the last writer of a cell wins, as in the reference's
        // sequential copies
        for (int cix = 0; cix < ncase; cix++) {
            const int s0 = case_first[cix];
            const CaseSpec &cs = cases[s0];
            std::map<long long, size_t> last, last_sa;
            std::vector<std::pair<PeriodicIO, bool>> pairs;
            for (auto &p : cs.interiors) pairs.push_back({level_pair(p, l), false});
            for (auto &p : cs.periodics) pairs.push_back({level_pair(p, l), true});
            for (auto &pp : pairs) {
                const PeriodicIO &pr = pp.first;
                const bool rotate = pp.second;
                const int sa = s0 + pr.b1 - 1, sb = s0 + pr.b2 - 1;
                const Lvl &va = Lv.lv[sa], &vb = Lv.lv[sb];
                const LevelCase &ca = lc[sa], &cb = lc[sb];
                if (rotate) {
                    long long pa = ix(va, pr.r1[0], pr.r1[2], pr.r1[4]), pb = ix(vb, pr.r2[0], pr.r2[2], pr.r2[4]);
                    double th1 = std::atan(hy[pa] / hx[pa]), th2 = std::atan(hy[pb] / hx[pb]);
                    if ((th2 - th1) < 0.0)
                        throw std::runtime_error("periodic pair listed against the pitch direction (the reference flips the pitch sign on every call then); list the lower-theta face first");
                }
                for (int nd = 1; nd <= P.ndummy; nd++) {
                    for (int dir = 0; dir < 2; dir++) {
                        // side 1 -> side 2 rotated by +delta_th of block 1, then side 2 -> side 1 by
                        // -delta_th; an interface copies without rotation
                        const int *ra = dir == 0 ? pr.r1 : pr.r2, *rb = dir == 0 ? pr.r2 : pr.r1;
                        int fa = dir == 0 ? pr.f1 : pr.f2, fb = dir == 0 ? pr.f2 : pr.f1;
                        const Lvl &vs = dir == 0 ? va : vb, &vd = dir == 0 ? vb : va;
                        const LevelCase &cS = dir == 0 ? ca : cb, &cD = dir == 0 ? cb : ca;
                        int La, Ma, Lb, Mb;
                        auto A = patch_walk(fa, nd, ra, cS.IM, cS.JM, cS.KM, La, Ma);
                        auto Bw = patch_walk(fb, nd, rb, cD.IM, cD.JM, cD.KM, Lb, Mb);
                        std::map<std::pair<int, int>, long long> src;
                        for (auto &e : A) {
                            int l2, m2;
                            trans(pr.orient, e.l, e.m, La, Ma, l2, m2);
                            src[{l2, m2}] = ix(vs, e.ri, e.rj, e.rk);
                        }
                        const int sign = rotate ? (dir == 0 ? 1 : -1) : 0;
                        for (auto &e : Bw) {
                            auto it = src.find({e.l, e.m});
                            if (it == src.end()) throw std::runtime_error(rotate ? "periodic patches of different size" : "interface patches of different size");
                            long long dsts[2] = {ix(vd, e.gi, e.gj, e.gk), -1};
                            if (nd == 1) {
                                // the first layer also fills the ghost cell next to the face
                                int gi = e.gi, gj = e.gj, gk = e.gk;
                                if (gi < 0) gi = 0; else if (gi > cD.IM) gi = cD.IM;
                                if (gj < 0) gj = 0; else if (gj > cD.JM) gj = cD.JM;
                                if (gk < 0) gk = 0; else if (gk > cD.KM) gk = cD.KM;
                                if (gi == cD.IM + 1) gi = cD.IM;
                                dsts[1] = ix(vd, gi, gj, gk);
                            }
                            for (long long dd : dsts) {
                                if (dd < 0) continue;
                                // the rotation angle is block 1's pitch
                                const int meta = sa * 4 + sign + 1;
                                auto f = last.find(dd);
                                if (f != last.end()) { psrc[f->second] = it->second; pmeta[f->second] = meta; }
                                else { last[dd] = pdst.size(); pdst.push_back(dd); psrc.push_back(it->second); pmeta.push_back(meta); }
                            }
                            if (dsts[1] >= 0) {
                                // the Spalart-Allmaras variable goes to the first ghost layer only
                                auto f = last_sa.find(dsts[1]);
                                if (f != last_sa.end()) sa_src_h[f->second] = it->second;
                                else { last_sa[dsts[1]] = sa_dst_h.size(); sa_dst_h.push_back(dsts[1]); sa_src_h.push_back(it->second); }
                            }
                        }
                    }
                }
            }
        }
        // mixing planes of every case (applied last, source/BoundaryCondition.cpp:59-62)
        std::vector<DevMix> mixes;
        for (int cix = 0; cix < ncase; cix++) {
            const int s0 = case_first[cix];
            for (auto mp : cases[s0].mixing) {
                const PeriodicIO q = level_pair(mp, l);
                DevMix m{s0 + q.b1 - 1, s0 + q.b2 - 1, q.r1[0], q.r1[1], q.r1[2], q.r1[3], q.r2[2], q.r2[3]};
                const Lvl &v1 = Lv.lv[m.s1], &v2 = Lv.lv[m.s2];
                if (m.is < 1 || m.ie > v1.IM - 1 || m.ie > v2.IM - 1 || m.js1 < 1 || m.je1 > v1.JM - 1 || m.js2 < 1 || m.je2 > v2.JM - 1)
                    throw std::runtime_error("mixing plane range outside its blocks (rows of the first block are used on both sides)");
                mixes.push_back(m);
                bc.max_mix_rows = std::max(bc.max_mix_rows, m.ie - m.is + 1);
                bc.max_mix_j = std::max(bc.max_mix_j, std::max(m.je1 - m.js1 + 1, m.je2 - m.js2 + 1));
            }
        }
        // upload everything into one table buffer
        auto bytes = [](size_t n, size_t sz) { return (n * sz + 255) & ~(size_t)255; };
        size_t tot = bytes(inl.size(), sizeof(DevInOut)) + bytes(outl.size(), sizeof(DevInOut)) + bytes(inl1.size(), sizeof(DevInOut)) +
                     bytes(outl1.size(), sizeof(DevInOut)) + bytes(walls.size(), sizeof(DevWall)) + bytes(pdst.size(), 8) * 2 +
                     bytes(pmeta.size(), 4) + bytes(outl.size() * (size_t)(bc.max_outlet_im + 1), 8) +
                     bytes((size_t)nsolve * 2 * kIntegralBlocks * 3, 8) + bytes(sa_dst_h.size(), 8) * 2 +
                     bytes(mixes.size(), sizeof(DevMix)) + bytes(mixes.size() * (size_t)bc.max_mix_rows * kMixVals, 8) +
                     bytes((size_t)nsolve * 4, 8) + 256;
        CK(cudaMalloc(&Lv.tab_mem.p, tot));
        char *q = (char *)Lv.tab_mem.p;
        auto up = [&](const void *h, size_t n, size_t sz) {
            void *dptr = q;
            if (n) CK(cudaMemcpy(dptr, h, n * sz, cudaMemcpyHostToDevice));
            q += bytes(n, sz);
            return dptr;
        };
        bc.inlet = (const DevInOut *)up(inl.data(), inl.size(), sizeof(DevInOut)); bc.n_inlet = (int)inl.size();
        bc.outlet = (const DevInOut *)up(outl.data(), outl.size(), sizeof(DevInOut)); bc.n_outlet = (int)outl.size();
        bc.inlet_first = (const DevInOut *)up(inl1.data(), inl1.size(), sizeof(DevInOut));
        bc.outlet_first = (const DevInOut *)up(outl1.data(), outl1.size(), sizeof(DevInOut));
        bc.wall = (const DevWall *)up(walls.data(), walls.size(), sizeof(DevWall)); bc.n_wall = (int)walls.size();
        bc.per_dst = (const long long *)up(pdst.data(), pdst.size(), 8);
        bc.per_src = (const long long *)up(psrc.data(), psrc.size(), 8);
        bc.per_meta = (const int *)up(pmeta.data(), pmeta.size(), 4);
        bc.n_per = (long long)pdst.size();
        bc.sa_dst = (const long long *)up(sa_dst_h.data(), sa_dst_h.size(), 8);
        bc.sa_src = (const long long *)up(sa_src_h.data(), sa_src_h.size(), 8);
        bc.n_sa_gather = (long long)sa_dst_h.size();
        bc.mix = (const DevMix *)up(mixes.data(), mixes.size(), sizeof(DevMix));
        bc.n_mix = (int)mixes.size();
        bc.mix_avg = (double *)up(nullptr, 0, 8); q += bytes(mixes.size() * (size_t)bc.max_mix_rows * kMixVals, 8);
        bc.outlet_cu = (double *)up(nullptr, 0, 8); q += bytes(outl.size() * (size_t)(bc.max_outlet_im + 1), 8);
        bc.integ_part = (double *)up(nullptr, 0, 8); q += bytes((size_t)nsolve * 2 * kIntegralBlocks * 3, 8);
        double *trig = (double *)up(nullptr, 0, 8); q += bytes((size_t)nsolve * 4, 8);
        bc.per_trig = trig;
        launch_periodic_trig(ctx(l), trig);
        for (int f = 0; f < 3; f++)
            CK(cudaMemcpy((void *)Lv.W.wallf[f], wallf[f].data(), sizeof(int) * (size_t)Lv.pool_n, cudaMemcpyHostToDevice));
        Lv.walls_h = walls;
    }

    // ---------------------------------------------------------------- reference call surface
    void init_uniform() override
    {
        // source/Initialization.cpp:34-68 (nondimensional inlet totals; FP64 like the reference),
        // with each case's initial Mach number
        const double Gamma = P.gamma, Rgas = P.rgas;
        std::vector<double> init((size_t)nsolve * 5);
        for (int s = 0; s < nsolve; s++) {
            const CaseSpec &c = cases[s];
            const double Ma0 = c.Ma0;
            const double press = P.ptin * std::pow(1.0f + (Gamma - 1.0f) / 2.0f * Ma0 * Ma0, 0.0f - Gamma / (Gamma - 1.0f));
            const double temp = P.ttin * std::pow(1.0f + (Gamma - 1.0f) / 2.0f * Ma0 * Ma0, 0.0f - 1.0f);
            const double dens = press / (Rgas * temp);
            const double Vel = std::pow(Gamma * Rgas * temp, 0.5f) * Ma0;
            const double *a = c.inlet_dir;
            const double n_m = std::pow(a[0] * a[0] + a[1] * a[1] + a[2] * a[2], 0.5);
            const double u = Vel * a[0] / n_m, v = Vel * a[1] / n_m, w = Vel * a[2] / n_m;
            const double V2 = u * u + v * v + w * w;
            const double ener = press / (dens * (Gamma - 1.0f)) + V2 / 2.0f;
            const double q[5] = {dens, dens * u, dens * v, dens * w, dens * ener};
            for (int m = 0; m < 5; m++) init[(size_t)s * 5 + m] = q[m];
        }
        int l = ng == 1 ? 1 : 2;
        LaunchCtx cx = ctx(l);
        Flow<T> &W = lev[l].W;
        CK(cudaMemcpyAsync(init_q, init.data(), sizeof(double) * init.size(), cudaMemcpyHostToDevice, stream));
        k_fill_uniform<<<cx.grid_cells(256), 256, 0, stream>>>(cx.batch, W.cv[0], W.cv[1], W.cv[2], W.cv[3], W.cv[4], init_q);
        if (W.ev) launch_sa_init(cx, W.ev, P.ev_ratio);        // Initialization.cpp:40,70-71
        launch_primitive<T>(cx, P, W);
        CK(cudaStreamSynchronize(stream));
        CK(cudaGetLastError());
    }
    void resflux(int l) override
    {
        launch_resflux<T>(ctx(l), P, PC, lev[l].G, lev[l].GW, lev[l].W, lev[l].bc, l, dtmin);
    }
    void time_marching(int l) override
    {
        LaunchCtx cx = ctx(l);
        Level<T> &Lv = lev[l];
        if (!Lv.use_force) resflux(l);
        else { Mark m(this, "mg_forcing"); launch_forcing<T>(cx, Lv.W); }
        sweep_update(l);
    }
    void sweep_update(int l)
    {
        LaunchCtx cx = ctx(l);
        Level<T> &Lv = lev[l];
        launch_lusgs_sweeps<T>(cx, PC, Lv.G, Lv.W, Lv.planes, Lv.sweep);
        launch_update<T>(cx, P, Lv.G, Lv.W, l, bad_list, bad_cap, bad_count);
    }
    // transfers between level lf and the next coarser one
    void restrict_lv(int lf)
    {
        Mark m(this, "mg_restrict");
        launch_restrict<T>(ctx(lf), ctx(lf + 1), lev[lf].G, lev[lf + 1].G, lev[lf].W, lev[lf + 1].W);
    }
    void interpolate_lv(int lf, int init)
    {
        Mark m(this, "mg_prolong");
        launch_interpolate<T>(ctx(lf), ctx(lf + 1), lev[lf].W, lev[lf + 1].W, init);
    }
    void delta_lv(int lc) { Mark m(this, "mg_delta"); launch_delta<T>(ctx(lc), lev[lc].W); }
    // FAS smoothing of coarse level l (three-level extension): residual at the restricted state,
    // forcing kept, sweeps and update
    void smooth_fas(int l)
    {
        resflux(l);
        { Mark m(this, "mg_forcing"); launch_forcing_keep<T>(ctx(l), lev[l].W); }
        sweep_update(l);
    }
    void res_calculate(int l) override { launch_res_norm<T>(ctx(l), lev[l].G, lev[l].W, lev[l].totalvol, norm_part, norm_blk); }
    void sweep_shape(int l, int out[2]) const override { out[0] = lev[l].planes.cpw; out[1] = lev[l].planes.wpb; }
    bool face_staged(int l) const override
    {
        return lev[l].tma_mem.p != nullptr && P.recon_var == 200 && P.recon == 500 && P.scheme == 300;
    }
    void res_calculate_static(int l, double *host_out) override
    {
        launch_res_norm_static<T>(ctx(l), lev[l].G, lev[l].W, lev[l].totalvol, ncase, host_out);
    }
    void primitive_vars(int l) override { Mark m(this, "primitive"); launch_primitive<T>(ctx(l), P, lev[l].W); }
    void limit_vars(int l) override { Mark m(this, "limiter", 2); launch_limiter<T>(ctx(l), P, lev[l].W, l, bad_list, bad_cap, bad_count); }
    void corner_treatment(int l) override { Mark m(this, "mg_corner", 2); launch_corner<T>(ctx(l), lev[l].W); }
    void restrict_to_coarse() override
    {
        need_mg();
        Mark m(this, "mg_restrict");
        launch_restrict<T>(ctx(1), ctx(2), lev[1].G, lev[2].G, lev[1].W, lev[2].W);
    }
    void interpolate(int init) override
    {
        need_mg();
        Mark m(this, "mg_prolong");
        launch_interpolate<T>(ctx(1), ctx(2), lev[1].W, lev[2].W, init);
    }
    void delta_cons() override { need_mg(); Mark m(this, "mg_delta"); launch_delta<T>(ctx(2), lev[2].W); }
    void integrals(int l) override { Mark m(this, "integrals", 2); launch_integrals<T>(ctx(l), P, lev[l].G, lev[l].W, lev[l].bc); }
    void set_use_force(int l, bool on) override { lev[l].use_force = on; }
    void need_mg() const { if (ng < 2) throw std::runtime_error("the case runs on a single grid level"); }

    void begin_iteration() { k_iter_begin<<<(nsolve + 127) / 128, 128, 0, stream>>>(batch(1)); }
    void mass_flow_imposed() override
    {
        if (any_mass) k_mass_control<<<(nsolve + 127) / 128, 128, 0, stream>>>(batch(1));
    }
    void outlet_pressure(double *out) override
    {
        std::vector<SolveState> st(ncase);
        states(st.data());
        for (int c = 0; c < ncase; c++) out[c] = st[c].pout;
    }

    // CSolver::Solver (source/Solver.cpp:47-140) for the current iteration number
    void step_body()
    {
        if (ng == 1) { time_marching(1); res_calculate(1); return; }
        if (!reuse && iter < coarse_iter) { time_marching(2); res_calculate(2); }
        else if (!reuse && iter == coarse_iter) {
            time_marching(2); res_calculate(2); corner_treatment(2);
            interpolate(1); primitive_vars(1); limit_vars(1);
        } else if (ng == 2) {
            lev[2].use_force = true;
            time_marching(1); res_calculate(1);
            resflux(1);
            restrict_to_coarse();
            primitive_vars(2); limit_vars(2);
            time_marching(2);
            delta_cons();
            corner_treatment(2);
            interpolate(0);
            primitive_vars(1); limit_vars(1);
        } else {
            // three-level V-cycle (extension): the fine step as in the two-level cycle, then FAS
            // on levels 2 and 3 with the coarse residuals evaluated at the restricted states
            time_marching(1); res_calculate(1);
            resflux(1);
            restrict_lv(1);
            primitive_vars(2); limit_vars(2);
            smooth_fas(2);
            resflux(2);
            { Mark m(this, "mg_forcing"); launch_add_forcing<T>(ctx(2), lev[2].W); }
            restrict_lv(2);
            primitive_vars(3); limit_vars(3);
            smooth_fas(3);
            delta_lv(3);
            corner_treatment(3);
            interpolate_lv(2, 0);
            primitive_vars(2); limit_vars(2);
            delta_lv(2);
            corner_treatment(2);
            interpolate_lv(1, 0);
            primitive_vars(1); limit_vars(1);
        }
    }
    // the level whose integrals an iteration reports (source/Structured_FV3D.cpp:150-156: the coarse
    // one up to the start-up's last iteration); a start from a given fine field has no start-up
    bool fine_start = false;
    int report_level() const { return (ng != 1 && !fine_start && iter <= coarse_iter) ? 2 : 1; }
    // driver phase: single grid; coarse-only start-up; the start-up's last cycle (eager); FAS. A
    // restarted multigrid run goes straight to FAS cycles (source/Solver.cpp:67-140)
    int phase() const
    {
        if (ng == 1) return 0;
        if (reuse) return 2;
        return iter < coarse_iter ? 1 : (iter == coarse_iter ? -1 : 2);
    }

    void solver_step() override
    {
        iter++;
        begin_iteration();
        step_body();
    }

    // the driver loop (source/Structured_FV3D.cpp:142-219): step + integrals, one graph per phase
    void iterate(int n, double *hist) override
    {
        std::vector<SolveState> st(nsolve);
        for (int q = 0; q < n; q++) {
            iter++;
            int ph = phase();
            // a phase graph fixes the reporting level it was captured with: a restarted multigrid
            // case reports the coarse level for its first iterations, which therefore run eagerly
            const bool level_moves = reuse && report_level() != 1;
            // a phase is captured at its second iteration: the first runs eagerly, so that a phase
            // that runs once (the start-up of a two-iteration coarse start) costs no capture and
            // instantiation (eager launches and graph replay give the same bits)
            const bool capture_now = ph >= 0 && !graphs[ph] && phase_runs[ph]++ >= 1;
            if (use_graphs && ph >= 0 && !profiling && !level_moves && (graphs[ph] || capture_now)) {
                if (!graphs[ph]) {
                    cudaGraph_t g;
                    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                    begin_iteration();
                    step_body();
                    integrals(report_level());
                    mass_flow_imposed();
                    CK(cudaStreamEndCapture(stream, &g));
                    CK(cudaGraphInstantiate(&graphs[ph], g, 0));
                    cudaGraphDestroy(g);
                }
                CK(cudaGraphLaunch(graphs[ph], stream));
            } else {
                begin_iteration();
                step_body();
                integrals(report_level());
                mass_flow_imposed();
            }
            if (hist) {
                CK(cudaMemcpyAsync(st.data(), st_d, sizeof(SolveState) * nsolve, cudaMemcpyDeviceToHost, stream));
                CK(cudaStreamSynchronize(stream));
                for (int cix = 0; cix < ncase; cix++) {
                    const SolveState &a = st[case_first[cix]];
                    double *r = hist + ((size_t)q * ncase + cix) * 12;
                    r[0] = a.iter;
                    for (int c = 0; c < 5; c++) r[1 + c] = a.res[c];
                    r[6] = a.m_in; r[7] = a.m_out; r[8] = a.pr; r[9] = a.eff; r[10] = a.m_ratio;
                    r[11] = a.cfl;
                }
            }
        }
        CK(cudaGetLastError());
    }

    void states(SolveState *out) override
    {
        std::vector<SolveState> st(nsolve);
        CK(cudaMemcpyAsync(st.data(), st_d, sizeof(SolveState) * nsolve, cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        for (int c = 0; c < ncase; c++) {
            out[c] = st[case_first[c]];
            for (int b = 1; b < case_nblk[c]; b++) {
                out[c].status |= st[case_first[c] + b].status;
                out[c].limiter_hits += st[case_first[c] + b].limiter_hits;
            }
        }
    }

    void dims(int solve, int l, int out[4]) const override
    {
        const Lvl &v = lev[l].lv[solve];
        out[0] = v.IM; out[1] = v.JM; out[2] = v.KM; out[3] = ng;
    }

    // ---------------------------------------------------------------- field access (tests, I/O)
    template <typename U>
    void fetch(const U *dptr, const Lvl &v, std::vector<double> &out)
    {
        long long n = box_size(v.IM, v.JM, v.KM);
        std::vector<U> tmp((size_t)n);
        CK(cudaMemcpyAsync(tmp.data(), dptr + v.base, sizeof(U) * n, cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        out.assign(tmp.begin(), tmp.end());
    }

    // a box [i0,i1]x[j0,j1]x[k0,k1] of several component arrays, components fastest
    struct Comp { const double *d; const T *t; };
    long box(const Lvl &v, const std::vector<Comp> &cs, int i0, int i1, int j0, int j1, int k0, int k1, double *out, long cap)
    {
        long n = (long)(i1 - i0 + 1) * (j1 - j0 + 1) * (k1 - k0 + 1) * (long)cs.size();
        if (n > cap) return -1;
        std::vector<std::vector<double>> h(cs.size());
        for (size_t c = 0; c < cs.size(); c++) {
            if (cs[c].d) fetch(cs[c].d, v, h[c]);
            else fetch(cs[c].t, v, h[c]);
        }
        long q = 0;
        Lvl z = v;
        z.base = 0;
        for (int i = i0; i <= i1; i++)
            for (int j = j0; j <= j1; j++)
                for (int k = k0; k <= k1; k++) {
                    long long p = ix(z, i, j, k);
                    for (size_t c = 0; c < cs.size(); c++) out[q++] = h[c][(size_t)p];
                }
        return n;
    }

    long get_field(int solve, int l, const std::string &name, double *out, long cap) override
    {
        if (solve < 0 || solve >= nsolve || l < 1 || l > ng) return -1;
        CK(cudaStreamSynchronize(stream));
        const Lvl &v = lev[l].lv[solve];
        const Flow<T> &W = lev[l].W;
        const Geo &G = lev[l].G;
        const int IM = v.IM, JM = v.JM, KM = v.KM;
        auto D = [](const double *p) { return Comp{p, nullptr}; };
        auto Tt = [](const T *p) { return Comp{nullptr, p}; };
        std::vector<Comp> cs;
        if (name == "cv") { for (int c = 0; c < 5; c++) cs.push_back(D(W.cv[c])); return box(v, cs, 0, IM, 0, JM, 0, KM, out, cap); }
        if (name == "pv") { for (int c = 0; c < 6; c++) cs.push_back(Tt(W.pv[c])); return box(v, cs, 0, IM, 0, JM, 0, KM, out, cap); }
        if (name == "mut") return box(v, {Tt(W.mut)}, 0, IM, 0, JM, 0, KM, out, cap);
        if (name == "ev" || name == "res_ev" || name == "dwall") {
            if (!W.ev) return -1;                  // Spalart-Allmaras cases, fine level
            if (name == "ev") return box(v, {D(W.ev)}, 0, IM, 0, JM, 0, KM, out, cap);
            if (name == "res_ev") return box(v, {Tt(W.res_ev)}, 1, IM - 1, 1, JM - 1, 1, KM - 1, out, cap);
            return box(v, {D(W.dwall)}, 1, IM - 1, 1, JM - 1, 1, KM - 1, out, cap);
        }
        if (name == "res") { for (int c = 0; c < 5; c++) cs.push_back(Tt(W.res[c])); return box(v, cs, 1, IM - 1, 1, JM - 1, 1, KM - 1, out, cap); }
        if (name == "dq") { for (int c = 0; c < 5; c++) cs.push_back(Tt(W.dq[c])); return box(v, cs, 1, IM - 1, 1, JM - 1, 1, KM - 1, out, cap); }
        if (name == "dt") return box(v, {Tt(W.dt)}, 1, IM - 1, 1, JM - 1, 1, KM - 1, out, cap);
        if (name == "omega") return box(v, {Tt(W.omega)}, 1, IM - 1, 1, JM - 1, 1, KM - 1, out, cap);
        const char *lam[6] = {"lamcI", "lamcJ", "lamcK", "lamvI", "lamvJ", "lamvK"};
        for (int q = 0; q < 6; q++)
            if (name == lam[q]) return box(v, {Tt(q < 3 ? W.lamc[q] : W.lamv[q - 3])}, 1, IM - 1, 1, JM - 1, 1, KM - 1, out, cap);
        const char *fcn[3] = {"FcI", "FcJ", "FcK"}, *fvn[3] = {"FvI", "FvJ", "FvK"}, *gn[3] = {"faceI", "faceJ", "faceK"};
        for (int f = 0; f < 3; f++) {
            int i1 = f == 0 ? IM : IM - 1, j1 = f == 1 ? JM : JM - 1, k1 = f == 2 ? KM : KM - 1;
            if (name == fcn[f]) { for (int c = 0; c < 5; c++) cs.push_back(Tt(W.Ff[f][c])); return box(v, cs, 1, i1, 1, j1, 1, k1, out, cap); }
            if (name == fvn[f]) { for (int c = 0; c < 5; c++) cs.push_back(Tt(W.Vf[f][c])); return box(v, cs, 1, i1, 1, j1, 1, k1, out, cap); }
            if (name == gn[f]) {
                for (int c = 0; c < 3; c++) cs.push_back(D(G.S[f][c]));
                cs.push_back(D(G.s[f]));
                for (int c = 0; c < 3; c++) cs.push_back(D(G.c[f][c]));
                cs.push_back(D(G.r[f])); cs.push_back(D(G.th[f]));
                for (int c = 0; c < 9; c++) cs.push_back(D(G.m[f][c]));
                return box(v, cs, 1, i1, 1, j1, 1, k1, out, cap);
            }
        }
        if (name == "cell") {
            cs.push_back(D(G.vol));
            for (int c = 0; c < 3; c++) cs.push_back(D(G.cc[c]));
            for (int c = 0; c < 9; c++) cs.push_back(D(G.cm[c]));
            return box(v, cs, 1, IM - 1, 1, JM - 1, 1, KM - 1, out, cap);
        }
        if (name == "totalvol") {
            if (cap < 1) return -1;
            CK(cudaMemcpy(out, lev[l].totalvol + solve, sizeof(double), cudaMemcpyDeviceToHost));
            return 1;
        }
        // reconstruction layers, [layer 1..2] along the face normal
        const char *dn[6] = {"dIS", "dIP", "dJS", "dJP", "dKS", "dKP"};
        for (int q = 0; q < 6; q++) {
            bool is_cv = name == std::string(dn[q]) + "_cv", is_pv = name == std::string(dn[q]) + "_pv";
            if (!is_cv && !is_pv) continue;
            int dir = q / 2, hi = q % 2;
            if (is_cv) for (int c = 0; c < 5; c++) cs.push_back(D(W.cv[c]));
            else for (int c = 0; c < 6; c++) cs.push_back(Tt(W.pv[c]));
            int r0[3] = {1, 1, 1}, r1[3] = {IM - 1, JM - 1, KM - 1};
            int N = dir == 0 ? IM : (dir == 1 ? JM : KM);
            long cnt = 2L * (long)cs.size();
            for (int d = 0; d < 3; d++) if (d != dir) cnt *= (r1[d] - r0[d] + 1);
            if (cnt > cap) return -1;
            std::vector<std::vector<double>> h(cs.size());
            for (size_t c = 0; c < cs.size(); c++) { if (cs[c].d) fetch(cs[c].d, v, h[c]); else fetch(cs[c].t, v, h[c]); }
            r0[dir] = 1; r1[dir] = 2;
            Lvl z = v; z.base = 0;
            long o = 0;
            for (int a = r0[0]; a <= r1[0]; a++)
                for (int b = r0[1]; b <= r1[1]; b++)
                    for (int e = r0[2]; e <= r1[2]; e++) {
                        int ii[3] = {a, b, e};
                        int nd = ii[dir];
                        ii[dir] = hi ? N + nd : -nd;
                        long long p = ix(z, ii[0], ii[1], ii[2]);
                        for (size_t c = 0; c < cs.size(); c++) out[o++] = h[c][(size_t)p];
                    }
            return cnt;
        }
        return -1;
    }

    // ---- the reference's solution files (source/Ouput.cpp:109-259, source/UserInput.cpp:1118-1159)
    std::string default_path(int cix, const std::string &path, const char *name) const
    {
        return path.empty() ? cases[case_first[cix]].dir + "/" + name : path;
    }
    void check_case(int cix) const { if (cix < 0 || cix >= ncase) throw std::runtime_error("bad solve"); }
    void fine_state(int slot, std::vector<double> &pv, std::vector<double> &cv, std::vector<double> *mut)
    {
        const Lvl &v = lev[1].lv[slot];
        const size_t nb = (size_t)(v.IM + 1) * (v.JM + 1) * (v.KM + 1);
        pv.resize(nb * 6);
        cv.resize(nb * 5);
        if (get_field(slot, 1, "pv", pv.data(), (long)pv.size()) < 0 || get_field(slot, 1, "cv", cv.data(), (long)cv.size()) < 0)
            throw std::runtime_error("state download failed");
        if (mut) {
            mut->resize(nb);
            if (get_field(slot, 1, "mut", mut->data(), (long)mut->size()) < 0) throw std::runtime_error("state download failed");
        }
    }
    // the fine-level fields of every block of a case
    void case_fields(int cix, std::vector<std::vector<double>> &pv, std::vector<std::vector<double>> &cv,
                     std::vector<std::vector<double>> *mut, std::vector<BlockField> &blocks,
                     std::vector<std::vector<double>> *ev = nullptr)
    {
        const int nb = case_nblk[cix];
        pv.resize(nb); cv.resize(nb);
        if (ev) ev->resize(nb);
        if (mut) mut->resize(nb);
        blocks.resize(nb);
        for (int b = 0; b < nb; b++) {
            const int s = case_first[cix] + b;
            fine_state(s, pv[b], cv[b], mut ? &(*mut)[b] : nullptr);
            const Lvl &v = lev[1].lv[s];
            BlockField &f = blocks[b];
            f.IM = v.IM; f.JM = v.JM; f.KM = v.KM;
            f.pv = pv[b].data(); f.cv = cv[b].data(); f.mut = mut ? (*mut)[b].data() : nullptr;
            f.x = cases[s].x.data(); f.y = cases[s].y.data(); f.z = cases[s].z.data();
            f.w_rot = lev[1].sc[s].w_rot; f.delta_th = lev[1].sc[s].delta_th;
            if (ev && lev[1].W.ev) {
                (*ev)[b].resize((size_t)(v.IM + 1) * (v.JM + 1) * (v.KM + 1));
                if (get_field(s, 1, "ev", (*ev)[b].data(), (long)(*ev)[b].size()) < 0) throw std::runtime_error("state download failed");
                f.ev = (*ev)[b].data();
            }
        }
    }
    void write_restart(int cix, const std::string &path) override
    {
        check_case(cix);
        std::vector<std::vector<double>> pv, cv, ev;
        std::vector<BlockField> blocks;
        case_fields(cix, pv, cv, nullptr, blocks, &ev);
        write_restart_file(default_path(cix, path, "RestartSolution.dat"), blocks);
    }
    void write_solution(int cix, const std::string &path) override
    {
        check_case(cix);
        std::vector<std::vector<double>> pv, cv, mut;
        std::vector<BlockField> blocks;
        case_fields(cix, pv, cv, &mut, blocks);
        const CaseSpec &c = cases[case_first[cix]];
        SolutionScales sc;
        sc.gamma = P.gamma; sc.rgas = P.rgas;
        sc.len_ref = c.Len_ref; sc.dens_ref = nd_ref.dens_ref; sc.vel_ref = nd_ref.vel_ref; sc.temp_ref = nd_ref.temp_ref;
        sc.mue_ref = nd_ref.mue_ref; sc.re_ref = nd_ref.re_ref;
        write_solution_file(default_path(cix, path, "RelativeSolution.plt"), blocks, sc);
    }
    void read_restart(int cix, const std::string &path) override
    {
        check_case(cix);
        std::vector<BlockField> blocks(case_nblk[cix]);
        for (int b = 0; b < case_nblk[cix]; b++) {
            const Lvl &v = lev[1].lv[case_first[cix] + b];
            blocks[b].IM = v.IM; blocks[b].JM = v.JM; blocks[b].KM = v.KM;
        }
        std::vector<std::vector<double>> cvs, pvs, evs;
        Flow<T> &W = lev[1].W;
        read_restart_file(default_path(cix, path, "RestartSolution.dat"), blocks, cvs, pvs, W.ev != nullptr, &evs);
        // Q, the primitive variables (and the SA variable) exactly as read (CUserInput::ReadSolution)
        CK(cudaStreamSynchronize(stream));
        for (int b = 0; b < case_nblk[cix]; b++) {
            const Lvl &v = lev[1].lv[case_first[cix] + b];
            const std::vector<double> &cv = cvs[b], &pv = pvs[b];
            const long long bn = box_size(v.IM, v.JM, v.KM);
            Lvl z = v; z.base = 0;
            for (int c = 0; c < 5; c++) {
                std::vector<double> h((size_t)bn);
                CK(cudaMemcpy(h.data(), W.cv[c] + v.base, sizeof(double) * bn, cudaMemcpyDeviceToHost));
                size_t q = c;
                for (int i = 1; i <= v.IM - 1; i++)
                    for (int j = 1; j <= v.JM - 1; j++)
                        for (int k = 1; k <= v.KM - 1; k++, q += 5) h[(size_t)ix(z, i, j, k)] = cv[q];
                CK(cudaMemcpy(W.cv[c] + v.base, h.data(), sizeof(double) * bn, cudaMemcpyHostToDevice));
            }
            for (int c = 0; c < 6; c++) {
                std::vector<T> h((size_t)bn);
                CK(cudaMemcpy(h.data(), W.pv[c] + v.base, sizeof(T) * bn, cudaMemcpyDeviceToHost));
                size_t q = c;
                for (int i = 1; i <= v.IM - 1; i++)
                    for (int j = 1; j <= v.JM - 1; j++)
                        for (int k = 1; k <= v.KM - 1; k++, q += 6) h[(size_t)ix(z, i, j, k)] = (T)pv[q];
                CK(cudaMemcpy(W.pv[c] + v.base, h.data(), sizeof(T) * bn, cudaMemcpyHostToDevice));
            }
            if (W.ev) {
                std::vector<double> h((size_t)bn);
                CK(cudaMemcpy(h.data(), W.ev + v.base, sizeof(double) * bn, cudaMemcpyDeviceToHost));
                size_t q = 0;
                for (int i = 1; i <= v.IM - 1; i++)
                    for (int j = 1; j <= v.JM - 1; j++)
                        for (int k = 1; k <= v.KM - 1; k++, q++) h[(size_t)ix(z, i, j, k)] = evs[b][q];
                CK(cudaMemcpy(W.ev + v.base, h.data(), sizeof(double) * bn, cudaMemcpyHostToDevice));
            }
        }
    }

    FineView fine_view() override
    {
        FineView v;
        v.nslot = nsolve;
        v.lv = lev[1].lv;
        v.lv_dev = lev[1].lv_d;
        for (int c = 0; c < NQ; c++) v.cv[c] = lev[1].W.cv[c];
        for (int c = 0; c < 3; c++) v.cc[c] = lev[1].G.cc[c];
        v.mut = lev[1].W.mut;
        v.fp32 = sizeof(T) == 4;
        return v;
    }
    void fill_uniform_fine(const std::vector<int> &slots) override
    {
        LaunchCtx cx = ctx(1);
        Flow<T> &W = lev[1].W;
        std::vector<int> all;
        const std::vector<int> *list = &slots;
        if (slots.empty()) {
            for (int s = 0; s < nsolve; s++) all.push_back(s);
            list = &all;
        }
        for (int s : *list) {
            if (s < 0 || s >= nsolve) throw std::runtime_error("slot out of range");
            const Lvl &v = lev[1].lv[s];
            const long long n = (long long)(v.IM - 1) * (v.JM - 1) * (v.KM - 1);
            k_fill_uniform_slot<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(cx.batch, s, W.cv[0], W.cv[1], W.cv[2],
                                                                                W.cv[3], W.cv[4], init_q);
        }
        CK(cudaGetLastError());
    }
    void fine_primitive() override { launch_primitive<T>(ctx(1), P, lev[1].W); }
    void fine_residual(std::vector<double> &per_case) override
    {
        resflux(1);
        std::vector<double> part((size_t)nsolve * kAbsResBlocks);
        DevBuf d;
        d.bytes = sizeof(double) * part.size();
        CK(cudaMalloc(&d.p, d.bytes));
        k_abs_res_partial<T><<<dim3(kAbsResBlocks, nsolve), 256, 0, stream>>>(batch(1), lev[1].W.res[0], (double *)d.p);
        CK(cudaMemcpyAsync(part.data(), d.p, d.bytes, cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        per_case.assign(ncase, 0.0);
        for (int c = 0; c < ncase; c++)
            for (int b = 0; b < case_nblk[c]; b++)
                for (int q = 0; q < kAbsResBlocks; q++) per_case[c] += part[(size_t)(case_first[c] + b) * kAbsResBlocks + q];
    }
    void start_from_fine_state() override
    {
        if (iter != 0) throw std::runtime_error("a start field is set before the first iteration");
        if (ng >= 2) {
            // the two-level cycle keeps the coarse level's time steps and spectral radii from its
            // start-up (the coarse residual is not evaluated again, source/Solver.cpp:88-110); without
            // a start-up they are evaluated once here, at the fine field restricted to the coarse
            // level (and, with three levels, to the coarsest)
            resflux(1);
            restrict_to_coarse();
            primitive_vars(2); limit_vars(2);
            resflux(2);
            if (ng == 3) {
                restrict_lv(2);
                primitive_vars(3); limit_vars(3);
                resflux(3);
            }
            CK(cudaStreamSynchronize(stream));
            CK(cudaGetLastError());
        }
        reuse = true;
        fine_start = true;
    }
    DevBuf snap;
    void save_fine_state() override
    {
        Level<T> &L = lev[1];
        if (snap.p) { cudaFree(snap.p); snap.p = nullptr; snap.bytes = 0; }
        snap.bytes = L.flow_d_mem.bytes + L.flow_t_mem.bytes + L.sa_mem.bytes + sizeof(SolveState) * nsolve;
        CK(cudaMalloc(&snap.p, snap.bytes));
        char *q = (char *)snap.p;
        CK(cudaMemcpyAsync(q, L.flow_d_mem.p, L.flow_d_mem.bytes, cudaMemcpyDeviceToDevice, stream)); q += L.flow_d_mem.bytes;
        CK(cudaMemcpyAsync(q, L.flow_t_mem.p, L.flow_t_mem.bytes, cudaMemcpyDeviceToDevice, stream)); q += L.flow_t_mem.bytes;
        if (L.sa_mem.bytes) { CK(cudaMemcpyAsync(q, L.sa_mem.p, L.sa_mem.bytes, cudaMemcpyDeviceToDevice, stream)); q += L.sa_mem.bytes; }
        CK(cudaMemcpyAsync(q, st_d, sizeof(SolveState) * nsolve, cudaMemcpyDeviceToDevice, stream));
        CK(cudaStreamSynchronize(stream));
    }
    void restore_fine_state(bool put_back) override
    {
        if (!snap.p) throw std::runtime_error("no saved state");
        if (put_back) {
            Level<T> &L = lev[1];
            const char *q = (const char *)snap.p;
            CK(cudaMemcpyAsync(L.flow_d_mem.p, q, L.flow_d_mem.bytes, cudaMemcpyDeviceToDevice, stream)); q += L.flow_d_mem.bytes;
            CK(cudaMemcpyAsync(L.flow_t_mem.p, q, L.flow_t_mem.bytes, cudaMemcpyDeviceToDevice, stream)); q += L.flow_t_mem.bytes;
            if (L.sa_mem.bytes) { CK(cudaMemcpyAsync(L.sa_mem.p, q, L.sa_mem.bytes, cudaMemcpyDeviceToDevice, stream)); q += L.sa_mem.bytes; }
            CK(cudaMemcpyAsync(st_d, q, sizeof(SolveState) * nsolve, cudaMemcpyDeviceToDevice, stream));
            CK(cudaStreamSynchronize(stream));
        }
        if (snap.p) { cudaFree(snap.p); snap.p = nullptr; snap.bytes = 0; }
    }

    void set_cv(int solve, int l, const double *in, long n) override
    {
        if (solve < 0 || solve >= nsolve || l < 1 || l > ng) throw std::runtime_error("bad solve or level");
        const Lvl &v = lev[l].lv[solve];
        long need = (long)(v.IM - 1) * (v.JM - 1) * (v.KM - 1) * 5;
        if (n != need) throw std::runtime_error("state size does not match the level");
        CK(cudaStreamSynchronize(stream));
        long long bn = box_size(v.IM, v.JM, v.KM);
        Lvl z = v; z.base = 0;
        for (int c = 0; c < 5; c++) {
            std::vector<double> h((size_t)bn);
            CK(cudaMemcpy(h.data(), lev[l].W.cv[c] + v.base, sizeof(double) * bn, cudaMemcpyDeviceToHost));
            long q = c;
            for (int i = 1; i <= v.IM - 1; i++)
                for (int j = 1; j <= v.JM - 1; j++)
                    for (int k = 1; k <= v.KM - 1; k++, q += 5) h[(size_t)ix(z, i, j, k)] = in[q];
            CK(cudaMemcpy(lev[l].W.cv[c] + v.base, h.data(), sizeof(double) * bn, cudaMemcpyHostToDevice));
        }
        launch_primitive<T>(ctx(l), P, lev[l].W);
        CK(cudaStreamSynchronize(stream));
    }
};

std::unique_ptr<SolverBase> make_solver(const std::vector<std::string> &dirs, int precision, int max_levels)
{
    if (precision == 0) return std::unique_ptr<SolverBase>(new SolverT<double>(dirs, 0, max_levels));
    if (precision == 1) return std::unique_ptr<SolverBase>(new SolverT<float>(dirs, 1, max_levels));
    throw std::runtime_error("precision must be 0 (FP64) or 1 (mixed FP32/FP64)");
}

}  // namespace gbt
