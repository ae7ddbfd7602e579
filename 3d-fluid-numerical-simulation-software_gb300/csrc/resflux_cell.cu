// Cell-centred stages of the residual: spectral radii and vorticity magnitude
// (source/Spectral_curl_grad.cpp:9-83), Baldwin-Lomax eddy viscosity along wall-normal grid
// lines (source/BL_Model.cpp:8-329), local time step and viscous spectral radii
// (source/TimeStep.cpp:7-93), and the wall ghost of mu_t (source/WallFlux.cpp:106-109).
#include "gbt_common.cuh"
#include "kernels.hpp"
#include "flux.cuh"

namespace gbt {

// lambda_c per direction and |curl V| (needs ghosts of the velocity)
template <typename T, bool NS>   // NS: Navier-Stokes (the curl is needed), else Euler
__global__ void __launch_bounds__(256) k_cell_a(Batch B, PhysW<T> PC, GeoW<T> G, Flow<T> W)
{
    const int s = blockIdx.y;
    const Lvl L = B.lv[s];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
    const T w_rot = (T)B.sc[s].w_rot;
    const T u = W.pv[PU][p], v = W.pv[PV][p], w = W.pv[PW][p];
    const T ur = u + w_rot * G.cc[1][p];
    const T vr = v - w_rot * G.cc[0][p];
    const T cs = tsqrt(PC.gamma * PC.rgas * W.pv[PT][p]);
    T lam[3];                                  // stored after the curl's loads
#pragma unroll
    for (int d = 0; d < 3; d++) {
        T sx = G.sb[d][0][p], sy = G.sb[d][1][p], sz = G.sb[d][2][p];
        lam[d] = tabs(ur * sx + vr * sy + w * sz) + cs * tsqrt(sx * sx + sy * sy + sz * sz);
    }
    if constexpr (!NS) {
#pragma unroll
        for (int d = 0; d < 3; d++) W.lamc[d][p] = lam[d];
        return;
    }
    const long long sI = (long long)L.NJ * L.NK, sJ = L.NK;
    const T h = (T)0.5;
    T uk = h * (W.pv[PU][p + sI] - W.pv[PU][p - sI]), vk = h * (W.pv[PV][p + sI] - W.pv[PV][p - sI]), wk = h * (W.pv[PW][p + sI] - W.pv[PW][p - sI]);
    T ue = h * (W.pv[PU][p + sJ] - W.pv[PU][p - sJ]), ve = h * (W.pv[PV][p + sJ] - W.pv[PV][p - sJ]), we = h * (W.pv[PW][p + sJ] - W.pv[PW][p - sJ]);
    T uz = h * (W.pv[PU][p + 1] - W.pv[PU][p - 1]), vz = h * (W.pv[PV][p + 1] - W.pv[PV][p - 1]), wz = h * (W.pv[PW][p + 1] - W.pv[PW][p - 1]);
    T m0 = G.cm[0][p], m1 = G.cm[1][p], m2 = G.cm[2][p], m3 = G.cm[3][p], m4 = G.cm[4][p],
      m5 = G.cm[5][p], m6 = G.cm[6][p], m7 = G.cm[7][p], m8 = G.cm[8][p];
    T v_x = vk * m0 + ve * m3 + vz * m6, w_x = wk * m0 + we * m3 + wz * m6;
    T u_y = uk * m1 + ue * m4 + uz * m7, w_y = wk * m1 + we * m4 + wz * m7;
    T u_z = uk * m2 + ue * m5 + uz * m8, v_z = vk * m2 + ve * m5 + vz * m8;
    const T om = tsqrt(h * ((w_y - v_z) * (w_y - v_z) + (u_z - w_x) * (u_z - w_x) + (v_x - u_y) * (v_x - u_y)));
#pragma unroll
    for (int d = 0; d < 3; d++) W.lamc[d][p] = lam[d];
    W.omega[p] = om;
    // FP64 form: the cell's laminar viscosity, once for the Baldwin-Lomax lines that cross it (up to
    // four) and the viscous spectral radii (the same function of the same temperature, so the same
    // value; on the FP64 pipe it costs about 25 instructions). The mixed form forms it where it is used.
    if constexpr (sizeof(T) == 8) W.mul[p] = sutherland(PC, W.pv[PT][p]);
}

// Baldwin-Lomax inner/outer viscosity (source/BL_Model.cpp:283-329) along the wall-normal lines
// of one wall patch; each line runs across the whole block from the wall face. A block holds 32
// lines on its lanes (the coalesced tangential index) and BL_WARPS warps that split the points
// of every line; the line maxima go through shared memory. mu_t is merged as the minimum over
// all walls whose lines cross the cell; the wall-adjacent cell and its ghost are set to zero
// (source/BL_Model.cpp:101-119). The maxima keep the reference's first-occurrence rule (strict
// ">" in line order), so the result does not depend on how the points are split.
constexpr int BL_WARPS = 8;
constexpr int BL_CACHE = 16;         // points per thread whose damping pass 2 keeps for pass 3

// geometry of one wall-normal line of wall record wl (shared by the distance and BL kernels)
struct BlLine {
    int dirn, lo, N, lines;
    long long p0, sn, fw;
    bool live;
    long long t;
};
__device__ __forceinline__ BlLine bl_line(const Lvl &L, const DevWall &wl, int blk, int lane)
{
    BlLine r;
    r.dirn = (wl.face - 1) / 2;
    r.lo = wl.face % 2 == 1;
    int a0, a1, b0, b1;                  // a: fast (coalesced) tangential index, b: the other one
    if (r.dirn == 0) { a0 = wl.ks; a1 = wl.ke; b0 = wl.js; b1 = wl.je; }
    else if (r.dirn == 1) { a0 = wl.ks; a1 = wl.ke; b0 = wl.is; b1 = wl.ie; }
    else { a0 = wl.js; a1 = wl.je; b0 = wl.is; b1 = wl.ie; }
    const int na = a1 - a0 + 1, nb = b1 - b0 + 1;
    r.lines = na * nb;
    r.t = (long long)blk * 32 + lane;
    r.live = r.t < (long long)r.lines;
    const unsigned tq = r.live ? (unsigned)r.t / (unsigned)na : 0u;
    const int a = a0 + (int)(r.live ? (unsigned)r.t - tq * (unsigned)na : 0u), b = b0 + (int)tq;
    r.N = r.dirn == 0 ? L.IM : (r.dirn == 1 ? L.JM : L.KM);
    r.sn = r.dirn == 0 ? (long long)L.NJ * L.NK : (r.dirn == 1 ? (long long)L.NK : 1LL);
    if (r.dirn == 0) { r.p0 = ix(L, 0, b, a); r.fw = ix(L, r.lo ? 1 : L.IM, b, a); }
    else if (r.dirn == 1) { r.p0 = ix(L, b, 0, a); r.fw = ix(L, b, r.lo ? 1 : L.JM, a); }
    else { r.p0 = ix(L, b, a, 0); r.fw = ix(L, b, a, r.lo ? 1 : L.KM); }
    return r;
}

// distance of every line point from its wall-face centre, formed exactly as the BL kernel would
template <typename T>
__global__ void __launch_bounds__(32 * BL_WARPS) k_wall_dist(Batch B, Geo G, const DevWall *walls,
                                                             const long long *off, T *dist)
{
    const DevWall wl = walls[blockIdx.y];
    const Lvl L = B.lv[wl.solve];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const BlLine ln = bl_line(L, wl, blockIdx.x, lane);
    if (!ln.live) return;
    const double fx = G.c[ln.dirn][0][ln.fw], fy = G.c[ln.dirn][1][ln.fw], fz = G.c[ln.dirn][2][ln.fw];
    T *d = dist + off[blockIdx.y];
    for (int n0 = 1 + wp; n0 < ln.N; n0 += BL_WARPS) {
        const long long p = ln.p0 + (long long)(ln.lo ? n0 : ln.N - n0) * ln.sn;
        const T dx = (T)(G.cc[0][p] - fx), dy = (T)(G.cc[1][p] - fy), dz = (T)(G.cc[2][p] - fz);
        d[(long long)(n0 - 1) * ln.lines + ln.t] = tsqrt(dx * dx + dy * dy + dz * dz);
    }
}

template <typename T>
void launch_wall_distances(const LaunchCtx &ctx, const Geo &G, const BcTables &bc)
{
    if (!bc.n_wall || !bc.wall_dist) return;
    dim3 g((unsigned)((bc.max_wall + 31) / 32), bc.n_wall);
    k_wall_dist<T><<<g, 32 * BL_WARPS, 0, ctx.stream>>>(ctx.batch, G, bc.wall, bc.wall_dist_off, (T *)bc.wall_dist);
}
template void launch_wall_distances<double>(const LaunchCtx &, const Geo &, const BcTables &);
template void launch_wall_distances<float>(const LaunchCtx &, const Geo &, const BcTables &);

// mu_t as an unsigned integer that orders like the value for mu_t >= 0, and back
__device__ __forceinline__ unsigned long long bl_bits(double v) { return (unsigned long long)__double_as_longlong(v); }
__device__ __forceinline__ unsigned long long bl_bits(float v) { return (unsigned long long)__float_as_uint(v); }
template <typename T> __device__ __forceinline__ T bl_value(unsigned long long b);
template <> __device__ __forceinline__ double bl_value<double>(unsigned long long b) { return __longlong_as_double((long long)b); }
template <> __device__ __forceinline__ float bl_value<float>(unsigned long long b) { return __uint_as_float((unsigned)b); }

template <typename T>
__global__ void __launch_bounds__(32 * BL_WARPS) k_bl(Batch B, PhysW<T> PC, Flow<T> W, const DevWall *walls, int off,
                                                      const long long *dist_off, const T *dist_all)
{
    __shared__ T sh_a[BL_WARPS][32], sh_b[BL_WARPS][32], sh_u[BL_WARPS][32];
    __shared__ int sh_n[BL_WARPS][32];
    __shared__ T sh_d1[32], sh_m1[32], sh_ret[32], sh_ymax[32], sh_fwake[32];
    const DevWall wl = walls[off + blockIdx.y];
    const Lvl L = B.lv[wl.solve];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const BlLine ln = bl_line(L, wl, blockIdx.x, lane);
    if ((long long)blockIdx.x * 32 >= (long long)ln.lines) return;      // whole block past the patch
    const bool live = ln.live;
    const int N = ln.N, lo = ln.lo;
    const long long p0 = ln.p0, sn = ln.sn;
    // wall distance of point n0 of this line (precomputed once from the geometry)
    const T *dist = dist_all + dist_off[off + blockIdx.y] + ln.t;
#define DIST(n0) dist[(long long)((n0) - 1) * ln.lines]
    // line order n0 = 1..N-1 (n0 = 1 next to the wall); warp wp takes n0 = 1 + wp, 1 + wp + BL_WARPS, ...
#define CELL(n0) (p0 + (long long)(lo ? (n0) : N - (n0)) * sn)
    // pass 1: wall shear, taken as the largest |omega * mu_l| along the line
    // Each pass takes a thread's points in chunks of four whose loads are issued together (indices
    // clamped to the line, so that the loads need no guard) and then processed in line order; the
    // first BL_CACHE points in unrolled chunks, so that pass 2 keeps their damping in registers.
    T tmax = (T)0;
    bool any = false;
    if (live) {
        auto p1 = [&](int n0, T ml, T om) {
            const T tw = tabs(om * ml);
            if (n0 == 1) { sh_d1[lane] = W.pv[PD][CELL(1)]; sh_m1[lane] = ml; }   // first cell: density, mu_l
            if (!any || tw > tmax) tmax = tw;
            any = true;
        };
#pragma unroll
        for (int ch = 0; ch < BL_CACHE / 4; ch++) {
            const int nb = 1 + wp + ch * 4 * BL_WARPS;
            if (nb < N) {
                T tv[4], ov[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const long long p = CELL(min(nb + u * BL_WARPS, N - 1));
                    tv[u] = sizeof(T) == 8 ? W.mul[p] : sutherland(PC, W.pv[PT][p]); ov[u] = W.omega[p];
                }
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (nb + u * BL_WARPS < N) p1(nb + u * BL_WARPS, tv[u], ov[u]);
            }
        }
        for (int n0 = 1 + wp + BL_CACHE * BL_WARPS; n0 < N; n0 += BL_WARPS)
            p1(n0, sizeof(T) == 8 ? W.mul[CELL(n0)] : sutherland(PC, W.pv[PT][CELL(n0)]), W.omega[CELL(n0)]);
    }
    sh_a[wp][lane] = tmax;
    sh_n[wp][lane] = any;
    __syncthreads();
    if (wp == 0 && live) {
        T Tw = (T)0;
        bool got = false;
        for (int w = 0; w < BL_WARPS; w++)
            if (sh_n[w][lane] && (!got || sh_a[w][lane] > Tw)) { Tw = sh_a[w][lane]; got = true; }
        sh_ret[lane] = tsqrt(sh_d1[lane] * Tw) / sh_m1[lane];
    }
    __syncthreads();
    const T Ret = sh_ret[lane];
    const T Aplus = (T)26.0, kap = (T)(double)0.4f, Ckleb = (T)(double)0.3f;
    const T aCcp = (T)((double)0.0168f * (double)1.6f);
    // pass 2: largest speed, and F = y |omega| (1 - exp(-y+/A+)) with its first maximiser
    T Fmax = (T)0, ymax = (T)0, Udif = (T)0;
    int nmax = 0x7fffffff;
    // van Driest damping of this thread's first BL_CACHE points, reused by pass 3
    T c_damp[BL_CACHE];
    if (live) {
        auto p2 = [&](int n0, T dis, T u, T v, T w, T om) -> T {
            const T V = tsqrt(u * u + v * v + w * w);
            if (V > Udif) Udif = V;
            const T damp = (T)1 - exp(-(dis * Ret) / Aplus);
            const T F = dis * tabs(om) * damp;
            if (F > Fmax) { Fmax = F; ymax = dis; nmax = n0; }
            return damp;
        };
#pragma unroll
        for (int ch = 0; ch < BL_CACHE / 4; ch++) {
            const int nb = 1 + wp + ch * 4 * BL_WARPS;
            if (nb < N) {
                T dv[4], uv[4], vv[4], wv[4], ov[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int m = min(nb + u * BL_WARPS, N - 1);
                    const long long p = CELL(m);
                    dv[u] = DIST(m); uv[u] = W.pv[PU][p]; vv[u] = W.pv[PV][p]; wv[u] = W.pv[PW][p]; ov[u] = W.omega[p];
                }
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (nb + u * BL_WARPS < N) c_damp[ch * 4 + u] = p2(nb + u * BL_WARPS, dv[u], uv[u], vv[u], wv[u], ov[u]);
            }
        }
        for (int n0 = 1 + wp + BL_CACHE * BL_WARPS; n0 < N; n0 += BL_WARPS) {
            const long long p = CELL(n0);
            p2(n0, DIST(n0), W.pv[PU][p], W.pv[PV][p], W.pv[PW][p], W.omega[p]);
        }
    }
    __syncthreads();
    sh_a[wp][lane] = Fmax;
    sh_b[wp][lane] = ymax;
    sh_n[wp][lane] = nmax;
    sh_u[wp][lane] = Udif;
    __syncthreads();
    if (wp == 0 && live) {
        T F = (T)0, y = (T)0, U = (T)0;
        int n = 0x7fffffff;
        for (int w = 0; w < BL_WARPS; w++) {
            if (sh_u[w][lane] > U) U = sh_u[w][lane];
            const T f = sh_a[w][lane];
            const int m = sh_n[w][lane];
            if (f > F || (f == F && m < n && f > (T)0)) { F = f; y = sh_b[w][lane]; n = m; }
        }
        const T q = y * U * U / F;
        sh_ymax[lane] = y;
        sh_fwake[lane] = (y * F < q) ? y * F : q;
    }
    __syncthreads();
    if (!live) return;
    const T ym = sh_ymax[lane], Fwake = sh_fwake[lane];
    // (Ret * dis) equals (dis * Ret) exactly, so the cached damping is the value pass 3 would form
    // pass 3: inner and outer viscosity, the smaller one merged into mu_t
    auto p3 = [&](int n0, T dis, T damp, T om, T rho) {
        const long long p = CELL(n0);
        const T bL = kap * dis * damp;
        const T m_in = rho * bL * bL * om;
        const T r = Ckleb * dis / ym;
        const T r2 = r * r;
        const T Fk = (T)1 / ((T)1 + (T)5.5 * (r2 * r2 * r2));
        const T m_out = aCcp * rho * Fwake * Fk;
        const T mt = (tabs(m_in) > tabs(m_out)) ? m_out : m_in;
        if (n0 == 1) {
            atomicMin(&W.blmin[p], 0ull);                      // wall-adjacent cell: mu_t = 0
            W.mut[p0 + (long long)(lo ? 0 : N) * sn] = (T)0;   // its ghost
            return;
        }
        // the smallest mu_t over the walls whose lines reach the cell (the reference's merge,
        // BL_Model.cpp:88-96,163-171,239-247: the first wall sets it, later walls keep the minimum; mu_t >= 0, so
        // the minimum of the bit patterns is the minimum of the values and the walls' order is moot)
        atomicMin(&W.blmin[p], bl_bits(mt));
    };
#pragma unroll
    for (int ch = 0; ch < BL_CACHE / 4; ch++) {
        const int nb = 1 + wp + ch * 4 * BL_WARPS;
        if (nb < N) {
            T dv[4], ov[4], rv[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int m = min(nb + u * BL_WARPS, N - 1);
                const long long p = CELL(m);
                dv[u] = DIST(m); ov[u] = W.omega[p]; rv[u] = W.pv[PD][p];
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (nb + u * BL_WARPS < N) p3(nb + u * BL_WARPS, dv[u], c_damp[ch * 4 + u], ov[u], rv[u]);
        }
    }
    for (int n0 = 1 + wp + BL_CACHE * BL_WARPS; n0 < N; n0 += BL_WARPS) {
        const long long p = CELL(n0);
        const T dis = DIST(n0);
        p3(n0, dis, (T)1 - exp(-(Ret * dis) / Aplus), W.omega[p], W.pv[PD][p]);
    }
#undef CELL
#undef DIST
}

// mu_t of every cell a wall line reached: the merged minimum (other cells keep their mu_t)
template <typename T>
__global__ void __launch_bounds__(256) k_bl_merge(Flow<T> W, long long n)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const unsigned long long b = W.blmin[p];
    if (b != ~0ull) W.mut[p] = bl_value<T>(b);
}

// ghost mu_t mirrored across every wall face (source/WallFlux.cpp:106-109,137-140,168-171)
template <typename T>
__global__ void k_wall_mut(Batch B, Flow<T> W, const DevWall *walls)
{
    const DevWall wl = walls[blockIdx.y];
    const Lvl L = B.lv[wl.solve];
    const int ni = wl.ie - wl.is + 1, nj = wl.je - wl.js + 1, nk = wl.ke - wl.ks + 1;
    int i, j, k;
    if (!box_index(ni, nj, nk, i, j, k)) return;
    i += wl.is - 1; j += wl.js - 1; k += wl.ks - 1;
    const int f = (wl.face - 1) / 2;
    const long long p = ix(L, i, j, k);
    const long long m = f == 0 ? ix(L, i - 1, j, k) : (f == 1 ? ix(L, i, j - 1, k) : ix(L, i, j, k - 1));
    if (wl.face % 2 == 1) W.mut[m] = -W.mut[p];
    else W.mut[p] = -W.mut[m];
}

// viscous spectral radii and the local time step
template <typename T, bool NS>   // NS: Navier-Stokes (viscous radii), else Euler
__global__ void __launch_bounds__(256) k_cell_b(Batch B, PhysW<T> PC, GeoW<T> G, Flow<T> W, int level)
{
    const int s = blockIdx.y;
    const Lvl L = B.lv[s];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
    const int fl = B.st[s].flag_low_dt[level];
    const double cfl = B.st[s].cfl;
    const double dtf = fl == 0 ? 1.0 : (double)(1.0f / (1.0f + (float)fl));
    const T vol = G.vol[p];
    T lc = W.lamc[0][p] + W.lamc[1][p] + W.lamc[2][p];
    T lv = (T)0;
    if constexpr (NS) {
        const T ml = sizeof(T) == 8 ? W.mul[p] : sutherland(PC, W.pv[PT][p]);   // FP64: formed by k_cell_a
        const T mt = W.mut[p];
        const T rho = W.pv[PD][p];
        const T a = (T)(double)(4.0f / 3.0f) / rho, b = PC.gamma / rho;
        const T coef = (a > b ? a : b) * (ml / PC.pr_lam + mt / PC.pr_tur);
        T l[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            T sx = G.sb[d][0][p], sy = G.sb[d][1][p], sz = G.sb[d][2][p];
            l[d] = coef * (sx * sx + sy * sy + sz * sz) / vol;
        }
#pragma unroll
        for (int d = 0; d < 3; d++) W.lamv[d][p] = l[d];
        lv = l[0] + l[1] + l[2];
    }
    W.dt[p] = to_work<T>(dtf * cfl) * vol / (lc + PC.c_timestep * lv);
}

// global time stepping: minimum over the solve, then broadcast (source/TimeStep.cpp:64-87)
template <typename T>
__global__ void __launch_bounds__(1024) k_dt_min(Batch B, Flow<T> W, T *out)
{
    const Lvl L = B.lv[blockIdx.y];
    const int nI = L.IM - 1, nJ = L.JM - 1, nK = L.KM - 1;
    const unsigned n = (unsigned)nI * (unsigned)nJ * (unsigned)nK;
    T m = (T)1E10;
    for (unsigned t = threadIdx.x; t < n; t += blockDim.x) {
        const unsigned q = t / (unsigned)nK, r = q / (unsigned)nJ;
        const int k = (int)(t - q * (unsigned)nK) + 1, j = (int)(q - r * (unsigned)nJ) + 1, i = (int)r + 1;
        T v = W.dt[ix(L, i, j, k)];
        m = (m < v) ? m : v;
    }
    __shared__ T sh[1024];
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) { T v = sh[threadIdx.x + o]; sh[threadIdx.x] = sh[threadIdx.x] < v ? sh[threadIdx.x] : v; }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.y] = sh[0];
}
template <typename T>
__global__ void k_dt_set(Batch B, Flow<T> W, const T *mn)
{
    const Lvl L = B.lv[blockIdx.y];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    W.dt[ix(L, i, j, k)] = mn[blockIdx.y];
}

// decrement of the low-time-step counter after the time step used it
__global__ void k_after_timestep(Batch B, int level)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B.nsolve) return;
    if (B.st[s].flag_low_dt[level] > 0) B.st[s].flag_low_dt[level] -= 1;
}

template <typename T>
void launch_cell_stages(const LaunchCtx &ctx, const Phys &P, const PhysW<T> &PC, const Geo &G, const GeoW<T> &GW,
                        Flow<T> W, const BcTables &bc,
                        int level, T *scratch)
{
    const Batch &B = ctx.batch;
    ctx.mark("spectral_curl", 1);
    if (P.equation_ns) k_cell_a<T, true><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, PC, GW, W);
    else k_cell_a<T, false><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, PC, GW, W);
    ctx.mark("spectral_curl", 0);
    ctx.mark("baldwin_lomax", 1, 4);
    if (level == 1 && P.turb_bl && bc.n_wall > 0) {
        // every wall of every solve in one launch (32 lines per block, the points of each line split
        // over BL_WARPS warps), merged through the per-cell minimum, reset every evaluation
        cudaMemsetAsync(W.blmin, 0xFF, (size_t)ctx.pool_n * sizeof(unsigned long long), ctx.stream);
        dim3 g((unsigned)((bc.max_wall + 31) / 32), bc.n_wall);
        k_bl<T><<<g, 32 * BL_WARPS, 0, ctx.stream>>>(B, PC, W, bc.wall, 0, bc.wall_dist_off, (const T *)bc.wall_dist);
        k_bl_merge<T><<<(unsigned)((ctx.pool_n + 255) / 256), 256, 0, ctx.stream>>>(W, ctx.pool_n);
    }
    if (level == 1 && P.turb_sa && W.ev) launch_sa_model<T>(ctx, P, GW, W);
    if (bc.n_wall > 0) {
        dim3 g((unsigned)((bc.max_wall + 127) / 128), bc.n_wall);
        k_wall_mut<T><<<g, 128, 0, ctx.stream>>>(B, W, bc.wall);
    }
    ctx.mark("baldwin_lomax", 0, 4);
    ctx.mark("time_step", 1, 2);
    if (P.equation_ns) k_cell_b<T, true><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, PC, GW, W, level);
    else k_cell_b<T, false><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, PC, GW, W, level);
    if (P.global_dt) {
        k_dt_min<T><<<dim3(1, B.nsolve), 1024, 0, ctx.stream>>>(B, W, scratch);
        k_dt_set<T><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, W, scratch);
    }
    k_after_timestep<<<(B.nsolve + 127) / 128, 128, 0, ctx.stream>>>(B, level);
    ctx.mark("time_step", 0, 2);
}

template void launch_cell_stages<double>(const LaunchCtx &, const Phys &, const PhysW<double> &, const Geo &,
                                         const GeoW<double> &, Flow<double>, const BcTables &, int, double *);
template void launch_cell_stages<float>(const LaunchCtx &, const Phys &, const PhysW<float> &, const Geo &,
                                        const GeoW<float> &, Flow<float>, const BcTables &, int, float *);

}  // namespace gbt
