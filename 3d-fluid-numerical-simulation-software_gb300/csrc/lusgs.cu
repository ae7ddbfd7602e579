// LU-SGS on i+j+k hyperplanes (source/LU_SGS_Marching.cpp:10-419): the forward sweep visits
// planes 3 .. IM+JM+KM-3, the backward sweep the same planes in reverse; the cells of a plane
// are independent, so a plane is one launch over all cells of all solves of the batch. The
// off-diagonal terms use the matrix-free flux difference of the neighbour in the rotating
// frame. Followed by the update Q += dQ (FP64 accumulation in both precision forms), the
// primitive variables (source/PrimitiveVars.cpp:7-28), detection of out-of-range cells for the
// limiter (source/Limit_FlowVars.cpp:8-118), and the residual norm (source/ComputeAllBlockVars.cpp:318-372).
#include "gbt_common.cuh"
#include "kernels.hpp"
#include "flux.cuh"

namespace gbt {

// Programmatic dependent launch: every plane's kernel lets the next plane's kernel start as soon
// as all of its own blocks are resident, so the kernels of many planes are in flight at once; each
// reads everything the sweep does not write (indices, geometry, Q, spectral radii, residual)
// first, then waits for the previous plane's grid to finish before it reads dQ. The resident set
// is always a prefix of the plane sequence, so the oldest resident plane can always finish.
__device__ __forceinline__ void wait_previous_plane() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void release_next_plane() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Each warp handles CPW cells of a plane with three lanes per cell, lane d computing
// the off-diagonal term of neighbour direction d; the three terms are combined on the first lane.
// A plane's cells and their neighbours are read from the plane-order copy (SweepData), so a warp's
// loads are dense. The neighbour's old flux F_n(Q) and the diagonal do not depend on dQ and are
// formed before the wait, so only the new flux F_n(Q + dQ) and the combination sit on the
// plane-to-plane critical path. Each lane's term is formed as
//   u = ((|S|/2) (F_n(Q+dQ) - F_n(Q)) +- (relax lambda_c / 2 + lambda_v) dQ_n) / alpha
// (+ forward, - backward): the reference's A and V terms of the same neighbour, grouped per lane
// and divided by the cell's diagonal (source/LU_SGS_Marching.cpp:95-150, 293-419), so that the first
// lane forms
//   forward:  dQ = -R / alpha + (u_I + u_J + u_K)
//   backward: dQ = dQ* - (u_I + u_J + u_K).
// The terms that do not depend on dQ (the neighbour's old flux, the diagonal) are formed before the
// wait, in the reference's sequence.
template <typename T, int DIR, int CPW, int WPB>   // DIR = +1 forward, -1 backward; CPW cells per warp, WPB warps per block
__global__ void __launch_bounds__(32 * WPB) k_sweep(PhysW<T> P, SweepData<T> S, const int *__restrict__ pstart,
                                                    int pstride, int plane)
{
    release_next_plane();
    const int lane = threadIdx.x & 31, slot = lane / 3, d = lane - 3 * slot;
    const int s = blockIdx.y;
    const int base = pstart[s * pstride + plane], cnt = pstart[s * pstride + plane + 1] - base;
    const int idx = (blockIdx.x * WPB + (int)(threadIdx.x >> 5)) * CPW + slot;
    const bool active = lane < 3 * CPW && idx < cnt;
    const int q = base + idx;
    int nb = -1;
    T nx = 0, ny = 0, nz = 0, ve = 0, od = 0, omx = 0, omy = 0, omz = 0, oe = 0, sd = 0, rl = 0, lv = 0;
    T fo[5] = {(T)0, (T)0, (T)0, (T)0, (T)0}, rhs[5] = {(T)0, (T)0, (T)0, (T)0, (T)0};
    T inva = (T)1;
    if (active) {
        nb = S.nb[DIR > 0 ? 0 : 1][d][q];
        if (nb >= 0) {
            nx = S.gn[d][0][nb]; ny = S.gn[d][1][nb]; nz = S.gn[d][2][nb];
            ve = S.gve[d][nb];
            od = S.cv[0][nb]; omx = S.cv[1][nb]; omy = S.cv[2][nb]; omz = S.cv[3][nb]; oe = S.cv[4][nb];
            const T po = S.pp[nb];
            // (the FP64 form's quotients Newton-refined, as in its other kernels; the mixed form's IEEE)
            const T oinv = sizeof(T) == 8 ? frcp<T>(od) : (T)1 / od;
            const T Vo = omx * oinv * nx + omy * oinv * ny + omz * oinv * nz;
            const T dov = Vo - ve;
            fo[0] = od * dov;
            fo[1] = omx * dov + po * nx;
            fo[2] = omy * dov + po * ny;
            fo[3] = omz * dov + po * nz;
            fo[4] = (oe + po) * dov + po * ve;
            rl = P.relax * S.lamc[d][nb];
            sd = S.gs[d][nb];
            lv = S.lamv[d][nb];
        }
        // the cell's 1 / alpha on all three lanes (the warp executes these instructions once)
        if constexpr (sizeof(T) == 8) {
            const T alpha = fdiv<T>(S.gvol[q], S.dt[q]) + P.relax * (S.lamc[0][q] + S.lamc[1][q] + S.lamc[2][q]) +
                            (T)2 * (S.lamv[0][q] + S.lamv[1][q] + S.lamv[2][q]);
            inva = frcp<T>(alpha);
        } else {
            const T alpha = S.gvol[q] / S.dt[q] + P.relax * (S.lamc[0][q] + S.lamc[1][q] + S.lamc[2][q]) +
                            (T)2 * (S.lamv[0][q] + S.lamv[1][q] + S.lamv[2][q]);
            inva = (T)1 / alpha;
        }
        if (DIR > 0) {
            if constexpr (sizeof(T) == 8) {
                // lane d combines components d and d + 3 (below)
                rhs[0] = -S.res[d][q] * inva;
                if (d < 2) rhs[1] = -S.res[d + 3][q] * inva;
            } else if (d == 0) {
#pragma unroll
                for (int c = 0; c < 5; c++) rhs[c] = -S.res[c][q] * inva;
            }
        }
    }
    // the lane's coefficients, divided by alpha here so that the combination is three additions
    const T hs = ((T)0.5 * sd) * inva, cq = ((T)0.5 * rl + lv) * inva;
    wait_previous_plane();
    T dqp[5];                            // backward sweep: this cell's forward-sweep dQ
    if (DIR < 0 && active) {
        if constexpr (sizeof(T) == 8) {
            dqp[0] = S.dq[d][q];
            if (d < 2) dqp[1] = S.dq[d + 3][q];
        } else if (d == 0) {
#pragma unroll
            for (int c = 0; c < 5; c++) dqp[c] = S.dq[c][q];
        }
    }
    T u[5] = {(T)0, (T)0, (T)0, (T)0, (T)0};
    if (nb >= 0) {
        T dqn[5];
#pragma unroll
        for (int c = 0; c < 5; c++) dqn[c] = S.dq[c][nb];
        // flux difference F_n(Q+dQ) - F_n(Q) of the neighbour across its mean normal; the momentum
        // projection and |m|^2 are formed while the reciprocal of the density is computed, so that
        // only V_n = (m.n)/rho and p = (g-1)(rho E - |m|^2/(2 rho)) follow it, and the old flux is
        // taken off the pressure term, which does not wait for V_n
        const T nd = od + dqn[0], nmx = omx + dqn[1], nmy = omy + dqn[2], nmz = omz + dqn[3], ne = oe + dqn[4];
        const T mn = nmx * nx + nmy * ny + nmz * nz, m2 = nmx * nmx + nmy * nmy + nmz * nmz;
        const T inv = frcp<T>(nd);
        const T pn = P.gm1 * (ne - (T)0.5 * (m2 * inv));
        const T dn = mn * inv - ve;
        T dF[5];
        dF[0] = nd * dn - fo[0];
        dF[1] = nmx * dn + (pn * nx - fo[1]);
        dF[2] = nmy * dn + (pn * ny - fo[2]);
        dF[3] = nmz * dn + (pn * nz - fo[3]);
        dF[4] = (ne + pn) * dn + (pn * ve - fo[4]);
#pragma unroll
        for (int c = 0; c < 5; c++) u[c] = DIR > 0 ? hs * dF[c] + cq * dqn[c] : hs * dF[c] - cq * dqn[c];
    }
    if constexpr (sizeof(T) == 8) {
        // FP64: the three lanes of a cell share the combination, lane d taking components d and
        // d + 3, so that the warp runs two rounds of three FP64 additions instead of five (each FP64
        // instruction holds the sub-partition for about 70 cycles whatever the active lanes). In
        // sub-round r, lane d reads from lane (d + r) mod 3 of its cell the term of component d + 3t,
        // which that lane selects from its own terms; the sums keep the order (u_I + u_J) + u_K.
        const int base = lane - d;
#pragma unroll
        for (int t = 0; t < 2; t++) {
            T part[3] = {(T)0, (T)0, (T)0};
#pragma unroll
            for (int r = 1; r <= 2; r++) {
                const int src = d + r < 3 ? d + r : d + r - 3;        // the lane read from (its d)
                const int cs = (d >= r ? d - r : d - r + 3) + 3 * t;  // the component this lane sends
                T send = (T)0;
#pragma unroll
                for (int m = 0; m < 5; m++)
                    if (cs == m) send = u[m];
                const T got = __shfl_sync(0xffffffffu, send, base + src);
                if (src == 0) part[0] = got;
                else if (src == 1) part[1] = got;
                else part[2] = got;
            }
            const int c = d + 3 * t;
            T own = (T)0;
#pragma unroll
            for (int m = 0; m < 5; m++)
                if (c == m) own = u[m];
            if (d == 0) part[0] = own;
            else if (d == 1) part[1] = own;
            else part[2] = own;
            if (active && c < 5) {
                const T sum = (part[0] + part[1]) + part[2];
                S.dq[c][q] = DIR > 0 ? rhs[t] + sum : dqp[t] - sum;
            }
        }
    } else {
        T u1[5], u2[5];
#pragma unroll
        for (int c = 0; c < 5; c++) {
            u1[c] = __shfl_down_sync(0xffffffffu, u[c], 1);
            u2[c] = __shfl_down_sync(0xffffffffu, u[c], 2);
        }
        if (!active || d != 0) return;
#pragma unroll
        for (int c = 0; c < 5; c++) {
            const T sum = (u[c] + u1[c]) + u2[c];
            S.dq[c][q] = DIR > 0 ? rhs[c] + sum : dqp[c] - sum;
        }
    }
}

// Box <-> plane order through shared-memory tiles: the sweeps' flow inputs into plane order before
// the forward sweep, dQ back into the box after the backward sweep. A hyperplane's cells are never
// neighbours in the k-contiguous box (consecutive plane cells (i, j, k), (i, j+1, k-1) lie NK - 1
// apart), so a per-cell copy moves one DRAM sector per value on one side. A block here takes a
// 32 x 32 (j, k) tile of one i-row of one solve for a group of G arrays (grid.z): it moves the
// box's k-rows and the tile's j + k = const diagonals, which are runs of consecutive plane-order
// indices (the plane order enumerates i, then j), so both sides move whole sectors. The diagonals'
// starts are read once per block; the loads of all arrays of the group are issued before the first
// store. Batches take groups of five arrays, so that a block keeps some twenty loads per thread in
// flight (the 64-point batch's gather and scatter 0.68 ms faster per cycle than with one array per
// block); single solves keep one array per block, where the grid then has enough blocks to fill
// the GPU (five-array groups made the single FP64 solve's scatter 13 us slower). Values are converted on the
// way from the source to the destination type (FP64 Q to the working type with the conversion
// instructions' rounding).
constexpr int kTileArrays = 13;
template <typename Src, typename Dst> struct TileList {
    const Src *src[kTileArrays];
    Dst *dst[kTileArrays];
};
template <typename Dst, typename Src> __device__ __forceinline__ Dst tile_conv(Src v)
{
    if constexpr (sizeof(Src) == 8 && sizeof(Dst) == 4) return f64_to_f32_rn(v);
    else return (Dst)v;
}

template <typename Src, typename Dst, bool TO_PLANE, int G>
__global__ void __launch_bounds__(256) k_plane_tile(Batch B, const int *__restrict__ rq, const long long *__restrict__ rq_off,
                                                    TileList<Src, Dst> A, int n, int tj, int tk)
{
    const int s = blockIdx.y, a0 = (int)blockIdx.z * G;   // solve, first array of the group
    const int na = min(G, n - a0);
    const Lvl L = B.lv[s];
    const int nI = L.IM - 1, nJ = L.JM - 1, nK = L.KM - 1;
    const int kb = (int)(blockIdx.x % (unsigned)tk), jb = (int)((blockIdx.x / (unsigned)tk) % (unsigned)tj);
    const int i = (int)(blockIdx.x / ((unsigned)tk * (unsigned)tj)) + 1;
    const int j0 = jb * 32 + 1, k0 = kb * 32 + 1;
    if (i > nI || j0 > nJ || k0 > nK) return;
    // row stride 34: the diagonals (word offset 33 jj + dd) and the k-rows both hit 32 banks
    __shared__ Dst tile[G][32][34];
    __shared__ int qd[63];                               // plane-order index of (i, j0, k0 + dd) minus j0
    const int lane = threadIdx.x & 31, w = (int)(threadIdx.x >> 5);
    // (a diagonal beyond the solve's last plane holds no cell of the solve: its entry is clamped to
    // the table and never used)
    if (threadIdx.x < 63) qd[threadIdx.x] = rq[rq_off[s] + (long long)min(i + j0 + k0 + (int)threadIdx.x, nI + nJ + nK) * nI + (i - 1)];
    if (TO_PLANE) {
#pragma unroll
        for (int g = 0; g < G; g++) {
            if (g >= na) break;
            const Src *src = A.src[a0 + g];
#pragma unroll
            for (int r = w; r < 32; r += 8) {
                const int j = j0 + r, k = k0 + lane;
                if (j <= nJ && k <= nK) tile[g][r][lane] = tile_conv<Dst>(src[ix(L, i, j, k)]);
            }
        }
        __syncthreads();
#pragma unroll
        for (int g = 0; g < G; g++) {
            if (g >= na) break;
            Dst *dst = A.dst[a0 + g];
#pragma unroll
            for (int e = 0; e < 8; e++) {
                const int dd = w + 8 * e, kk = dd - lane, j = j0 + lane, k = k0 + kk;
                if (dd < 63 && kk >= 0 && kk < 32 && j <= nJ && k <= nK) dst[qd[dd] + j] = tile[g][lane][kk];
            }
        }
    } else {
        __syncthreads();
#pragma unroll
        for (int g = 0; g < G; g++) {
            if (g >= na) break;
            const Src *src = A.src[a0 + g];
#pragma unroll
            for (int e = 0; e < 8; e++) {
                const int dd = w + 8 * e, kk = dd - lane, j = j0 + lane, k = k0 + kk;
                if (dd < 63 && kk >= 0 && kk < 32 && j <= nJ && k <= nK) tile[g][lane][kk] = tile_conv<Dst>(src[qd[dd] + j]);
            }
        }
        __syncthreads();
#pragma unroll
        for (int g = 0; g < G; g++) {
            if (g >= na) break;
            Dst *dst = A.dst[a0 + g];
#pragma unroll
            for (int r = w; r < 32; r += 8) {
                const int j = j0 + r, k = k0 + lane;
                if (j <= nJ && k <= nK) dst[ix(L, i, j, k)] = tile[g][r][lane];
            }
        }
    }
}

template <typename Src, typename Dst, bool TO_PLANE>
static void launch_plane_tile(const LaunchCtx &ctx, const PlaneTables &pt, const TileList<Src, Dst> &A, int n)
{
    const int tj = (ctx.maxJM - 1 + 31) / 32, tk = (ctx.maxKM - 1 + 31) / 32;
    const dim3 grid((unsigned)((ctx.maxIM - 1) * tj * tk), ctx.batch.nsolve);
    if (ctx.batch.nsolve >= 4) {
        k_plane_tile<Src, Dst, TO_PLANE, 5><<<dim3(grid.x, grid.y, (n + 4) / 5), 256, 0, ctx.stream>>>(ctx.batch, pt.rq, pt.rq_off, A, n, tj, tk);
    } else {
        k_plane_tile<Src, Dst, TO_PLANE, 1><<<dim3(grid.x, grid.y, n), 256, 0, ctx.stream>>>(ctx.batch, pt.rq, pt.rq_off, A, n, tj, tk);
    }
}

// the sweeps' flow inputs into plane order (before every forward sweep): Q in the working type,
// the residual, lambda_c, lambda_v, p and dt (two launches)
template <typename T>
static void launch_sweep_gather(const LaunchCtx &ctx, const PlaneTables &pt, const Flow<T> &W, const SweepData<T> &S)
{
    TileList<double, T> q = {};
    for (int c = 0; c < NQ; c++) { q.src[c] = W.cv[c]; q.dst[c] = S.cv[c]; }
    launch_plane_tile<double, T, true>(ctx, pt, q, NQ);
    TileList<T, T> f = {};
    int n = 0;
    for (int c = 0; c < NQ; c++) { f.src[n] = W.res[c]; f.dst[n++] = S.res[c]; }
    for (int d = 0; d < 3; d++) { f.src[n] = W.lamc[d]; f.dst[n++] = S.lamc[d]; }
    for (int d = 0; d < 3; d++) { f.src[n] = W.lamv[d]; f.dst[n++] = S.lamv[d]; }
    f.src[n] = W.pv[PP]; f.dst[n++] = S.pp;
    f.src[n] = W.dt; f.dst[n++] = S.dt;
    launch_plane_tile<T, T, true>(ctx, pt, f, n);
}

// geometry of the sweeps into plane order, in the working precision (once per level)
template <typename T>
__global__ void __launch_bounds__(256) k_sweep_geometry(Geo G, SweepData<T> S, long long nq)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const long long p = S.cell[q];
#pragma unroll
    for (int d = 0; d < 3; d++) {
#pragma unroll
        for (int c = 0; c < 3; c++) S.gn[d][c][q] = (T)G.cn[d][c][p];
        S.gs[d][q] = (T)G.cs[d][p];
        S.gve[d][q] = (T)G.cve[d][p];
    }
    S.gvol[q] = (T)G.vol[p];
}

template <typename T, int DIR, int CPW, int WPB>
static void launch_plane_v(const LaunchCtx &ctx, const PhysW<T> &P, const PlaneTables &pt, const SweepData<T> &S, int pl,
                           bool first)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(max(1, (pt.max_count[pl] + CPW * WPB - 1) / (CPW * WPB)), ctx.batch.nsolve);
    cfg.blockDim = dim3(32 * WPB);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = ctx.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = first ? 0 : 1;     // the first plane of a sweep waits for everything before it
    cudaLaunchKernelEx(&cfg, k_sweep<T, DIR, CPW, WPB>, P, S, pt.start, pt.stride, pl);
}

// (cells per warp, warps per block) variants of the sweep kernels; the autotuner picks one per level
struct SweepShape { int cpw, wpb; };
constexpr SweepShape kSweepShapes[] = {{1, 1}, {2, 1}, {4, 1}, {10, 1}, {4, 4}, {10, 4}, {10, 8}};

bool sweep_shape_known(int cpw, int wpb)
{
    for (const SweepShape &sh : kSweepShapes)
        if (sh.cpw == cpw && sh.wpb == wpb) return true;
    return false;
}

template <typename T, int DIR>
static void launch_plane(const LaunchCtx &ctx, const PhysW<T> &P, const PlaneTables &pt, const SweepData<T> &S, int pl,
                         bool first)
{
    const int v = pt.cpw * 16 + pt.wpb;
    switch (v) {
    case 1 * 16 + 1: launch_plane_v<T, DIR, 1, 1>(ctx, P, pt, S, pl, first); break;
    case 2 * 16 + 1: launch_plane_v<T, DIR, 2, 1>(ctx, P, pt, S, pl, first); break;
    case 4 * 16 + 1: launch_plane_v<T, DIR, 4, 1>(ctx, P, pt, S, pl, first); break;
    case 4 * 16 + 4: launch_plane_v<T, DIR, 4, 4>(ctx, P, pt, S, pl, first); break;
    case 10 * 16 + 4: launch_plane_v<T, DIR, 10, 4>(ctx, P, pt, S, pl, first); break;
    case 10 * 16 + 8: launch_plane_v<T, DIR, 10, 8>(ctx, P, pt, S, pl, first); break;
    default: launch_plane_v<T, DIR, 10, 1>(ctx, P, pt, S, pl, first); break;
    }
}

// benign sweep inputs for timing (Q = rest state, unit time step and radii, zero residual)
template <typename T>
__global__ void __launch_bounds__(256) k_sweep_fill(SweepData<T> S, long long nq)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    S.cv[0][q] = (T)1; S.cv[1][q] = (T)0.1; S.cv[2][q] = (T)0.1; S.cv[3][q] = (T)0.1; S.cv[4][q] = (T)2.5;
    S.pp[q] = (T)0.7;
    for (int d = 0; d < 3; d++) { S.lamc[d][q] = (T)1; S.lamv[d][q] = (T)0.1; }
    S.dt[q] = (T)1;
    for (int c = 0; c < NQ; c++) { S.res[c][q] = (T)1e-3; S.dq[c][q] = (T)0; }
}

// Autotuner of the sweep's block shape (cells per warp, warps per block): times the forward and
// backward plane chains of this
// level on benign inputs written into the plane-order scratch (which every time step gathers
// afresh, so the solver's state is untouched) and returns the fastest candidate as
// cpw * 16 + wpb. Results do not depend on the choice: every cell is computed the same way.
template <typename T>
int tune_sweep_cpw(const LaunchCtx &ctx, const PhysW<T> &P, const PlaneTables &pt0, const SweepData<T> &S)
{
    PlaneTables pt = pt0;
    const int np = pt.max_plane;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_sweep_fill<T><<<(unsigned)((pt.nq + 255) / 256), 256, 0, ctx.stream>>>(S, pt.nq);
    SweepShape best = {10, 1};
    float best_ms = 1e30f;
    for (const SweepShape &sh : kSweepShapes) {
        pt.cpw = sh.cpw;
        pt.wpb = sh.wpb;
        float ms = 0.f;
        for (int rep = 0; rep < 3; rep++) {
            cudaEventRecord(e0, ctx.stream);
            for (int pl = 3; pl <= np; pl++) launch_plane<T, 1>(ctx, P, pt, S, pl, pl == 3);
            for (int pl = np; pl >= 3; pl--) launch_plane<T, -1>(ctx, P, pt, S, pl, pl == np);
            cudaEventRecord(e1, ctx.stream);
            cudaEventSynchronize(e1);
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            if (rep > 0) ms += t;           // first repetition warms up
        }
        if (ms < best_ms) { best_ms = ms; best = sh; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return best.cpw * 16 + best.wpb;
}

template <typename T>
void launch_lusgs_sweeps(const LaunchCtx &ctx, const PhysW<T> &P, const Geo &G, Flow<T> W, const PlaneTables &pt,
                         const SweepData<T> &S)
{
    const int np = pt.max_plane;
    ctx.mark("sweep_forward", 1, np);                 // two gather launches and the planes
    launch_sweep_gather<T>(ctx, pt, W, S);
    for (int pl = 3; pl <= np; pl++) launch_plane<T, 1>(ctx, P, pt, S, pl, pl == 3);
    ctx.mark("sweep_forward", 0, np);
    if (W.ev) {
        ctx.mark("sa_sweeps", 1, np - 2);
        launch_sa_sweep<T>(ctx, P, G, W, pt, S, 1);
        ctx.mark("sa_sweeps", 0, np - 2);
    }
    ctx.mark("sweep_backward", 1, np - 1);
    for (int pl = np; pl >= 3; pl--) launch_plane<T, -1>(ctx, P, pt, S, pl, pl == np);
    ctx.mark("sweep_backward", 0, np - 1);
    if (W.ev) {
        ctx.mark("sa_sweeps", 1, np - 2);
        launch_sa_sweep<T>(ctx, P, G, W, pt, S, -1);
        ctx.mark("sa_sweeps", 0, np - 2);
    }
    ctx.mark("sweep_scatter", 1, 1);
    TileList<T, T> dq = {};
    for (int c = 0; c < NQ; c++) { dq.src[c] = S.dq[c]; dq.dst[c] = W.dq[c]; }
    launch_plane_tile<T, T, false>(ctx, pt, dq, NQ);
    ctx.mark("sweep_scatter", 0, 1);
}

template <typename T>
void launch_sweep_geometry(const LaunchCtx &ctx, const Geo &G, const PlaneTables &pt, const SweepData<T> &S)
{
    k_sweep_geometry<T><<<(unsigned)((pt.nq + 255) / 256), 256, 0, ctx.stream>>>(G, S, pt.nq);
}

// primitive variables from the conserved ones
template <typename T>
__device__ __forceinline__ void prim_from_cons(const Phys &P, const double c[5], T q[6])
{
    if constexpr (sizeof(T) == 4) {
        // mixed form: primitives are stored in FP32, so they are formed in FP32 from the FP64 Q
        // (conversions by integer operations: the same roundings as the conversion instructions)
        const float d = f64_to_f32_rn(c[0]), rd = 1.0f / d;
        const float u = f64_to_f32_rn(c[1]) * rd, v = f64_to_f32_rn(c[2]) * rd, w = f64_to_f32_rn(c[3]) * rd;
        const float V2 = u * u + v * v + w * w;
        const float pr = ((float)P.gamma - 1.0f) * (f64_to_f32_rn(c[4]) - d * V2 * 0.5f);
        q[PD] = d; q[PU] = u; q[PV] = v; q[PW] = w; q[PP] = pr; q[PT] = pr * rd / (float)P.rgas;
    } else {
        // one FP64 division by the density, products with its reciprocal (within rounding)
        const double d = c[0], rd = 1.0 / d, u = c[1] * rd, v = c[2] * rd, w = c[3] * rd;
        const double V2 = u * u + v * v + w * w;
        const double pr = (P.gamma - 1.0) * (c[4] - d * V2 * 0.5);
        q[PD] = (T)d; q[PU] = (T)u; q[PV] = (T)v; q[PW] = (T)w; q[PP] = (T)pr; q[PT] = (T)(pr * rd / P.rgas);
    }
}

template <typename T>
__device__ __forceinline__ bool out_of_range(const T q[6])
{
    const T dmin = (T)(double)1.0E-6f, dmax = (T)1000, pmin = (T)(double)1.0E-6f, pmax = (T)1000, vmax = (T)1000;
    return q[PD] < dmin || q[PD] > dmax || q[PP] < pmin || q[PP] > pmax || q[PU] > vmax || q[PV] > vmax || q[PW] > vmax;
}

// Q_old = Q; Q += dQ; primitive variables; out-of-range cells appended to the solve's list
template <typename T>
__global__ void __launch_bounds__(256) k_update(Batch B, Phys P, Flow<T> W, int *bad_list, int bad_cap, int *bad_count)
{
    const int s = blockIdx.y;
    const Lvl L = B.lv[s];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
    double c[5];
#pragma unroll
    for (int n = 0; n < 5; n++) {
        const double o = W.cv[n][p];
        W.cvold[n][p] = o;
        c[n] = o + to_f64<T>(W.dq[n][p]);
        W.cv[n][p] = c[n];
    }
    T q[6];
    prim_from_cons<T>(P, c, q);
#pragma unroll
    for (int n = 0; n < 6; n++) W.pv[n][p] = q[n];
    if (P.limiter && out_of_range(q)) {
        int slot = atomicAdd(&bad_count[s], 1);
        if (slot < bad_cap) bad_list[(long long)s * bad_cap + slot] = (int)(((long long)(i - 1) * (L.JM - 1) + (j - 1)) * (L.KM - 1) + (k - 1));
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_primitive(Batch B, Phys P, Flow<T> W)
{
    const Lvl L = B.lv[blockIdx.y];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
    double c[5];
#pragma unroll
    for (int n = 0; n < 5; n++) c[n] = W.cv[n][p];
    T q[6];
    prim_from_cons<T>(P, c, q);
#pragma unroll
    for (int n = 0; n < 6; n++) W.pv[n][p] = q[n];
}

template <typename T>
__global__ void __launch_bounds__(256) k_detect(Batch B, Phys P, Flow<T> W, int *bad_list, int bad_cap, int *bad_count)
{
    const int s = blockIdx.y;
    const Lvl L = B.lv[s];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
    T q[6];
#pragma unroll
    for (int n = 0; n < 6; n++) q[n] = W.pv[n][p];
    if (out_of_range(q)) {
        int slot = atomicAdd(&bad_count[s], 1);
        if (slot < bad_cap) bad_list[(long long)s * bad_cap + slot] = (int)(((long long)(i - 1) * (L.JM - 1) + (j - 1)) * (L.KM - 1) + (k - 1));
    }
}

// The reference repairs limited cells one after another in i, j, k order, each from the mean of
// its in-range neighbours as they are at that moment, so a repaired cell can feed a later one.
// Rare; one thread per solve replays that order over the (sorted) list of flagged cells. When
// the list overflowed, the thread scans every cell instead.
template <typename T>
__global__ void k_limiter(Batch B, Phys P, Flow<T> W, int level, int *bad_list, int bad_cap, int *bad_count)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B.nsolve) return;
    const int n = bad_count[s];
    if (n == 0) { B.st[s].status &= ~GBT_STATUS_LIMITER; return; }
    const Lvl L = B.lv[s];
    const int nI = L.IM - 1, nJ = L.JM - 1, nK = L.KM - 1;
    int *lst = bad_list + (long long)s * bad_cap;
    const bool full = n > bad_cap;
    if (!full) {
        for (int a = 1; a < n; a++) {                 // insertion sort: lists are short
            int v = lst[a], b = a - 1;
            while (b >= 0 && lst[b] > v) { lst[b + 1] = lst[b]; b--; }
            lst[b + 1] = v;
        }
    }
    const long long total = (long long)nI * nJ * nK;
    const long long m = full ? total : n;
    for (long long e = 0; e < m; e++) {
        const long long lin = full ? e : lst[e];
        const int i = 1 + (int)(lin / ((long long)nJ * nK)), j = 1 + (int)((lin / nK) % nJ), k = 1 + (int)(lin % nK);
        const long long p = ix(L, i, j, k);
        T q[6];
        for (int c = 0; c < 6; c++) q[c] = W.pv[c][p];
        if (!out_of_range(q)) continue;
        double d = 0, u = 0, v = 0, w = 0, pr = 0;
        int kn = 0, i1 = 0, j1 = 0, k1 = 0;
        for (int ia = -1; ia <= 1; ia++)
            for (int ja = -1; ja <= 1; ja++)
                for (int ka = -1; ka <= 1; ka++) {
                    k1 = k + ka; j1 = j + ja; i1 = i + ia;
                    if (i1 > 0 && i1 < L.IM && j1 > 0 && j1 < L.JM && k1 > 0 && k1 < L.KM) {
                        const long long r = ix(L, i1, j1, k1);
                        T qq[6];
                        for (int c = 0; c < 6; c++) qq[c] = W.pv[c][r];
                        if (!out_of_range(qq)) {
                            d += qq[PD]; u += qq[PU]; v += qq[PV]; w += qq[PW]; pr += qq[PP]; kn++;
                        }
                    }
                }
        if (kn == 0) {
            // last visited neighbour (i+1, j+1, k+1), clipped to the admissible range
            const long long r = ix(L, i1, j1, k1);
            d = W.pv[PD][r]; u = W.pv[PU][r]; v = W.pv[PV][r]; w = W.pv[PW][r]; pr = W.pv[PP][r];
            const double lo = (double)1.0E-6f;
            if (d < lo) d = lo;
            if (d > 1000.0) d = 1000.0;
            if (pr < lo) pr = lo;
            if (pr > 1000.0) pr = 1000.0;
            if (fabs(u) > 1000.0) u = u < 0 ? -1000.0 : 1000.0;
            if (fabs(v) > 1000.0) v = v < 0 ? -1000.0 : 1000.0;
            if (fabs(w) > 1000.0) w = w < 0 ? -1000.0 : 1000.0;
        } else {
            const double sn1 = (double)(1.0f / (float)kn);
            d *= sn1; u *= sn1; v *= sn1; w *= sn1; pr *= sn1;
        }
        W.pv[PD][p] = (T)d; W.pv[PU][p] = (T)u; W.pv[PV][p] = (T)v; W.pv[PW][p] = (T)w; W.pv[PP][p] = (T)pr;
        W.pv[PT][p] = (T)(pr / d / P.rgas);
        W.cv[0][p] = d; W.cv[1][p] = d * u; W.cv[2][p] = d * v; W.cv[3][p] = d * w;
        W.cv[4][p] = pr / (P.gamma - 1.0) + d * (u * u + v * v + w * w) / 2.0;
    }
    B.st[s].flag_low_dt[level] = 10;
    B.st[s].status |= GBT_STATUS_LIMITER | (full ? GBT_STATUS_LIMITER_OVF : 0);
    B.st[s].limiter_hits += n;
}

template <typename T>
void launch_update(const LaunchCtx &ctx, const Phys &P, const Geo &G, Flow<T> W, int level, int *bad_list,
                   int bad_cap, int *bad_count)
{
    (void)G;
    const Batch &B = ctx.batch;
    ctx.mark("update_limiter", 1, 2);
    cudaMemsetAsync(bad_count, 0, sizeof(int) * B.nsolve, ctx.stream);
    k_update<T><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, P, W, bad_list, bad_cap, bad_count);
    if (P.limiter) k_limiter<T><<<(B.nsolve + 31) / 32, 32, 0, ctx.stream>>>(B, P, W, level, bad_list, bad_cap, bad_count);
    if (W.ev) {
        // the variable's update and Limit_SA after the mean flow's (source/LU_SGS_Marching.cpp:275-277,
        // source/ComputeAllBlockVars.cpp:257-266); the limiter list is reused
        launch_sa_update<T>(ctx, P, W, bad_list, bad_cap, bad_count);
        if (P.limiter) launch_sa_limit<T>(ctx, W, bad_list, bad_cap, bad_count);
    }
    ctx.mark("update_limiter", 0, 2);
}

template <typename T>
void launch_primitive(const LaunchCtx &ctx, const Phys &P, Flow<T> W)
{
    k_primitive<T><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(ctx.batch, P, W);
}

template <typename T>
void launch_limiter(const LaunchCtx &ctx, const Phys &P, Flow<T> W, int level, int *bad_list, int bad_cap,
                    int *bad_count)
{
    if (!P.limiter) return;
    const Batch &B = ctx.batch;
    cudaMemsetAsync(bad_count, 0, sizeof(int) * B.nsolve, ctx.stream);
    k_detect<T><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, P, W, bad_list, bad_cap, bad_count);
    k_limiter<T><<<(B.nsolve + 31) / 32, 32, 0, ctx.stream>>>(B, P, W, level, bad_list, bad_cap, bad_count);
}

// ---- residual norm: sum |(Q_old - Q)/Q_old| * Vol / V_total, FP64, fixed-order two-stage sum ----
template <typename T>
__global__ void __launch_bounds__(256) k_norm_partial(Batch B, Geo G, Flow<T> W, double *partials, int nblk)
{
    const int s = blockIdx.y;
    const Lvl L = B.lv[s];
    const int nI = L.IM - 1, nJ = L.JM - 1, nK = L.KM - 1;
    const unsigned n = (unsigned)nI * (unsigned)nJ * (unsigned)nK;
    double acc[5] = {0, 0, 0, 0, 0};
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (unsigned)nblk * blockDim.x) {
        const unsigned q = t / (unsigned)nK, r = q / (unsigned)nJ;
        const int k = (int)(t - q * (unsigned)nK) + 1, j = (int)(q - r * (unsigned)nJ) + 1, i = (int)r + 1;
        const long long p = ix(L, i, j, k);
        const double vol = G.vol[p];
#pragma unroll
        for (int c = 0; c < 5; c++) {
            const double o = W.cvold[c][p];
            acc[c] += rel_change_t<T>(o, W.cv[c][p]) * vol;
        }
    }
    __shared__ double sh[8][5];
#pragma unroll
    for (int c = 0; c < 5; c++) {
        double v = acc[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double v = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += sh[w][threadIdx.x];
        partials[((long long)s * nblk + blockIdx.x) * 5 + threadIdx.x] = v;
    }
}

// the norm of a case: the partials of its blocks in block order, over the case's volume (every
// slot of the case computes the same sum and keeps it)
__global__ void k_norm_final(Batch B, const double *partials, int nblk, const double *totalvol)
{
    const int s = blockIdx.x;
    if (threadIdx.x >= 5) return;
    const SolveConst &sc = B.sc[s];
    double v = 0;
    for (int q = sc.lead; q < sc.lead + sc.nblk; q++)
        for (int b = 0; b < nblk; b++) v += partials[((long long)q * nblk + b) * 5 + threadIdx.x];
    v = v / totalvol[s];
    B.st[s].res[threadIdx.x] = v;
    if (threadIdx.x == 0 && !isfinite(v)) B.st[s].status |= GBT_STATUS_NAN;
}

template <typename T>
void launch_res_norm(const LaunchCtx &ctx, const Geo &G, Flow<T> W, const double *totalvol, double *partials, int nblk)
{
    const Batch &B = ctx.batch;
    ctx.mark("res_norm", 1, 2);
    k_norm_partial<T><<<dim3(nblk, B.nsolve), 256, 0, ctx.stream>>>(B, G, W, partials, nblk);
    k_norm_final<<<B.nsolve, 32, 0, ctx.stream>>>(B, partials, nblk, totalvol);
    ctx.mark("res_norm", 0, 2);
}

// ---- inlet/outlet integrals (source/Ouput.cpp:9-107,282-300) ----
// partial sums over one section (inlet or outlet k face): mass flow, sum Pt^((g-1)/g) * m and
// sum Tt * m; grid (kIntegralBlocks, solves, 2 sections), so the FP64 powers spread over the SMs
template <typename T>
__global__ void __launch_bounds__(128) k_section_partial(Batch B, Phys P, Geo G, Flow<T> W, const DevInOut *inl,
                                                         const DevInOut *outl, double *part)
{
    const int s = blockIdx.y, sec = blockIdx.z;
    // the section's block: the case's Inlet[1] / Outlet[1] may lie in any of its blocks
    const DevInOut &sp = sec == 0 ? inl[s] : outl[s];
    const Lvl L = B.lv[sp.solve];
    const int K = sp.ks;
    const int nI = L.IM - 1, nJ = L.JM - 1;
    const double g = P.gamma, g1 = g - 1.0, R = P.rgas;
    double m = 0, pm = 0, tm = 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nI * nJ; t += kIntegralBlocks * blockDim.x) {
        const int i = 1 + t / nJ, j = 1 + t % nJ;
        const long long p = ix(L, i, j, K), q = ix(L, i, j, K - 1);
        const double d = 0.5 * ((double)W.pv[PD][p] + (double)W.pv[PD][q]);
        const double u = 0.5 * ((double)W.pv[PU][p] + (double)W.pv[PU][q]);
        const double v = 0.5 * ((double)W.pv[PV][p] + (double)W.pv[PV][q]);
        const double w = 0.5 * ((double)W.pv[PW][p] + (double)W.pv[PW][q]);
        const double mc = d * (u * G.S[2][0][p] + v * G.S[2][1][p] + w * G.S[2][2][p]);
        const double tf = 0.5 * ((double)W.pv[PT][p] + (double)W.pv[PT][q]);
        const double Ma = sqrt(u * u + v * v + w * w) / sqrt(g * R * tf);
        const double fac = 1.0 + g1 / 2.0 * Ma * Ma;
        const double Pt = (double)W.pv[PP][p] * pow(fac, g / g1);
        m += mc;
        pm += pow(Pt, g1 / g) * mc;
        tm += (double)W.pv[PT][p] * fac * mc;
    }
    __shared__ double sh[3][4];
    double v3[3] = {m, pm, tm};
    for (int c = 0; c < 3; c++) {
        double v = v3[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) sh[c][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double v = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += sh[threadIdx.x][w];
        part[(((long long)s * 2 + sec) * kIntegralBlocks + blockIdx.x) * 3 + threadIdx.x] = v;
    }
}

// inlet/outlet integrals (source/Ouput.cpp:9-107,282-300): partials summed in block order
__global__ void k_integrals(Batch B, Phys P, const DevInOut *inl, const DevInOut *outl, const double *part)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B.nsolve) return;
    double a[3] = {0, 0, 0}, b[3] = {0, 0, 0};
    for (int blk = 0; blk < kIntegralBlocks; blk++)
        for (int c = 0; c < 3; c++) {
            a[c] += part[(((long long)s * 2 + 0) * kIntegralBlocks + blk) * 3 + c];
            b[c] += part[(((long long)s * 2 + 1) * kIntegralBlocks + blk) * 3 + c];
        }
    const double g = P.gamma, g1 = g - 1.0, R = P.rgas;
    // blade count of the inlet's and of the outlet's block (source/Ouput.cpp:288,294)
    const double mi = a[0] * P.dens_ref * P.vel_ref * B.sc[inl[s].solve].nblade;
    const double mo = b[0] * P.dens_ref * P.vel_ref * B.sc[outl[s].solve].nblade;
    const double pti = pow(a[1] / a[0], g / g1) * P.dens_ref * P.vel_ref * P.vel_ref;
    const double pto = pow(b[1] / b[0], g / g1) * P.dens_ref * P.vel_ref * P.vel_ref;
    const double tti = a[2] / a[0] * P.temp_ref, tto = b[2] / b[0] * P.temp_ref;
    const double PR = pto / pti;
    const double Ladk = g / g1 * R * tti * (pow(PR, g1 / g) - 1.0);
    const double Lk = g / g1 * R * tti * (tto / tti - 1.0);
    SolveState &st = B.st[s];
    st.m_in = mi; st.m_out = mo; st.pr = PR; st.eff = Ladk / Lk;
    st.m_ratio = fabs((mi - mo) / mi);
    if (!isfinite(mi) || !isfinite(mo)) st.status |= GBT_STATUS_NAN;
}

template <typename T>
void launch_integrals(const LaunchCtx &ctx, const Phys &P, const Geo &G, Flow<T> W, const BcTables &bc)
{
    // first inlet and first outlet patch of every solve (the reference reports Inlet[1], Outlet[1])
    const Batch &B = ctx.batch;
    k_section_partial<T><<<dim3(kIntegralBlocks, B.nsolve, 2), 128, 0, ctx.stream>>>(B, P, G, W, bc.inlet_first,
                                                                                      bc.outlet_first, bc.integ_part);
    k_integrals<<<(B.nsolve + 31) / 32, 32, 0, ctx.stream>>>(B, P, bc.inlet_first, bc.outlet_first, bc.integ_part);
}

// CFL ramp of the driver (source/Solver.cpp:49-60): x1.2 whenever the density residual falls
// below a threshold that then drops tenfold; capped at 10
__global__ void k_cfl_ramp(Batch B, int iter)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B.nsolve || iter <= 1) return;
    SolveState &st = B.st[s];
    if (st.res[0] <= st.cfl_res) {
        st.cfl = st.cfl * (double)1.2f;
        st.cfl_res = st.cfl_res / 10.0;
    }
    if (st.cfl > 10.0) st.cfl = 10.0;
}
void launch_cfl_ramp(const LaunchCtx &ctx, int iter)
{
    k_cfl_ramp<<<(ctx.batch.nsolve + 127) / 128, 128, 0, ctx.stream>>>(ctx.batch, iter);
}

#define GBT_INST(T)                                                                                                   \
    template void launch_lusgs_sweeps<T>(const LaunchCtx &, const PhysW<T> &, const Geo &, Flow<T>, const PlaneTables &, const SweepData<T> &); \
    template void launch_sweep_geometry<T>(const LaunchCtx &, const Geo &, const PlaneTables &, const SweepData<T> &); \
    template int tune_sweep_cpw<T>(const LaunchCtx &, const PhysW<T> &, const PlaneTables &, const SweepData<T> &); \
    template void launch_update<T>(const LaunchCtx &, const Phys &, const Geo &, Flow<T>, int, int *, int, int *);     \
    template void launch_primitive<T>(const LaunchCtx &, const Phys &, Flow<T>);                                       \
    template void launch_limiter<T>(const LaunchCtx &, const Phys &, Flow<T>, int, int *, int, int *);                 \
    template void launch_res_norm<T>(const LaunchCtx &, const Geo &, Flow<T>, const double *, double *, int);          \
    template void launch_integrals<T>(const LaunchCtx &, const Phys &, const Geo &, Flow<T>, const BcTables &);
GBT_INST(double)
GBT_INST(float)

}  // namespace gbt
