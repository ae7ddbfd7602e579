// Two-level multigrid transfer (source/Prolong_Interpolate.cpp:7-176,
// source/ComputeAllBlockVars.cpp:269-309,374-438): volume-weighted restriction of Q and summed
// restriction of the residual, forcing term on the coarse level, coarse correction dQ, edge and
// corner fill of the coarse ghosts, trilinear 27/9/3/1 prolongation.
#include "gbt_common.cuh"
#include "kernels.hpp"
#include <algorithm>

namespace gbt {

template <typename T>
__global__ void __launch_bounds__(256) k_restrict(Batch Bf, Batch Bc, Geo Gf, Geo Gc, Flow<T> Wf, Flow<T> Wc)
{
    const int s = blockIdx.y;
    const Lvl F = Bf.lv[s], C = Bc.lv[s];
    int i, j, k;
    if (!box_index(C.IM - 1, C.JM - 1, C.KM - 1, i, j, k)) return;
    const int i1 = 2 * i - 1, j1 = 2 * j - 1, k1 = 2 * k - 1, i2 = 2 * i, j2 = 2 * j, k2 = 2 * k;
    const long long f[8] = {ix(F, i1, j1, k1), ix(F, i1, j1, k2), ix(F, i1, j2, k1), ix(F, i1, j2, k2),
                            ix(F, i2, j1, k1), ix(F, i2, j1, k2), ix(F, i2, j2, k1), ix(F, i2, j2, k2)};
    const long long p = ix(C, i, j, k);
    const double vc = Gc.vol[p];
#pragma unroll
    for (int c = 0; c < NQ; c++) {
        double a = Wf.cv[c][f[0]] * Gf.vol[f[0]];
        T r = Wf.res[c][f[0]];
#pragma unroll
        for (int q = 1; q < 8; q++) { a = a + Wf.cv[c][f[q]] * Gf.vol[f[q]]; r = r + Wf.res[c][f[q]]; }
        a = a / vc;
        Wc.cv2h[c][p] = a;
        Wc.cv[c][p] = a;
        Wc.res2h[c][p] = r;
    }
}

// coarse residual replaced by the restricted fine residual through the forcing function:
// Qf = R_2h - R_c; R_c = R_c + Qf
template <typename T>
__global__ void __launch_bounds__(256) k_forcing(Batch B, Flow<T> W)
{
    const Lvl L = B.lv[blockIdx.y];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
#pragma unroll
    for (int c = 0; c < NQ; c++) {
        const T qf = W.res2h[c][p] - W.res[c][p];
        W.res[c][p] = W.res[c][p] + qf;
    }
}

// three-level V-cycle extension (proper FAS on the coarse levels): the forcing Qf = R_2h - R_c at
// the restricted state replaces the residual by the restricted one and is kept (in res2h) for the
// level's own FAS residual R_c(Q') + Qf after its smoothing, which is restricted further
template <typename T>
__global__ void __launch_bounds__(256) k_forcing_keep(Batch B, Flow<T> W)
{
    const Lvl L = B.lv[blockIdx.y];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
#pragma unroll
    for (int c = 0; c < NQ; c++) {
        const T qf = W.res2h[c][p] - W.res[c][p];
        W.res[c][p] = W.res[c][p] + qf;
        W.res2h[c][p] = qf;
    }
}
template <typename T>
__global__ void __launch_bounds__(256) k_add_forcing(Batch B, Flow<T> W)
{
    const Lvl L = B.lv[blockIdx.y];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
#pragma unroll
    for (int c = 0; c < NQ; c++) W.res[c][p] = W.res[c][p] + W.res2h[c][p];
}

template <typename T>
__global__ void __launch_bounds__(256) k_delta(Batch B, Flow<T> W)
{
    const Lvl L = B.lv[blockIdx.y];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
#pragma unroll
    for (int c = 0; c < NQ; c++) W.dq2h[c][p] = to_work<T>(W.cv[c][p] - W.cv2h[c][p]);
}

// 12 edges then 8 corners of the ghost layer, for Q and for the coarse correction
// (source/Corner_Treatment.cpp): edges in one launch (one thread per edge cell, all values read
// before any is written), then the corners, which read the edges, in a second one
template <typename T>
__global__ void __launch_bounds__(64) k_edges(Batch B, Flow<T> W)
{
    const Lvl L = B.lv[blockIdx.z];
    const int IM = L.IM, JM = L.JM, KM = L.KM;
    const int e = blockIdx.y, n = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    long long dst, a, b;
    switch (e) {
    case 0: if (n > IM - 1) return; dst = ix(L, n, 0, 0); a = ix(L, n, 1, 0); b = ix(L, n, 0, 1); break;
    case 1: if (n > IM - 1) return; dst = ix(L, n, JM, 0); a = ix(L, n, JM - 1, 0); b = ix(L, n, JM, 1); break;
    case 2: if (n > IM - 1) return; dst = ix(L, n, 0, KM); a = ix(L, n, 0, KM - 1); b = ix(L, n, 1, KM); break;
    case 3: if (n > IM - 1) return; dst = ix(L, n, JM, KM); a = ix(L, n, JM - 1, KM); b = ix(L, n, JM, KM - 1); break;
    case 4: if (n > JM - 1) return; dst = ix(L, 0, n, 0); a = ix(L, 1, n, 0); b = ix(L, 0, n, 1); break;
    case 5: if (n > JM - 1) return; dst = ix(L, 0, n, KM); a = ix(L, 1, n, KM); b = ix(L, 0, n, KM - 1); break;
    case 6: if (n > JM - 1) return; dst = ix(L, IM, n, KM); a = ix(L, IM - 1, n, KM); b = ix(L, IM, n, KM - 1); break;
    case 7: if (n > JM - 1) return; dst = ix(L, IM, n, 0); a = ix(L, IM - 1, n, 0); b = ix(L, IM, n, 1); break;
    case 8: if (n > KM - 1) return; dst = ix(L, 0, 0, n); a = ix(L, 1, 0, n); b = ix(L, 0, 1, n); break;
    case 9: if (n > KM - 1) return; dst = ix(L, IM, 0, n); a = ix(L, IM, 1, n); b = ix(L, IM - 1, 0, n); break;
    case 10: if (n > KM - 1) return; dst = ix(L, 0, JM, n); a = ix(L, 1, JM, n); b = ix(L, 0, JM - 1, n); break;
    default: if (n > KM - 1) return; dst = ix(L, IM, JM, n); a = ix(L, IM - 1, JM, n); b = ix(L, IM, JM - 1, n); break;
    }
    double qa[NQ], qb[NQ];
    T da[NQ], db[NQ];
#pragma unroll
    for (int c = 0; c < NQ; c++) { qa[c] = W.cv[c][a]; qb[c] = W.cv[c][b]; da[c] = W.dq2h[c][a]; db[c] = W.dq2h[c][b]; }
#pragma unroll
    for (int c = 0; c < NQ; c++) {
        W.cv[c][dst] = 0.5 * (qa[c] + qb[c]);
        W.dq2h[c][dst] = (T)0.5 * (da[c] + db[c]);
    }
}

// corner (ci,cj,ck) from its three edge neighbours and three face-diagonal neighbours; thread
// corner * NQ + c of the block of its solve
template <typename T>
__global__ void __launch_bounds__(64) k_corners(Batch B, Flow<T> W)
{
    const Lvl L = B.lv[blockIdx.x];
    const int IM = L.IM, JM = L.JM, KM = L.KM;
    if (threadIdx.x >= 8 * NQ) return;
    const int corner = threadIdx.x / NQ, c = threadIdx.x % NQ;
    const int ci = (corner & 1) ? IM : 0, cj = (corner & 2) ? JM : 0, ck = (corner & 4) ? KM : 0;
    const int i1 = ci ? IM - 1 : 1, j1 = cj ? JM - 1 : 1, k1 = ck ? KM - 1 : 1;
    const long long e1 = ix(L, i1, cj, ck), e2 = ix(L, ci, j1, ck), e3 = ix(L, ci, cj, k1);
    const long long d1 = ix(L, i1, j1, ck), d2 = ix(L, i1, cj, k1), d3 = ix(L, ci, j1, k1);
    const long long dst = ix(L, ci, cj, ck);
    const double q = (2.0 * (W.cv[c][e1] + W.cv[c][e2] + W.cv[c][e3]) - (W.cv[c][d1] + W.cv[c][d2] + W.cv[c][d3])) / 3.0;
    const T d = ((T)2 * (W.dq2h[c][e1] + W.dq2h[c][e2] + W.dq2h[c][e3]) - (W.dq2h[c][d1] + W.dq2h[c][d2] + W.dq2h[c][d3])) / (T)3;
    W.cv[c][dst] = q;
    W.dq2h[c][dst] = d;
}

// fine Q (+)= sum of 27/64, 9/64, 3/64, 1/64 weighted coarse values around the fine cell; the
// first call after the coarse start-up phase interpolates Q itself, later calls the correction
template <typename T>
__global__ void __launch_bounds__(256) k_interpolate(Batch Bf, Batch Bc, Flow<T> Wf, Flow<T> Wc, int init)
{
    const int s = blockIdx.y;
    const Lvl F = Bf.lv[s], C = Bc.lv[s];
    int i, j, k;
    if (!box_index(F.IM - 1, F.JM - 1, F.KM - 1, i, j, k)) return;
    // nearest coarse cell and the next one (source/Prolong_Interpolate.cpp:90-119): for an odd
    // fine index n, (n+1)/2 and (n-1)/2; for an even one, n/2 and n/2+1
    const int ia1 = (i + 1) >> 1, ia2 = (i & 1) ? (i - 1) >> 1 : (i >> 1) + 1;
    const int ja1 = (j + 1) >> 1, ja2 = (j & 1) ? (j - 1) >> 1 : (j >> 1) + 1;
    const int ka1 = (k + 1) >> 1, ka2 = (k & 1) ? (k - 1) >> 1 : (k >> 1) + 1;
    const long long c111 = ix(C, ia1, ja1, ka1), c112 = ix(C, ia1, ja1, ka2), c121 = ix(C, ia1, ja2, ka1),
                    c211 = ix(C, ia2, ja1, ka1), c221 = ix(C, ia2, ja2, ka1), c122 = ix(C, ia1, ja2, ka2),
                    c212 = ix(C, ia2, ja1, ka2), c222 = ix(C, ia2, ja2, ka2);
    const double a1 = 27.0 / 64.0, a2 = 9.0 / 64.0, a3 = 3.0 / 64.0, a4 = 1.0 / 64.0;
    const long long p = ix(F, i, j, k);
#pragma unroll
    for (int c = 0; c < NQ; c++) {
        double v;
        if (init) {
            const double *q = Wc.cv[c];
            v = a1 * q[c111] + a2 * (q[c112] + q[c121] + q[c211]) + a3 * (q[c221] + q[c122] + q[c212]) + a4 * q[c222];
            Wf.cv[c][p] = v;
        } else {
            const T *q = Wc.dq2h[c];
            if constexpr (sizeof(T) == 4) {
                // mixed form: the correction is summed in FP32 (the weights are exact there) and
                // accumulated into the FP64 Q
                const T w = (T)a1 * q[c111] + (T)a2 * (q[c112] + q[c121] + q[c211]) +
                            (T)a3 * (q[c221] + q[c122] + q[c212]) + (T)a4 * q[c222];
                v = (double)w;
            } else {
                v = a1 * (double)q[c111] + a2 * ((double)q[c112] + (double)q[c121] + (double)q[c211]) +
                    a3 * ((double)q[c221] + (double)q[c122] + (double)q[c212]) + a4 * (double)q[c222];
            }
            Wf.cv[c][p] = Wf.cv[c][p] + v;
        }
    }
}

template <typename T>
void launch_restrict(const LaunchCtx &cf, const LaunchCtx &cc, const Geo &Gf, const Geo &Gc, Flow<T> Ff, Flow<T> Fc)
{
    k_restrict<T><<<cc.grid_cells(256), 256, 0, cc.stream>>>(cf.batch, cc.batch, Gf, Gc, Ff, Fc);
}
template <typename T>
void launch_forcing(const LaunchCtx &cc, Flow<T> Fc)
{
    k_forcing<T><<<cc.grid_cells(256), 256, 0, cc.stream>>>(cc.batch, Fc);
}
template <typename T>
void launch_forcing_keep(const LaunchCtx &cc, Flow<T> Fc)
{
    k_forcing_keep<T><<<cc.grid_cells(256), 256, 0, cc.stream>>>(cc.batch, Fc);
}
template <typename T>
void launch_add_forcing(const LaunchCtx &cc, Flow<T> Fc)
{
    k_add_forcing<T><<<cc.grid_cells(256), 256, 0, cc.stream>>>(cc.batch, Fc);
}
template <typename T>
void launch_delta(const LaunchCtx &cc, Flow<T> Fc)
{
    k_delta<T><<<cc.grid_cells(256), 256, 0, cc.stream>>>(cc.batch, Fc);
}
template <typename T>
void launch_corner(const LaunchCtx &cc, Flow<T> Fc)
{
    const int mx = std::max(cc.maxIM, std::max(cc.maxJM, cc.maxKM));
    k_edges<T><<<dim3((mx + 63) / 64, 12, cc.batch.nsolve), 64, 0, cc.stream>>>(cc.batch, Fc);
    k_corners<T><<<cc.batch.nsolve, 64, 0, cc.stream>>>(cc.batch, Fc);
}
template <typename T>
void launch_interpolate(const LaunchCtx &cf, const LaunchCtx &cc, Flow<T> Ff, Flow<T> Fc, int init)
{
    k_interpolate<T><<<cf.grid_cells(256), 256, 0, cf.stream>>>(cf.batch, cc.batch, Ff, Fc, init);
}

#define GBT_INST(T)                                                                                                       \
    template void launch_restrict<T>(const LaunchCtx &, const LaunchCtx &, const Geo &, const Geo &, Flow<T>, Flow<T>); \
    template void launch_forcing<T>(const LaunchCtx &, Flow<T>);                                                         \
    template void launch_forcing_keep<T>(const LaunchCtx &, Flow<T>);                                                    \
    template void launch_add_forcing<T>(const LaunchCtx &, Flow<T>);                                                     \
    template void launch_delta<T>(const LaunchCtx &, Flow<T>);                                                           \
    template void launch_corner<T>(const LaunchCtx &, Flow<T>);                                                          \
    template void launch_interpolate<T>(const LaunchCtx &, const LaunchCtx &, Flow<T>, Flow<T>, int);
GBT_INST(double)
GBT_INST(float)

}  // namespace gbt
