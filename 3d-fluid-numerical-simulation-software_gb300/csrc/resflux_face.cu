// Face stage of the residual: one thread per face computes the convective flux (4-cell stencil
// with the dummy-layer switch of source/Upwind_Convective.cpp:38-97, reconstruction, Roe or
// Steger-Warming in the face frame, rotation back, times |S|; on wall faces the wall flux of
// source/WallFlux.cpp:70-175 instead) and the viscous flux from the face gradients
// (source/Spectral_curl_grad.cpp:85-493, source/ViscousFlux.cpp:9-269). The cell stage sums the
// face fluxes, subtracts the rotation source and forms the residual
// (source/ComputeAllBlockVars.cpp:73-119,223-255, source/ViscousFlux.cpp:271-281).
#include "gbt_common.cuh"
#include "kernels.hpp"
#include "flux.cuh"
#include "face_body.cuh"

namespace gbt {

// one thread per face of family F, inputs read from the padded boxes in HBM
template <typename T, int F, int MODE>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 8 : 4) k_face(Batch B, Phys P, PhysW<T> PC, GeoW<T> G, Flow<T> W, const DevWall *walls)
{
    const int s = blockIdx.y;
    const Lvl L = B.lv[s];
    int ni, nj, nk, i, j, k;
    face_extent(L, F, ni, nj, nk);
    if (!box_index(ni, nj, nk, i, j, k)) return;
    const int p = (int)ix(L, i, j, k);
    const int sI = L.NJ * L.NK, sJ = L.NK, sK = 1;
    FaceGeo<T> g;
#pragma unroll
    for (int c = 0; c < 3; c++) { g.S[c] = G.S[F][c]; g.nrm[c] = G.nrm[F][c]; g.t1[c] = G.t1[F][c]; g.t2[c] = G.t2[F][c]; }
    g.s = G.s[F];
    g.qe = G.qe[F];
#pragma unroll
    for (int c = 0; c < 9; c++) g.m[c] = G.m[F][c];
    g.q = p;
    const int wq = W.wallf[F][p];
    const bool central = !MODE && P.scheme == 100;
    T rot = (T)0, cx = (T)0, cy = (T)0;
    if (wq || central) {
        rot = wq ? (walls[wq - 1].rotate ? (T)B.sc[s].w_rot : (T)0) : (T)B.sc[s].w_rot;
        cx = G.c[F][0][p];
        cy = G.c[F][1][p];
    }
    CellSrc<T> C;
#pragma unroll
    for (int c = 0; c < NPV; c++) C.pv[c] = W.pv[c];
    C.mut = W.mut;
    T out[10];
    face_body<T, F, MODE>(P, PC, C, W.cv, p, sI, sJ, sK, i, j, k, L.IM, L.JM, L.KM, g, wq, rot, cx, cy, out);
    // the flux is stored after every load of the viscous part
#pragma unroll
    for (int c = 0; c < NQ; c++) W.Ff[F][c][p] = out[c];
    if (!P.equation_ns) return;
#pragma unroll
    for (int c = 0; c < NQ; c++) W.Vf[F][c][p] = out[5 + c];
}

// JST artificial dissipation (source/JST_Dissip.cpp:5-431). Positions along a grid line follow
// the reference's switch between cells and reconstruction layers (position c <= 0 is dummy layer
// 1 - c, c >= N dummy layer c - N + 1), which in the padded box is index c - 1 / c + 1.
__device__ __forceinline__ int jst_pos(int c, int NN) { return c <= 0 ? c - 1 : (c >= NN ? c + 1 : c); }

// pressure sensor of every position -1 .. N + 1 of every line of direction F (sensorI/J/K, :5-190);
// the k-direction sensor's range check compares j with KM, as the reference's does
template <typename T, int F>
__global__ void __launch_bounds__(256) k_jst_sensor(Batch B, Flow<T> W)
{
    const Lvl L = B.lv[blockIdx.y];
    const int NN = F == 0 ? L.IM : (F == 1 ? L.JM : L.KM);
    const int n1 = F == 0 ? L.JM - 1 : L.IM - 1, n2 = F == 2 ? L.JM - 1 : L.KM - 1;
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned np = (unsigned)(NN + 3);
    if (t >= np * (unsigned)n1 * (unsigned)n2) return;
    const int c = (int)(t % np) - 1;
    const unsigned r = t / np;
    const int a1 = 1 + (int)(r % (unsigned)n1), a2 = 1 + (int)(r / (unsigned)n1);
    int i, j, k;
    if (F == 0) { j = a1; k = a2; i = 0; }
    else if (F == 1) { i = a1; k = a2; j = 0; }
    else { i = a1; j = a2; k = 0; }
    const long long sn = F == 0 ? (long long)L.NJ * L.NK : (F == 1 ? (long long)L.NK : 1LL);
    const long long p0 = ix(L, i, j, k);
    T v = (T)0;
    if (!(F == 2 && j > L.KM)) {
        const T pf = W.pv[PP][p0 + jst_pos(c + 1, NN) * sn], pc = W.pv[PP][p0 + jst_pos(c, NN) * sn],
                pb = W.pv[PP][p0 + jst_pos(c - 1, NN) * sn];
        v = fabs((pf - (T)2 * pc + pb) / (pf + (T)2 * pc + pb));
    }
    W.jsens[F][p0 + jst_pos(c, NN) * sn] = v;
}

// anisotropy-weighted spectral radius phi * lambda of every cell and direction (:198-216); the
// two other directions in the reference's order of the sum: I faces J, K; J faces I, K; K faces J, I
template <typename T>
__global__ void __launch_bounds__(256) k_jst_weights(Batch B, Flow<T> W)
{
    const Lvl L = B.lv[blockIdx.y];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
    const T ex = (T)(double)0.4f;
    const T l0 = W.lamc[0][p], l1 = W.lamc[1][p], l2 = W.lamc[2][p];
    W.jva[0][p] = ((T)1 + pow(l1 / l0, ex) + pow(l2 / l0, ex)) * l0;
    W.jva[1][p] = ((T)1 + pow(l0 / l1, ex) + pow(l2 / l1, ex)) * l1;
    W.jva[2][p] = ((T)1 + pow(l1 / l2, ex) + pow(l0 / l2, ex)) * l2;
}

// dissipation of one face: blended second and fourth differences of Q (:193-413)
template <typename T, int F>
__global__ void __launch_bounds__(128) k_jst_dissip(Batch B, Phys P, Flow<T> W)
{
    const int s = blockIdx.y;
    const Lvl L = B.lv[s];
    int ni, nj, nk, i, j, k;
    face_extent(L, F, ni, nj, nk);
    if (!box_index(ni, nj, nk, i, j, k)) return;
    const long long p = ix(L, i, j, k);
    const long long sn = F == 0 ? (long long)L.NJ * L.NK : (F == 1 ? (long long)L.NK : 1LL);
    const int NN = F == 0 ? L.IM : (F == 1 ? L.JM : L.KM);
    const int a = F == 0 ? i : (F == 1 ? j : k);
    const long long p0 = p - (long long)a * sn;
    const long long c1 = p0 + jst_pos(a + 1, NN) * sn, c2 = p0 + jst_pos(a, NN) * sn, c3 = p0 + jst_pos(a - 1, NN) * sn,
                    c4 = p0 + jst_pos(a - 2, NN) * sn;
    const T *sen = W.jsens[F];
    const T e2 = (T)P.k2 * fmax(fmax(sen[c1], sen[c2]), fmax(sen[c3], sen[c4]));
    const T e4 = fmax((T)0, (T)P.k4 - e2);
    T alpha;
    if (a == 1) alpha = W.jva[F][p];
    else if (a == NN) alpha = W.jva[F][p - sn];
    else alpha = (T)0.5 * (W.jva[F][p] + W.jva[F][p - sn]);
    T d[NQ];
#pragma unroll
    for (int c = 0; c < NQ; c++) {
        const T q1 = (T)W.cv[c][c1], q2 = (T)W.cv[c][c2], q3 = (T)W.cv[c][c3], q4 = (T)W.cv[c][c4];
        d[c] = alpha * (e2 * (q2 - q3) - e4 * (q1 - (T)3 * q2 + (T)3 * q3 - q4));
    }
#pragma unroll
    for (int c = 0; c < NQ; c++) W.Fd[F][c][p] = d[c];
}

// face sums, rotation source, residual R = Fc - Fv (- Fd with JST). The viscous and dissipation
// terms are compile-time switches (NS, JST), so that every load of a cell is issued before the
// first sum instead of behind a branch.
template <typename T, bool NS, bool JST>
__global__ void __launch_bounds__(256) k_cell_sum(Batch B, GeoW<T> G, Flow<T> W)
{
    const int s = blockIdx.y;
    const Lvl L = B.lv[s];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
    const long long pI = p + (long long)L.NJ * L.NK, pJ = p + L.NK, pK = p + 1;
    const T w = (T)B.sc[s].w_rot;
    const T rv = W.pv[PD][p] * G.vol[p];
    T src[5] = {(T)0, rv * (w * W.pv[PV][p]), -(rv * (w * W.pv[PU][p])), (T)0, (T)0};
    T r[NQ];                                   // all loads first, then the stores
#pragma unroll
    for (int c = 0; c < NQ; c++) {
        T fc = W.Ff[0][c][pI] - W.Ff[0][c][p] + W.Ff[1][c][pJ] - W.Ff[1][c][p] + W.Ff[2][c][pK] - W.Ff[2][c][p] - src[c];
        T fv = (T)0;
        if constexpr (NS)
            fv = W.Vf[0][c][pI] - W.Vf[0][c][p] + W.Vf[1][c][pJ] - W.Vf[1][c][p] + W.Vf[2][c][pK] - W.Vf[2][c][p];
        r[c] = fc - fv;
        if constexpr (JST)
            r[c] = r[c] - (W.Fd[0][c][pI] - W.Fd[0][c][p] + W.Fd[1][c][pJ] - W.Fd[1][c][p] + W.Fd[2][c][pK] - W.Fd[2][c][p]);
    }
#pragma unroll
    for (int c = 0; c < NQ; c++) W.res[c][p] = r[c];
}

template <typename T>
void launch_cell_stages(const LaunchCtx &ctx, const Phys &P, const PhysW<T> &PC, const Geo &G, const GeoW<T> &GW,
                        Flow<T> W, const BcTables &bc, int level, T *scratch);

template <typename T>
void launch_resflux(const LaunchCtx &ctx, const Phys &P, const PhysW<T> &PC, const Geo &G, const GeoW<T> &GW, Flow<T> W,
                    const BcTables &bc, int level, T *scratch)
{
    const int nbc = (bc.n_inlet > 0) + 3 * (bc.n_outlet > 0) + (bc.n_wall > 0) + (bc.n_per > 0);
    ctx.mark("boundary", 1, nbc);
    launch_boundary<T>(ctx, P, G, W, bc);
    ctx.mark("boundary", 0, nbc);
    launch_cell_stages<T>(ctx, P, PC, G, GW, W, bc, level, scratch);
    const Batch &B = ctx.batch;
    ctx.mark("face_flux", 1, 3);
    bool staged = false;
    if constexpr (sizeof(T) == 4) {
        if (ctx.face_tma && P.recon_var == 200 && P.recon == 500 && P.scheme == 300) {
            launch_face_tma(ctx, P, PC, GW, W, bc.wall);
            staged = true;
        }
    }
    if (staged) {
    } else if (P.recon_var == 200 && P.recon == 500 && P.scheme == 300) {
        k_face<T, 0, 1><<<ctx.grid_faces(0, 128), 128, 0, ctx.stream>>>(B, P, PC, GW, W, bc.wall);
        k_face<T, 1, 1><<<ctx.grid_faces(1, 128), 128, 0, ctx.stream>>>(B, P, PC, GW, W, bc.wall);
        k_face<T, 2, 1><<<ctx.grid_faces(2, 128), 128, 0, ctx.stream>>>(B, P, PC, GW, W, bc.wall);
    } else {
        k_face<T, 0, 0><<<ctx.grid_faces(0, 128), 128, 0, ctx.stream>>>(B, P, PC, GW, W, bc.wall);
        k_face<T, 1, 0><<<ctx.grid_faces(1, 128), 128, 0, ctx.stream>>>(B, P, PC, GW, W, bc.wall);
        k_face<T, 2, 0><<<ctx.grid_faces(2, 128), 128, 0, ctx.stream>>>(B, P, PC, GW, W, bc.wall);
    }
    ctx.mark("face_flux", 0, 3);
    if (P.scheme == 100) {
        ctx.mark("jst_dissipation", 1, 7);
        const long long ls0 = (long long)(ctx.maxIM + 3) * (ctx.maxJM - 1) * (ctx.maxKM - 1);
        const long long ls1 = (long long)(ctx.maxJM + 3) * (ctx.maxIM - 1) * (ctx.maxKM - 1);
        const long long ls2 = (long long)(ctx.maxKM + 3) * (ctx.maxIM - 1) * (ctx.maxJM - 1);
        k_jst_sensor<T, 0><<<ctx.grid_n(ls0, 256), 256, 0, ctx.stream>>>(B, W);
        k_jst_sensor<T, 1><<<ctx.grid_n(ls1, 256), 256, 0, ctx.stream>>>(B, W);
        k_jst_sensor<T, 2><<<ctx.grid_n(ls2, 256), 256, 0, ctx.stream>>>(B, W);
        k_jst_weights<T><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, W);
        k_jst_dissip<T, 0><<<ctx.grid_faces(0, 128), 128, 0, ctx.stream>>>(B, P, W);
        k_jst_dissip<T, 1><<<ctx.grid_faces(1, 128), 128, 0, ctx.stream>>>(B, P, W);
        k_jst_dissip<T, 2><<<ctx.grid_faces(2, 128), 128, 0, ctx.stream>>>(B, P, W);
        ctx.mark("jst_dissipation", 0, 7);
    }
    ctx.mark("cell_sum", 1);
    const bool jst = W.Fd[0][0] != nullptr;
    if (P.equation_ns && !jst) k_cell_sum<T, true, false><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, GW, W);
    else if (P.equation_ns) k_cell_sum<T, true, true><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, GW, W);
    else if (!jst) k_cell_sum<T, false, false><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, GW, W);
    else k_cell_sum<T, false, true><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, GW, W);
    ctx.mark("cell_sum", 0);
}

template void launch_resflux<double>(const LaunchCtx &, const Phys &, const PhysW<double> &, const Geo &,
                                     const GeoW<double> &, Flow<double>, const BcTables &, int, double *);
template void launch_resflux<float>(const LaunchCtx &, const Phys &, const PhysW<float> &, const Geo &,
                                    const GeoW<float> &, Flow<float>, const BcTables &, int, float *);

}  // namespace gbt
