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

namespace gbt {

template <typename T>
__device__ __forceinline__ P6<T> ld_pv(const Flow<T> &W, long long p)
{
    P6<T> q = {W.pv[PD][p], W.pv[PU][p], W.pv[PV][p], W.pv[PW][p], W.pv[PP][p], W.pv[PT][p]};
    return q;
}
template <typename T>
__device__ __forceinline__ C5<T> ld_cv(const Flow<T> &W, long long p)
{
    C5<T> q = {(T)W.cv[0][p], (T)W.cv[1][p], (T)W.cv[2][p], (T)W.cv[3][p], (T)W.cv[4][p]};
    return q;
}

// tangential difference of component c across a face of family F along tangential direction
// DT: mean of the four cells on the + side minus mean of the four on the - side, leaving out the
// ghost corner cell where the face is on the block boundary and the line ends
// (source/Spectral_curl_grad.cpp:115-203 and the J/K counterparts, including the extra 0.25 of
// :311-314 on J faces at j = JM, k = 1).
template <typename T, int F, int DT>
__device__ __forceinline__ T tan_diff(const T *__restrict__ c, long long p, long long sn, long long st, int a, int NN,
                                      int b, int TT)
{
    // cells: (0,0)=p, (-1,0)=p-sn, (0,+1)=p+st, (-1,+1)=p-sn+st, (0,-1)=p-st, (-1,-1)=p-sn-st
    const T c00 = c[p], cm0 = c[p - sn];
    const T c0p = c[p + st], cmp = c[p - sn + st], c0m = c[p - st], cmm = c[p - sn - st];
    T plus, minus;
    const bool lo_n = (a == 1), hi_n = (a == NN), lo_t = (b == 1), hi_t = (b == TT - 1);
    if (lo_n && hi_t) plus = (c00 + c0p + cm0) / (T)3;                 // no (-1,+1)
    else if (hi_n && hi_t) plus = (c00 + cmp + cm0) / (T)3;            // no (0,+1)
    else plus = (T)0.25 * (c00 + c0p + cmp + cm0);
    if (lo_n && lo_t) minus = (c00 + cm0 + c0m) / (T)3;                // no (-1,-1)
    else if (hi_n && lo_t) {
        minus = (c00 + cm0 + cmm) / (T)3;                               // no (0,-1)
        if (F == 1 && DT == 2) minus = (T)0.25 * minus;
    } else minus = (T)0.25 * (c00 + cm0 + cmm + c0m);
    return plus - minus;
}

// MODE 1 is the default scheme (MUSCL3 on primitive variables, Roe) with the option switches
// resolved at compile time; MODE 0 reads them from P
template <typename T, int F, int MODE>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 8 : 4) k_face(Batch B, Phys P, PhysW<T> PC, GeoW<T> G, Flow<T> W, const DevWall *walls)
{
    const int recon_var = MODE ? 200 : P.recon_var, recon = MODE ? 500 : P.recon, scheme = MODE ? 300 : P.scheme;
    const int s = blockIdx.y;
    const Lvl L = B.lv[s];
    int ni, nj, nk, i, j, k;
    face_extent(L, F, ni, nj, nk);
    if (!box_index(ni, nj, nk, i, j, k)) return;
    const long long p = ix(L, i, j, k);
    const long long sI = (long long)L.NJ * L.NK, sJ = L.NK, sK = 1;
    const long long sn = F == 0 ? sI : (F == 1 ? sJ : sK);
    const int NN = F == 0 ? L.IM : (F == 1 ? L.JM : L.KM);
    const int a = F == 0 ? i : (F == 1 ? j : k);
    const T gamma = PC.gamma, g1 = PC.gm1;
    const T Sx = G.S[F][0][p], Sy = G.S[F][1][p], Sz = G.S[F][2][p];
    const int wq = W.wallf[F][p];
    T f0, f1, f2, f3, f4;
    if (wq || (!MODE && scheme == 100)) {
        // wall face: flux from the face average of ghost and interior, in the wall's frame
        // (source/WallFlux.cpp:70-175); the JST central flux has the same form in the block's
        // frame (source/JST_Convective.cpp:53-95)
        const T rot = wq ? (walls[wq - 1].rotate ? (T)B.sc[s].w_rot : (T)0) : (T)B.sc[s].w_rot;
        const long long m = p - sn;
        const P6<T> A = ld_pv(W, p), Bq = ld_pv(W, m);
        const T d = (T)0.5 * (A.d + Bq.d), u = (T)0.5 * (A.u + Bq.u), v = (T)0.5 * (A.v + Bq.v),
                w = (T)0.5 * (A.w + Bq.w), pr = (T)0.5 * (A.p + Bq.p);
        const T ue = -G.c[F][1][p] * rot, ve = G.c[F][0][p] * rot;
        const T Vna = u * Sx + v * Sy + w * Sz, Vne = ue * Sx + ve * Sy;
        const T e = pr / g1 + d * (u * u + v * v + w * w) / (T)2;
        const T dv = Vna - Vne;
        f0 = d * dv; f1 = d * u * dv + pr * Sx; f2 = d * v * dv + pr * Sy; f3 = d * w * dv + pr * Sz;
        f4 = (e + pr) * dv + pr * Vne;
    } else {
        // stencil FF, F, B, BB along the face normal; the first ghost layer is skipped in favour of
        // the reconstruction layers
        const long long p0 = p - (long long)a * sn;
        auto rm = [NN](int c) { return c <= 0 ? c - 1 : (c >= NN ? c + 1 : c); };
        const long long q0 = p0 + rm(a - 2) * sn, q1 = p0 + rm(a - 1) * sn, q2 = p0 + rm(a) * sn, q3 = p0 + rm(a + 1) * sn;
        C5<T> cl, cr;
        if (recon_var == 100) recon_cons(recon, gamma, ld_cv(W, q0), ld_cv(W, q1), ld_cv(W, q2), ld_cv(W, q3), cl, cr);
        else recon_prim(recon, gamma, ld_pv(W, q0), ld_pv(W, q1), ld_pv(W, q2), ld_pv(W, q3), cl, cr);
        const T nx = G.nrm[F][0][p], ny = G.nrm[F][1][p], nz = G.nrm[F][2][p];
        const T ax = G.t1[F][0][p], ay = G.t1[F][1][p], az = G.t1[F][2][p];
        const T bx = G.t2[F][0][p], by = G.t2[F][1][p], bz = G.t2[F][2][p];
        C5<T> QL = {cl.d, cl.mx * nx + cl.my * ny + cl.mz * nz, cl.mx * ax + cl.my * ay + cl.mz * az,
                    cl.mx * bx + cl.my * by + cl.mz * bz, cl.e};
        C5<T> QR = {cr.d, cr.mx * nx + cr.my * ny + cr.mz * nz, cr.mx * ax + cr.my * ay + cr.mz * az,
                    cr.mx * bx + cr.my * by + cr.mz * bz, cr.e};
        const T qe = G.qe[F][p];
        C5<T> Fc;
        if (scheme == 300) Fc = roe(gamma, QL, QR, qe);
        else {
            C5<T> fp = sw_half(gamma, QL, qe, (T)1), fm = sw_half(gamma, QR, qe, (T)-1);
            Fc.d = fp.d + fm.d; Fc.mx = fp.mx + fm.mx; Fc.my = fp.my + fm.my; Fc.mz = fp.mz + fm.mz; Fc.e = fp.e + fm.e;
        }
        const T sa = G.s[F][p];
        f0 = Fc.d * sa;
        f1 = (Fc.mx * nx + Fc.my * ax + Fc.mz * bx) * sa;
        f2 = (Fc.mx * ny + Fc.my * ay + Fc.mz * by) * sa;
        f3 = (Fc.mx * nz + Fc.my * az + Fc.mz * bz) * sa;
        f4 = Fc.e * sa;
    }
    // the flux is stored after every load of the viscous part (the compiler cannot move those loads
    // above a store to memory it cannot tell apart)
    if (!P.equation_ns) {
        W.Ff[F][0][p] = f0; W.Ff[F][1][p] = f1; W.Ff[F][2][p] = f2; W.Ff[F][3][p] = f3; W.Ff[F][4][p] = f4;
        return;
    }

    // ---- viscous flux ----
    const int iD1 = F == 0 ? 1 : 0, iD2 = F == 2 ? 1 : 2;   // tangential directions (kesi/yita/zita order)
    const long long st1 = iD1 == 0 ? sI : sJ, st2 = iD2 == 1 ? sJ : sK;
    const int b1 = iD1 == 0 ? i : j, T1 = iD1 == 0 ? L.IM : L.JM;
    const int b2 = iD2 == 1 ? j : k, T2 = iD2 == 1 ? L.JM : L.KM;
    T dn[4], d1[4], d2[4];
    const int comp[4] = {PU, PV, PW, PT};
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const T *c = W.pv[comp[q]];
        dn[q] = c[p] - c[p - sn];
        d1[q] = tan_diff<T, F, (F == 0 ? 1 : 0)>(c, p, sn, st1, a, NN, b1, T1);
        d2[q] = tan_diff<T, F, (F == 2 ? 1 : 2)>(c, p, sn, st2, a, NN, b2, T2);
    }
    // derivatives along kesi, yita, zita
    T dk[4], de[4], dz[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        if (F == 0) { dk[q] = dn[q]; de[q] = d1[q]; dz[q] = d2[q]; }
        else if (F == 1) { dk[q] = d1[q]; de[q] = dn[q]; dz[q] = d2[q]; }
        else { dk[q] = d1[q]; de[q] = d2[q]; dz[q] = dn[q]; }
    }
    const T m0 = G.m[F][0][p], m1 = G.m[F][1][p], m2 = G.m[F][2][p], m3 = G.m[F][3][p], m4 = G.m[F][4][p],
            m5 = G.m[F][5][p], m6 = G.m[F][6][p], m7 = G.m[F][7][p], m8 = G.m[F][8][p];
    T gx[4], gy[4], gz[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        gx[q] = dk[q] * m0 + de[q] * m3 + dz[q] * m6;
        gy[q] = dk[q] * m1 + de[q] * m4 + dz[q] * m7;
        gz[q] = dk[q] * m2 + de[q] * m5 + dz[q] * m8;
    }
    const long long m = p - sn;
    const T h = (T)0.5;
    const T uf = h * (W.pv[PU][p] + W.pv[PU][m]), vf = h * (W.pv[PV][p] + W.pv[PV][m]);
    const T wf = h * (W.pv[PW][p] + W.pv[PW][m]), tf = h * (W.pv[PT][p] + W.pv[PT][m]);
    const T mul = sutherland(PC, tf);
    const T gR = gamma * PC.rgas / g1;
    T mu = mul, cond = mul * gR / PC.pr_lam;
    if (P.turb_bl || P.turb_sa) {
        const T mt = (W.mut[m] + W.mut[p]) / (T)2;
        mu = mul + mt;
        cond = cond + mt * gR / PC.pr_tur;
    }
    const T c43 = (T)(double)(4.0f / 3.0f), c23 = (T)(double)(2.0f / 3.0f);
    const T txx = mu * (c43 * gx[0] - c23 * (gy[1] + gz[2]));
    const T txy = mu * (gy[0] + gx[1]);
    const T txz = mu * (gz[0] + gx[2]);
    const T tyy = mu * (c43 * gy[1] - c23 * (gx[0] + gz[2]));
    const T tyz = mu * (gz[1] + gy[2]);
    const T tzz = mu * (c43 * gz[2] - c23 * (gx[0] + gy[1]));
    const T qx = uf * txx + vf * txy + wf * txz + cond * gx[3];
    const T qy = uf * txy + vf * tyy + wf * tyz + cond * gy[3];
    const T qz = uf * txz + vf * tyz + wf * tzz + cond * gz[3];
    W.Ff[F][0][p] = f0; W.Ff[F][1][p] = f1; W.Ff[F][2][p] = f2; W.Ff[F][3][p] = f3; W.Ff[F][4][p] = f4;
    W.Vf[F][0][p] = (T)0;
    W.Vf[F][1][p] = txx * Sx + txy * Sy + txz * Sz;
    W.Vf[F][2][p] = txy * Sx + tyy * Sy + tyz * Sz;
    W.Vf[F][3][p] = txz * Sx + tyz * Sy + tzz * Sz;
    W.Vf[F][4][p] = qx * Sx + qy * Sy + qz * Sz;
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

// face sums, rotation source, residual R = Fc - Fv (- Fd with JST)
template <typename T>
__global__ void __launch_bounds__(256) k_cell_sum(Batch B, Phys P, GeoW<T> G, Flow<T> W)
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
        if (P.equation_ns)
            fv = W.Vf[0][c][pI] - W.Vf[0][c][p] + W.Vf[1][c][pJ] - W.Vf[1][c][p] + W.Vf[2][c][pK] - W.Vf[2][c][p];
        r[c] = fc - fv;
        if (W.Fd[0][0])
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
    if (P.recon_var == 200 && P.recon == 500 && P.scheme == 300) {
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
    k_cell_sum<T><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, P, GW, W);
    ctx.mark("cell_sum", 0);
}

template void launch_resflux<double>(const LaunchCtx &, const Phys &, const PhysW<double> &, const Geo &,
                                     const GeoW<double> &, Flow<double>, const BcTables &, int, double *);
template void launch_resflux<float>(const LaunchCtx &, const Phys &, const PhysW<float> &, const Geo &,
                                    const GeoW<float> &, Flow<float>, const BcTables &, int, float *);

}  // namespace gbt
