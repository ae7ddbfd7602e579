// Arithmetic of one face of the face stage (convective flux from the 4-cell stencil with the
// dummy-layer switch of source/Upwind_Convective.cpp:38-97, reconstruction, Roe or
// Steger-Warming in the face frame, rotation back, times |S|; on wall faces the wall flux of
// source/WallFlux.cpp:70-175; then the viscous flux from the face gradients of
// source/Spectral_curl_grad.cpp:85-493 and source/ViscousFlux.cpp:9-269), written once for the
// two ways the face stage reads its inputs: straight from the padded boxes in HBM (k_face) and from
// a tile staged in shared memory by the tensor memory accelerator (k_face_tma). Cells are addressed
// as base index + offsets with the strides of whichever array holds them. Indices are 32-bit: a
// level's pool holds fewer than 2^31 cells of every field (the solver refuses larger batches).
#pragma once
#include "gbt_common.cuh"
#include "flux.cuh"

namespace gbt {

// where the face stage reads the per-face geometry (area vector, |S|, face frame, entrainment
// speed, metric coefficients): arrays and the face's index in them, read where the arithmetic
// needs each value
template <typename T> struct FaceGeo {
    const T *S[3], *s, *nrm[3], *t1[3], *t2[3], *qe, *m[9];
    int q;
};

// cell fields the face stage reads: the six primitive variables and mu_t (or the conserved
// variables for conservative reconstruction, read from the FP64 boxes by the plain form only)
template <typename T> struct CellSrc {
    const T *pv[NPV];
    const T *mut;
};

template <typename T>
__device__ __forceinline__ P6<T> ld_p6(const CellSrc<T> &C, int q)
{
    P6<T> v = {C.pv[PD][q], C.pv[PU][q], C.pv[PV][q], C.pv[PW][q], C.pv[PP][q], C.pv[PT][q]};
    return v;
}

// tangential difference of component c across a face of family F along tangential direction
// DT: mean of the four cells on the + side minus mean of the four on the - side, leaving out the
// ghost corner cell where the face is on the block boundary and the line ends
// (source/Spectral_curl_grad.cpp:115-203 and the J/K counterparts, including the extra 0.25 of
// :311-314 on J faces at j = JM, k = 1).
template <typename T, int F, int DT>
__device__ __forceinline__ T tan_diff(const T *__restrict__ c, int p, int sn, int st, int a, int NN,
                                      int b, int TT)
{
    // cells: (0,0)=p, (-1,0)=p-sn, (0,+1)=p+st, (-1,+1)=p-sn+st, (0,-1)=p-st, (-1,-1)=p-sn-st
    const T c00 = c[p], cm0 = c[p - sn];
    const T c0p = c[p + st], cmp = c[p - sn + st], c0m = c[p - st], cmm = c[p - sn - st];
    const bool lo_n = (a == 1), hi_n = (a == NN), lo_t = (b == 1), hi_t = (b == TT - 1);
    // away from the corners both means hold the two cells across the face, which cancel: in exact
    // arithmetic the reference's difference of means is 1/4 of the difference of the remaining
    // pairs, which is formed here without the rounding of the cancelled terms
    if (!((lo_n || hi_n) && (lo_t || hi_t))) return (T)0.25 * ((c0p + cmp) - (cmm + c0m));
    const T third = (T)(1.0 / 3.0);
    T plus, minus;
    if (lo_n && hi_t) plus = (c00 + c0p + cm0) * third;                // no (-1,+1)
    else if (hi_n && hi_t) plus = (c00 + cmp + cm0) * third;           // no (0,+1)
    else plus = (T)0.25 * (c00 + c0p + cmp + cm0);
    if (lo_n && lo_t) minus = (c00 + cm0 + c0m) * third;               // no (-1,-1)
    else if (hi_n && lo_t) {
        minus = (c00 + cm0 + cmm) * third;                              // no (0,-1)
        if (F == 1 && DT == 2) minus = (T)0.25 * minus;
    } else minus = (T)0.25 * (c00 + cm0 + cmm + c0m);
    return plus - minus;
}

// Fluxes of one face of family F at node indices (i, j, k) of a block with node counts (IM, JM, KM).
// p: the face's + side cell in C's index space, strides sI, sJ, sK there; g: the face's geometry;
// wq: its wall patch (1-based) or 0; rot: rotation speed of the frame of the wall flux (the wall's
// own, or the block's for the JST central flux); cx, cy: the face centre (read on wall faces and
// by the central flux only). out[0..4]: convective flux, out[5..9]: viscous flux.
// MODE 1 is the default scheme (MUSCL3 on primitive variables, Roe) with the option switches
// resolved at compile time; MODE 0 reads them from P (conservative reconstruction reads cv, the
// FP64 conserved variables, through the plain form's global indices).
template <typename T, int F, int MODE>
__device__ __forceinline__ void face_body(const Phys &P, const PhysW<T> &PC, const CellSrc<T> &C, const double *const *cv,
                                          int p, int sI, int sJ, int sK, int i, int j, int k,
                                          int IM, int JM, int KM, const FaceGeo<T> &g, int wq, T rot, T cx, T cy, T out[10])
{
    const int recon_var = MODE ? 200 : P.recon_var, recon = MODE ? 500 : P.recon, scheme = MODE ? 300 : P.scheme;
    const int sn = F == 0 ? sI : (F == 1 ? sJ : sK);
    const int NN = F == 0 ? IM : (F == 1 ? JM : KM);
    const int a = F == 0 ? i : (F == 1 ? j : k);
    const T gamma = PC.gamma, g1 = PC.gm1;
    const T Sx = g.S[0][g.q], Sy = g.S[1][g.q], Sz = g.S[2][g.q];
    T f0, f1, f2, f3, f4;
    if (wq || (!MODE && scheme == 100)) {
        // wall face: flux from the face average of ghost and interior, in the wall's frame
        // (source/WallFlux.cpp:70-175); the JST central flux has the same form in the block's
        // frame (source/JST_Convective.cpp:53-95)
        const int m = p - sn;
        const P6<T> A = ld_p6(C, p), Bq = ld_p6(C, m);
        const T d = (T)0.5 * (A.d + Bq.d), u = (T)0.5 * (A.u + Bq.u), v = (T)0.5 * (A.v + Bq.v),
                w = (T)0.5 * (A.w + Bq.w), pr = (T)0.5 * (A.p + Bq.p);
        const T ue = -cy * rot, ve = cx * rot;
        const T Vna = u * Sx + v * Sy + w * Sz, Vne = ue * Sx + ve * Sy;
        const T e = pr * PC.rgm1 + d * (u * u + v * v + w * w) / (T)2;
        const T dv = Vna - Vne;
        f0 = d * dv; f1 = d * u * dv + pr * Sx; f2 = d * v * dv + pr * Sy; f3 = d * w * dv + pr * Sz;
        f4 = (e + pr) * dv + pr * Vne;
    } else {
        // stencil FF, F, B, BB along the face normal; the first ghost layer is skipped in favour of
        // the reconstruction layers
        const int p0 = p - a * sn;
        auto rm = [NN](int c) { return c <= 0 ? c - 1 : (c >= NN ? c + 1 : c); };
        const int q0 = p0 + rm(a - 2) * sn, q1 = p0 + rm(a - 1) * sn, q2 = p0 + rm(a) * sn, q3 = p0 + rm(a + 1) * sn;
        C5<T> cl, cr;
        if (!MODE && recon_var == 100) {
            auto ldc = [cv](int q) {
                C5<T> v = {(T)cv[0][q], (T)cv[1][q], (T)cv[2][q], (T)cv[3][q], (T)cv[4][q]};
                return v;
            };
            recon_cons(recon, gamma, ldc(q0), ldc(q1), ldc(q2), ldc(q3), cl, cr);
        } else {
            recon_prim(recon, PC.rgm1, ld_p6(C, q0), ld_p6(C, q1), ld_p6(C, q2), ld_p6(C, q3), cl, cr);
        }
        const T nx = g.nrm[0][g.q], ny = g.nrm[1][g.q], nz = g.nrm[2][g.q];
        const T ax = g.t1[0][g.q], ay = g.t1[1][g.q], az = g.t1[2][g.q];
        const T bx = g.t2[0][g.q], by = g.t2[1][g.q], bz = g.t2[2][g.q];
        C5<T> QL = {cl.d, cl.mx * nx + cl.my * ny + cl.mz * nz, cl.mx * ax + cl.my * ay + cl.mz * az,
                    cl.mx * bx + cl.my * by + cl.mz * bz, cl.e};
        C5<T> QR = {cr.d, cr.mx * nx + cr.my * ny + cr.mz * nz, cr.mx * ax + cr.my * ay + cr.mz * az,
                    cr.mx * bx + cr.my * by + cr.mz * bz, cr.e};
        const T qe = g.qe[g.q];
        C5<T> Fc;
        if (scheme == 300) Fc = roe(gamma, QL, QR, qe);
        else {
            C5<T> fp = sw_half(gamma, QL, qe, (T)1), fm = sw_half(gamma, QR, qe, (T)-1);
            Fc.d = fp.d + fm.d; Fc.mx = fp.mx + fm.mx; Fc.my = fp.my + fm.my; Fc.mz = fp.mz + fm.mz; Fc.e = fp.e + fm.e;
        }
        const T sa = g.s[g.q];
        f0 = Fc.d * sa;
        f1 = (Fc.mx * nx + Fc.my * ax + Fc.mz * bx) * sa;
        f2 = (Fc.mx * ny + Fc.my * ay + Fc.mz * by) * sa;
        f3 = (Fc.mx * nz + Fc.my * az + Fc.mz * bz) * sa;
        f4 = Fc.e * sa;
    }
    out[0] = f0; out[1] = f1; out[2] = f2; out[3] = f3; out[4] = f4;
    if (!P.equation_ns) return;

    // ---- viscous flux ----
    const int iD1 = F == 0 ? 1 : 0, iD2 = F == 2 ? 1 : 2;   // tangential directions (kesi/yita/zita order)
    const int st1 = iD1 == 0 ? sI : sJ, st2 = iD2 == 1 ? sJ : sK;
    const int b1 = iD1 == 0 ? i : j, T1 = iD1 == 0 ? IM : JM;
    const int b2 = iD2 == 1 ? j : k, T2 = iD2 == 1 ? JM : KM;
    T dn[4], d1[4], d2[4];
    const int comp[4] = {PU, PV, PW, PT};
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const T *c = C.pv[comp[q]];
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
    const int gq = g.q;
    const T m0 = g.m[0][gq], m1 = g.m[1][gq], m2 = g.m[2][gq], m3 = g.m[3][gq], m4 = g.m[4][gq], m5 = g.m[5][gq],
            m6 = g.m[6][gq], m7 = g.m[7][gq], m8 = g.m[8][gq];
    T gx[4], gy[4], gz[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        gx[q] = dk[q] * m0 + de[q] * m3 + dz[q] * m6;
        gy[q] = dk[q] * m1 + de[q] * m4 + dz[q] * m7;
        gz[q] = dk[q] * m2 + de[q] * m5 + dz[q] * m8;
    }
    const int m = p - sn;
    const T h = (T)0.5;
    const T uf = h * (C.pv[PU][p] + C.pv[PU][m]), vf = h * (C.pv[PV][p] + C.pv[PV][m]);
    const T wf = h * (C.pv[PW][p] + C.pv[PW][m]), tf = h * (C.pv[PT][p] + C.pv[PT][m]);
    const T mul = sutherland_face(PC, tf);
    T mu = mul, cond = mul * PC.cond_lam;
    if (P.turb_bl || P.turb_sa) {
        const T mt = (C.mut[m] + C.mut[p]) / (T)2;
        mu = mul + mt;
        cond = cond + mt * PC.cond_tur;
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
    out[5] = (T)0;
    out[6] = txx * Sx + txy * Sy + txz * Sz;
    out[7] = txy * Sx + tyy * Sy + tyz * Sz;
    out[8] = txz * Sx + tyz * Sy + tzz * Sz;
    out[9] = qx * Sx + qy * Sy + qz * Sz;
}

}  // namespace gbt
