// Point-wise numerics of the face flux: MUSCL/NND reconstruction
// (source/Reconstruction.cpp:7-68, 70-265), Roe (source/Flux_Split_Scheme.cpp:568-635) and
// Steger-Warming (:82-149) fluxes in the rotated face frame (:728-776), the wall flux
// (source/WallFlux.cpp:70-175). Templated on the working type.
#pragma once
#include "gbt_common.cuh"

namespace gbt {

template <typename T> struct C5 { T d, mx, my, mz, e; };
template <typename T> struct P6 { T d, u, v, w, p, t; };

template <typename T> __device__ __forceinline__ T tabs(T x) { return x < (T)0 ? -x : x; }

// minmod of one component (source/Reconstruction.cpp:472-560)
template <typename T> __device__ __forceinline__ T mm(T a, T b)
{
    if (a * b < (T)0) return (T)0;
    return (tabs(a) <= tabs(b)) ? a : b;
}
template <typename T> __device__ __forceinline__ T min3t(T a, T b, T c) { T m = a; if (m > b) m = b; if (m > c) m = c; return m; }
template <typename T> __device__ __forceinline__ T max2t(T a, T b) { return a > b ? a : b; }

// One scalar of the MUSCL family: left state at the face from (FF, F, B) and right state from
// (F, B, BB). Component-wise, identical for primitive and conserved variables apart from eta.
template <typename T>
__device__ __forceinline__ void recon1(int type, T eta, T FF, T F, T B, T BB, T &L, T &R)
{
    const T eps = (T)(double)1E-6f;
    L = (T)0; R = (T)0;
    if (type == 100) {                      // NND
        L = F + (T)0.5 * mm(B - F, F - FF);
        R = B - (T)0.5 * mm(B - F, BB - B);
    } else if (type == 200) {               // MUSCL2u, k = -1
        L = F + (T)0.25 * ((T)2 * mm((T)2 * (B - F), F - FF) + (T)0 * mm((T)2 * (F - FF), B - F));
        R = B - (T)0.25 * ((T)2 * mm((T)2 * (B - F), BB - B) + (T)0 * mm((T)2 * (BB - B), B - F));
    } else if (type == 300) {               // MUSCL2c, k = 1
        L = F + (T)0.25 * ((T)0 * mm((T)2 * (B - F), F - FF) + (T)2 * mm(B - F, (T)2 * (F - FF)));
        R = B - (T)0.25 * ((T)0 * mm((T)2 * (B - F), BB - B) + (T)2 * mm(B - F, (T)2 * (BB - B)));
    } else if (type == 400) {               // MUSCL2o
        T r1 = (F - FF + eps) / (B - F + eps), r2 = (B - F + eps) / (BB - B + eps);
        T f1 = (((T)1 - eta) + ((eta - (T)(double)0.55f) / (T)2) / r2) + r1 * ((eta + (T)(double)0.55f) / (T)2);
        T f = max2t((T)0, min3t((T)2, f1, (T)2 * r1));
        L = F + ((T)0.5 * f) * (B - F);
        r1 = (BB - B + eps) / (B - F + eps); r2 = (B - F + eps) / (F - FF + eps);
        f1 = (((T)1 - eta) + ((eta - (T)(double)0.55f) / (T)2) / r2) + r1 * ((eta + (T)(double)0.55f) / (T)2);
        f = max2t((T)0, min3t((T)2, f1, (T)2 * r1));
        R = B - ((T)0.5 * f) * (B - F);
    } else if (type == 500) {               // MUSCL3 with the smooth (van Albada-type) limiter
        T a = F - FF, b = B - F, c = BB - B;
        T SL = fdiv<T>((T)2 * a * b + eps, a * a + b * b + eps);
        T SR = fdiv<T>((T)2 * c * b + eps, c * c + b * b + eps);
        // S/3 as a product with 1/3 (the FP64 divide is the costly instruction here; within rounding)
        const T third = (T)(1.0 / 3.0);
        const T sl3 = SL * third, sr3 = SR * third;
        L = F + SL * (T)0.25 * (((T)1 - sl3) * a + (sl3 + (T)1) * b);
        R = B - SR * (T)0.25 * (((T)1 - sr3) * c + (sr3 + (T)1) * b);
    }
}

// primitive reconstruction + positivity fallback + conversion to conserved variables
template <typename T>
__device__ __forceinline__ void recon_prim(int type, T rgm1, const P6<T> &FF, const P6<T> &F, const P6<T> &B,
                                           const P6<T> &BB, C5<T> &cl, C5<T> &cr)
{
    const T eta = (T)(double)0.2f, lz = (T)(double)1E-20f;
    P6<T> l, r;
    recon1(type, eta, FF.d, F.d, B.d, BB.d, l.d, r.d);
    recon1(type, eta, FF.u, F.u, B.u, BB.u, l.u, r.u);
    recon1(type, eta, FF.v, F.v, B.v, BB.v, l.v, r.v);
    recon1(type, eta, FF.w, F.w, B.w, BB.w, l.w, r.w);
    recon1(type, eta, FF.p, F.p, B.p, BB.p, l.p, r.p);
    if (l.d <= lz || l.p <= lz) l = F;
    if (r.d <= lz || r.p <= lz) r = B;
    cl.d = l.d; cl.mx = l.d * l.u; cl.my = l.d * l.v; cl.mz = l.d * l.w;
    cl.e = l.p * rgm1 + l.d * (l.u * l.u + l.v * l.v + l.w * l.w) * (T)0.5;
    cr.d = r.d; cr.mx = r.d * r.u; cr.my = r.d * r.v; cr.mz = r.d * r.w;
    cr.e = r.p * rgm1 + r.d * (r.u * r.u + r.v * r.v + r.w * r.w) * (T)0.5;
}

template <typename T>
__device__ __forceinline__ void recon_cons(int type, T gamma, const C5<T> &FF, const C5<T> &F, const C5<T> &B,
                                           const C5<T> &BB, C5<T> &cl, C5<T> &cr)
{
    const T eta = (T)(double)0.05f, lz = (T)(double)1E-20f;
    recon1(type, eta, FF.d, F.d, B.d, BB.d, cl.d, cr.d);
    recon1(type, eta, FF.mx, F.mx, B.mx, BB.mx, cl.mx, cr.mx);
    recon1(type, eta, FF.my, F.my, B.my, BB.my, cl.my, cr.my);
    recon1(type, eta, FF.mz, F.mz, B.mz, BB.mz, cl.mz, cr.mz);
    recon1(type, eta, FF.e, F.e, B.e, BB.e, cl.e, cr.e);
    const T gm1 = gamma - (T)1;
    T pL = gm1 * (cl.e - (T)0.5 * (cl.mx * cl.mx + cl.my * cl.my + cl.mz * cl.mz) / cl.d);
    T pR = gm1 * (cr.e - (T)0.5 * (cr.mx * cr.mx + cr.my * cr.my + cr.mz * cr.mz) / cr.d);
    if (cl.d <= lz || pL <= lz) cl = F;
    if (cr.d <= lz || pR <= lz) cr = B;
}

// Harten's entropy fix z > d ? z : 0.5 (z^2 + d^2) / d at the Roe flux's d = 0.5, where it is
// z^2 + 0.25 bit for bit (the halving and the division by one half are exact)
template <typename T>
__device__ __forceinline__ T entropy_corr_half(T z) { return z > (T)0.5 ? z : z * z + (T)0.25; }

// Roe flux in the face frame with Harten's fix (delta fixed at 0.5) and the reference's wave
// strengths arr[2], arr[3] divided by (v+1e-8), (w+1e-8)
template <typename T>
__device__ __forceinline__ C5<T> roe(T gamma, const C5<T> &QL, const C5<T> &QR, T qe)
{
    const T g1 = gamma - (T)1;
    // divisions by the densities as products with their reciprocals (within rounding)
    T dL = QL.d, rdL = frcp<T>(dL), uL = QL.mx * rdL, vL = QL.my * rdL, wL = QL.mz * rdL, EL = QL.e * rdL;
    T pL = g1 * dL * (EL - (T)0.5 * (uL * uL + vL * vL + wL * wL));
    T HL = EL + pL * rdL;
    T dR = QR.d, rdR = frcp<T>(dR), uR = QR.mx * rdR, vR = QR.my * rdR, wR = QR.mz * rdR, ER = QR.e * rdR;
    T pR = g1 * dR * (ER - (T)0.5 * (uR * uR + vR * vR + wR * wR));
    T HR = ER + pR * rdR;
    T unL = uL - qe, unR = uR - qe;
    T tmp = fsqrt<T>(dR * rdL);
    T inv = frcp<T>((T)1 + tmp);
    T ua = (uL + tmp * uR) * inv, va = (vL + tmp * vR) * inv, wa = (wL + tmp * wR) * inv, Ha = (HL + tmp * HR) * inv;
    T q2 = ua * ua + va * va + wa * wa;
    T ca = fsqrt<T>(g1 * (Ha - (T)0.5 * q2));
    T una = ua - qe;
    T l1 = entropy_corr_half(tabs(una - ca)), l2 = entropy_corr_half(tabs(una)), l5 = entropy_corr_half(tabs(una + ca));
    T dd = dR - dL, dmx = QR.mx - QL.mx, dmy = QR.my - QL.my, dmz = QR.mz - QL.mz, de = QR.e - QL.e;
    T a2, a3;
    if constexpr (sizeof(T) == 8) {
        a2 = fdiv<T>(dmy, va + (T)(double)1E-8f) - dd;
        a3 = fdiv<T>(dmz, wa + (T)(double)1E-8f) - dd;
    } else {
        // mixed form: the FP32 round-off of a near-zero tangential velocity (about 1e-8 of the
        // speed) is as large as the reference's 1e-8 regularisation, so v + 1e-8 can reach 0 and the
        // wave strength infinity where FP64 round-off (1e-16) stays far from it; below half the
        // regularisation the denominator is held there, sign kept (|v / den| <= 3 in that band)
        const T eps = (T)(double)1E-8f, h = (T)0.5 * eps;
        T d2 = va + eps, d3 = wa + eps;
        if (tabs(d2) < h) d2 = d2 < (T)0 ? -h : h;
        if (tabs(d3) < h) d3 = d3 < (T)0 ? -h : h;
        a2 = fdiv<T>(dmy, d2) - dd;
        a3 = fdiv<T>(dmz, d3) - dd;
    }
    const T rca = frcp<T>(ca);
    T a4 = g1 * (dd * (Ha - ua * ua - va * va - wa * wa) + ua * dmx + va * dmy + wa * dmz - de) * (rca * rca);
    T a1 = ((ua + ca) * dd - dmx - ca * a4) * ((T)0.5 * rca);
    T a5 = dd - (a1 + a4);
    C5<T> F;
    F.d = (T)0.5 * (QL.d * unL + QR.d * unR) - (T)0.5 * (l1 * a1 + l2 * a4 + l5 * a5);
    F.mx = (T)0.5 * ((QL.mx * unL + pL) + (QR.mx * unR + pR)) -
           (T)0.5 * (l1 * a1 * (ua - ca) + l2 * a4 * ua + l5 * a5 * (ua + ca));
    F.my = (T)0.5 * (QL.my * unL + QR.my * unR) - (T)0.5 * (l1 * a1 * va + l2 * a2 * va + l2 * a4 * va + l5 * a5 * va);
    F.mz = (T)0.5 * (QL.mz * unL + QR.mz * unR) - (T)0.5 * (l1 * a1 * wa + l2 * a3 * wa + l2 * a4 * wa + l5 * a5 * wa);
    F.e = (T)0.5 * (((QL.e + pL) * unL + qe * pL) + ((QR.e + pR) * unR + qe * pR)) -
          (T)0.5 * (l1 * a1 * (Ha - ua * ca) + l2 * a2 * va * va + l2 * a3 * wa * wa + l2 * a4 * (T)0.5 * q2 +
                    l5 * a5 * (Ha + ua * ca));
    return F;
}

// Steger-Warming split flux of one side: sgn = +1 for the left state (positive eigenvalues),
// -1 for the right state (negative ones); epsilon = 1e-6 smooths |lambda|
template <typename T>
__device__ __forceinline__ C5<T> sw_half(T gamma, const C5<T> &Q, T qe, T sgn)
{
    const T eps = (T)(double)1E-6f;
    const T g1 = gamma - (T)1;
    T d = Q.d, u = Q.mx / d, v = Q.my / d, w = Q.mz / d, e = Q.e / d;
    T t = gamma * g1 * (e - (T)0.5 * (u * u + v * v + w * w));
    t = tsqrt(t * t);
    T c = tsqrt(t);
    T un = u - qe;
    T l1 = (T)0.5 * (un + sgn * tsqrt(un * un + eps * eps));
    T l4 = (T)0.5 * ((un - c) + sgn * tsqrt((un - c) * (un - c) + eps * eps));
    T l5 = (T)0.5 * ((un + c) + sgn * tsqrt((un + c) * (un + c) + eps * eps));
    T W2 = ((T)3 - gamma) * (l4 + l5) * c * c / (T)2 / g1;
    T A = (u - c) * (u - c) + v * v + w * w;
    T Bq = (u + c) * (u + c) + v * v + w * w;
    T f = d / (T)2 / gamma;
    C5<T> F;
    F.d = f * ((T)2 * g1 * l1 + l4 + l5);
    F.mx = f * ((T)2 * g1 * l1 * u + l4 * (u - c) + l5 * (u + c));
    F.my = f * ((T)2 * g1 * l1 * v + l4 * v + l5 * v);
    F.mz = f * ((T)2 * g1 * l1 * w + l4 * w + l5 * w);
    F.e = f * (g1 * l1 * (u * u + v * v + w * w) + (T)0.5 * l4 * A + (T)0.5 * l5 * Bq + W2);
    return F;
}

}  // namespace gbt
