// Spalart-Allmaras turbulence model of the reference (config turbulence model 200), fine level
// only, single grid level:
//  - wall distances, once (CMesh::WallDistanceSA, source/WallDistanceSA.cpp:6-160): distance of
//    every cell centre to the nearest wall-face centre of any block of the case;
//  - the eddy-viscosity variable's ghost cells (inlet, outlet, wall, interfaces and periodic pairs:
//    source/BndCondInlet.cpp:104-105, source/BndCondOutlet.cpp:102-103, source/BndCondWall.cpp:104-107,
//    source/ShadowOutIn.cpp);
//  - the model (CSpaceDiscr::SA_Model, source/SA_Model.cpp:6-257): mu_t from the variable, the
//    clipping of both, first-order upwind convective and viscous face fluxes with the face
//    gradient of the variable (source/Spectral_curl_grad.cpp:85-493, taken before the clipping),
//    the source term, the residual Res_ev = Cell_Fc_tur - Cell_Fv_tur
//    (source/ComputeAllBlockVars.cpp:109-113, 237-249), and mu_t of the ghost layer;
//  - the variable's LU-SGS sweeps (source/LU_SGS_Marching.cpp:76-258, delt_Fn_up/down :293-419)
//    as a scalar hyperplane chain after each of the mean-flow sweeps, whose dQ it reads;
//  - its update and limiter (source/LU_SGS_Marching.cpp:262-287, CFluidProps::Limit_SA,
//    source/Limit_FlowVars.cpp:122-166).
// The reference's quirks are kept: the I-face viscous flux uses the x derivative for all three
// components, the K-face one has its y and z derivatives swapped (aliased pointers at
// source/SA_Model.cpp:19-29).
#include "gbt_common.cuh"
#include "kernels.hpp"

namespace gbt {

namespace {

// model constants as the reference declares them (float literals assigned to REAL)
struct SAConst {
    double Cb1, Cb2, Cv1, sigma, kavf, Cw1, Cw2, Cw3, Ct3, Ct4;
};
__host__ __device__ inline SAConst sa_const()
{
    SAConst c;
    c.Cb1 = (double)0.1355f; c.Cb2 = (double)0.622f; c.Cv1 = (double)7.1f; c.sigma = (double)(2.0f / 3.0f);
    c.kavf = (double)0.41f;
    c.Cw1 = c.Cb1 / c.kavf / c.kavf + (1.0 + c.Cb2) / c.sigma;
    c.Cw2 = (double)0.3f; c.Cw3 = (double)2.0f; c.Ct3 = (double)1.2f; c.Ct4 = (double)0.5f;
    return c;
}

template <typename T>
__device__ __forceinline__ T fv1_of(T X, T Cv1)
{
    const T x3 = pow(X, (T)3);
    return x3 / (x3 + Cv1 * Cv1 * Cv1);
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// wall distances: cell centre to the nearest wall-face centre of the case
// ---------------------------------------------------------------------------------------------
__global__ void k_sa_wall_points(Geo G, const long long *face_p, const int *face_f, long long n, double *wx, double *wy,
                                 double *wz)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const long long p = face_p[t];
    const int f = face_f[t];
    wx[t] = G.c[f][0][p]; wy[t] = G.c[f][1][p]; wz[t] = G.c[f][2][p];
}

__global__ void __launch_bounds__(256) k_sa_wall_dist(Batch B, Geo G, const double *wx, const double *wy, const double *wz,
                                                      const long long *case_off, double *dwall)
{
    const int s = blockIdx.y;
    const Lvl L = B.lv[s];
    int i, j, k;
    const bool in = box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k);
    const long long p = in ? ix(L, i, j, k) : 0;
    const double cx = in ? G.cc[0][p] : 0.0, cy = in ? G.cc[1][p] : 0.0, cz = in ? G.cc[2][p] : 0.0;
    const int c = B.sc[s].cix;
    const long long a = case_off[c], b = case_off[c + 1];
    __shared__ double sx[256], sy[256], sz[256];
    // the nearest point by squared distance, one root at the end: the root is monotone and
    // correctly rounded, so this is the reference's minimum of the roots
    double d2min = 1.0e8;                      // (the reference's initial 10000)^2
    for (long long t0 = a; t0 < b; t0 += 256) {
        const long long t = t0 + threadIdx.x;
        __syncthreads();
        if (t < b) { sx[threadIdx.x] = wx[t]; sy[threadIdx.x] = wy[t]; sz[threadIdx.x] = wz[t]; }
        __syncthreads();
        const int m = (int)min((long long)256, b - t0);
        if (in)
            for (int q = 0; q < m; q++) {
                const double dx = cx - sx[q], dy = cy - sy[q], dz = cz - sz[q];
                const double d2 = dx * dx + dy * dy + dz * dz;
                if (d2min >= d2) d2min = d2;
            }
    }
    if (in) dwall[p] = sqrt(d2min);
}

void launch_sa_wall_distance(const LaunchCtx &ctx, const Geo &G, const long long *face_p, const int *face_f, long long n,
                             double *scratch_xyz, const long long *case_off, double *dwall)
{
    double *wx = scratch_xyz, *wy = scratch_xyz + n, *wz = scratch_xyz + 2 * n;
    if (n > 0) k_sa_wall_points<<<(unsigned)((n + 255) / 256), 256, 0, ctx.stream>>>(G, face_p, face_f, n, wx, wy, wz);
    k_sa_wall_dist<<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(ctx.batch, G, wx, wy, wz, case_off, dwall);
}

// ---------------------------------------------------------------------------------------------
// uniform start and ghost cells of the variable
// ---------------------------------------------------------------------------------------------
__global__ void k_sa_fill(Batch B, double *ev, double v)
{
    const Lvl L = B.lv[blockIdx.y];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    ev[ix(L, i, j, k)] = v;
}

void launch_sa_init(const LaunchCtx &ctx, double *ev, double ev_ratio)
{
    k_sa_fill<<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(ctx.batch, ev, ev_ratio);
}

// inlet: the ghost holds the configured ratio; outlet: the ghost copies the last cell
__global__ void k_sa_bc_inout(Batch B, double *ev, const DevInOut *pat, int outlet, double ev_ratio)
{
    const DevInOut pt = pat[blockIdx.y];
    const Lvl L = B.lv[pt.solve];
    if (outlet) {
        const int t = blockIdx.x * blockDim.x + threadIdx.x;
        if (t >= (L.IM - 1) * (L.JM - 1)) return;
        const int i = 1 + t / (L.JM - 1), j = 1 + t % (L.JM - 1);
        ev[ix(L, i, j, L.KM)] = ev[ix(L, i, j, L.KM - 1)];
        return;
    }
    const int ni = pt.ie - pt.is + 1, nj = pt.je - pt.js + 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ni * nj) return;
    const int i = pt.is + t / nj, j = pt.js + t % nj;
    const int kv = pt.ks == 1 ? 0 : L.KM;
    ev[ix(L, i, j, kv)] = ev_ratio * (double)1.0f;
}

__global__ void k_sa_bc_wall(Batch B, double *ev, const DevWall *walls)
{
    const DevWall wl = walls[blockIdx.y];
    const Lvl L = B.lv[wl.solve];
    const int ni = wl.ie - wl.is + 1, nj = wl.je - wl.js + 1, nk = wl.ke - wl.ks + 1;
    int i, j, k;
    if (!box_index(ni, nj, nk, i, j, k)) return;
    i += wl.is - 1; j += wl.js - 1; k += wl.ks - 1;
    const int f = (wl.face - 1) / 2;
    const bool lo = wl.face % 2 == 1;
    const long long sn = f == 0 ? (long long)L.NJ * L.NK : (f == 1 ? (long long)L.NK : 1LL);
    const long long fp = ix(L, i, j, k);
    ev[lo ? fp - sn : fp] = 0.0;
}

__global__ void k_sa_gather(double *ev, const long long *dst, const long long *src, long long n)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) ev[dst[t]] = ev[src[t]];
}

template <typename T>
void launch_sa_boundary(const LaunchCtx &ctx, const Phys &P, Flow<T> W, const BcTables &bc)
{
    const Batch &B = ctx.batch;
    if (bc.n_inlet)
        k_sa_bc_inout<<<dim3((bc.max_inlet + 127) / 128, bc.n_inlet), 128, 0, ctx.stream>>>(B, W.ev, bc.inlet, 0, P.ev_ratio);
    if (bc.n_outlet)
        k_sa_bc_inout<<<dim3((bc.max_outlet_im * bc.max_outlet_jm + 127) / 128, bc.n_outlet), 128, 0, ctx.stream>>>(
            B, W.ev, bc.outlet, 1, P.ev_ratio);
    if (bc.n_wall) k_sa_bc_wall<<<dim3((bc.max_wall + 127) / 128, bc.n_wall), 128, 0, ctx.stream>>>(B, W.ev, bc.wall);
    if (bc.n_sa_gather)
        k_sa_gather<<<(unsigned)((bc.n_sa_gather + 255) / 256), 256, 0, ctx.stream>>>(W.ev, bc.sa_dst, bc.sa_src, bc.n_sa_gather);
}

// ---------------------------------------------------------------------------------------------
// the model
// ---------------------------------------------------------------------------------------------
// mu_t from the variable, then the clipping of mu_t and of the variable (source/SA_Model.cpp:44-83)
template <typename T>
__global__ void __launch_bounds__(256) k_sa_mut(Batch B, Phys P, Flow<T> W)
{
    const Lvl L = B.lv[blockIdx.y];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
    const SAConst C = sa_const();
    const T Re = (T)P.re_ref, Cv1 = (T)C.Cv1;
    const T d = W.pv[PD][p], tt = W.pv[PT][p];
    T ev = (T)W.ev[p];
    const T mlam = sutherland<T>(P, tt);
    T ev_lam = Re * mlam / d;
    const T X = ev / ev_lam;
    T mt = fv1_of<T>(X, Cv1) * d * ev / Re;
    const T Max = (T)200.0;
    if (mt < (T)0) mt = (T)0;
    bool changed = false;
    if (ev < (T)0) { ev = (T)0; changed = true; }
    ev_lam = Re * mlam / d;
    if (mlam > (T)0 && mt > Max * mlam) mt = Max * mlam;
    if (ev_lam > (T)0 && ev > Max * ev_lam) { ev = Max * ev_lam; changed = true; }
    W.mut[p] = mt;
    if (changed) W.ev[p] = (double)ev;
}

// tangential difference across a face (the gradient stencil of the mean flow, applied to the
// variable; source/Spectral_curl_grad.cpp:112-204 and the J, K counterparts)
template <typename T, int F, int DT>
__device__ __forceinline__ T sa_tan_diff(const double *__restrict__ c, long long p, long long sn, long long st, int a,
                                         int NN, int b, int TT)
{
    const T c00 = (T)c[p], cm0 = (T)c[p - sn];
    const T c0p = (T)c[p + st], cmp = (T)c[p - sn + st], c0m = (T)c[p - st], cmm = (T)c[p - sn - st];
    T plus, minus;
    const bool lo_n = (a == 1), hi_n = (a == NN), lo_t = (b == 1), hi_t = (b == TT - 1);
    if (lo_n && hi_t) plus = (c00 + c0p + cm0) / (T)3;
    else if (hi_n && hi_t) plus = (c00 + cmp + cm0) / (T)3;
    else plus = (T)0.25 * (c00 + c0p + cmp + cm0);
    if (lo_n && lo_t) minus = (c00 + cm0 + c0m) / (T)3;
    else if (hi_n && lo_t) {
        minus = (c00 + cm0 + cmm) / (T)3;
        if (F == 1 && DT == 2) minus = (T)0.25 * minus;
    } else minus = (T)0.25 * (c00 + cm0 + cmm + c0m);
    return plus - minus;
}

// face fluxes of the variable (source/SA_Model.cpp:85-180): first-order upwind convective flux
// (zero on wall faces, source/WallFlux.cpp:104-105), viscous flux and the gradient flux of the
// cross-diffusion term
template <typename T, int F>
__global__ void __launch_bounds__(128) k_sa_face(Batch B, Phys P, GeoW<T> G, Flow<T> W)
{
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
    const long long m = p - sn;
    const SAConst C = sa_const();
    const T Re = (T)P.re_ref;
    // face gradient of the variable before the clipping (W.evg)
    const int iD1 = F == 0 ? 1 : 0, iD2 = F == 2 ? 1 : 2;
    const long long st1 = iD1 == 0 ? sI : sJ, st2 = iD2 == 1 ? sJ : sK;
    const int b1 = iD1 == 0 ? i : j, T1 = iD1 == 0 ? L.IM : L.JM;
    const int b2 = iD2 == 1 ? j : k, T2 = iD2 == 1 ? L.JM : L.KM;
    const T dn = (T)W.evg[p] - (T)W.evg[m];
    const T d1 = sa_tan_diff<T, F, (F == 0 ? 1 : 0)>(W.evg, p, sn, st1, a, NN, b1, T1);
    const T d2 = sa_tan_diff<T, F, (F == 2 ? 1 : 2)>(W.evg, p, sn, st2, a, NN, b2, T2);
    T dk, de, dz;
    if (F == 0) { dk = dn; de = d1; dz = d2; }
    else if (F == 1) { dk = d1; de = dn; dz = d2; }
    else { dk = d1; de = d2; dz = dn; }
    const T gx = dk * G.m[F][0][p] + de * G.m[F][3][p] + dz * G.m[F][6][p];
    const T gy = dk * G.m[F][1][p] + de * G.m[F][4][p] + dz * G.m[F][7][p];
    const T gz = dk * G.m[F][2][p] + de * G.m[F][5][p] + dz * G.m[F][8][p];
    // the model reads the I-face x derivative for all three components and the K-face y and z
    // derivatives swapped
    const T ux = gx, uy = F == 0 ? gx : (F == 2 ? gz : gy), uz = F == 0 ? gx : (F == 2 ? gy : gz);
    const T h = (T)0.5;
    const T densf = h * (W.pv[PD][p] + W.pv[PD][m]);
    const T tempf = h * (W.pv[PT][p] + W.pv[PT][m]);
    const T evp = (T)W.ev[p], evm = (T)W.ev[m];
    const T evf = h * (evp + evm);
    const T ev_lam = Re * sutherland<T>(P, tempf) / densf;
    const T cf = (T)((1.0 + C.Cb2) / C.sigma) * (ev_lam + evf);
    const T tx = cf * ux, ty = cf * uy, tz = cf * uz;
    const T Sx = G.S[F][0][p], Sy = G.S[F][1][p], Sz = G.S[F][2][p], sa = G.s[F][p];
    const T nx = Sx / sa, ny = Sy / sa, nz = Sz / sa;
    const T Vn1 = W.pv[PU][m] * nx + W.pv[PV][m] * ny + W.pv[PW][m] * nz;
    const T Vn2 = W.pv[PU][p] * nx + W.pv[PV][p] * ny + W.pv[PW][p] * nz;
    T fc = (h * (Vn1 + fabs(Vn1)) * evm + h * (Vn2 - fabs(Vn2)) * evp) * sa;
    if (W.wallf[F][p]) fc = (T)0;
    W.Fct[F][p] = fc;
    W.Fvt[F][p] = (tx * Sx + ty * Sy + tz * Sz) / Re;
    W.Fv1t[F][p] = ux * Sx + uy * Sy + uz * Sz;
}

// source term, cell sums and the residual of the variable (source/SA_Model.cpp:182-205,
// source/ComputeAllBlockVars.cpp:109-113, 245-248)
template <typename T>
__global__ void __launch_bounds__(256) k_sa_cell(Batch B, Phys P, GeoW<T> G, Flow<T> W)
{
    const Lvl L = B.lv[blockIdx.y];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
    const long long pI = p + (long long)L.NJ * L.NK, pJ = p + L.NK, pK = p + 1;
    const SAConst C = sa_const();
    const T Re = (T)P.re_ref, Cv1 = (T)C.Cv1, kv = (T)C.kavf, Cb1 = (T)C.Cb1, Cb2 = (T)C.Cb2, sigma = (T)C.sigma;
    const T Cw1 = (T)C.Cw1, Cw2 = (T)C.Cw2, Cw3 = (T)C.Cw3, Ct3 = (T)C.Ct3, Ct4 = (T)C.Ct4;
    const T ev = (T)W.ev[p];
    const T ev_lam = Re * sutherland<T>(P, W.pv[PT][p]) / W.pv[PD][p];
    const T X = ev / ev_lam;
    const T fv1 = fv1_of<T>(X, Cv1);
    const T fv2 = (T)1 - X / ((T)1 + X * fv1);
    const T ft2 = Ct3 * exp((T)0 - Ct4 * X * X);
    const T om = W.omega[p];
    const T dw = (T)W.dwall[p];
    const T Sbar = fmax(om + ev * fv2 / (pow(kv * dw, (T)2) * Re), (T)(double)0.3f * om);
    const T r = fmin(ev / (Sbar * kv * kv * dw * dw * Re), (T)10);
    const T g = r + Cw2 * (pow(r, (T)6) - r);
    const T cw36 = pow(Cw3, (T)6);
    const T fw = g * pow(((T)1 + cw36) / (pow(g, (T)6) + cw36), (T)(double)(1.0f / 6.0f));
    const T Qc = (Cb1 * ((T)1 - ft2) * Sbar * ev -
                  (Cw1 * fw - Cb1 * (((T)1 - ft2) * fv2 + ft2) / (kv * kv)) * pow(ev / dw, (T)2) / Re) * G.vol[p];
    const T fv = Qc + W.Fvt[0][pI] - W.Fvt[0][p] + W.Fvt[1][pJ] - W.Fvt[1][p] + W.Fvt[2][pK] - W.Fvt[2][p] -
                 Cb2 * (ev_lam + ev) / sigma / Re *
                     (W.Fv1t[0][pI] - W.Fv1t[0][p] + W.Fv1t[1][pJ] - W.Fv1t[1][p] + W.Fv1t[2][pK] - W.Fv1t[2][p]);
    const T fc = W.Fct[0][pI] - W.Fct[0][p] + W.Fct[1][pJ] - W.Fct[1][p] + W.Fct[2][pK] - W.Fct[2][p];
    W.res_ev[p] = fc - fv;
}

// mu_t of the ghost layer from its variable (source/SA_Model.cpp:208-256): threads over the six
// faces' interior ranges
template <typename T>
__global__ void k_sa_ghost_mut(Batch B, Phys P, Flow<T> W)
{
    const Lvl L = B.lv[blockIdx.y];
    const int nI = L.IM - 1, nJ = L.JM - 1, nK = L.KM - 1;
    const int nf0 = nJ * nK, nf1 = nI * nK, nf2 = nI * nJ;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * (nf0 + nf1 + nf2)) return;
    int i, j, k;
    if (t < 2 * nf0) {
        const int side = t / nf0, r = t % nf0;
        i = side ? L.IM : 0; j = 1 + r / nK; k = 1 + r % nK;
    } else if ((t -= 2 * nf0) < 2 * nf1) {
        const int side = t / nf1, r = t % nf1;
        j = side ? L.JM : 0; i = 1 + r / nK; k = 1 + r % nK;
    } else {
        t -= 2 * nf1;
        const int side = t / nf2, r = t % nf2;
        k = side ? L.KM : 0; i = 1 + r / nJ; j = 1 + r % nJ;
    }
    const long long p = ix(L, i, j, k);
    const SAConst C = sa_const();
    const T Re = (T)P.re_ref;
    const T d = W.pv[PD][p], ev = (T)W.ev[p];
    const T ev_lam = Re * sutherland<T>(P, W.pv[PT][p]) / d;
    W.mut[p] = fv1_of<T>(ev / ev_lam, (T)C.Cv1) * d * ev / Re;
}

template <typename T>
void launch_sa_model(const LaunchCtx &ctx, const Phys &P, const GeoW<T> &GW, Flow<T> W)
{
    const Batch &B = ctx.batch;
    // the gradients of the variable are those of the state before the model clips it
    cudaMemcpyAsync(W.evg, W.ev, sizeof(double) * (size_t)ctx.pool_n, cudaMemcpyDeviceToDevice, ctx.stream);
    k_sa_mut<T><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, P, W);
    k_sa_face<T, 0><<<ctx.grid_faces(0, 128), 128, 0, ctx.stream>>>(B, P, GW, W);
    k_sa_face<T, 1><<<ctx.grid_faces(1, 128), 128, 0, ctx.stream>>>(B, P, GW, W);
    k_sa_face<T, 2><<<ctx.grid_faces(2, 128), 128, 0, ctx.stream>>>(B, P, GW, W);
    k_sa_cell<T><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, P, GW, W);
    const long long ng = 2LL * ((long long)(ctx.maxJM - 1) * (ctx.maxKM - 1) + (long long)(ctx.maxIM - 1) * (ctx.maxKM - 1) +
                                (long long)(ctx.maxIM - 1) * (ctx.maxJM - 1));
    k_sa_ghost_mut<T><<<ctx.grid_n(ng, 256), 256, 0, ctx.stream>>>(B, P, W);
}

// ---------------------------------------------------------------------------------------------
// LU-SGS sweeps of the variable (source/LU_SGS_Marching.cpp:76-258, delt_Fn_up/down :293-419). They
// run after the mean-flow chain of the same direction, so every neighbour's mean-flow dQ is final:
// a parallel pass first forms, for every cell as somebody's neighbour, the parts of
// delt_Fn_ev = ev_new * Vn_new - ev_old * Vn_old that do not depend on the variable's own update
// (Vn_new, ev_old * Vn_old) and the diagonal; the hyperplane chain then only adds the neighbours'
// updates. One launch per plane, chained by programmatic dependent launch like the mean flow.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void sa_wait_previous() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void sa_release_next() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename T, int DIR>
__global__ void __launch_bounds__(256) k_sa_sweep_prep(PhysW<T> PC, Geo G, Flow<T> W, SweepData<T> S, long long nq)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const long long p = S.cell[q];
    const double o0 = W.cv[0][p], o1 = W.cv[1][p], o2 = W.cv[2][p], o3 = W.cv[3][p];
    const T dn0 = (T)(o0 + (double)S.dq[0][q]), dn1 = (T)(o1 + (double)S.dq[1][q]), dn2 = (T)(o2 + (double)S.dq[2][q]),
            dn3 = (T)(o3 + (double)S.dq[3][q]);
    const T evo = (T)W.ev[p];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const T nx = (T)G.cn[d][0][p], ny = (T)G.cn[d][1][p], nz = (T)G.cn[d][2][p];
        S.sa_vn[d][q] = dn1 / dn0 * nx + dn2 / dn0 * ny + dn3 / dn0 * nz;
        if (DIR > 0) {
            const T Vold = (T)o1 / (T)o0 * nx + (T)o2 / (T)o0 * ny + (T)o3 / (T)o0 * nz;
            S.sa_eb[d][q] = evo * Vold;
            S.sa_s[d][q] = (T)G.cs[d][p];
            S.sa_rl[d][q] = PC.relax * W.lamc[d][p];
            S.sa_lv[d][q] = W.lamv[d][p];
        }
    }
    if (DIR > 0) {
        const T lc = W.lamc[0][p] + W.lamc[1][p] + W.lamc[2][p];
        const T lv = W.lamv[0][p] + W.lamv[1][p] + W.lamv[2][p];
        S.sa_alpha[q] = (T)G.vol[p] / W.dt[p] + PC.relax * lc + (T)3 * lv;
        S.sa_ev0[q] = evo;
        S.sa_res[q] = W.res_ev[p];
    }
}

template <typename T, int DIR>
__global__ void __launch_bounds__(32) k_sa_sweep(SweepData<T> S, const int *start, int stride, int plane)
{
    sa_release_next();
    const int s = blockIdx.y;
    const int q0 = start[(long long)s * stride + plane], q1 = start[(long long)s * stride + plane + 1];
    const int q = q0 + blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = q < q1;
    T alpha = (T)1, own = (T)0;
    int qn[3] = {-1, -1, -1};
    if (in) {
        alpha = S.sa_alpha[q];
        own = DIR > 0 ? -S.sa_res[q] : alpha * S.sa_dq[q];
#pragma unroll
        for (int d = 0; d < 3; d++) qn[d] = S.nb[DIR > 0 ? 0 : 1][d][q];
    }
    sa_wait_previous();
    if (!in) return;
    T aws[3], vws[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        aws[d] = (T)0; vws[d] = (T)0;
        const int n = qn[d];
        if (n < 0) continue;
        const T dqn = S.sa_dq[n];
        const T dF = (S.sa_ev0[n] + dqn) * S.sa_vn[d][n] - S.sa_eb[d][n];
        aws[d] = (T)0.5 * (dF * S.sa_s[d][n] + (DIR > 0 ? S.sa_rl[d][n] : -S.sa_rl[d][n]) * dqn);
        vws[d] = S.sa_lv[d][n] * dqn;
    }
    if (DIR > 0)
        S.sa_dq[q] = (own + aws[0] + aws[1] + aws[2] + vws[0] + vws[1] + vws[2]) / alpha;
    else
        S.sa_dq[q] = (own - aws[0] - aws[1] - aws[2] + vws[0] + vws[1] + vws[2]) / alpha;
}

template <typename T>
__global__ void __launch_bounds__(256) k_sa_sweep_scatter(Flow<T> W, SweepData<T> S, long long nq)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nq) W.dq_ev[S.cell[q]] = S.sa_dq[q];
}

template <typename T, int DIR>
static void launch_sa_plane(const LaunchCtx &ctx, const SweepData<T> &S, const PlaneTables &pt, int pl, bool first)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(max(1, (pt.max_count[pl] + 31) / 32), ctx.batch.nsolve);
    cfg.blockDim = dim3(32);
    cfg.stream = ctx.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = first ? 0 : 1;
    cudaLaunchKernelEx(&cfg, k_sa_sweep<T, DIR>, S, pt.start, pt.stride, pl);
}

template <typename T>
void launch_sa_sweep(const LaunchCtx &ctx, const PhysW<T> &PC, const Geo &G, Flow<T> W, const PlaneTables &pt,
                     const SweepData<T> &S, int dir)
{
    const int np = pt.max_plane;
    const unsigned gq = (unsigned)((pt.nq + 255) / 256);
    if (dir > 0) {
        k_sa_sweep_prep<T, 1><<<gq, 256, 0, ctx.stream>>>(PC, G, W, S, pt.nq);
        for (int pl = 3; pl <= np; pl++) launch_sa_plane<T, 1>(ctx, S, pt, pl, pl == 3);
    } else {
        k_sa_sweep_prep<T, -1><<<gq, 256, 0, ctx.stream>>>(PC, G, W, S, pt.nq);
        for (int pl = np; pl >= 3; pl--) launch_sa_plane<T, -1>(ctx, S, pt, pl, pl == np);
        k_sa_sweep_scatter<T><<<gq, 256, 0, ctx.stream>>>(W, S, pt.nq);
    }
}

// ---------------------------------------------------------------------------------------------
// update and limiter of the variable
// ---------------------------------------------------------------------------------------------
constexpr double kSAmin = (double)1.0E-8f, kSAmax = (double)1000.0f;

template <typename T>
__global__ void __launch_bounds__(256) k_sa_update(Batch B, Flow<T> W, int limit, int *bad_list, int bad_cap, int *bad_count)
{
    const int s = blockIdx.y;
    const Lvl L = B.lv[s];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
    const double e = W.ev[p] + (double)W.dq_ev[p];
    W.ev[p] = e;
    if (limit && e > kSAmax) {
        const int slot = atomicAdd(&bad_count[s], 1);
        if (slot < bad_cap) bad_list[(long long)s * bad_cap + slot] = (int)(((long long)(i - 1) * (L.JM - 1) + (j - 1)) * (L.KM - 1) + (k - 1));
    }
}

// CFluidProps::Limit_SA replayed in the reference's i, j, k order for the cells above the upper
// bound: a neighbour earlier in that order already holds its clamped (or repaired) value, a later
// one its value from the update; one thread per solve, a full scan if the list overflowed
template <typename T>
__global__ void k_sa_limit_serial(Batch B, Flow<T> W, int *bad_list, int bad_cap, int *bad_count)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B.nsolve) return;
    const int n = bad_count[s];
    if (n == 0) return;
    const Lvl L = B.lv[s];
    const int nI = L.IM - 1, nJ = L.JM - 1, nK = L.KM - 1;
    int *lst = bad_list + (long long)s * bad_cap;
    const bool full = n > bad_cap;
    if (!full)
        for (int a = 1; a < n; a++) {
            int v = lst[a], b = a - 1;
            while (b >= 0 && lst[b] > v) { lst[b + 1] = lst[b]; b--; }
            lst[b + 1] = v;
        }
    const long long total = (long long)nI * nJ * nK;
    const long long m = full ? total : n;
    for (long long e = 0; e < m; e++) {
        const long long lin = full ? e : lst[e];
        const int i = 1 + (int)(lin / ((long long)nJ * nK)), j = 1 + (int)((lin / nK) % nJ), k = 1 + (int)(lin % nK);
        const long long p = ix(L, i, j, k);
        if (!(W.ev[p] > kSAmax)) continue;
        double s0 = 0.0;
        int kn = 0;
        for (int ka = -1; ka <= 1; ka++)
            for (int ja = -1; ja <= 1; ja++)
                for (int ia = -1; ia <= 1; ia++) {
                    const int k1 = k + ka, j1 = j + ja, i1 = i + ia;
                    if (i1 > 0 && i1 < L.IM && j1 > 0 && j1 < L.JM && k1 > 0 && k1 < L.KM) {
                        const long long l1 = ((long long)(i1 - 1) * nJ + (j1 - 1)) * nK + (k1 - 1);
                        double v = W.ev[ix(L, i1, j1, k1)];
                        if (l1 < lin && v < kSAmin) v = kSAmin;      // already clamped in the reference's order
                        if (v >= kSAmin && v <= kSAmax) { s0 = s0 + v; kn = kn + 1; }
                    }
                }
        W.ev[p] = kn == 0 ? kSAmax : s0 / kn;
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_sa_limit_clamp(Batch B, Flow<T> W)
{
    const Lvl L = B.lv[blockIdx.y];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    const long long p = ix(L, i, j, k);
    if (W.ev[p] < kSAmin) W.ev[p] = kSAmin;
}

template <typename T>
void launch_sa_update(const LaunchCtx &ctx, const Phys &P, Flow<T> W, int *bad_list, int bad_cap, int *bad_count)
{
    const Batch &B = ctx.batch;
    if (P.limiter) cudaMemsetAsync(bad_count, 0, sizeof(int) * B.nsolve, ctx.stream);
    k_sa_update<T><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, W, P.limiter, bad_list, bad_cap, bad_count);
}

template <typename T>
void launch_sa_limit(const LaunchCtx &ctx, Flow<T> W, int *bad_list, int bad_cap, int *bad_count)
{
    const Batch &B = ctx.batch;
    k_sa_limit_serial<T><<<(B.nsolve + 31) / 32, 32, 0, ctx.stream>>>(B, W, bad_list, bad_cap, bad_count);
    k_sa_limit_clamp<T><<<ctx.grid_cells(256), 256, 0, ctx.stream>>>(B, W);
}

#define GBT_SA_INST(T)                                                                                                 \
    template void launch_sa_boundary<T>(const LaunchCtx &, const Phys &, Flow<T>, const BcTables &);                  \
    template void launch_sa_model<T>(const LaunchCtx &, const Phys &, const GeoW<T> &, Flow<T>);                      \
    template void launch_sa_sweep<T>(const LaunchCtx &, const PhysW<T> &, const Geo &, Flow<T>, const PlaneTables &, \
                                     const SweepData<T> &, int);                                                        \
    template void launch_sa_update<T>(const LaunchCtx &, const Phys &, Flow<T>, int *, int, int *);                    \
    template void launch_sa_limit<T>(const LaunchCtx &, Flow<T>, int *, int, int *);
GBT_SA_INST(double)
GBT_SA_INST(float)

}  // namespace gbt
