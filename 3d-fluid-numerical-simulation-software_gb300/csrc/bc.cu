// Ghost and reconstruction-layer fill before every residual evaluation, in the reference's order
// (source/BoundaryCondition.cpp:9-63): total-condition inlet (source/BndCondInlet.cpp:7-127),
// axial outlet with radial equilibrium (source/BndCondOutlet.cpp:13-113), no-slip wall
// (source/BndCondWall.cpp:20-285) and rotational periodicity as a precomputed gather list
// equivalent to the shadow copies of source/ShadowOutIn.cpp and
// source/BndCondInteriorPeriodic.cpp:36-69.
#include "gbt_common.cuh"
#include "kernels.hpp"
#include "flux.cuh"

namespace gbt {

template <typename T>
__device__ __forceinline__ void st_state(Flow<T> &W, long long g, const double c[5], const T q[6])
{
#pragma unroll
    for (int n = 0; n < 5; n++) W.cv[n][g] = c[n];
#pragma unroll
    for (int n = 0; n < 6; n++) W.pv[n][g] = q[n];
}

// inlet: Riemann invariant from the interior, total pressure/temperature and flow direction
template <typename T>
__global__ void __launch_bounds__(32) k_bc_inlet(Batch B, Phys P, Geo G, Flow<T> W, const DevInOut *pat)
{
    const DevInOut pt = pat[blockIdx.y];
    const Lvl L = B.lv[pt.solve];
    const int ni = pt.ie - pt.is + 1, nj = pt.je - pt.js + 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ni * nj) return;
    const int i = pt.is + t / nj, j = pt.js + t % nj;
    const bool low = (pt.ks == 1);
    const int k = low ? 1 : L.KM - 1, kv = low ? 0 : L.KM;
    const long long fp = ix(L, i, j, low ? 1 : L.KM);
    const double Sx = G.S[2][0][fp], Sy = G.S[2][1][fp], Sz = G.S[2][2][fp];
    const double n_m = sqrt(Sx * Sx + Sy * Sy + Sz * Sz);
    const long long p = ix(L, i, j, k), g = ix(L, i, j, kv);
    const double u = W.pv[PU][p], v = W.pv[PV][p], w = W.pv[PW][p];
    double vdn = (u * Sx / n_m + v * Sy / n_m + w * Sz / n_m);
    if (low) vdn = -1.0 * vdn;
    const double gam = P.gamma, g1 = gam - 1.0, R = P.rgas, Ttin = P.ttin, Ptin = P.ptin;
    const double c_d = sqrt(gam * R * (double)W.pv[PT][p]);
    const double V2 = u * u + v * v + w * w;
    const double costh = -1.0 * vdn / sqrt(V2);
    const double c02 = c_d * c_d + g1 * V2 / 2.0;
    const double Rm = vdn - 2.0 * c_d / g1;
    const double mA = (-Rm * g1) / (g1 * costh * costh + 2.0);
    const double mB = sqrt(c02 * (g1 * costh * costh + 2.0) / g1 / (Rm * Rm) - g1 / 2.0);
    const double cb = mA * (1.0 + costh * mB);
    double Tb = Ttin * (cb * cb / c02);
    if (Tb > Ttin) Tb = (double)0.99f * Ttin;
    const double pb = Ptin * pow(Tb / Ttin, gam / g1);
    const double db = pb / R / Tb;
    const double Vb = sqrt(2.0 * gam / g1 * R * (Ttin - Tb));
    const double gu = Vb * P.inlet_dir[0] / P.inlet_vnm, gv = Vb * P.inlet_dir[1] / P.inlet_vnm,
                 gw = Vb * P.inlet_dir[2] / P.inlet_vnm;
    const double e = pb / db / g1 + (gu * gu + gv * gv + gw * gw) / 2.0;
    const double c[5] = {db, db * gu, db * gv, db * gw, db * e};
    const T q[6] = {(T)db, (T)gu, (T)gv, (T)gw, (T)pb, (T)Tb};
    st_state(W, g, c, q);
    for (int nd = 1; nd <= P.ndummy; nd++) st_state(W, ix(L, i, j, low ? -nd : L.KM + nd), c, q);
}

// axial outlet in three launches spread over the SMs: mass-weighted swirl per radial row (one
// warp per row, lanes over the pitch), radial equilibrium marched from p_out at i = IM/2 using
// the previous ghost density (one warp per pitch line), then ghosts extrapolated from the last
// interior layer (one thread per face)
template <typename T>
__global__ void __launch_bounds__(256) k_outlet_swirl(Batch B, Geo G, Flow<T> W, const DevInOut *pat, double *cu_all,
                                                      int cu_stride)
{
    const DevInOut pt = pat[blockIdx.y];
    const Lvl L = B.lv[pt.solve];
    const int JM = L.JM, KM = L.KM;
    const int lane = threadIdx.x & 31;
    const int i = 1 + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i > L.IM - 1) return;
    double acc = 0.0, sa = 0.0;
    for (int j = 1 + lane; j <= JM - 1; j += 32) {
        const long long p = ix(L, i, j, KM - 1), f = ix(L, i, j, KM);
        const double th = G.th[2][f];
        double sn, cs;
        sincos(th, &sn, &cs);
        const double ct = -1.0 * (double)W.pv[PU][p] * sn + (double)W.pv[PV][p] * cs;
        acc = acc + ct * G.s[2][f];
        sa = sa + G.s[2][f];
    }
    for (int o = 16; o > 0; o >>= 1) {
        acc += __shfl_down_sync(0xffffffffu, acc, o);
        sa += __shfl_down_sync(0xffffffffu, sa, o);
    }
    if (lane == 0) cu_all[(long long)blockIdx.y * cu_stride + i] = acc / sa;
}

// The march p_i = p_(i+1) - t_i (towards the hub) and p_i = p_(i-1) + u_i (towards the casing)
// has increments that do not depend on p, so one warp per pitch line forms them for 32 radial
// rows at a time and adds them up with a warp scan (a different association of the same sums
// than the reference's running total).
template <typename T>
__global__ void __launch_bounds__(32) k_outlet_march(Batch B, Geo G, Flow<T> W, const DevInOut *pat, const double *cu_all,
                                                     int cu_stride)
{
    const DevInOut pt = pat[blockIdx.y];
    const Lvl L = B.lv[pt.solve];
    const int IM = L.IM, KM = L.KM;
    const int j = 1 + blockIdx.x, lane = threadIdx.x;
    if (j > L.JM - 1) return;
    const double *cu = cu_all + (long long)blockIdx.y * cu_stride;
    const int iref = (int)(0.5 * IM);
    const double pout = B.st[pt.solve].pout;
    if (lane == 0) W.pv[PP][ix(L, iref, j, KM)] = (T)pout;
    // towards the hub: i = iref-1, iref-2, ..., 1
    double carry = 0.0;
    for (int base = 0; base < iref - 1; base += 32) {
        const int i = iref - 1 - base - lane;
        double t = 0.0;
        if (i >= 1) {
            const double rn = G.r[2][ix(L, i, j, KM)], rn1 = G.r[2][ix(L, i + 1, j, KM)];
            const double dpdr = W.cv[0][ix(L, i, j, KM)] * cu[i] * cu[i] / rn;
            t = dpdr * (rn1 - rn);
        }
        for (int o = 1; o < 32; o <<= 1) {
            const double v = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += v;
        }
        if (i >= 1) W.pv[PP][ix(L, i, j, KM)] = (T)(pout - (carry + t));
        carry += __shfl_sync(0xffffffffu, t, 31);
    }
    // towards the casing: i = iref+1, ..., IM-1, radii of the k = KM-1 face row as the reference takes them
    carry = 0.0;
    for (int base = 0; base < IM - 1 - iref; base += 32) {
        const int i = iref + 1 + base + lane;
        double u = 0.0;
        if (i <= IM - 1) {
            const double rn1 = G.r[2][ix(L, i, j, KM - 1)], rn = G.r[2][ix(L, i - 1, j, KM - 1)];
            const double dpdr = W.cv[0][ix(L, i, j, KM)] * cu[i] * cu[i] / rn;
            u = dpdr * (rn1 - rn);
        }
        for (int o = 1; o < 32; o <<= 1) {
            const double v = __shfl_up_sync(0xffffffffu, u, o);
            if (lane >= o) u += v;
        }
        if (i <= IM - 1) W.pv[PP][ix(L, i, j, KM)] = (T)(pout + (carry + u));
        carry += __shfl_sync(0xffffffffu, u, 31);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_outlet_fill(Batch B, Phys P, Flow<T> W, const DevInOut *pat)
{
    const DevInOut pt = pat[blockIdx.y];
    const Lvl L = B.lv[pt.solve];
    const int IM = L.IM, JM = L.JM, KM = L.KM;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (IM - 1) * (JM - 1)) return;
    const double g1 = P.gamma - 1.0;
    const int i = 1 + t / (JM - 1), j = 1 + t % (JM - 1);
    const long long g = ix(L, i, j, KM), p = ix(L, i, j, KM - 1);
    const double d = W.cv[0][p];
    const double pr = (double)W.pv[PP][g];
    const double u = W.pv[PU][p], v = W.pv[PV][p], w = W.pv[PW][p];
    const double c[5] = {d, W.cv[1][p], W.cv[2][p], W.cv[3][p], pr / g1 + d * (u * u + v * v + w * w) / 2.0};
    const T q[6] = {(T)d, (T)u, (T)v, (T)w, (T)pr, (T)(pr / P.rgas / d)};
    st_state(W, g, c, q);
    for (int nd = 1; nd <= P.ndummy; nd++) st_state(W, ix(L, i, j, KM + nd), c, q);
}

// no-slip wall: ghost keeps p, T, rho, rho*E of the first cell, relative velocity reflected;
// reconstruction layers = mean of ghost and first cell
template <typename T>
__global__ void k_bc_wall(Batch B, Phys P, Geo G, Flow<T> W, const DevWall *walls)
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
    // (i,j,k) is the wall face; interior cell next to it and the ghost on the other side
    const long long fp = ix(L, i, j, k);
    const long long pin = lo ? fp : fp - sn, g = lo ? fp - sn : fp;
    const long long step = lo ? -sn : sn;           // from the ghost outwards
    const double rot = wl.rotate ? B.sc[wl.solve].w_rot : 0.0;
    const double x = G.c[f][0][fp], y = G.c[f][1][fp];
    const double vwx = -rot * y, vwy = rot * x;
    const double u = W.pv[PU][pin], v = W.pv[PV][pin], w = W.pv[PW][pin];
    const double gu = (0.0 - (u - vwx)) + vwx, gv = (0.0 - (v - vwy)) + vwy, gw = (0.0 - (w - 0.0)) + 0.0;
    const double d = W.cv[0][pin];
    const double c[5] = {d, gu * d, gv * d, gw * d, W.cv[4][pin]};
    const T q[6] = {W.pv[PD][pin], (T)gu, (T)gv, (T)gw, W.pv[PP][pin], W.pv[PT][pin]};
    st_state(W, g, c, q);
    double cm[5];
    T qm[6];
#pragma unroll
    for (int n = 0; n < 5; n++) cm[n] = 0.5 * (c[n] + W.cv[n][pin]);
#pragma unroll
    for (int n = 0; n < 6; n++) qm[n] = (T)0.5 * (q[n] + W.pv[n][pin]);
    for (int nd = 1; nd <= P.ndummy; nd++) st_state(W, g + nd * step, cm, qm);
}

// periodic exchange: ghost/dummy <- interior cell of the partner face, velocity and momentum
// rotated about z by +-delta_th
template <typename T>
__global__ void k_bc_periodic(Batch B, Flow<T> W, const long long *dst, const long long *src, const int *meta,
                              const double *trig, long long n)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int mt = meta[t];
    const int s = mt >> 2, sg = (mt & 3) - 1;
    const long long a = src[t], b = dst[t];
    const double dr = sg * B.sc[s].delta_th;
    double c[5];
    T q[6];
#pragma unroll
    for (int m = 0; m < 5; m++) c[m] = W.cv[m][a];
#pragma unroll
    for (int m = 0; m < 6; m++) q[m] = W.pv[m][a];
    if (dr != 0.0) {
        // cos(dr) and sin(dr), formed once per solve by k_periodic_trig with the same functions
        const double *tr = trig + 4 * s + (sg > 0 ? 0 : 2);
        const double cs = tr[0], sn = tr[1];
        const double mx = c[1], my = c[2];
        c[1] = mx * cs - my * sn;
        c[2] = my * cs + mx * sn;
        const double u = q[PU], v = q[PV];
        q[PU] = (T)(u * cs - v * sn);
        q[PV] = (T)(v * cs + u * sn);
    }
    st_state(W, b, c, q);
}

// cosine and sine of the periodic rotation +-delta_th of every solve (the entries of the gather
// list read them instead of evaluating FP64 trigonometric functions per ghost cell)
__global__ void k_periodic_trig(Batch B, double *trig)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B.nsolve) return;
    const double x = B.sc[s].delta_th;
    const double p = 1.0 * x, m = -1.0 * x;
    trig[4 * s + 0] = cos(p);
    trig[4 * s + 1] = sin(p);
    trig[4 * s + 2] = cos(m);
    trig[4 * s + 3] = sin(m);
}

void launch_periodic_trig(const LaunchCtx &ctx, double *trig)
{
    k_periodic_trig<<<(ctx.batch.nsolve + 127) / 128, 128, 0, ctx.stream>>>(ctx.batch, trig);
}

// mixing plane (CMesh::BndCondMixingPlane, source/BndCondMixingPlane.cpp:287-520), one warp per
// radial row and side: flux averages over the pitch of the last cell layer upstream (block 1,
// k = KM - 1, normals of the k = KM faces) and of the first layer downstream (block 2, k = 1), each
// turned into a mixed-out state by the quadratic for the pressure (the pitch sums are formed as a
// warp reduction, not in the reference's sequential order)
template <typename T>
__global__ void __launch_bounds__(32) k_mix_average(Batch B, Phys P, Geo G, Flow<T> W, const DevMix *mix, int max_rows, double *avg)
{
    const DevMix m = mix[blockIdx.y];
    const int r = blockIdx.x, side = blockIdx.z;
    if (r > m.ie - m.is) return;
    const int i = m.is + r;
    const double g = P.gamma, R = P.rgas;
    double *o = avg + ((long long)blockIdx.y * max_rows + r) * kMixVals;
    const int s = side ? m.s2 : m.s1;
    const Lvl L = B.lv[s];
    const int kf = side ? 1 : L.KM, kc = side ? 1 : L.KM - 1;
    const int j0 = side ? m.js2 : m.js1, j1 = side ? m.je2 : m.je1;
    double acc[10] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};   // I1..I6, n*s (3), s
    for (int j = j0 + (int)threadIdx.x; j <= j1; j += 32) {
        const long long f = ix(L, i, j, kf), c = ix(L, i, j, kc);
        const double sa = G.s[2][f];
        const double nx = G.S[2][0][f] / sa, ny = G.S[2][1][f] / sa, nz = G.S[2][2][f] / sa;
        const double u = W.pv[PU][c], v = W.pv[PV][c], w = W.pv[PW][c], pr = W.pv[PP][c];
        const double Vn = u * nx + v * ny + w * nz;
        acc[0] += W.cv[0][c] * Vn * sa;
        acc[1] += (W.cv[1][c] * Vn + nx * pr) * sa;
        acc[2] += (W.cv[2][c] * Vn + ny * pr) * sa;
        acc[3] += (W.cv[3][c] * Vn + nz * pr) * sa;
        acc[4] += (W.cv[4][c] + pr) * Vn * sa;
        if (W.ev) acc[5] += W.cv[0][c] * W.ev[c] * Vn * sa;
        acc[6] += nx * sa; acc[7] += ny * sa; acc[8] += nz * sa;
        acc[9] += sa;
    }
#pragma unroll
    for (int q = 0; q < 10; q++)
        for (int off = 16; off > 0; off >>= 1) acc[q] += __shfl_down_sync(0xffffffffu, acc[q], off);
    if (threadIdx.x != 0) return;
    const double ss = acc[9];
    const double I1 = acc[0] / ss, I2 = acc[1] / ss, I3 = acc[2] / ss, I4 = acc[3] / ss, I5 = acc[4] / ss;
    if (side == 0) o[12] = W.ev ? (acc[5] / ss) / I1 : 0.0;
    const double nux = acc[6] / ss, nuy = acc[7] / ss, nuz = acc[8] / ss;
    const double A = I2 * nux + I3 * nuy + I4 * nuz;
    const double Bq = 2.0 * I1 * I5 - (I2 * I2 + I3 * I3 + I4 * I4);
    const double C = nux * nux + nuy * nuy + nuz * nuz;
    const double pr = (A / C + sqrt(A * A / C / C - (g * g - 1.0) * Bq / C)) / (g + 1.0);
    const double u = (I2 - pr * nux) / I1, v = (I3 - pr * nuy) / I1, w = (I4 - pr * nuz) / I1;
    const double d = I1 / (u * nux + v * nuy + w * nuz);
    const double t = pr / R / d;
    double *q = o + 6 * side;
    q[0] = d; q[1] = u; q[2] = v; q[3] = w; q[4] = pr; q[5] = sqrt(g * R * t);
}

// ghost and reconstruction layers of both sides from the other side's mixed-out state and the
// outgoing characteristics (:431-518); the SA variable of both ghosts is the upstream average
template <typename T>
__global__ void k_mix_fill(Batch B, Phys P, Flow<T> W, const DevMix *mix, int max_rows, int max_j, const double *avg)
{
    const DevMix m = mix[blockIdx.y];
    const int side = blockIdx.z;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int j0 = side ? m.js2 : m.js1, nj = (side ? m.je2 : m.je1) - j0 + 1;
    const int nr = m.ie - m.is + 1;
    if (t >= nr * nj) return;
    const int r = t / nj, i = m.is + r, j = j0 + t % nj;
    const double *o = avg + ((long long)blockIdx.y * max_rows + r) * kMixVals;
    const double *pu = o, *pd = o + 6;                         // d u v w p c of the upstream / downstream average
    const double g = P.gamma, R = P.rgas;
    const Lvl L = B.lv[side ? m.s2 : m.s1];
    double d, u, v, w, pr;
    long long gp, step;
    if (side == 0) {
        const long long c = ix(L, i, j, L.KM - 1);
        const double cu = pu[5], cd = pd[5];
        const double C1 = -cu * cu * ((double)W.pv[PD][c] - pu[0]) + ((double)W.pv[PP][c] - pu[4]);
        const double C2 = pu[0] * cu * ((double)W.pv[PW][c] - pu[3]) + ((double)W.pv[PP][c] - pu[4]);
        const double C5 = 0.0;
        d = pd[0] + (-C1 + (C2 + C5) / 2.0) / (cd * cd);
        w = pd[3] + (C2 - C5) / (2.0 * pd[0] * cd);
        v = W.pv[PV][c];
        u = W.pv[PU][c];
        pr = pd[4] + (C2 + C5) / 2.0;
        gp = ix(L, i, j, L.KM);
        step = 1;
    } else {
        const long long c = ix(L, i, j, 1);
        const double cu = pu[5], cd = pd[5];
        const double C5 = (0.0 - pd[0] * cd * ((double)W.pv[PW][c] - pd[3]) + ((double)W.pv[PP][c] - pd[4]));
        d = pu[0] + (-0.0 + (0.0 + C5) / 2.0) / (cu * cu);
        w = pu[3] - C5 / (2.0 * pu[0] * cu);
        v = pu[2] + 0.0 / (pu[0] * cu);
        u = pu[1] + 0.0 / (pu[0] * cu);
        pr = pu[4] + (0.0 + C5) / 2.0;
        gp = ix(L, i, j, 0);
        step = -1;
    }
    const double V2 = pow(u, 2.0) + pow(v, 2.0) + pow(w, 2.0);
    const double c[5] = {d, d * u, d * v, d * w, pr / (g - 1.0) + d * V2 / 2.0};
    const T q[6] = {(T)d, (T)u, (T)v, (T)w, (T)pr, (T)(pr / R / d)};
    st_state(W, gp, c, q);
    if (W.ev) W.ev[gp] = o[12];
    for (int nd = 1; nd <= P.ndummy; nd++) st_state(W, gp + step * nd, c, q);
}

template <typename T>
void launch_boundary(const LaunchCtx &ctx, const Phys &P, const Geo &G, Flow<T> W, const BcTables &bc)
{
    const Batch &B = ctx.batch;
    // 32-thread blocks: the FP64 powers and roots of the inlet state spread over many SMs
    if (bc.n_inlet) k_bc_inlet<T><<<dim3((bc.max_inlet + 31) / 32, bc.n_inlet), 32, 0, ctx.stream>>>(B, P, G, W, bc.inlet);
    if (bc.n_outlet) {
        const int cs = bc.max_outlet_im + 1;
        k_outlet_swirl<T><<<dim3((bc.max_outlet_im + 7) / 8, bc.n_outlet), 256, 0, ctx.stream>>>(B, G, W, bc.outlet, bc.outlet_cu, cs);
        k_outlet_march<T><<<dim3(bc.max_outlet_jm, bc.n_outlet), 32, 0, ctx.stream>>>(B, G, W, bc.outlet, bc.outlet_cu, cs);
        k_outlet_fill<T><<<dim3((bc.max_outlet_im * bc.max_outlet_jm + 255) / 256, bc.n_outlet), 256, 0, ctx.stream>>>(B, P, W, bc.outlet);
    }
    if (bc.n_wall) k_bc_wall<T><<<dim3((bc.max_wall + 127) / 128, bc.n_wall), 128, 0, ctx.stream>>>(B, P, G, W, bc.wall);
    if (bc.n_per)
        k_bc_periodic<T><<<(unsigned)((bc.n_per + 255) / 256), 256, 0, ctx.stream>>>(B, W, bc.per_dst, bc.per_src, bc.per_meta,
                                                                                   bc.per_trig, bc.n_per);
    if (W.ev) launch_sa_boundary<T>(ctx, P, W, bc);
    if (bc.n_mix) {
        k_mix_average<T><<<dim3(bc.max_mix_rows, bc.n_mix, 2), 32, 0, ctx.stream>>>(B, P, G, W, bc.mix, bc.max_mix_rows, bc.mix_avg);
        k_mix_fill<T><<<dim3((bc.max_mix_rows * bc.max_mix_j + 127) / 128, bc.n_mix, 2), 128, 0, ctx.stream>>>(
            B, P, W, bc.mix, bc.max_mix_rows, bc.max_mix_j, bc.mix_avg);
    }
}

template void launch_boundary<double>(const LaunchCtx &, const Phys &, const Geo &, Flow<double>, const BcTables &);
template void launch_boundary<float>(const LaunchCtx &, const Phys &, const Geo &, Flow<float>, const BcTables &);

}  // namespace gbt
