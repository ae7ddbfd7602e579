// Setup-time geometry of every level, FP64 on the device (source/GeometryVariables.cpp:10-391),
// plus the per-face and per-cell quantities the hot kernels would otherwise recompute every
// iteration: face frames of the flux rotation (source/Flux_Split_Scheme.cpp:728-776), mean area
// vectors of the spectral radii and time step (source/Spectral_curl_grad.cpp:28-38,
// source/TimeStep.cpp:34-36) and mean normals / areas / entrainment speeds of the LU-SGS
// off-diagonal terms (source/LU_SGS_Marching.cpp:88,293-341). Every stored value is the same
// expression the reference evaluates in place.
#include "gbt_common.cuh"
#include "kernels.hpp"
#include <algorithm>

namespace gbt {

struct V3 { double x, y, z; };
__device__ __forceinline__ V3 v3(double x, double y, double z) { V3 r = {x, y, z}; return r; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(double s, V3 a) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 node(const Geo &G, const Lvl &L, int i, int j, int k)
{
    long long p = ix(L, i, j, k);
    return v3(G.x[p], G.y[p], G.z[p]);
}
__device__ __forceinline__ V3 fS(const Geo &G, int f, long long p) { return v3(G.S[f][0][p], G.S[f][1][p], G.S[f][2][p]); }
__device__ __forceinline__ V3 fC(const Geo &G, int f, long long p) { return v3(G.c[f][0][p], G.c[f][1][p], G.c[f][2][p]); }

// :17-76 face vector (diagonal cross product), centre, polar coordinates, |S|; face frame
__global__ void k_face_geo(Batch B, Geo G, int f)
{
    const Lvl L = B.lv[blockIdx.y];
    int ni, nj, nk, i, j, k;
    face_extent(L, f, ni, nj, nk);
    if (!box_index(ni, nj, nk, i, j, k)) return;
    V3 A, Bv, c, r;
    if (f == 0) {
        A = node(G, L, i, j + 1, k) - node(G, L, i, j, k + 1);
        Bv = node(G, L, i, j + 1, k + 1) - node(G, L, i, j, k);
        c = 0.25 * (((node(G, L, i, j, k) + node(G, L, i, j + 1, k)) + node(G, L, i, j + 1, k + 1)) + node(G, L, i, j, k + 1));
        r = node(G, L, i, j + 1, k + 1) - node(G, L, i, j, k);
    } else if (f == 1) {
        A = node(G, L, i, j, k + 1) - node(G, L, i + 1, j, k);
        Bv = node(G, L, i + 1, j, k + 1) - node(G, L, i, j, k);
        c = 0.25 * (((node(G, L, i, j, k) + node(G, L, i + 1, j, k)) + node(G, L, i + 1, j, k + 1)) + node(G, L, i, j, k + 1));
        r = node(G, L, i + 1, j, k + 1) - node(G, L, i, j, k);
    } else {
        A = node(G, L, i + 1, j + 1, k) - node(G, L, i, j, k);
        Bv = node(G, L, i, j + 1, k) - node(G, L, i + 1, j, k);
        c = 0.25 * (((node(G, L, i, j, k) + node(G, L, i + 1, j, k)) + node(G, L, i + 1, j + 1, k)) + node(G, L, i, j + 1, k));
        r = node(G, L, i + 1, j + 1, k) - node(G, L, i, j, k);
    }
    long long p = ix(L, i, j, k);
    V3 S = v3(0.5 * (A.y * Bv.z - Bv.y * A.z), 0.5 * (A.z * Bv.x - A.x * Bv.z), 0.5 * (A.x * Bv.y - Bv.x * A.y));
    double s = sqrt(S.x * S.x + S.y * S.y + S.z * S.z);
    G.S[f][0][p] = S.x; G.S[f][1][p] = S.y; G.S[f][2][p] = S.z; G.s[f][p] = s;
    G.c[f][0][p] = c.x; G.c[f][1][p] = c.y; G.c[f][2][p] = c.z;
    G.r[f][p] = sqrt(c.x * c.x + c.y * c.y);
    G.th[f][p] = atan(c.y / c.x);
    // frame: n = S/|S|, tau1 along the node diagonal, tau2 = n x tau1 (both normalised)
    V3 n = v3(S.x / s, S.y / s, S.z / s);
    double rl = sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
    V3 t1 = v3(r.x / rl, r.y / rl, r.z / rl);
    V3 q = v3(n.y * t1.z - n.z * t1.y, n.z * t1.x - n.x * t1.z, n.x * t1.y - n.y * t1.x);
    double ql = sqrt(q.x * q.x + q.y * q.y + q.z * q.z);
    V3 t2 = v3(q.x / ql, q.y / ql, q.z / ql);
    G.nrm[f][0][p] = n.x; G.nrm[f][1][p] = n.y; G.nrm[f][2][p] = n.z;
    G.t1[f][0][p] = t1.x; G.t1[f][1][p] = t1.y; G.t1[f][2][p] = t1.z;
    G.t2[f][0][p] = t2.x; G.t2[f][1][p] = t2.y; G.t2[f][2][p] = t2.z;
    double w = B.sc[blockIdx.y].w_rot;
    double ue = -1.0 * c.y * w, ve = c.x * w;
    G.qe[f][p] = ue * n.x + ve * n.y + 0.0 * n.z;
}

// :77-103 volume by the divergence theorem and centre; derived per-cell quantities
__global__ void k_cell_geo(Batch B, Geo G)
{
    const Lvl L = B.lv[blockIdx.y];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    long long p = ix(L, i, j, k);
    long long q[3] = {ix(L, i + 1, j, k), ix(L, i, j + 1, k), ix(L, i, j, k + 1)};
    double v = dot(fC(G, 0, q[0]), fS(G, 0, q[0])) - dot(fC(G, 0, p), fS(G, 0, p)) +
               dot(fC(G, 1, q[1]), fS(G, 1, q[1])) - dot(fC(G, 1, p), fS(G, 1, p)) +
               dot(fC(G, 2, q[2]), fS(G, 2, q[2])) - dot(fC(G, 2, p), fS(G, 2, p));
    v = v / 3.0;
    G.vol[p] = v;
    V3 c = node(G, L, i, j, k) + node(G, L, i + 1, j, k);
    c = c + node(G, L, i, j + 1, k);
    c = c + node(G, L, i + 1, j + 1, k);
    c = c + node(G, L, i, j, k + 1);
    c = c + node(G, L, i + 1, j, k + 1);
    c = c + node(G, L, i, j + 1, k + 1);
    c = c + node(G, L, i + 1, j + 1, k + 1);
    c = 0.125 * c;
    G.cc[0][p] = c.x; G.cc[1][p] = c.y; G.cc[2][p] = c.z;
    double w = B.sc[blockIdx.y].w_rot;
    double ue = -1.0 * c.y * w, ve = c.x * w;
    for (int d = 0; d < 3; d++) {
        V3 sb = 0.5 * (fS(G, d, p) + fS(G, d, q[d]));
        G.sb[d][0][p] = sb.x; G.sb[d][1][p] = sb.y; G.sb[d][2][p] = sb.z;
        V3 cn = v3((G.nrm[d][0][q[d]] + G.nrm[d][0][p]) / 2.0, (G.nrm[d][1][q[d]] + G.nrm[d][1][p]) / 2.0,
                   (G.nrm[d][2][q[d]] + G.nrm[d][2][p]) / 2.0);
        G.cn[d][0][p] = cn.x; G.cn[d][1][p] = cn.y; G.cn[d][2][p] = cn.z;
        G.cs[d][p] = 0.5 * (G.s[d][p] + G.s[d][q[d]]);
        G.cve[d][p] = ue * cn.x + ve * cn.y + 0.0 * cn.z;
    }
}

// metric coefficients; gradz_kesi repeats the gradx_kesi expression (:201-209 etc.)
__device__ void metrics(double *out, double xk, double yk, double zk, double xe, double ye, double ze,
                        double xz, double yz, double zz)
{
    const double lim_zero = (double)1E-20f;
    double partA = (xk * (ye * zz - yz * ze));
    double partB = (xe * (yk * zz - yz * zk));
    double partC = (xz * (yk * ze - ye * zk));
    double J1 = (partA - partB + partC);
    if (fabs(J1) <= lim_zero) J1 = lim_zero;
    double J = 1.0 / J1;
    out[0] = J * (ye * zz - yz * ze);
    out[1] = J * (ze * xz - zz * xe);
    out[2] = J * (ye * zz - yz * ze);
    out[3] = J * (yz * zk - yk * zz);
    out[4] = J * (zz * xk - zk * xz);
    out[5] = J * (xz * yk - xk * yz);
    out[6] = J * (yk * ze - ye * zk);
    out[7] = J * (zk * xe - ze * xk);
    out[8] = J * (xk * ye - xe * yk);
}

// one-sided at the first/last cell, central inside (:133-192)
__device__ V3 cdiff(const Geo &G, const Lvl &L, int i, int j, int k, int d)
{
    int n = d == 0 ? L.IM : (d == 1 ? L.JM : L.KM);
    int a = d == 0 ? i : (d == 1 ? j : k);
    int o[3] = {0, 0, 0};
    o[d] = 1;
    long long p = ix(L, i, j, k), pp = ix(L, i + o[0], j + o[1], k + o[2]), pm = ix(L, i - o[0], j - o[1], k - o[2]);
    V3 c0 = v3(G.cc[0][p], G.cc[1][p], G.cc[2][p]);
    if (a == 1) return v3(G.cc[0][pp], G.cc[1][pp], G.cc[2][pp]) - c0;
    if (a == n - 1) return c0 - v3(G.cc[0][pm], G.cc[1][pm], G.cc[2][pm]);
    V3 dd = v3(G.cc[0][pp], G.cc[1][pp], G.cc[2][pp]) - v3(G.cc[0][pm], G.cc[1][pm], G.cc[2][pm]);
    return 0.5 * dd;
}

__global__ void k_cell_metrics(Batch B, Geo G)
{
    const Lvl L = B.lv[blockIdx.y];
    int i, j, k;
    if (!box_index(L.IM - 1, L.JM - 1, L.KM - 1, i, j, k)) return;
    V3 dk = cdiff(G, L, i, j, k, 0), de = cdiff(G, L, i, j, k, 1), dz = cdiff(G, L, i, j, k, 2);
    double m[9];
    metrics(m, dk.x, dk.y, dk.z, de.x, de.y, de.z, dz.x, dz.y, dz.z);
    long long p = ix(L, i, j, k);
    for (int c = 0; c < 9; c++) G.cm[c][p] = m[c];
}

// :214-389 face metrics: the derivative along the face normal from neighbouring face centres,
// the two tangential ones from edge midpoints of the face
__global__ void k_face_metrics(Batch B, Geo G, int f)
{
    const Lvl L = B.lv[blockIdx.y];
    int ni, nj, nk, i, j, k;
    face_extent(L, f, ni, nj, nk);
    if (!box_index(ni, nj, nk, i, j, k)) return;
    long long p = ix(L, i, j, k);
    int o[3] = {0, 0, 0};
    o[f] = 1;
    int a = f == 0 ? i : (f == 1 ? j : k);
    int n = f == 0 ? L.IM : (f == 1 ? L.JM : L.KM);
    long long pp = ix(L, i + o[0], j + o[1], k + o[2]), pm = ix(L, i - o[0], j - o[1], k - o[2]);
    V3 dn;
    if (a == 1) dn = fC(G, f, pp) - fC(G, f, p);
    else if (a == n) dn = fC(G, f, p) - fC(G, f, pm);
    else dn = 0.5 * (fC(G, f, pp) - fC(G, f, pm));
    V3 d1, d2;     // the two tangential derivatives in (kesi, yita, zita) order
    if (f == 0) {
        V3 n0 = node(G, L, i, j, k), n1 = node(G, L, i, j + 1, k), n2 = node(G, L, i, j + 1, k + 1), n3 = node(G, L, i, j, k + 1);
        d1 = 0.5 * (n1 + n2) - 0.5 * (n0 + n3);
        d2 = 0.5 * (n3 + n2) - 0.5 * (n0 + n0);          // Node[i][j][k] taken twice (:248-250)
    } else if (f == 1) {
        V3 n0 = node(G, L, i, j, k), n1 = node(G, L, i + 1, j, k), n2 = node(G, L, i + 1, j, k + 1), n3 = node(G, L, i, j, k + 1);
        d1 = 0.5 * (n1 + n2) - 0.5 * (n0 + n3);
        d2 = 0.5 * (n3 + n2) - 0.5 * (n0 + n1);
    } else {
        V3 n0 = node(G, L, i, j, k), n1 = node(G, L, i + 1, j, k), n2 = node(G, L, i + 1, j + 1, k), n3 = node(G, L, i, j + 1, k);
        d1 = 0.5 * (n2 + n1) - 0.5 * (n0 + n3);
        d2 = 0.5 * (n2 + n3) - 0.5 * (n1 + n0);
    }
    V3 dk, de, dz;
    if (f == 0) { dk = dn; de = d1; dz = d2; }
    else if (f == 1) { dk = d1; de = dn; dz = d2; }
    else { dk = d1; de = d2; dz = dn; }
    double m[9];
    metrics(m, dk.x, dk.y, dk.z, de.x, de.y, de.z, dz.x, dz.y, dz.z);
    for (int c = 0; c < 9; c++) G.m[f][c][p] = m[c];
}

// total volume per solve (ComputeAllBlockVars.cpp:28-33), one block per solve
__global__ void __launch_bounds__(1024) k_total_volume(Batch B, Geo G, double *out)
{
    const Lvl L = B.lv[blockIdx.y];
    int nI = L.IM - 1, nJ = L.JM - 1, nK = L.KM - 1;
    long long n = (long long)nI * nJ * nK;
    double acc = 0.0;
    for (long long t = threadIdx.x; t < n; t += blockDim.x) {
        int k = (int)(t % nK) + 1;
        long long q = t / nK;
        int j = (int)(q % nJ) + 1, i = (int)(q / nJ) + 1;
        acc += G.vol[ix(L, i, j, k)];
    }
    __shared__ double sh[32];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) out[blockIdx.y] = acc;
    }
}

void launch_geometry(const LaunchCtx &ctx, const Geo &G, double *totalvol)
{
    Batch B = ctx.batch;
    dim3 blk(256);
    for (int f = 0; f < 3; f++)
        k_face_geo<<<ctx.grid_faces(f, 256), blk, 0, ctx.stream>>>(B, G, f);
    k_cell_geo<<<ctx.grid_cells(256), blk, 0, ctx.stream>>>(B, G);
    k_cell_metrics<<<ctx.grid_cells(256), blk, 0, ctx.stream>>>(B, G);
    for (int f = 0; f < 3; f++)
        k_face_metrics<<<ctx.grid_faces(f, 256), blk, 0, ctx.stream>>>(B, G, f);
    k_total_volume<<<dim3(1, B.nsolve), dim3(1024), 0, ctx.stream>>>(B, G, totalvol);
}

// ---- FP32 copies of the geometry read by the working-precision kernels (mixed form) ----
__global__ void __launch_bounds__(256) k_to_float(const double *__restrict__ src, float *__restrict__ dst, long long n)
{
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        dst[t] = (float)src[t];
}

void launch_geometry_working(const LaunchCtx &ctx, const Geo &G, const GeoW<float> &W)
{
    const long long n = ctx.pool_n;
    const unsigned g = (unsigned)std::min<long long>((n + 255) / 256, 152LL * 16);
    auto cv = [&](const double *a, float *b) { k_to_float<<<g, 256, 0, ctx.stream>>>(a, b, n); };
    for (int f = 0; f < 3; f++) {
        for (int c = 0; c < 3; c++) {
            cv(G.S[f][c], W.S[f][c]); cv(G.nrm[f][c], W.nrm[f][c]); cv(G.t1[f][c], W.t1[f][c]); cv(G.t2[f][c], W.t2[f][c]);
            cv(G.sb[f][c], W.sb[f][c]);
        }
        for (int c = 0; c < 2; c++) cv(G.c[f][c], W.c[f][c]);
        cv(G.s[f], W.s[f]);
        cv(G.qe[f], W.qe[f]);
        for (int c = 0; c < 9; c++) cv(G.m[f][c], W.m[f][c]);
    }
    cv(G.vol, W.vol);
    for (int c = 0; c < 2; c++) cv(G.cc[c], W.cc[c]);
    for (int c = 0; c < 9; c++) cv(G.cm[c], W.cm[c]);
}

}  // namespace gbt
