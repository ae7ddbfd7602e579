// Shared device-side definitions of the GB300 residual-and-update path.
//
// Data layout: every array of one mesh level of one operating point ("solve") lives on a padded
// box i in [-3, IM+3] x j in [-3, JM+3] x k in [-3, KM+3] with k contiguous (the axial index is
// the longest one on turbomachinery passages, so warps read along it). Cell (i,j,k) spans nodes
// i..i+1; index 0 and IM hold the first ghost layer of the reference solver and the two
// reconstruction layers ("dummies") sit at -1,-2 and IM+1, IM+2 (a third at -3, IM+3 with JST). Face family f (0=I, 1=J, 2=K)
// at (i,j,k) is the reference's FaceI/J/K[i][j][k]. All solves of a batch share one pool per
// field; a solve's box starts at Lvl::base.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "dfloat.cuh"

namespace gbt {

constexpr int PAD = 3;
constexpr int NQ = 5;
constexpr int NPV = 6;                 // dens u v w press temp
enum { PD = 0, PU, PV, PW, PP, PT };

struct Lvl {
    int IM, JM, KM;                    // node counts
    int NJ, NK;                        // padded extents (strides)
    long long base;                    // offset of this solve's box in every pool of the level
};

__host__ __device__ inline long long ix(const Lvl &L, int i, int j, int k)
{
    return L.base + ((long long)(i + PAD) * L.NJ + (j + PAD)) * (long long)L.NK + (k + PAD);
}
__host__ __device__ inline long long box_size(int IM, int JM, int KM)
{
    return (long long)(IM + 1 + 2 * PAD) * (JM + 1 + 2 * PAD) * (KM + 1 + 2 * PAD);
}

// Geometry of a level (FP64 in both precision forms).
struct Geo {
    double *x, *y, *z;                        // nodes
    double *S[3][3], *s[3], *c[3][3];          // face area vector, |S|, face centre
    double *r[3], *th[3];                      // face polar radius / angle
    double *m[3][9];                           // face metric coefficients
    double *nrm[3][3], *t1[3][3], *t2[3][3];   // face frame: unit normal, tau1, tau2
    double *qe[3];                             // normal entrainment speed of the face
    double *vol, *cc[3], *cm[9];               // cell volume, centre, metrics
    double *sb[3][3];                          // per cell, per direction: mean area vector
    double *cn[3][3];                          // per cell, per direction: mean unit normal
    double *cs[3];                             // per cell, per direction: mean |S|
    double *cve[3];                            // per cell, per direction: entrainment speed
};

// Flow arrays of a level. T is the working type (double, or float in the mixed form).
template <typename T>
struct Flow {
    double *cv[NQ];                                  // conserved variables (FP64 in both forms)
    double *cvold[NQ];
    T *pv[NPV];
    T *mut, *omega, *dt;
    T *mul;                                          // FP64 form: laminar viscosity (Sutherland) per cell, formed
                                                     // with the spectral radii for Baldwin-Lomax and the viscous radii
    T *lamc[3], *lamv[3];
    T *Ff[3][NQ], *Vf[3][NQ];                        // face convective / viscous fluxes
    T *Fd[3][NQ];                                    // face artificial dissipation (JST only, else null)
    T *jsens[3], *jva[3];                            // JST per cell and direction: pressure sensor, phi * lambda
    T *res[NQ], *dq[NQ];
    double *cv2h[NQ];                                // multigrid (coarse level only)
    T *res2h[NQ], *dq2h[NQ];
    // Baldwin-Lomax merge over the walls: per cell the bit pattern of the smallest mu_t of the
    // lines that reach it (mu_t >= 0 orders as an unsigned integer; all ones = not reached)
    unsigned long long *blmin;
    const int *wallf[3];                             // per face: wall patch (1-based) or 0
    // Spalart-Allmaras (fine level of a case with turbulence model 200; null otherwise): the
    // eddy-viscosity variable (FP64 like Q) and its copy before the model's clipping, its
    // residual and update, face fluxes (convective, viscous, gradient) and the wall distance
    double *ev, *evg;
    T *res_ev, *dq_ev;
    T *Fct[3], *Fvt[3], *Fv1t[3];
    double *dwall;
};

// Per-solve scalars that evolve on the device (one record per solve).
struct SolveState {
    double cfl, cfl_res;
    double res[NQ];
    double m_in, m_out, pr, eff, m_ratio;
    int flag_low_dt[4];                              // per level (index = level)
    int iter;
    int status;                                      // bit flags, see GBT_STATUS_*
    int limiter_hits;
    int pad_;
    double pout;                                     // current nondimensional back pressure (mass-flow control moves it)
};

// Per-solve constants (copied once).
struct SolveConst {
    double w_rot;                                    // nondimensional rotation speed
    double delta_th;                                 // periodic pitch angle (sign as used)
    double pout;                                     // nondimensional back pressure
    double nblade;
    // imposed mass flow (source/Solver.cpp:142-145, source/Structured_FV3D.cpp:186-193)
    double m_imposed, relax_press, resc_mass_imp;
    int iter_mass_imp, mass_imposed;
    // the case this block belongs to: its first slot and its number of blocks (the case-wide
    // residual norm and integrals combine these slots; every slot of a case holds the same
    // case-wide state)
    int lead, nblk, cix;                             // cix: the case's index
    int pad_;
};

// Global (per handle) physical constants, in the reference's nondimensional units.
struct Phys {
    double gamma, rgas, pr_lam, pr_tur, re_ref;
    double ptin, ttin;
    double dens_ref, vel_ref, temp_ref;
    double inlet_dir[3], inlet_vnm;
    double c_timestep, relax;
    double suth_c1, suth_c2;                         // (1 + 110.4/288.15) and 110.4/288.15 (float-rounded)
    double k2, k4;                                   // JST coefficients (k4 as the reciprocal of the config value)
    double ev_ratio;                                 // Spalart-Allmaras inlet / initial value of the variable
    int equation_ns, turb_bl, recon_var, recon, scheme, limiter, global_dt, ndummy;
    int turb_sa;
};

// Geometry in the working precision T, the copy the T-arithmetic kernels (face fluxes, spectral
// radii, curl, time step, residual sum) read: for T = double the pointers alias the FP64 arrays
// of Geo; for T = float they point at FP32 copies made once at set-up, holding exactly the values
// that converting the FP64 arrays at every use would give. (Converting at use costs one FP64-pipe
// instruction per value, and the FP64 pipe is GB300's narrowest.)
template <typename T>
struct GeoW {
    T *S[3][3], *s[3], *c[3][2], *nrm[3][3], *t1[3][3], *t2[3][3], *qe[3], *m[3][9];   // faces
    T *vol, *cc[2], *sb[3][3], *cm[9];                                                 // cells
};

// Physical constants in the working precision, converted (and the reciprocal Reynolds number
// formed) once on the host.
template <typename T>
struct PhysW {
    T gamma, gm1, rgas, pr_lam, pr_tur, c_timestep, relax, inv_re, suth_c1, suth_c2;
    // formed once in FP64 on the host: 1 / (gamma - 1) and the conductivity factors
    // gamma R / (gamma - 1) / Pr of the laminar and turbulent parts
    T rgm1, cond_lam, cond_tur;
};

template <typename T>
inline PhysW<T> phys_working(const Phys &P)
{
    PhysW<T> w;
    w.gamma = (T)P.gamma;
    w.gm1 = w.gamma - (T)1;
    w.rgas = (T)P.rgas;
    w.pr_lam = (T)P.pr_lam;
    w.pr_tur = (T)P.pr_tur;
    w.c_timestep = (T)P.c_timestep;
    w.relax = (T)P.relax;
    w.inv_re = (T)(1.0 / P.re_ref);
    w.suth_c1 = (T)P.suth_c1;
    w.suth_c2 = (T)P.suth_c2;
    const double g1 = (double)w.gamma - 1.0, cp = (double)w.gamma * (double)w.rgas / g1;
    w.rgm1 = (T)(1.0 / g1);
    w.cond_lam = (T)(cp / (double)w.pr_lam);
    w.cond_tur = (T)(cp / (double)w.pr_tur);
    return w;
}

// Status bits reported per solve.
enum {
    GBT_STATUS_NAN = 1,          // a residual norm or an integral is not finite
    GBT_STATUS_LIMITER = 2,      // the positivity limiter replaced cells in the last step
    GBT_STATUS_LIMITER_OVF = 4,  // more limited cells than the list holds (processed by a full scan)
    GBT_STATUS_WAIT_TIMEOUT = 8, // a kernel's bounded wait for its own asynchronous copies ran out
};

// an FP64 value in the working precision, and a working-precision value in FP64, with the
// conversion instructions' rounding but without the FP64 pipe (dfloat.cuh)
template <typename T> __device__ __forceinline__ T to_work(double x)
{
    if constexpr (sizeof(T) == 8) return x;
    else return f64_to_f32_rn(x);
}
template <typename T> __device__ __forceinline__ double to_f64(T x)
{
    if constexpr (sizeof(T) == 8) return x;
    else return f32_to_f64(x);
}

template <typename T> __device__ __forceinline__ T tsqrt(T x);
template <> __device__ __forceinline__ double tsqrt<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float tsqrt<float>(float x) { return sqrtf(x); }

// Reciprocal, quotient and square root for the FP64 form's compute-bound kernels. GB300 runs FP64
// at about 1/64 of its FP32 rate and every FP64 instruction (add, multiply, FMA) holds the pipe
// equally long, so the IEEE-rounded division and root (a hardware approximation followed by a long
// refinement and correction) are among the costliest steps of the face flux. These forms keep the
// hardware approximation and refine it by Newton-Raphson iteration (the textbook method; see
// e.g. P. Markstein, "Computation of elementary functions on the IBM RISC System/6000 processor",
// IBM J. Res. Dev. 34(1), 1990), to within two units in the last place of the IEEE results
// (checked against them by gb_fp64_arith_check):
//   1/b: r0 from rcp.approx.ftz.f64, e = 1 - b r0, then the third-order step r1 = r0 + r0 (e + e^2),
//        whose relative error is about e^3 -- three FMAs;
//   sqrt(x): y0 from rsqrt.approx.ftz.f64, s0 = x y0, then two Heron steps s <- s + (x - s^2) y0 / 2
//        with the approximate 1/(2 sqrt x) held fixed -- one multiply and four FMAs.
// The FP32 (mixed) form, whose results are held to FP32-level tolerances against the FP64 solve,
// takes the hardware approximations themselves (rcp.approx.ftz.f32, sqrt.approx.ftz.f32: a
// relative error of a few units in the last place, one instruction each, where the IEEE forms take
// a refinement sequence and a slow-path test). The arguments here are positive normal numbers
// (densities, sums of squares plus a regularisation, speeds of sound, temperatures) or regularised
// quotients; like the IEEE forms, 1/0 gives a non-finite value.
__device__ __forceinline__ double rcp_nr(double b)
{
    double r0;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r0) : "d"(b));
    const double e = fma(-b, r0, 1.0);
    return fma(fma(e, e, e), r0, r0);
}
__device__ __forceinline__ double sqrt_nr(double x)
{
    double y0;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y0) : "d"(x));
    const double h = 0.5 * y0;
    double s = x * y0;
    s = fma(fma(-s, s, x), h, s);
    return fma(fma(-s, s, x), h, s);
}
template <typename T> __device__ __forceinline__ T frcp(T b);
template <> __device__ __forceinline__ double frcp<double>(double b) { return rcp_nr(b); }
template <> __device__ __forceinline__ float frcp<float>(float b)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
    return r;
}
template <typename T> __device__ __forceinline__ T fdiv(T a, T b);
template <> __device__ __forceinline__ double fdiv<double>(double a, double b) { return a * rcp_nr(b); }
template <> __device__ __forceinline__ float fdiv<float>(float a, float b) { return a * frcp<float>(b); }
template <typename T> __device__ __forceinline__ T fsqrt(T x);
template <> __device__ __forceinline__ double fsqrt<double>(double x) { return sqrt_nr(x); }
template <> __device__ __forceinline__ float fsqrt<float>(float x)
{
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Sutherland law of the reference (include/FluidProps.h:107-112); T^1.5 as T*sqrt(T).
// |(o - c) / o| for the residual norm: the reciprocal of o is seeded by an FP32 division and
// refined by one Newton-Raphson step, r1 = r0 (2 - o r0), which takes the 2^-24 relative error of
// the seed to about 1e-14 for two FP64 fused multiply-adds instead of an FP64 division (the norm
// sums some 1e5 such terms, so this is far below what it resolves).
__device__ __forceinline__ double rel_change(double o, double c)
{
    const double r0 = (double)(1.0f / (float)o);
    const double r1 = r0 * fma(-o, r0, 2.0);
    return fabs((o - c) * r1);
}
// the mixed form's term, |o - c| / |o| to FP32 accuracy without FP64 instructions: o and c split
// into double-float pairs by integer operations (dfloat.cuh), their difference formed in FP32
// (o.hi - c.hi is exact where the two are within a factor of two, so the difference keeps about
// 2^-47 |o| absolute accuracy), times the approximate reciprocal of o.hi, widened to FP64 exactly
// for the FP64 accumulation. Relative error of the term about 2^-22 wherever |o - c| > 2^-24 |o|.
__device__ __forceinline__ double rel_change_mixed(double o, double c)
{
    const dfloat a = df_from(o), b = df_from(c);
    const float diff = __fadd_rn(__fsub_rn(a.hi, b.hi), __fsub_rn(a.lo, b.lo));
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a.hi));
    return f32_to_f64(fabsf(__fmul_rn(diff, r)));
}
template <typename T>
__device__ __forceinline__ double rel_change_t(double o, double c)
{
    if constexpr (sizeof(T) == 8) return rel_change(o, c);
    else return rel_change_mixed(o, c);
}

template <typename T>
__device__ __forceinline__ T sutherland(const PhysW<T> &P, T temp)
{
    return P.inv_re * (temp * tsqrt(temp)) * P.suth_c1 / (temp + P.suth_c2);
}

// the face flux's evaluation, with the FP64 form's refined root and quotient
template <typename T>
__device__ __forceinline__ T sutherland_face(const PhysW<T> &P, T temp)
{
    return fdiv<T>(P.inv_re * (temp * fsqrt<T>(temp)) * P.suth_c1, temp + P.suth_c2);
}

template <typename T>
__device__ __forceinline__ T sutherland(const Phys &P, T temp)
{
    return (T)(1.0 / P.re_ref) * (temp * tsqrt(temp)) * (T)P.suth_c1 / (temp + (T)P.suth_c2);
}

// block -> (solve, local block) mapping: grid.y enumerates solves, grid.x covers the largest one
struct Batch {
    const Lvl *lv;               // per-solve level descriptors (device)
    const SolveConst *sc;        // per-solve constants (device)
    SolveState *st;              // per-solve state (device)
    int nsolve;
};

// Thread -> (i,j,k) over the box [1, 1+ni) x [1, 1+nj) x [1, 1+nk), k fastest. Returns false for
// threads past the end of the box of this solve.
// (32-bit arithmetic: a solve's box has far fewer than 2^32 cells, and a 64-bit division costs
// several times a 32-bit one on the GPU)
__device__ __forceinline__ bool box_index(int ni, int nj, int nk, int &i, int &j, int &k)
{
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned n = (unsigned)ni * (unsigned)nj * (unsigned)nk;
    if (t >= n) return false;
    const unsigned q = t / (unsigned)nk;
    k = (int)(t - q * (unsigned)nk) + 1;
    const unsigned r = q / (unsigned)nj;
    j = (int)(q - r * (unsigned)nj) + 1;
    i = (int)r + 1;
    return true;
}

// number of faces of family f / of cells in each direction
__host__ __device__ inline void face_extent(const Lvl &L, int f, int &ni, int &nj, int &nk)
{
    ni = L.IM - 1 + (f == 0);
    nj = L.JM - 1 + (f == 1);
    nk = L.KM - 1 + (f == 2);
}

}  // namespace gbt
