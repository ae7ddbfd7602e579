/* CPU oracle for the residual-and-update hot path -- TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Layout: every array of a level lives on one padded index box i in [-3, IM+3] (same for j, k),
 * k fastest. Cell (i,j,k) spans nodes i..i+1; the reference's first ghost layer is index 0 / IM,
 * its reconstruction layers Dummy{I,J,K}S[nd] sit at index -nd and Dummy*P[nd] at IM+nd.
 * Face family f (0=I, 1=J, 2=K) at (i,j,k) is FaceI/J/K[i][j][k] of the reference.
 *
 * Arithmetic follows the reference expression by expression (same association, same float
 * literals widened to double) so that the results are bitwise those of the reference's FP64
 * build when both are compiled without FP contraction.
 */
#include "oracle.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdarg.h>

#define PAD 3
#define NQ 5
#define NP 6
enum { PD = 0, PU, PV, PW, PP, PT };       /* TPrimVars order: dens uvel vvel wvel press temp */
/* The reference's REAL is float unless SINGLE is defined (include/defs.h:28-54). The default build
 * here is its FP64 build (the parity form); ORC_FP32 gives its default FP32 build, used only as the
 * CPU timing beside the GPU's mixed form (not pinned bit for bit). */
#ifdef ORC_FP32
typedef float REAL;
#define RSCAN "%f"
#else
typedef double REAL;
#define RSCAN "%lf"
#endif
#define MAXV(a, b) (((a) > (b)) ? (a) : (b))
#define MINV(a, b) (((a) < (b)) ? (a) : (b))
#define PIF 3.1415926535897932f           /* include/defs.h:204 (float literal) */

typedef struct { REAL d, mx, my, mz, e; } cons_t;
typedef struct { REAL d, u, v, w, p, t; } prim_t;
typedef struct { REAL x, y, z; } vec_t;

typedef struct { int face, is, ie, js, je, ks, ke; } inout_t;
typedef struct { int face, rotate, is, ie, js, je, ks, ke; REAL rot; } wall_t;
typedef struct { int orient, f1, r1[6], f2, r2[6]; } per_t;

typedef struct {
    int IM, JM, KM, NI, NJ, NK;
    size_t n;
    REAL *x, *y, *z;                          /* nodes */
    REAL *fS[3][3], *fs[3], *fc[3][3], *fr[3], *fth[3], *fm[3][9];
    REAL *vol, *cc[3], *cm[9];
    REAL totalvol;
    REAL *cv[NQ], *pv[NP], *mut, *omega, *lamc[3], *lamv[3], *dt;
    REAL *Ff[3][NQ], *Vf[3][NQ], *Fc[NQ], *Fv[NQ], *res[NQ];
    REAL *Fdf[3][NQ], *Fd[NQ];                /* JST artificial dissipation: faces, cells */
    REAL *cvold[NQ], *dq[NQ];
    REAL *cv2h[NQ], *dq2h[NQ], *res2h[NQ], *qf2h[NQ];
    int *flag;
    REAL w_rot, delta_th;
    int nblade, flag_low_dt, use_force, id;
    int n_in, n_out, n_wall, n_per;
    inout_t *in, *out;
    wall_t *wall;
    per_t *per;
} level_t;

struct orc_solver {
    /* configuration (static members of the reference classes) */
    int equation_ns, turb_bl, recon_var, recon, scheme, time_scheme, limiter, global_dt, nt;
    int use_mg, ng, coarse_iter, maxiter, ndummy, turbo_axial;
    REAL Rgas, Gamma, Pr_lam, Pr_tur, Ma0, Ptin, Ttin, Pout, Pout_static, P21, Len_ref, ev_ratio;
    REAL Vel_ref, dens_ref, Temp_ref, Press_ref, mue_ref, Ma_ref, Re_ref;
    vec_t inlet_dir;
    REAL convtol, CFL, C_timestep, relax, epsEntr, k2, k4, CFL_res;
    int iter;
    REAL res[NQ];
    REAL m_in, m_out, eff, m_ratio, pr;
    level_t L[3];
};

/* ------------------------------------------------------------------------------------- */
static inline size_t IX(const level_t *L, int i, int j, int k)
{
    return ((size_t)(i + PAD) * L->NJ + (size_t)(j + PAD)) * L->NK + (size_t)(k + PAD);
}
static REAL *alloc_arr(const level_t *L) { return (REAL *)calloc(L->n, sizeof(REAL)); }

static cons_t ld_cv(REAL *const a[NQ], size_t p) { cons_t c = {a[0][p], a[1][p], a[2][p], a[3][p], a[4][p]}; return c; }
static void st_cv(REAL *const a[NQ], size_t p, cons_t c) { a[0][p] = c.d; a[1][p] = c.mx; a[2][p] = c.my; a[3][p] = c.mz; a[4][p] = c.e; }
static prim_t ld_pv(REAL *const a[NP], size_t p) { prim_t c = {a[0][p], a[1][p], a[2][p], a[3][p], a[4][p], a[5][p]}; return c; }
static void st_pv(REAL *const a[NP], size_t p, prim_t c) { a[0][p] = c.d; a[1][p] = c.u; a[2][p] = c.v; a[3][p] = c.w; a[4][p] = c.p; a[5][p] = c.t; }
static vec_t node(const level_t *L, int i, int j, int k) { size_t p = IX(L, i, j, k); vec_t v = {L->x[p], L->y[p], L->z[p]}; return v; }
static vec_t vsub(vec_t a, vec_t b) { vec_t c = {a.x - b.x, a.y - b.y, a.z - b.z}; return c; }
static vec_t vadd(vec_t a, vec_t b) { vec_t c = {a.x + b.x, a.y + b.y, a.z + b.z}; return c; }
static vec_t vscale(REAL s, vec_t a) { vec_t c = {a.x * s, a.y * s, a.z * s}; return c; }
static REAL vdot(vec_t a, vec_t b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static vec_t fS(const level_t *L, int f, size_t p) { vec_t v = {L->fS[f][0][p], L->fS[f][1][p], L->fS[f][2][p]}; return v; }
static vec_t fC(const level_t *L, int f, size_t p) { vec_t v = {L->fc[f][0][p], L->fc[f][1][p], L->fc[f][2][p]}; return v; }

/* cons/prim operators of include/defs.h restated component-wise (source/defs.cpp:36-300) */
static cons_t c_add(cons_t a, cons_t b) { cons_t c = {a.d + b.d, a.mx + b.mx, a.my + b.my, a.mz + b.mz, a.e + b.e}; return c; }
static cons_t c_sub(cons_t a, cons_t b) { cons_t c = {a.d - b.d, a.mx - b.mx, a.my - b.my, a.mz - b.mz, a.e - b.e}; return c; }
static cons_t c_mul(cons_t a, cons_t b) { cons_t c = {a.d * b.d, a.mx * b.mx, a.my * b.my, a.mz * b.mz, a.e * b.e}; return c; }
static cons_t c_div(cons_t a, cons_t b) { cons_t c = {a.d / b.d, a.mx / b.mx, a.my / b.my, a.mz / b.mz, a.e / b.e}; return c; }
static cons_t c_scl(cons_t a, REAL s) { cons_t c = {a.d * s, a.mx * s, a.my * s, a.mz * s, a.e * s}; return c; }
static cons_t c_divs(cons_t a, REAL s) { cons_t c = {a.d / s, a.mx / s, a.my / s, a.mz / s, a.e / s}; return c; }
static cons_t c_adds(cons_t a, REAL s) { cons_t c = {a.d + s, a.mx + s, a.my + s, a.mz + s, a.e + s}; return c; }
static cons_t c_rsub(REAL s, cons_t a) { cons_t c = {s - a.d, s - a.mx, s - a.my, s - a.mz, s - a.e}; return c; }
static cons_t c_sdiv(REAL s, cons_t a) { cons_t c = {s / a.d, s / a.mx, s / a.my, s / a.mz, s / a.e}; return c; }
/* The reference's component-wise POW lives out of line (source/defs.cpp:146-155,272-282), so
 * its pow(x, 2.0) is a run-time libm call that the compiler cannot fold into x*x; calling
 * through a volatile pointer keeps that here too. */
static double (*volatile pow_rt)(double, double) = pow;
static cons_t c_pow(cons_t a, REAL b) { cons_t c = {pow_rt(a.d, b), pow_rt(a.mx, b), pow_rt(a.my, b), pow_rt(a.mz, b), pow_rt(a.e, b)}; return c; }
static prim_t p_add(prim_t a, prim_t b) { prim_t c = {a.d + b.d, a.u + b.u, a.v + b.v, a.w + b.w, a.p + b.p, a.t + b.t}; return c; }
static prim_t p_sub(prim_t a, prim_t b) { prim_t c = {a.d - b.d, a.u - b.u, a.v - b.v, a.w - b.w, a.p - b.p, a.t - b.t}; return c; }
static prim_t p_mul(prim_t a, prim_t b) { prim_t c = {a.d * b.d, a.u * b.u, a.v * b.v, a.w * b.w, a.p * b.p, a.t * b.t}; return c; }
static prim_t p_div(prim_t a, prim_t b) { prim_t c = {a.d / b.d, a.u / b.u, a.v / b.v, a.w / b.w, a.p / b.p, a.t / b.t}; return c; }
static prim_t p_scl(REAL s, prim_t a) { prim_t c = {s * a.d, s * a.u, s * a.v, s * a.w, s * a.p, s * a.t}; return c; }
static prim_t p_divs(prim_t a, REAL s) { prim_t c = {a.d / s, a.u / s, a.v / s, a.w / s, a.p / s, a.t / s}; return c; }
static prim_t p_adds(prim_t a, REAL s) { prim_t c = {a.d + s, a.u + s, a.v + s, a.w + s, a.p + s, a.t + s}; return c; }
static prim_t p_rsub(REAL s, prim_t a) { prim_t c = {s - a.d, s - a.u, s - a.v, s - a.w, s - a.p, s - a.t}; return c; }
static prim_t p_sdiv(REAL s, prim_t a) { prim_t c = {s / a.d, s / a.u, s / a.v, s / a.w, s / a.p, s / a.t}; return c; }
static prim_t p_pow(prim_t a, REAL b) { prim_t c = {pow_rt(a.d, b), pow_rt(a.u, b), pow_rt(a.v, b), pow_rt(a.w, b), pow_rt(a.p, b), pow_rt(a.t, b)}; return c; }

static REAL mm1(REAL a, REAL b)          /* source/Reconstruction.cpp:472-511 per component */
{
    if (a * b < 0.0) return 0.0;
    else if (fabs(a) <= fabs(b)) return a;
    else return b;
}
static cons_t c_minmod(cons_t a, cons_t b) { cons_t c = {mm1(a.d, b.d), mm1(a.mx, b.mx), mm1(a.my, b.my), mm1(a.mz, b.mz), mm1(a.e, b.e)}; return c; }
static prim_t p_minmod(prim_t a, prim_t b) { prim_t c = {mm1(a.d, b.d), mm1(a.u, b.u), mm1(a.v, b.v), mm1(a.w, b.w), mm1(a.p, b.p), mm1(a.t, b.t)}; return c; }
static REAL min3(REAL a, REAL b, REAL c) { REAL m = a; if (m > b) m = b; if (m > c) m = c; return m; }

/* include/FluidProps.h:107-112 */
static REAL sutherland(const orc_solver *s, REAL temp)
{
    return 1.0f / s->Re_ref * pow(temp, 3.0f / 2.0f) * (1.0f + 110.4f / 288.15f) / (temp + 110.4f / 288.15f);
}

/* ====================================================================================
 * input (source/UserInput.cpp, include/fstringIO.h)
 * ==================================================================================== */
typedef struct { FILE *f; int eof; } rd_t;
/* include/fstringIO.h:15-42: strip from '#', leading and trailing blanks (not tabs). A
 * trailing carriage return is dropped first, as a text-mode read of a CRLF file does. */
static int read_line(rd_t *r, char *buf, int cap)
{
    if (!fgets(buf, cap, r->f)) { buf[0] = 0; r->eof = 1; return 0; }
    size_t n = strlen(buf);
    while (n && (buf[n - 1] == '\n' || buf[n - 1] == '\r')) buf[--n] = 0;
    char *h = strchr(buf, '#');
    if (h) *h = 0;
    char *p = buf;
    while (*p == ' ') p++;
    if (p != buf) memmove(buf, p, strlen(p) + 1);
    n = strlen(buf);
    while (n && buf[n - 1] == ' ') buf[--n] = 0;
    return 1;
}
static REAL stof_(const char *s) { return (REAL)strtof(s, NULL); }
static int yes(const char *s) { return strcmp(s, "y") == 0 || strcmp(s, "Y") == 0; }

static void seterr(char *err, int len, const char *fmt, ...)
{
    if (!err || len <= 0) return;
    va_list ap; va_start(ap, fmt); vsnprintf(err, len, fmt, ap); va_end(ap);
}

static int alloc_level(level_t *L, int IM, int JM, int KM)
{
    L->IM = IM; L->JM = JM; L->KM = KM;
    L->NI = IM + 1 + 2 * PAD; L->NJ = JM + 1 + 2 * PAD; L->NK = KM + 1 + 2 * PAD;
    L->n = (size_t)L->NI * L->NJ * L->NK;
    L->x = alloc_arr(L); L->y = alloc_arr(L); L->z = alloc_arr(L);
    for (int f = 0; f < 3; f++) {
        for (int c = 0; c < 3; c++) { L->fS[f][c] = alloc_arr(L); L->fc[f][c] = alloc_arr(L); }
        L->fs[f] = alloc_arr(L); L->fr[f] = alloc_arr(L); L->fth[f] = alloc_arr(L);
        for (int c = 0; c < 9; c++) L->fm[f][c] = alloc_arr(L);
        for (int c = 0; c < NQ; c++) { L->Ff[f][c] = alloc_arr(L); L->Vf[f][c] = alloc_arr(L); L->Fdf[f][c] = alloc_arr(L); }
        L->lamc[f] = alloc_arr(L); L->lamv[f] = alloc_arr(L);
    }
    for (int c = 0; c < NQ; c++) L->Fd[c] = alloc_arr(L);
    L->vol = alloc_arr(L);
    for (int c = 0; c < 3; c++) L->cc[c] = alloc_arr(L);
    for (int c = 0; c < 9; c++) L->cm[c] = alloc_arr(L);
    for (int c = 0; c < NQ; c++) {
        L->cv[c] = alloc_arr(L); L->Fc[c] = alloc_arr(L); L->Fv[c] = alloc_arr(L);
        L->res[c] = alloc_arr(L); L->cvold[c] = alloc_arr(L); L->dq[c] = alloc_arr(L);
        L->cv2h[c] = alloc_arr(L); L->dq2h[c] = alloc_arr(L); L->res2h[c] = alloc_arr(L);
        L->qf2h[c] = alloc_arr(L);
    }
    for (int c = 0; c < NP; c++) L->pv[c] = alloc_arr(L);
    L->mut = alloc_arr(L); L->omega = alloc_arr(L); L->dt = alloc_arr(L);
    L->flag = (int *)calloc(L->n, sizeof(int));
    return L->flag != NULL;
}

static void free_level(level_t *L)
{
    if (!L->x) return;
    free(L->x); free(L->y); free(L->z);
    for (int f = 0; f < 3; f++) {
        for (int c = 0; c < 3; c++) { free(L->fS[f][c]); free(L->fc[f][c]); }
        free(L->fs[f]); free(L->fr[f]); free(L->fth[f]);
        for (int c = 0; c < 9; c++) free(L->fm[f][c]);
        for (int c = 0; c < NQ; c++) { free(L->Ff[f][c]); free(L->Vf[f][c]); free(L->Fdf[f][c]); }
        free(L->lamc[f]); free(L->lamv[f]);
    }
    for (int c = 0; c < NQ; c++) free(L->Fd[c]);
    free(L->vol);
    for (int c = 0; c < 3; c++) free(L->cc[c]);
    for (int c = 0; c < 9; c++) free(L->cm[c]);
    for (int c = 0; c < NQ; c++) {
        free(L->cv[c]); free(L->Fc[c]); free(L->Fv[c]); free(L->res[c]); free(L->cvold[c]);
        free(L->dq[c]); free(L->cv2h[c]); free(L->dq2h[c]); free(L->res2h[c]); free(L->qf2h[c]);
    }
    for (int c = 0; c < NP; c++) free(L->pv[c]);
    free(L->mut); free(L->omega); free(L->dt); free(L->flag);
    free(L->in); free(L->out); free(L->wall); free(L->per);
    memset(L, 0, sizeof(*L));
}

/* source/UserInput.cpp:17-239 */
static int read_config(orc_solver *s, const char *dir, char *grid, char *bcf, char *err, int el)
{
    char path[4096], b[1024];
    snprintf(path, sizeof path, "%s/config.dat", dir);
    rd_t r = {fopen(path, "r"), 0};
    if (!r.f) { seterr(err, el, "cannot open %s", path); return -1; }
#define RL() do { if (!read_line(&r, b, sizeof b)) { seterr(err, el, "config.dat ended early"); fclose(r.f); return -1; } } while (0)
    RL(); RL(); strcpy(grid, b);
    RL(); RL(); RL(); strcpy(bcf, b);
    RL(); RL(); RL();
    RL(); s->turbo_axial = (strcmp(b, "a") == 0 || strcmp(b, "A") == 0);
    RL(); s->equation_ns = !(strcmp(b, "e") == 0 || strcmp(b, "E") == 0);
    RL();                                                           /* uniform / interpolate */
    RL(); s->Rgas = stof_(b);
    RL(); s->Gamma = stof_(b);
    RL(); s->Pr_lam = stof_(b);
    RL(); s->Pr_tur = stof_(b);
    RL(); RL(); RL();
    RL(); s->Ptin = stof_(b);
    RL(); s->Ttin = stof_(b);
    RL(); s->Pout = stof_(b); s->Pout_static = s->Pout;
    RL(); s->P21 = stof_(b);
    RL(); s->Ma0 = stof_(b);
    RL(); s->Len_ref = stof_(b);
    RL(); s->ev_ratio = stof_(b);
    RL(); s->inlet_dir.x = s->inlet_dir.y = s->inlet_dir.z = 0;
    sscanf(b, RSCAN " " RSCAN " " RSCAN, &s->inlet_dir.x, &s->inlet_dir.y, &s->inlet_dir.z);
    RL();                                                           /* outlet angle */
    RL();                                                           /* mass flow imposed */
    RL();
    RL(); RL(); RL();
    RL(); s->maxiter = atoi(b);
    RL(); s->coarse_iter = atoi(b);
    RL();                                                           /* OutStep */
    RL(); s->convtol = stof_(b);
    RL(); s->nt = atoi(b);
    RL(); s->use_mg = yes(b);
    RL();
    RL();
    RL(); RL(); RL();
    RL(); s->CFL = stof_(b);
    RL(); s->C_timestep = stof_(b);
    RL(); s->relax = stof_(b);
    RL(); s->epsEntr = stof_(b);
    RL(); s->k2 = stof_(b);
    RL(); s->k4 = stof_(b); s->k4 = 1.0f / s->k4;
    RL();                                                           /* IRS */
    RL(); s->limiter = yes(b);
    RL(); s->global_dt = !(strcmp(b, "l") == 0 || strcmp(b, "L") == 0);
    RL(); s->recon_var = atoi(b);
    RL(); s->recon = atoi(b);
    RL(); s->scheme = atoi(b);
    RL(); s->time_scheme = atoi(b);
    RL(); {
        int t = atoi(b);
        if (t != 0 && t != 100) { seterr(err, el, "turbulence model %d is not on this path", t); fclose(r.f); return -1; }
        s->turb_bl = (t == 100);
    }
#undef RL
    fclose(r.f);
    s->ndummy = (s->recon == 0) ? 3 : 2;
    if (s->scheme == 100) s->ndummy = 3;                            /* JST: UserInput.cpp:158-161 */
    if (s->scheme != 100 && s->scheme != 200 && s->scheme != 300) { seterr(err, el, "space scheme %d is not on this path (JST 100, Roe 300, Steger-Warming 200)", s->scheme); return -1; }
    if (s->time_scheme >= 100 && s->time_scheme <= 400) { seterr(err, el, "Runge-Kutta marching is not on this path (LU-SGS only)"); return -1; }
    if (s->use_mg && s->coarse_iter < 1) { seterr(err, el, "multigrid needs at least one coarse-grid iteration (the fine level is initialised from it)"); return -1; }
    if (s->recon_var != 100 && s->recon_var != 200) { seterr(err, el, "reconstruction variables %d not supported", s->recon_var); return -1; }
    return 0;
}

static int rd_ints(const char *b, int *v, int n)
{
    const char *p = b;
    for (int i = 0; i < n; i++) {
        char *e;
        long x = strtol(p, &e, 10);
        if (e == p) return i;
        v[i] = (int)x;
        p = e;
    }
    return n;
}

/* source/UserInput.cpp:336-446 (fine level), :799-1068 (number of levels) */
static int read_bc(orc_solver *s, const char *dir, const char *bcf, int *IMb, int *JMb, int *KMb,
                   int *nblade, REAL *rpm, char *err, int el)
{
    char path[4096], b[2048];
    snprintf(path, sizeof path, "%s/%s", dir, bcf);
    rd_t r = {fopen(path, "r"), 0};
    if (!r.f) { seterr(err, el, "cannot open %s", path); return -1; }
    level_t *L = &s->L[1];
    int NG = 4, v[20], n;
#define RL() do { if (!read_line(&r, b, sizeof b)) { seterr(err, el, "%s ended early", bcf); fclose(r.f); return -1; } } while (0)
#define NGCHECK(is, ie, js, je, ks, ke) do { int a0 = is, a1 = ie, b0 = js, b1 = je, c0 = ks, c1 = ke, num = 1; \
        if (a0 != a1) { a1 = a1 + 1; } if (b0 != b1) { b1 = b1 + 1; } if (c0 != c1) { c1 = c1 + 1; } \
        if ((a0 - 1) % 2 == 0 && (a1 - 1) % 2 == 0 && (b0 - 1) % 2 == 0 && (b1 - 1) % 2 == 0 && (c0 - 1) % 2 == 0 && (c1 - 1) % 2 == 0) num = 2; \
        NG = MINV(num, NG); } while (0)
    RL(); RL(); RL(); RL(); RL(); L->n_in = atoi(b);
    L->in = (inout_t *)calloc(L->n_in + 1, sizeof(inout_t));
    RL();
    for (int q = 1; q <= L->n_in; q++) {
        RL(); n = rd_ints(b, v, 9);
        if (n < 9) { seterr(err, el, "bad inlet line"); fclose(r.f); return -1; }
        if (v[1] != 1) { seterr(err, el, "multi-block cases are not supported"); fclose(r.f); return -1; }
        inout_t p = {v[2], v[3], v[4], v[5], v[6], v[7], v[8]};
        L->in[q] = p; NGCHECK(v[3], v[4], v[5], v[6], v[7], v[8]);
    }
    RL(); RL(); RL(); RL(); L->n_out = atoi(b);
    L->out = (inout_t *)calloc(L->n_out + 1, sizeof(inout_t));
    RL();
    for (int q = 1; q <= L->n_out; q++) {
        RL(); n = rd_ints(b, v, 9);
        if (n < 9) { seterr(err, el, "bad outlet line"); fclose(r.f); return -1; }
        inout_t p = {v[2], v[3], v[4], v[5], v[6], v[7], v[8]};
        L->out[q] = p; NGCHECK(v[3], v[4], v[5], v[6], v[7], v[8]);
    }
    RL(); RL(); RL(); RL(); L->n_wall = atoi(b);
    L->wall = (wall_t *)calloc(L->n_wall + 1, sizeof(wall_t));
    RL();
    for (int q = 1; q <= L->n_wall; q++) {
        RL(); n = rd_ints(b, v, 10);
        if (n < 10) { seterr(err, el, "bad wall line"); fclose(r.f); return -1; }
        wall_t w = {v[2], v[3] != 0, v[4], v[5], v[6], v[7], v[8], v[9], 0.0};
        L->wall[q] = w; NGCHECK(v[4], v[5], v[6], v[7], v[8], v[9]);
    }
    RL(); RL(); RL(); RL(); L->n_per = atoi(b);
    L->per = (per_t *)calloc(L->n_per + 1, sizeof(per_t));
    RL();
    for (int q = 1; q <= L->n_per; q++) {
        RL(); n = rd_ints(b, v, 18);
        if (n < 18) { seterr(err, el, "bad periodic line"); fclose(r.f); return -1; }
        per_t p;
        p.orient = v[1]; p.f1 = v[3]; p.f2 = v[11];
        for (int c = 0; c < 6; c++) { p.r1[c] = v[4 + c]; p.r2[c] = v[12 + c]; }
        L->per[q] = p; NGCHECK(v[4], v[5], v[6], v[7], v[8], v[9]);
    }
    RL(); RL(); RL(); RL(); if (atoi(b) != 0) { seterr(err, el, "interior interfaces are not supported"); fclose(r.f); return -1; }
    RL();
    RL(); RL(); RL(); RL(); if (atoi(b) != 0) { seterr(err, el, "mixing planes are not supported"); fclose(r.f); return -1; }
    RL();
    RL(); RL(); RL(); RL(); if (atoi(b) != 1) { seterr(err, el, "only single-block cases are supported"); fclose(r.f); return -1; }
    RL();
    RL();
    {
        /* BID IM JM KM NBlade rpm; rpm is read as a REAL by a stream (exact decimal parse) */
        char *p = b, *e;
        long id = strtol(p, &e, 10); p = e; (void)id;
        *IMb = (int)strtol(p, &e, 10); p = e;
        *JMb = (int)strtol(p, &e, 10); p = e;
        *KMb = (int)strtol(p, &e, 10); p = e;
        *nblade = (int)strtol(p, &e, 10); p = e;
        *rpm = strtod(p, &e);
        int IM = *IMb, JM = *JMb, KM = *KMb, num = 1;
        for (int j = 1; j <= MINV(MINV(IM, JM), KM); j++) {
            int nn = 2 * j;
            if ((IM - 1) % nn == 0 && (JM - 1) % nn == 0 && (KM - 1) % nn == 0 && (IM - 1) / nn > 2 && (JM - 1) / nn > 2 && (KM - 1) / nn > 2)
                num = j + 1;
            else
                break;
            NG = MINV(num, NG);
        }
    }
#undef RL
#undef NGCHECK
    fclose(r.f);
    s->ng = s->use_mg ? MINV(NG, 2) : 1;
    return 0;
}

/* source/UserInput.cpp:241-334 */
static int read_grid(orc_solver *s, const char *dir, const char *grid, int IMb, int JMb, int KMb, char *err, int el)
{
    char path[4096], b[1024];
    snprintf(path, sizeof path, "%s/%s", dir, grid);
    rd_t r = {fopen(path, "r"), 0};
    if (!r.f) { seterr(err, el, "cannot open grid %s", path); return -1; }
    int nb, id, IM, JM, KM;
    read_line(&r, b, sizeof b); nb = atoi(b);
    if (nb != 1) { seterr(err, el, "only single-block grids are supported"); fclose(r.f); return -1; }
    read_line(&r, b, sizeof b); id = atoi(b); (void)id;
    read_line(&r, b, sizeof b);
    if (sscanf(b, "%d %d %d", &IM, &JM, &KM) != 3) { seterr(err, el, "bad grid header"); fclose(r.f); return -1; }
    if (IM != IMb || JM != JMb || KM != KMb) { seterr(err, el, "grid and boundary file disagree on block size"); fclose(r.f); return -1; }
    if (IM < 4 || JM < 4 || KM < 4) { seterr(err, el, "each direction needs at least 4 nodes"); fclose(r.f); return -1; }
    level_t *L = &s->L[1];
    if (!alloc_level(L, IM, JM, KM)) { seterr(err, el, "out of memory"); fclose(r.f); return -1; }
    for (int k = 1; k <= KM; k++)
        for (int j = 1; j <= JM; j++)
            for (int i = 1; i <= IM; i++) {
                if (!read_line(&r, b, sizeof b)) { seterr(err, el, "grid file ended early"); fclose(r.f); return -1; }
                size_t p = IX(L, i, j, k);
                if (sscanf(b, RSCAN " " RSCAN " " RSCAN, &L->x[p], &L->y[p], &L->z[p]) != 3) { seterr(err, el, "bad grid line"); fclose(r.f); return -1; }
            }
    fclose(r.f);
    return 0;
}

static int coarse_index(int s0, int e0, int *s1, int *e1)
{
    if (s0 == e0) { *s1 = (s0 + 1) / 2; *e1 = (e0 + 1) / 2; }
    else { *s1 = (s0 + 1) / 2; *e1 = e0 / 2; }
    return 0;
}

/* coarse level: nodes injected from the fine level (source/UserInput.cpp:291-331), patches
 * re-indexed (source/UserInput.cpp:449-796) */
static int make_coarse(orc_solver *s)
{
    level_t *F = &s->L[1], *C = &s->L[2];
    if (!alloc_level(C, (F->IM + 1) / 2, (F->JM + 1) / 2, (F->KM + 1) / 2)) return -1;
    for (int k = 1; k <= C->KM; k++)
        for (int j = 1; j <= C->JM; j++)
            for (int i = 1; i <= C->IM; i++) {
                size_t p = IX(C, i, j, k), q = IX(F, 2 * i - 1, 2 * j - 1, 2 * k - 1);
                C->x[p] = F->x[q]; C->y[p] = F->y[q]; C->z[p] = F->z[q];
            }
    C->nblade = F->nblade; C->delta_th = F->delta_th; C->w_rot = F->w_rot;
    C->n_in = F->n_in; C->n_out = F->n_out; C->n_wall = F->n_wall; C->n_per = F->n_per;
    C->in = (inout_t *)calloc(C->n_in + 1, sizeof(inout_t));
    C->out = (inout_t *)calloc(C->n_out + 1, sizeof(inout_t));
    C->wall = (wall_t *)calloc(C->n_wall + 1, sizeof(wall_t));
    C->per = (per_t *)calloc(C->n_per + 1, sizeof(per_t));
    for (int q = 1; q <= F->n_in; q++) {
        inout_t a = F->in[q], c = a;
        coarse_index(a.is, a.ie, &c.is, &c.ie); coarse_index(a.js, a.je, &c.js, &c.je); coarse_index(a.ks, a.ke, &c.ks, &c.ke);
        C->in[q] = c;
    }
    for (int q = 1; q <= F->n_out; q++) {
        inout_t a = F->out[q], c = a;
        coarse_index(a.is, a.ie, &c.is, &c.ie); coarse_index(a.js, a.je, &c.js, &c.je); coarse_index(a.ks, a.ke, &c.ks, &c.ke);
        C->out[q] = c;
    }
    for (int q = 1; q <= F->n_wall; q++) {
        wall_t a = F->wall[q], c = a;
        coarse_index(a.is, a.ie, &c.is, &c.ie); coarse_index(a.js, a.je, &c.js, &c.je); coarse_index(a.ks, a.ke, &c.ks, &c.ke);
        C->wall[q] = c;
    }
    for (int q = 1; q <= F->n_per; q++) {
        per_t a = F->per[q], c = a;
        for (int d = 0; d < 3; d++) {
            coarse_index(a.r1[2 * d], a.r1[2 * d + 1], &c.r1[2 * d], &c.r1[2 * d + 1]);
            coarse_index(a.r2[2 * d], a.r2[2 * d + 1], &c.r2[2 * d], &c.r2[2 * d + 1]);
        }
        C->per[q] = c;
    }
    return 0;
}

/* ====================================================================================
 * geometry (source/GeometryVariables.cpp)
 * ==================================================================================== */
static void face_common(level_t *L, int f, size_t p, vec_t A, vec_t B, vec_t c)
{
    L->fS[f][0][p] = 0.5f * (A.y * B.z - B.y * A.z);
    L->fS[f][1][p] = 0.5f * (A.z * B.x - A.x * B.z);
    L->fS[f][2][p] = 0.5f * (A.x * B.y - B.x * A.y);
    L->fc[f][0][p] = c.x; L->fc[f][1][p] = c.y; L->fc[f][2][p] = c.z;
    L->fr[f][p] = sqrt(c.x * c.x + c.y * c.y);
    L->fth[f][p] = atan(c.y / c.x);
    L->fs[f][p] = sqrt(L->fS[f][0][p] * L->fS[f][0][p] + L->fS[f][1][p] * L->fS[f][1][p] + L->fS[f][2][p] * L->fS[f][2][p]);
}

static void face_vector_volume(level_t *L)        /* :10-105 */
{
    int IM = L->IM, JM = L->JM, KM = L->KM;
    for (int i = 1; i <= IM; i++)
        for (int j = 1; j <= JM - 1; j++)
            for (int k = 1; k <= KM - 1; k++) {
                vec_t A = vsub(node(L, i, j + 1, k), node(L, i, j, k + 1));
                vec_t B = vsub(node(L, i, j + 1, k + 1), node(L, i, j, k));
                vec_t c = vscale(0.25, vadd(vadd(vadd(node(L, i, j, k), node(L, i, j + 1, k)), node(L, i, j + 1, k + 1)), node(L, i, j, k + 1)));
                face_common(L, 0, IX(L, i, j, k), A, B, c);
            }
    for (int i = 1; i <= IM - 1; i++)
        for (int j = 1; j <= JM; j++)
            for (int k = 1; k <= KM - 1; k++) {
                vec_t A = vsub(node(L, i, j, k + 1), node(L, i + 1, j, k));
                vec_t B = vsub(node(L, i + 1, j, k + 1), node(L, i, j, k));
                vec_t c = vscale(0.25, vadd(vadd(vadd(node(L, i, j, k), node(L, i + 1, j, k)), node(L, i + 1, j, k + 1)), node(L, i, j, k + 1)));
                face_common(L, 1, IX(L, i, j, k), A, B, c);
            }
    for (int i = 1; i <= IM - 1; i++)
        for (int j = 1; j <= JM - 1; j++)
            for (int k = 1; k <= KM; k++) {
                vec_t A = vsub(node(L, i + 1, j + 1, k), node(L, i, j, k));
                vec_t B = vsub(node(L, i, j + 1, k), node(L, i + 1, j, k));
                vec_t c = vscale(0.25, vadd(vadd(vadd(node(L, i, j, k), node(L, i + 1, j, k)), node(L, i + 1, j + 1, k)), node(L, i, j + 1, k)));
                face_common(L, 2, IX(L, i, j, k), A, B, c);
            }
    REAL cellvol = 0.0;
    for (int i = 1; i <= IM - 1; i++)
        for (int j = 1; j <= JM - 1; j++)
            for (int k = 1; k <= KM - 1; k++) {
                size_t p = IX(L, i, j, k);
                size_t pi = IX(L, i + 1, j, k), pj = IX(L, i, j + 1, k), pk = IX(L, i, j, k + 1);
                REAL v = vdot(fC(L, 0, pi), fS(L, 0, pi)) - vdot(fC(L, 0, p), fS(L, 0, p)) +
                         vdot(fC(L, 1, pj), fS(L, 1, pj)) - vdot(fC(L, 1, p), fS(L, 1, p)) +
                         vdot(fC(L, 2, pk), fS(L, 2, pk)) - vdot(fC(L, 2, p), fS(L, 2, p));
                v = v / 3.0f;
                L->vol[p] = v;
                vec_t c = vadd(vadd(vadd(vadd(vadd(vadd(vadd(node(L, i, j, k), node(L, i + 1, j, k)), node(L, i, j + 1, k)), node(L, i + 1, j + 1, k)),
                                               node(L, i, j, k + 1)), node(L, i + 1, j, k + 1)), node(L, i, j + 1, k + 1)), node(L, i + 1, j + 1, k + 1));
                c = vscale(0.125, c);
                L->cc[0][p] = c.x; L->cc[1][p] = c.y; L->cc[2][p] = c.z;
                cellvol = cellvol + v;
            }
    L->totalvol = 0.0 + cellvol;                     /* ComputeAllBlockVars.cpp:28-33 */
}

/* metric coefficients from the three coordinate derivatives; gradz_kesi repeats the
 * gradx_kesi formula as the reference does (:201-209, :260-268, :318-326, :378-386) */
static void metrics(REAL *out, REAL xk, REAL yk, REAL zk, REAL xe, REAL ye, REAL ze, REAL xz, REAL yz, REAL zz)
{
    REAL lim_zero = 1E-20f;
    REAL partA = (xk * (ye * zz - yz * ze));
    REAL partB = (xe * (yk * zz - yz * zk));
    REAL partC = (xz * (yk * ze - ye * zk));
    REAL J1 = (partA - partB + partC);
    if (fabs(J1) <= lim_zero) J1 = lim_zero;
    REAL J = 1.0f / J1;
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

static void jacobi_convert(level_t *L)               /* :108-391 */
{
    int IM = L->IM, JM = L->JM, KM = L->KM;
    REAL m[9];
    for (int i = 1; i <= IM - 1; i++)
        for (int j = 1; j <= JM - 1; j++)
            for (int k = 1; k <= KM - 1; k++) {
                size_t p = IX(L, i, j, k);
                REAL xk, yk, zk, xe, ye, ze, xz, yz, zz;
                size_t a, b;
                if (i == 1) { a = IX(L, i + 1, j, k); b = p; xk = L->cc[0][a] - L->cc[0][b]; yk = L->cc[1][a] - L->cc[1][b]; zk = L->cc[2][a] - L->cc[2][b]; }
                else if (i == IM - 1) { a = p; b = IX(L, i - 1, j, k); xk = L->cc[0][a] - L->cc[0][b]; yk = L->cc[1][a] - L->cc[1][b]; zk = L->cc[2][a] - L->cc[2][b]; }
                else { a = IX(L, i + 1, j, k); b = IX(L, i - 1, j, k); xk = 0.5f * (L->cc[0][a] - L->cc[0][b]); yk = 0.5f * (L->cc[1][a] - L->cc[1][b]); zk = 0.5f * (L->cc[2][a] - L->cc[2][b]); }
                if (j == 1) { a = IX(L, i, j + 1, k); b = p; xe = (L->cc[0][a] - L->cc[0][b]); ye = (L->cc[1][a] - L->cc[1][b]); ze = (L->cc[2][a] - L->cc[2][b]); }
                else if (j == JM - 1) { a = p; b = IX(L, i, j - 1, k); xe = (L->cc[0][a] - L->cc[0][b]); ye = (L->cc[1][a] - L->cc[1][b]); ze = (L->cc[2][a] - L->cc[2][b]); }
                else { a = IX(L, i, j + 1, k); b = IX(L, i, j - 1, k); xe = 0.5f * (L->cc[0][a] - L->cc[0][b]); ye = 0.5f * (L->cc[1][a] - L->cc[1][b]); ze = 0.5f * (L->cc[2][a] - L->cc[2][b]); }
                if (k == 1) { a = IX(L, i, j, k + 1); b = p; xz = (L->cc[0][a] - L->cc[0][b]); yz = (L->cc[1][a] - L->cc[1][b]); zz = (L->cc[2][a] - L->cc[2][b]); }
                else if (k == KM - 1) { a = p; b = IX(L, i, j, k - 1); xz = (L->cc[0][a] - L->cc[0][b]); yz = (L->cc[1][a] - L->cc[1][b]); zz = (L->cc[2][a] - L->cc[2][b]); }
                else { a = IX(L, i, j, k + 1); b = IX(L, i, j, k - 1); xz = 0.5f * (L->cc[0][a] - L->cc[0][b]); yz = 0.5f * (L->cc[1][a] - L->cc[1][b]); zz = 0.5f * (L->cc[2][a] - L->cc[2][b]); }
                metrics(m, xk, yk, zk, xe, ye, ze, xz, yz, zz);
                for (int c = 0; c < 9; c++) L->cm[c][p] = m[c];
            }
    /* I faces */
    for (int i = 1; i <= IM; i++)
        for (int j = 1; j <= JM - 1; j++)
            for (int k = 1; k <= KM - 1; k++) {
                size_t p = IX(L, i, j, k), a, b;
                REAL xk, yk, zk, xe, ye, ze, xz, yz, zz;
                if (i == 1) { a = IX(L, i + 1, j, k); b = p; xk = L->fc[0][0][a] - L->fc[0][0][b]; yk = L->fc[0][1][a] - L->fc[0][1][b]; zk = L->fc[0][2][a] - L->fc[0][2][b]; }
                else if (i == IM) { a = p; b = IX(L, i - 1, j, k); xk = L->fc[0][0][a] - L->fc[0][0][b]; yk = L->fc[0][1][a] - L->fc[0][1][b]; zk = L->fc[0][2][a] - L->fc[0][2][b]; }
                else { a = IX(L, i + 1, j, k); b = IX(L, i - 1, j, k); xk = 0.5f * (L->fc[0][0][a] - L->fc[0][0][b]); yk = 0.5f * (L->fc[0][1][a] - L->fc[0][1][b]); zk = 0.5f * (L->fc[0][2][a] - L->fc[0][2][b]); }
                vec_t n0 = node(L, i, j, k), n1 = node(L, i, j + 1, k), n2 = node(L, i, j + 1, k + 1), n3 = node(L, i, j, k + 1);
                xe = 0.5f * (n1.x + n2.x) - 0.5f * (n0.x + n3.x);
                ye = 0.5f * (n1.y + n2.y) - 0.5f * (n0.y + n3.y);
                ze = 0.5f * (n1.z + n2.z) - 0.5f * (n0.z + n3.z);
                /* the second average repeats Node[i][j][k] (:248-250) */
                xz = 0.5f * (n3.x + n2.x) - 0.5f * (n0.x + n0.x);
                yz = 0.5f * (n3.y + n2.y) - 0.5f * (n0.y + n0.y);
                zz = 0.5f * (n3.z + n2.z) - 0.5f * (n0.z + n0.z);
                metrics(m, xk, yk, zk, xe, ye, ze, xz, yz, zz);
                for (int c = 0; c < 9; c++) L->fm[0][c][p] = m[c];
            }
    /* J faces */
    for (int i = 1; i <= IM - 1; i++)
        for (int j = 1; j <= JM; j++)
            for (int k = 1; k <= KM - 1; k++) {
                size_t p = IX(L, i, j, k), a, b;
                REAL xk, yk, zk, xe, ye, ze, xz, yz, zz;
                vec_t n0 = node(L, i, j, k), n1 = node(L, i + 1, j, k), n2 = node(L, i + 1, j, k + 1), n3 = node(L, i, j, k + 1);
                xk = 0.5f * (n1.x + n2.x) - 0.5f * (n0.x + n3.x);
                yk = 0.5f * (n1.y + n2.y) - 0.5f * (n0.y + n3.y);
                zk = 0.5f * (n1.z + n2.z) - 0.5f * (n0.z + n3.z);
                if (j == 1) { a = IX(L, i, j + 1, k); b = p; xe = (L->fc[1][0][a] - L->fc[1][0][b]); ye = (L->fc[1][1][a] - L->fc[1][1][b]); ze = (L->fc[1][2][a] - L->fc[1][2][b]); }
                else if (j == JM) { a = p; b = IX(L, i, j - 1, k); xe = (L->fc[1][0][a] - L->fc[1][0][b]); ye = (L->fc[1][1][a] - L->fc[1][1][b]); ze = (L->fc[1][2][a] - L->fc[1][2][b]); }
                else { a = IX(L, i, j + 1, k); b = IX(L, i, j - 1, k); xe = 0.5f * (L->fc[1][0][a] - L->fc[1][0][b]); ye = 0.5f * (L->fc[1][1][a] - L->fc[1][1][b]); ze = 0.5f * (L->fc[1][2][a] - L->fc[1][2][b]); }
                xz = 0.5f * (n3.x + n2.x) - 0.5f * (n0.x + n1.x);
                yz = 0.5f * (n3.y + n2.y) - 0.5f * (n0.y + n1.y);
                zz = 0.5f * (n3.z + n2.z) - 0.5f * (n0.z + n1.z);
                metrics(m, xk, yk, zk, xe, ye, ze, xz, yz, zz);
                for (int c = 0; c < 9; c++) L->fm[1][c][p] = m[c];
            }
    /* K faces */
    for (int i = 1; i <= IM - 1; i++)
        for (int j = 1; j <= JM - 1; j++)
            for (int k = 1; k <= KM; k++) {
                size_t p = IX(L, i, j, k), a, b;
                REAL xk, yk, zk, xe, ye, ze, xz, yz, zz;
                vec_t n0 = node(L, i, j, k), n1 = node(L, i + 1, j, k), n2 = node(L, i + 1, j + 1, k), n3 = node(L, i, j + 1, k);
                xk = 0.5f * (n2.x + n1.x) - 0.5f * (n0.x + n3.x);
                yk = 0.5f * (n2.y + n1.y) - 0.5f * (n0.y + n3.y);
                zk = 0.5f * (n2.z + n1.z) - 0.5f * (n0.z + n3.z);
                xe = 0.5f * (n2.x + n3.x) - 0.5f * (n1.x + n0.x);
                ye = 0.5f * (n2.y + n3.y) - 0.5f * (n1.y + n0.y);
                ze = 0.5f * (n2.z + n3.z) - 0.5f * (n1.z + n0.z);
                if (k == 1) { a = IX(L, i, j, k + 1); b = p; xz = (L->fc[2][0][a] - L->fc[2][0][b]); yz = (L->fc[2][1][a] - L->fc[2][1][b]); zz = (L->fc[2][2][a] - L->fc[2][2][b]); }
                else if (k == KM) { a = p; b = IX(L, i, j, k - 1); xz = (L->fc[2][0][a] - L->fc[2][0][b]); yz = (L->fc[2][1][a] - L->fc[2][1][b]); zz = (L->fc[2][2][a] - L->fc[2][2][b]); }
                else { a = IX(L, i, j, k + 1); b = IX(L, i, j, k - 1); xz = 0.5f * (L->fc[2][0][a] - L->fc[2][0][b]); yz = 0.5f * (L->fc[2][1][a] - L->fc[2][1][b]); zz = 0.5f * (L->fc[2][2][a] - L->fc[2][2][b]); }
                metrics(m, xk, yk, zk, xe, ye, ze, xz, yz, zz);
                for (int c = 0; c < 9; c++) L->fm[2][c][p] = m[c];
            }
}

/* ====================================================================================
 * state, boundary conditions
 * ==================================================================================== */
/* source/Initialization.cpp:17-76 */
static void initial_uniform(orc_solver *s, level_t *L)
{
    REAL Gamma = s->Gamma, Rgas = s->Rgas, Ma0 = s->Ma0;
    REAL press = s->Ptin * pow(1.0f + (Gamma - 1.0f) / 2.0f * Ma0 * Ma0, 0.0f - Gamma / (Gamma - 1.0f));
    REAL temp = s->Ttin * pow(1.0f + (Gamma - 1.0f) / 2.0f * Ma0 * Ma0, 0.0f - 1.0f);
    REAL dens = press / (Rgas * temp);
    REAL Vel = pow(Gamma * Rgas * temp, 0.5f) * Ma0;
    vec_t a = s->inlet_dir;
    REAL n_m = pow(a.x * a.x + a.y * a.y + a.z * a.z, 0.5);
    for (int i = 1; i <= L->IM - 1; i++)
        for (int j = 1; j <= L->JM - 1; j++)
            for (int k = 1; k <= L->KM - 1; k++) {
                REAL u = Vel * a.x / n_m, v = Vel * a.y / n_m, w = Vel * a.z / n_m;
                size_t p = IX(L, i, j, k);
                prim_t q = {dens, u, v, w, press, temp};
                st_pv(L->pv, p, q);
                REAL V2 = u * u + v * v + w * w;
                REAL ener = press / (dens * (Gamma - 1.0f)) + V2 / 2.0f;
                cons_t c = {dens, dens * u, dens * v, dens * w, dens * ener};
                st_cv(L->cv, p, c);
            }
}

/* source/PrimitiveVars.cpp:7-28 */
static void primitive_vars(orc_solver *s, level_t *L)
{
    for (int i = 1; i < L->IM; i++)
        for (int j = 1; j < L->JM; j++)
            for (int k = 1; k < L->KM; k++) {
                size_t p = IX(L, i, j, k);
                cons_t c = ld_cv(L->cv, p);
                prim_t q;
                q.d = c.d; q.u = c.mx / c.d; q.v = c.my / c.d; q.w = c.mz / c.d;
                REAL V2 = q.u * q.u + q.v * q.v + q.w * q.w;
                q.p = (s->Gamma - 1.0f) * (c.e - c.d * V2 / 2.0f);
                q.t = q.p / q.d / s->Rgas;
                st_pv(L->pv, p, q);
            }
}

static int lim_bad(const level_t *L, size_t p)
{
    REAL LdensMin = 1.0E-6f, LdensMax = 1000.0f, LpressMin = 1.0E-6f, LpressMax = 1000.0f, LVvelMax = 1000.0f;
    return (L->pv[PD][p] < LdensMin || L->pv[PD][p] > LdensMax || L->pv[PP][p] < LpressMin || L->pv[PP][p] > LpressMax ||
            L->pv[PU][p] > LVvelMax || L->pv[PV][p] > LVvelMax || L->pv[PW][p] > LVvelMax);
}

/* source/Limit_FlowVars.cpp:8-118 (in place, lexicographic order) */
static void limit_vars(orc_solver *s, level_t *L)
{
    int IM = L->IM, JM = L->JM, KM = L->KM, nneg = 0;
    REAL LdensMin = 1.0E-6f, LdensMax = 1000.0f, LpressMin = 1.0E-6f, LpressMax = 1000.0f, LVvelMax = 1000.0f;
    for (int i = 1; i <= IM - 1; i++)
        for (int j = 1; j <= JM - 1; j++)
            for (int k = 1; k <= KM - 1; k++) {
                size_t p = IX(L, i, j, k);
                if (!lim_bad(L, p)) continue;
                nneg++;
                int kn = 0, i1 = 0, j1 = 0, k1 = 0;
                REAL dens = 0.0, u = 0.0, v = 0.0, w = 0.0, press = 0.0;
                for (int ia = -1; ia <= 1; ia++)
                    for (int ja = -1; ja <= 1; ja++)
                        for (int ka = -1; ka <= 1; ka++) {
                            k1 = k + ka; j1 = j + ja; i1 = i + ia;
                            if (i1 > 0 && i1 < IM && j1 > 0 && j1 < JM && k1 > 0 && k1 < KM) {
                                size_t q = IX(L, i1, j1, k1);
                                if (!lim_bad(L, q)) {
                                    dens = dens + L->pv[PD][q]; u = u + L->pv[PU][q]; v = v + L->pv[PV][q];
                                    w = w + L->pv[PW][q]; press = press + L->pv[PP][q]; kn = kn + 1;
                                }
                            }
                        }
                if (kn == 0) {
                    size_t q = IX(L, i1, j1, k1);      /* last visited neighbour, as the reference does */
                    dens = L->pv[PD][q]; u = L->pv[PU][q]; v = L->pv[PV][q]; w = L->pv[PW][q]; press = L->pv[PP][q];
                    if (dens < LdensMin) dens = LdensMin;
                    if (dens > LdensMax) dens = LdensMax;
                    if (press < LpressMin) press = LpressMin;
                    if (press > LpressMax) press = LpressMax;
                    if (fabs(u) > LVvelMax) u = (u < 0) ? -1.0f * fabs(LVvelMax) : fabs(LVvelMax);
                    if (fabs(v) > LVvelMax) v = (v < 0) ? -1.0f * fabs(LVvelMax) : fabs(LVvelMax);
                    if (fabs(w) > LVvelMax) w = (w < 0) ? -1.0f * fabs(LVvelMax) : fabs(LVvelMax);
                } else {
                    REAL sn1 = 1.0f / kn;
                    dens = dens * sn1; u = u * sn1; v = v * sn1; w = w * sn1; press = press * sn1;
                }
                prim_t q = {dens, u, v, w, press, press / dens / s->Rgas};
                st_pv(L->pv, p, q);
                cons_t c = {dens, dens * u, dens * v, dens * w, press / (s->Gamma - 1.0f) + dens * (u * u + v * v + w * w) / 2.0f};
                st_cv(L->cv, p, c);
            }
    if (nneg > 0) L->flag_low_dt = 10;
}

/* source/BndCondInlet.cpp:7-127 */
static void bc_inlet(orc_solver *s, level_t *L, const inout_t *in)
{
    if (in->ks != in->ke) return;
    if (in->ks != 1 && in->ks != L->KM) return;
    REAL Rgas = s->Rgas, Gamma = s->Gamma, Ttin = s->Ttin, Ptin = s->Ptin;
    vec_t ang = s->inlet_dir;
    REAL Vn_m = sqrt(ang.x * ang.x + ang.y * ang.y + ang.z * ang.z);
    for (int i = in->is; i <= in->ie; i++)
        for (int j = in->js; j <= in->je; j++) {
            int k, kv;
            REAL u, v, w, vdn, n_m;
            vec_t S;
            if (in->ks == 1) {
                k = 1; kv = 0; S = fS(L, 2, IX(L, i, j, k));
                n_m = sqrt(S.x * S.x + S.y * S.y + S.z * S.z);
                size_t p = IX(L, i, j, k);
                u = L->pv[PU][p]; v = L->pv[PV][p]; w = L->pv[PW][p];
                vdn = -1.0f * (u * S.x / n_m + v * S.y / n_m + w * S.z / n_m);
            } else {
                k = L->KM - 1; kv = L->KM; S = fS(L, 2, IX(L, i, j, kv));
                n_m = sqrt(S.x * S.x + S.y * S.y + S.z * S.z);
                size_t p = IX(L, i, j, k);
                u = L->pv[PU][p]; v = L->pv[PV][p]; w = L->pv[PW][p];
                vdn = (u * S.x / n_m + v * S.y / n_m + w * S.z / n_m);
            }
            size_t p = IX(L, i, j, k), g = IX(L, i, j, kv);
            REAL c_d = sqrt(Gamma * Rgas * L->pv[PT][p]);
            REAL V2_d = u * u + v * v + w * w;
            REAL costh = -1.0f * vdn / sqrt(V2_d);
            REAL c_02 = c_d * c_d + (Gamma - 1.0f) * V2_d / 2.0f;
            REAL R_minus = vdn - 2.0f * c_d / (Gamma - 1.0f);
            REAL meduA = (-R_minus * (Gamma - 1.0f)) / ((Gamma - 1.0f) * costh * costh + 2.0f);
            REAL meduB = sqrt(c_02 * ((Gamma - 1.0f) * costh * costh + 2.0f) / (Gamma - 1.0f) / (R_minus * R_minus) - (Gamma - 1.0f) / 2.0f);
            REAL c_b = meduA * (1.0f + costh * meduB);
            REAL TempBC = Ttin * (c_b * c_b / c_02);
            if (TempBC > Ttin) TempBC = 0.99f * Ttin;
            REAL PressBC = Ptin * pow(TempBC / Ttin, Gamma / (Gamma - 1.0f));
            REAL DensBC = PressBC / Rgas / TempBC;
            REAL VBC = sqrt(2.0f * Gamma / (Gamma - 1) * Rgas * (Ttin - TempBC));
            REAL gu = VBC * ang.x / Vn_m, gv = VBC * ang.y / Vn_m, gw = VBC * ang.z / Vn_m;
            REAL V2 = gu * gu + gv * gv + gw * gw;
            REAL ener = PressBC / DensBC / (Gamma - 1.0f) + V2 / 2.0f;
            prim_t q = {DensBC, gu, gv, gw, PressBC, TempBC};
            st_pv(L->pv, g, q);
            cons_t c = {DensBC, DensBC * gu, DensBC * gv, DensBC * gw, DensBC * ener};
            st_cv(L->cv, g, c);
            for (int nd = 1; nd <= s->ndummy; nd++) {
                size_t dpos = (in->ks == 1) ? IX(L, i, j, -nd) : IX(L, i, j, L->KM + nd);
                st_pv(L->pv, dpos, q); st_cv(L->cv, dpos, c);
            }
        }
}

/* source/BndCondOutlet.cpp:13-113 (axial machine: whole k = KM face) */
static void bc_outlet_axial(orc_solver *s, level_t *L, const inout_t *o)
{
    int IM = L->IM, JM = L->JM, KM = L->KM;
    if (o->ks != o->ke || o->ke != KM) return;
    int kv = KM, k = KM - 1;
    REAL Rgas = s->Rgas, Gamma = s->Gamma;
    REAL *cu = (REAL *)calloc(IM + 1, sizeof(REAL));
    for (int i = 1; i <= IM - 1; i++) {
        REAL S_temp = 0.0;
        cu[i] = 0.0;
        for (int j = 1; j <= JM - 1; j++) {
            size_t p = IX(L, i, j, k), f = IX(L, i, j, KM);
            REAL u = L->pv[PU][p], v = L->pv[PV][p];
            REAL th = L->fth[2][f];
            REAL cu_temp = -1.0f * u * sin(th) + v * cos(th);
            cu[i] = cu[i] + cu_temp * L->fs[2][f];
            S_temp = S_temp + L->fs[2][f];
        }
        cu[i] = cu[i] / S_temp;
    }
    int iref = (int)(0.5 * IM);
    for (int j = 1; j <= JM - 1; j++) {
        L->pv[PP][IX(L, iref, j, KM)] = s->Pout;
        for (int i = iref - 1; i >= 1; i--) {
            REAL rn = L->fr[2][IX(L, i, j, KM)], rn_1 = L->fr[2][IX(L, i + 1, j, KM)];
            REAL dp_dr = L->cv[0][IX(L, i, j, KM)] * cu[i] * cu[i] / rn;
            L->pv[PP][IX(L, i, j, KM)] = L->pv[PP][IX(L, i + 1, j, KM)] - dp_dr * (rn_1 - rn);
        }
        for (int i = iref + 1; i <= IM - 1; i++) {
            /* radii taken on the k = KM-1 face row here (:74-75) */
            REAL rn_1 = L->fr[2][IX(L, i, j, k)], rn = L->fr[2][IX(L, i - 1, j, k)];
            REAL dp_dr = L->cv[0][IX(L, i, j, KM)] * cu[i] * cu[i] / rn;
            L->pv[PP][IX(L, i, j, KM)] = L->pv[PP][IX(L, i - 1, j, KM)] + dp_dr * (rn_1 - rn);
        }
    }
    for (int i = 1; i <= IM - 1; i++)
        for (int j = 1; j <= JM - 1; j++) {
            size_t g = IX(L, i, j, KM), p = IX(L, i, j, KM - 1);
            L->cv[0][g] = L->cv[0][p]; L->cv[1][g] = L->cv[1][p]; L->cv[2][g] = L->cv[2][p]; L->cv[3][g] = L->cv[3][p];
            L->pv[PD][g] = L->cv[0][p];
            L->pv[PU][g] = L->pv[PU][p]; L->pv[PV][g] = L->pv[PV][p]; L->pv[PW][g] = L->pv[PW][p];
            L->pv[PT][g] = L->pv[PP][g] / Rgas / L->cv[0][g];
            REAL u = L->pv[PU][g], v = L->pv[PV][g], w = L->pv[PW][g];
            REAL V2 = u * u + v * v + w * w;
            L->cv[4][g] = L->pv[PP][g] / (Gamma - 1.0f) + L->pv[PD][g] * V2 / 2.0f;
            for (int nd = 1; nd <= s->ndummy; nd++) {
                size_t d = IX(L, i, j, KM + nd);
                st_cv(L->cv, d, ld_cv(L->cv, g)); st_pv(L->pv, d, ld_pv(L->pv, g));
            }
        }
    (void)kv;
    free(cu);
}

/* source/BndCondWall.cpp:20-285; ghost = reflected relative velocity, dummies = average of
 * ghost and first cell */
static void wall_cell(orc_solver *s, level_t *L, const wall_t *w, size_t pi, size_t pg, size_t pfirst, vec_t fcrd,
                      size_t d1, size_t d2)
{
    REAL x = fcrd.x, y = fcrd.y;
    L->pv[PP][pg] = L->pv[PP][pi]; L->pv[PT][pg] = L->pv[PT][pi]; L->pv[PD][pg] = L->pv[PD][pi];
    REAL Vwall_x = -w->rot * y, Vwall_y = w->rot * x;
    vec_t Vin = {L->pv[PU][pi] - Vwall_x, L->pv[PV][pi] - Vwall_y, L->pv[PW][pi] - 0.0f};
    vec_t Vout = {0.0f - Vin.x, 0.0f - Vin.y, 0.0f - Vin.z};
    L->pv[PU][pg] = Vout.x + Vwall_x; L->pv[PV][pg] = Vout.y + Vwall_y; L->pv[PW][pg] = Vout.z + 0.0f;
    L->cv[0][pg] = L->cv[0][pi];
    L->cv[1][pg] = L->pv[PU][pg] * L->cv[0][pg];
    L->cv[2][pg] = L->pv[PV][pg] * L->cv[0][pg];
    L->cv[3][pg] = L->pv[PW][pg] * L->cv[0][pg];
    L->cv[4][pg] = L->cv[4][pi];
    prim_t dp = p_scl(0.5, p_add(ld_pv(L->pv, pg), ld_pv(L->pv, pfirst)));
    cons_t dc = c_scl(c_add(ld_cv(L->cv, pg), ld_cv(L->cv, pfirst)), 0.5);
    st_pv(L->pv, d1, dp); st_cv(L->cv, d1, dc);
    if (s->ndummy >= 2) { st_pv(L->pv, d2, dp); st_cv(L->cv, d2, dc); }
    if (s->ndummy >= 3) {
        /* third layer (first-order schemes) lies beyond d2 in the same direction */
        size_t d3 = d2 + (d2 - d1);
        st_pv(L->pv, d3, dp); st_cv(L->cv, d3, dc);
    }
}

static void bc_wall(orc_solver *s, level_t *L, const wall_t *w)
{
    int IM = L->IM, JM = L->JM, KM = L->KM;
    if (w->is == w->ie) {
        for (int k = w->ks; k <= w->ke; k++)
            for (int j = w->js; j <= w->je; j++) {
                if (w->is == 1) {
                    vec_t c = fC(L, 0, IX(L, 1, j, k));
                    wall_cell(s, L, w, IX(L, 1, j, k), IX(L, 0, j, k), IX(L, 1, j, k), c, IX(L, -1, j, k), IX(L, -2, j, k));
                } else if (w->is == IM) {
                    vec_t c = fC(L, 0, IX(L, IM, j, k));
                    wall_cell(s, L, w, IX(L, IM - 1, j, k), IX(L, IM, j, k), IX(L, IM - 1, j, k), c, IX(L, IM + 1, j, k), IX(L, IM + 2, j, k));
                }
            }
    } else if (w->js == w->je) {
        for (int k = w->ks; k <= w->ke; k++)
            for (int i = w->is; i <= w->ie; i++) {
                if (w->js == 1) {
                    vec_t c = fC(L, 1, IX(L, i, 1, k));
                    wall_cell(s, L, w, IX(L, i, 1, k), IX(L, i, 0, k), IX(L, i, 1, k), c, IX(L, i, -1, k), IX(L, i, -2, k));
                } else if (w->js == JM) {
                    vec_t c = fC(L, 1, IX(L, i, JM, k));
                    wall_cell(s, L, w, IX(L, i, JM - 1, k), IX(L, i, JM, k), IX(L, i, JM - 1, k), c, IX(L, i, JM + 1, k), IX(L, i, JM + 2, k));
                }
            }
    } else if (w->ks == w->ke) {
        for (int j = w->js; j <= w->je; j++)
            for (int i = w->is; i <= w->ie; i++) {
                if (w->ks == 1) {
                    vec_t c = fC(L, 2, IX(L, i, j, 1));
                    wall_cell(s, L, w, IX(L, i, j, 1), IX(L, i, j, 0), IX(L, i, j, 1), c, IX(L, i, j, -1), IX(L, i, j, -2));
                } else if (w->ks == KM) {
                    vec_t c = fC(L, 2, IX(L, i, j, KM));
                    wall_cell(s, L, w, IX(L, i, j, KM - 1), IX(L, i, j, KM), IX(L, i, j, KM - 1), c, IX(L, i, j, KM + 1), IX(L, i, j, KM + 2));
                }
            }
    }
}

/* rotational periodicity through face-local shadow buffers (source/ShadowOutIn.cpp) */
typedef struct { int lmax, mmax; cons_t *c; prim_t *p; } shadow_t;
#define SH(sh, l, m) ((size_t)(l) * 400 + (size_t)(m))

/* face-local traversal of a patch: face type fc, layer nd; calls back with (l, m, cell, write
 * target) so ShadowOut and ShadowIn share the orderings of :15-164 and :324-497 */
static void patch_walk(level_t *L, int fc, int nd, const int *r, int out, shadow_t *sh)
{
    int is = r[0], ie = r[1], js = r[2], je = r[3], ks = r[4], ke = r[5];
    int IM = L->IM, JM = L->JM, KM = L->KM;
    int l, m, a, b;
#define VISIT(I, J, K, GI, GJ, GK) do { \
        if (out) { size_t p = IX(L, I, J, K); sh->c[SH(sh, l, m)] = ld_cv(L->cv, p); sh->p[SH(sh, l, m)] = ld_pv(L->pv, p); } \
        else { size_t g = IX(L, GI, GJ, GK); if (nd == 1) { size_t g0 = IX(L, I, J, K); st_cv(L->cv, g0, sh->c[SH(sh, l, m)]); st_pv(L->pv, g0, sh->p[SH(sh, l, m)]); } \
               st_cv(L->cv, g, sh->c[SH(sh, l, m)]); st_pv(L->pv, g, sh->p[SH(sh, l, m)]); } } while (0)
    switch (fc) {
    case 1:
        if (out) { sh->lmax = abs(ke - ks) + 1; sh->mmax = abs(je - js) + 1; }
        l = 1; a = ks; do { m = 1; b = js; do {
            if (out) VISIT(nd, b, a, 0, 0, 0); else VISIT(0, b, a, -nd, b, a);
            m++; b++; } while (b <= je); l++; a++; } while (a <= ke);
        break;
    case 2:
        if (out) { sh->lmax = abs(je - js) + 1; sh->mmax = abs(ke - ks) + 1; }
        l = 1; a = js; do { m = 1; b = ks; do {
            if (out) VISIT(IM - nd, a, b, 0, 0, 0); else VISIT(IM, a, b, IM + nd, a, b);
            m++; b++; } while (b <= ke); l++; a++; } while (a <= je);
        break;
    case 3:
        if (out) { sh->lmax = abs(ie - is) + 1; sh->mmax = abs(ke - ks) + 1; }
        l = 1; a = is; do { m = 1; b = ks; do {
            if (out) VISIT(a, nd, b, 0, 0, 0); else VISIT(a, 0, b, a, -nd, b);
            m++; b++; } while (b <= ke); l++; a++; } while (a <= ie);
        break;
    case 4:
        if (out) { sh->lmax = abs(ke - ks) + 1; sh->mmax = abs(ie - is) + 1; }
        l = 1; a = ks; do { m = 1; b = is; do {
            if (out) VISIT(b, JM - nd, a, 0, 0, 0); else VISIT(b, JM, a, b, JM + nd, a);
            m++; b++; } while (b <= ie); l++; a++; } while (a <= ke);
        break;
    case 5:
        if (out) { sh->lmax = abs(je - js) + 1; sh->mmax = abs(ie - is) + 1; }
        l = 1; a = js; do { m = 1; b = is; do {
            if (out) VISIT(b, a, nd, 0, 0, 0); else VISIT(b, a, 0, b, a, -nd);
            m++; b++; } while (b <= ie); l++; a++; } while (a <= je);
        break;
    case 6:
        if (out) { sh->lmax = abs(ie - is) + 1; sh->mmax = abs(je - js) + 1; }
        l = 1; a = is; do { m = 1; b = js; do {
            if (out) VISIT(a, b, KM - nd, 0, 0, 0); else VISIT(a, b, KM, a, b, KM + nd);
            m++; b++; } while (b <= je); l++; a++; } while (a <= ie);
        break;
    }
#undef VISIT
}

/* source/ShadowOutIn.cpp:167-321 */
static void shadow_trans(shadow_t *A, shadow_t *B, int ori, REAL dr)
{
    int L1 = A->lmax, M1 = A->mmax;
    for (int l1 = 1; l1 <= L1; l1++)
        for (int m1 = 1; m1 <= M1; m1++) {
            int l2 = 0, m2 = 0;
            switch (ori) {
            case 1: l2 = l1; m2 = M1 + 1 - m1; break;
            case 2: l2 = m1; m2 = l1; break;
            case 3: l2 = L1 + 1 - l1; m2 = m1; break;
            case 4: l2 = M1 + 1 - m1; m2 = L1 + 1 - l1; break;
            }
            cons_t c = A->c[SH(A, l1, m1)];
            prim_t p = A->p[SH(A, l1, m1)];
            if (!(dr == 0.0)) {
                cons_t c0 = c; prim_t p0 = p;
                c.mx = c0.mx * cos(dr) - c0.my * sin(dr);
                c.my = c0.my * cos(dr) + c0.mx * sin(dr);
                p.u = p0.u * cos(dr) - p0.v * sin(dr);
                p.v = p0.v * cos(dr) + p0.u * sin(dr);
            }
            B->c[SH(B, l2, m2)] = c;
            B->p[SH(B, l2, m2)] = p;
        }
    if (ori == 1 || ori == 3) { B->lmax = L1; B->mmax = M1; } else { B->lmax = M1; B->mmax = L1; }
}

/* source/BndCondInteriorPeriodic.cpp:36-69 */
static void bc_periodic(orc_solver *s, level_t *L, const per_t *pr)
{
    static shadow_t A, B;
    if (!A.c) {
        A.c = (cons_t *)calloc(400 * 400, sizeof(cons_t)); A.p = (prim_t *)calloc(400 * 400, sizeof(prim_t));
        B.c = (cons_t *)calloc(400 * 400, sizeof(cons_t)); B.p = (prim_t *)calloc(400 * 400, sizeof(prim_t));
    }
    vec_t na = node(L, pr->r1[0], pr->r1[2], pr->r1[4]), nb = node(L, pr->r2[0], pr->r2[2], pr->r2[4]);
    REAL th_1 = atan(na.y / na.x), th_2 = atan(nb.y / nb.x);
    if ((th_2 - th_1) < 0.0) L->delta_th = 0.0f - L->delta_th;
    for (int nd = 1; nd <= s->ndummy; nd++) {
        patch_walk(L, pr->f1, nd, pr->r1, 1, &A);
        shadow_trans(&A, &B, pr->orient, L->delta_th);
        patch_walk(L, pr->f2, nd, pr->r2, 0, &B);
        patch_walk(L, pr->f2, nd, pr->r2, 1, &A);
        shadow_trans(&A, &B, pr->orient, 0.0f - L->delta_th);
        patch_walk(L, pr->f1, nd, pr->r1, 0, &B);
    }
}

/* source/BoundaryCondition.cpp:9-63 */
static void boundary_condition(orc_solver *s, level_t *L)
{
    for (int q = 1; q <= L->n_in; q++) bc_inlet(s, L, &L->in[q]);
    for (int q = 1; q <= L->n_out; q++) bc_outlet_axial(s, L, &L->out[q]);
    for (int q = 1; q <= L->n_wall; q++) {
        L->wall[q].rot = L->wall[q].rotate ? L->w_rot : 0.0;
        bc_wall(s, L, &L->wall[q]);
    }
    for (int q = 1; q <= L->n_per; q++) bc_periodic(s, L, &L->per[q]);
}

/* ====================================================================================
 * residual (source/Spectral_curl_grad.cpp, BL_Model.cpp, TimeStep.cpp, Upwind_Convective.cpp,
 * Reconstruction.cpp, Flux_Split_Scheme.cpp, WallFlux.cpp, ViscousFlux.cpp,
 * ComputeAllBlockVars.cpp)
 * ==================================================================================== */
static void spectral_radii(orc_solver *s, level_t *L)      /* :9-42 */
{
    for (int i = 1; i <= L->IM - 1; i++)
        for (int j = 1; j <= L->JM - 1; j++)
            for (int k = 1; k <= L->KM - 1; k++) {
                size_t p = IX(L, i, j, k);
                REAL ur = L->pv[PU][p] + L->w_rot * L->cc[1][p];
                REAL vr = L->pv[PV][p] - L->w_rot * L->cc[0][p];
                REAL wr = L->pv[PW][p];
                REAL cs = sqrt(s->Gamma * s->Rgas * L->pv[PT][p]);
                size_t q[3] = {IX(L, i + 1, j, k), IX(L, i, j + 1, k), IX(L, i, j, k + 1)};
                for (int f = 0; f < 3; f++) {
                    vec_t S = vscale(0.5f, vadd(fS(L, f, p), fS(L, f, q[f])));
                    REAL CS = cs * sqrt(S.x * S.x + S.y * S.y + S.z * S.z);
                    L->lamc[f][p] = fabs(ur * S.x + vr * S.y + wr * S.z) + CS;
                }
            }
}

static void curl(level_t *L)                                 /* :44-83 */
{
    for (int k = 1; k <= L->KM - 1; k++)
        for (int j = 1; j <= L->JM - 1; j++)
            for (int i = 1; i <= L->IM - 1; i++) {
                size_t p = IX(L, i, j, k);
                size_t ip = IX(L, i + 1, j, k), im = IX(L, i - 1, j, k), jp = IX(L, i, j + 1, k), jm = IX(L, i, j - 1, k), kp = IX(L, i, j, k + 1), km = IX(L, i, j, k - 1);
                REAL u_k = 0.5f * (L->pv[PU][ip] - L->pv[PU][im]), v_k = 0.5f * (L->pv[PV][ip] - L->pv[PV][im]), w_k = 0.5f * (L->pv[PW][ip] - L->pv[PW][im]);
                REAL u_e = 0.5f * (L->pv[PU][jp] - L->pv[PU][jm]), v_e = 0.5f * (L->pv[PV][jp] - L->pv[PV][jm]), w_e = 0.5f * (L->pv[PW][jp] - L->pv[PW][jm]);
                REAL u_z = 0.5f * (L->pv[PU][kp] - L->pv[PU][km]), v_z = 0.5f * (L->pv[PV][kp] - L->pv[PV][km]), w_z = 0.5f * (L->pv[PW][kp] - L->pv[PW][km]);
                REAL *m[9]; for (int c = 0; c < 9; c++) m[c] = L->cm[c];
                REAL v_x = v_k * m[0][p] + v_e * m[3][p] + v_z * m[6][p];
                REAL w_x = w_k * m[0][p] + w_e * m[3][p] + w_z * m[6][p];
                REAL u_y = u_k * m[1][p] + u_e * m[4][p] + u_z * m[7][p];
                REAL w_y = w_k * m[1][p] + w_e * m[4][p] + w_z * m[7][p];
                REAL u_zz = u_k * m[2][p] + u_e * m[5][p] + u_z * m[8][p];
                REAL v_zz = v_k * m[2][p] + v_e * m[5][p] + v_z * m[8][p];
                L->omega[p] = sqrt(0.5f * ((w_y - v_zz) * (w_y - v_zz) + (u_zz - w_x) * (u_zz - w_x) + (v_x - u_y) * (v_x - u_y)));
            }
}

/* face gradient helpers: component c of the primitive state */
#define PC(c, p) (L->pv[c][p])
static REAL a4(const level_t *L, int c, size_t a, size_t b, size_t d, size_t e) { return (PC(c, a) + PC(c, b) + PC(c, d) + PC(c, e)) / 4.0f; }
static REAL q4(const level_t *L, int c, size_t a, size_t b, size_t d, size_t e) { return 0.25f * (PC(c, a) + PC(c, b) + PC(c, d) + PC(c, e)); }
static REAL a3(const level_t *L, int c, size_t a, size_t b, size_t d) { return (PC(c, a) + PC(c, b) + PC(c, d)) / 3.0f; }

/* gradients of u, v, w, T at a face from the three index derivatives and the face metrics */
static void grad_store(const level_t *L, int f, size_t p, const REAL dk[4], const REAL de[4], const REAL dz[4], REAL g[3][4])
{
    for (int c = 0; c < 4; c++) {
        g[0][c] = dk[c] * L->fm[f][0][p] + de[c] * L->fm[f][3][p] + dz[c] * L->fm[f][6][p];
        g[1][c] = dk[c] * L->fm[f][1][p] + de[c] * L->fm[f][4][p] + dz[c] * L->fm[f][7][p];
        g[2][c] = dk[c] * L->fm[f][2][p] + de[c] * L->fm[f][5][p] + dz[c] * L->fm[f][8][p];
    }
}
static const int GC[4] = {PU, PV, PW, PT};

/* :85-227 (I faces) */
static void grad_faceI(const level_t *L, int i, int j, int k, REAL g[3][4])
{
    int IM = L->IM, JM = L->JM, KM = L->KM;
    REAL dk[4], de[4], dz[4];
    size_t c0 = IX(L, i, j, k), cm = IX(L, i - 1, j, k);
    for (int q = 0; q < 4; q++) {
        int c = GC[q];
        dk[q] = PC(c, c0) - PC(c, cm);
        size_t jp = IX(L, i, j + 1, k), mjp = IX(L, i - 1, j + 1, k), jm = IX(L, i, j - 1, k), mjm = IX(L, i - 1, j - 1, k);
        if (i == 1 && j == 1) de[q] = a4(L, c, c0, jp, mjp, cm) - a3(L, c, c0, cm, jm);
        else if (i == 1 && j == JM - 1) de[q] = a3(L, c, c0, jp, cm) - a4(L, c, c0, cm, mjm, jm);
        else if (i == IM && j == 1) de[q] = a4(L, c, c0, jp, mjp, cm) - a3(L, c, c0, cm, mjm);
        else if (i == IM && j == JM - 1) de[q] = a3(L, c, c0, mjp, cm) - a4(L, c, c0, cm, mjm, jm);
        else de[q] = a4(L, c, c0, jp, mjp, cm) - a4(L, c, c0, cm, mjm, jm);
        size_t kp = IX(L, i, j, k + 1), mkp = IX(L, i - 1, j, k + 1), km = IX(L, i, j, k - 1), mkm = IX(L, i - 1, j, k - 1);
        if (i == 1 && k == 1) dz[q] = a4(L, c, c0, kp, mkp, cm) - a3(L, c, c0, cm, km);
        else if (i == 1 && k == KM - 1) dz[q] = a3(L, c, c0, kp, cm) - a4(L, c, c0, cm, mkm, km);
        else if (i == IM && k == 1) dz[q] = a4(L, c, c0, kp, mkp, cm) - a3(L, c, c0, cm, mkm);
        else if (i == IM && k == KM - 1) dz[q] = a3(L, c, c0, mkp, cm) - a4(L, c, c0, cm, mkm, km);
        else dz[q] = a4(L, c, c0, kp, mkp, cm) - a4(L, c, c0, cm, mkm, km);
    }
    grad_store(L, 0, c0, dk, de, dz, g);
}

/* :229-359 (J faces) */
static void grad_faceJ(const level_t *L, int i, int j, int k, REAL g[3][4])
{
    int IM = L->IM, JM = L->JM, KM = L->KM;
    REAL dk[4], de[4], dz[4];
    size_t c0 = IX(L, i, j, k), cm = IX(L, i, j - 1, k);
    for (int q = 0; q < 4; q++) {
        int c = GC[q];
        size_t ip = IX(L, i + 1, j, k), ipm = IX(L, i + 1, j - 1, k), im = IX(L, i - 1, j, k), imm = IX(L, i - 1, j - 1, k);
        if (j == 1 && i == 1) dk[q] = q4(L, c, c0, ip, ipm, cm) - a3(L, c, c0, im, cm);
        else if (j == 1 && i == IM - 1) dk[q] = a3(L, c, c0, ip, cm) - q4(L, c, c0, im, imm, cm);
        else if (j == JM && i == 1) dk[q] = q4(L, c, c0, ip, ipm, cm) - a3(L, c, c0, imm, cm);
        else if (j == JM && i == IM - 1) dk[q] = a3(L, c, c0, ipm, cm) - q4(L, c, c0, im, imm, cm);
        else dk[q] = q4(L, c, c0, ip, ipm, cm) - q4(L, c, c0, im, imm, cm);
        de[q] = PC(c, c0) - PC(c, cm);
        size_t kp = IX(L, i, j, k + 1), mkp = IX(L, i, j - 1, k + 1), km = IX(L, i, j, k - 1), mkm = IX(L, i, j - 1, k - 1);
        if (j == 1 && k == 1) dz[q] = q4(L, c, c0, kp, mkp, cm) - a3(L, c, c0, cm, km);
        else if (j == 1 && k == KM - 1) dz[q] = a3(L, c, c0, kp, cm) - q4(L, c, c0, cm, mkm, km);
        else if (j == JM && k == 1) dz[q] = q4(L, c, c0, kp, mkp, cm) - 0.25f * (PC(c, c0) + PC(c, cm) + PC(c, mkm)) / 3.0f;   /* extra 0.25 (:311-314) */
        else if (j == JM && k == KM - 1) dz[q] = a3(L, c, c0, mkp, cm) - q4(L, c, c0, cm, mkm, km);
        else dz[q] = q4(L, c, c0, kp, mkp, cm) - q4(L, c, c0, cm, mkm, km);
    }
    grad_store(L, 1, c0, dk, de, dz, g);
}

/* :361-490 (K faces) */
static void grad_faceK(const level_t *L, int i, int j, int k, REAL g[3][4])
{
    int IM = L->IM, JM = L->JM, KM = L->KM;
    REAL dk[4], de[4], dz[4];
    size_t c0 = IX(L, i, j, k), cm = IX(L, i, j, k - 1);
    for (int q = 0; q < 4; q++) {
        int c = GC[q];
        size_t ip = IX(L, i + 1, j, k), ipm = IX(L, i + 1, j, k - 1), im = IX(L, i - 1, j, k), imm = IX(L, i - 1, j, k - 1);
        if (k == 1 && i == 1) dk[q] = q4(L, c, c0, ip, ipm, cm) - a3(L, c, c0, im, cm);
        else if (k == 1 && i == IM - 1) dk[q] = a3(L, c, c0, ip, cm) - q4(L, c, c0, im, imm, cm);
        else if (k == KM && i == 1) dk[q] = q4(L, c, c0, ip, ipm, cm) - a3(L, c, c0, imm, cm);
        else if (k == KM && i == IM - 1) dk[q] = a3(L, c, c0, ipm, cm) - q4(L, c, c0, im, imm, cm);
        else dk[q] = q4(L, c, c0, ip, ipm, cm) - q4(L, c, c0, im, imm, cm);
        size_t jp = IX(L, i, j + 1, k), jpm = IX(L, i, j + 1, k - 1), jm = IX(L, i, j - 1, k), jmm = IX(L, i, j - 1, k - 1);
        if (k == 1 && j == 1) de[q] = q4(L, c, c0, jp, jpm, cm) - a3(L, c, c0, jm, cm);
        else if (k == 1 && j == JM - 1) de[q] = a3(L, c, c0, jp, cm) - q4(L, c, c0, jm, jmm, cm);
        else if (k == KM && j == 1) de[q] = q4(L, c, c0, jp, jpm, cm) - a3(L, c, c0, jmm, cm);
        else if (k == KM && j == JM - 1) de[q] = a3(L, c, c0, jpm, cm) - q4(L, c, c0, jm, jmm, cm);
        else de[q] = q4(L, c, c0, jp, jpm, cm) - q4(L, c, c0, jm, jmm, cm);
        dz[q] = PC(c, c0) - PC(c, cm);
    }
    grad_store(L, 2, c0, dk, de, dz, g);
}
#undef PC

/* source/BL_Model.cpp:283-329 */
static void bl_model_1d(int M, const REAL *dens, const REAL *Vvel, const REAL *dis, const REAL *Om, const REAL *mul, REAL *mut)
{
    REAL A_plus = 26.0f, Cwk = 1.0f, kap = 0.4f, Ckleb = 0.3f, alpha = 0.0168f, Ccp = 1.6f;
    REAL Tw = fabs(Om[1] * mul[1]);
    for (int i = 1; i < M; i++)
        if (fabs(Om[i] * mul[i]) > Tw) Tw = fabs(Om[i] * mul[i]);
    REAL Ret = sqrt(dens[1] * Tw) / mul[1];
    REAL Fmax = 0.0, y_max = 0.0, Udif = 0.0;
    for (int i = 1; i < M; i++) {
        if (Vvel[i] > Udif) Udif = Vvel[i];
        REAL y_plus = dis[i] * Ret;
        REAL F = dis[i] * fabs(Om[i]) * (1.0f - exp(-y_plus / A_plus));
        if (F > Fmax) { Fmax = F; y_max = dis[i]; }
    }
    REAL Fwake = MINV(y_max * Fmax, Cwk * y_max * Udif * Udif / Fmax);
    for (int i = 1; i < M; i++) {
        REAL y_plus = Ret * dis[i];
        REAL bL = kap * dis[i] * (1.0f - exp(-y_plus / A_plus));
        REAL mue_in = dens[i] * bL * bL * Om[i];
        REAL Fkleb = 1.0f / (1.0f + 5.5f * pow((Ckleb * dis[i] / y_max), 6.0));
        REAL mue_out = alpha * Ccp * dens[i] * Fwake * Fkleb;
        if (fabs(mue_in) > fabs(mue_out)) mut[i] = mue_out;
        else mut[i] = mue_in;
    }
}

/* source/BL_Model.cpp:8-279: one line per wall face, normal to the wall across the whole
 * block, min-merged over walls; wall-adjacent cells and ghosts get zero */
static void bl_model(orc_solver *s, level_t *L)
{
    int IM = L->IM, JM = L->JM, KM = L->KM;
    int MM = MAXV(MAXV(IM, JM), KM);
    REAL *dens = (REAL *)calloc(MM + 1, sizeof(REAL)), *Vv = (REAL *)calloc(MM + 1, sizeof(REAL));
    REAL *dis = (REAL *)calloc(MM + 1, sizeof(REAL)), *Om = (REAL *)calloc(MM + 1, sizeof(REAL));
    REAL *mul = (REAL *)calloc(MM + 1, sizeof(REAL)), *mt = (REAL *)calloc(MM + 1, sizeof(REAL));
    for (int i = 1; i <= IM - 1; i++)
        for (int j = 1; j <= JM - 1; j++)
            for (int k = 1; k <= KM - 1; k++) L->flag[IX(L, i, j, k)] = 0;
    for (int q = 1; q <= L->n_wall; q++) {
        const wall_t *w = &L->wall[q];
        int ft = w->face, dirn = (ft - 1) / 2;         /* 0: i-wall, 1: j-wall, 2: k-wall */
        int N = dirn == 0 ? IM : (dirn == 1 ? JM : KM);
        int lo = ft % 2 == 1;                         /* wall at index 1 */
        int a0, a1, b0, b1;                           /* ranges of the two tangential indices */
        if (dirn == 0) { a0 = w->ks; a1 = w->ke; b0 = w->js; b1 = w->je; }
        else if (dirn == 1) { a0 = w->ks; a1 = w->ke; b0 = w->is; b1 = w->ie; }
        else { a0 = w->js; a1 = w->je; b0 = w->is; b1 = w->ie; }
        for (int a = a0; a <= a1; a++)
            for (int b = b0; b <= b1; b++) {
                for (int n = 1; n <= N - 1; n++) {
                    int i, j, k;
                    size_t f;
                    if (dirn == 0) { i = n; j = b; k = a; f = IX(L, lo ? 1 : IM, j, k); }
                    else if (dirn == 1) { i = b; j = n; k = a; f = IX(L, i, lo ? 1 : JM, k); }
                    else { i = b; j = a; k = n; f = IX(L, i, j, lo ? 1 : KM); }
                    int n0 = lo ? n : N - n;
                    size_t p = IX(L, i, j, k);
                    dis[n0] = sqrt(pow((L->cc[0][p] - L->fc[dirn][0][f]), 2.0) + pow((L->cc[1][p] - L->fc[dirn][1][f]), 2.0) +
                                   pow((L->cc[2][p] - L->fc[dirn][2][f]), 2.0));
                    dens[n0] = L->pv[PD][p];
                    REAL u = L->pv[PU][p], v = L->pv[PV][p], ww = L->pv[PW][p];
                    Vv[n0] = sqrt(u * u + v * v + ww * ww);
                    Om[n0] = L->omega[p];
                    mul[n0] = sutherland(s, L->pv[PT][p]);
                }
                bl_model_1d(N, dens, Vv, dis, Om, mul, mt);
                for (int n = 1; n <= N - 1; n++) {
                    int i, j, k;
                    if (dirn == 0) { i = n; j = b; k = a; }
                    else if (dirn == 1) { i = b; j = n; k = a; }
                    else { i = b; j = a; k = n; }
                    int n0 = lo ? n : N - n;
                    size_t p = IX(L, i, j, k);
                    if (L->flag[p] == 0) { L->flag[p] = 1; L->mut[p] = mt[n0]; }
                    else L->mut[p] = MINV(L->mut[p], mt[n0]);
                }
            }
        for (int a = a0; a <= a1; a++)
            for (int b = b0; b <= b1; b++) {
                int n1 = lo ? 1 : N - 1, ng = lo ? 0 : N;
                if (dirn == 0) { L->mut[IX(L, n1, b, a)] = 0.0; L->mut[IX(L, ng, b, a)] = 0.0; }
                else if (dirn == 1) { L->mut[IX(L, b, n1, a)] = 0.0; L->mut[IX(L, b, ng, a)] = 0.0; }
                else { L->mut[IX(L, b, a, n1)] = 0.0; L->mut[IX(L, b, a, ng)] = 0.0; }
            }
    }
    free(dens); free(Vv); free(dis); free(Om); free(mul); free(mt);
}

/* source/TimeStep.cpp:7-93 */
static void time_step(orc_solver *s, level_t *L)
{
    REAL dt_factor;
    if (L->flag_low_dt == 0) dt_factor = 1.0f;
    else dt_factor = 1.0f / (1.0f + L->flag_low_dt);
    for (int i = 1; i <= L->IM - 1; i++)
        for (int j = 1; j <= L->JM - 1; j++)
            for (int k = 1; k <= L->KM - 1; k++) {
                size_t p = IX(L, i, j, k);
                size_t q[3] = {IX(L, i + 1, j, k), IX(L, i, j + 1, k), IX(L, i, j, k + 1)};
                REAL eq[3];
                for (int f = 0; f < 3; f++) {
                    vec_t S = vscale(0.5, vadd(fS(L, f, p), fS(L, f, q[f])));
                    eq[f] = S.x * S.x + S.y * S.y + S.z * S.z;
                }
                REAL lc, lv;
                if (s->equation_ns) {
                    REAL mul = sutherland(s, L->pv[PT][p]);
                    REAL mt = L->mut[p];
                    REAL dens = L->pv[PD][p];
                    for (int f = 0; f < 3; f++)
                        L->lamv[f][p] = MAXV(4.0f / 3.0f / dens, s->Gamma / dens) * (mul / s->Pr_lam + mt / s->Pr_tur) * eq[f] / L->vol[p];
                    lc = L->lamc[0][p] + L->lamc[1][p] + L->lamc[2][p];
                    lv = L->lamv[0][p] + L->lamv[1][p] + L->lamv[2][p];
                } else {
                    lc = L->lamc[0][p] + L->lamc[1][p] + L->lamc[2][p];
                    lv = 0.0;
                }
                L->dt[p] = dt_factor * s->CFL * L->vol[p] / (lc + s->C_timestep * lv);
            }
    if (s->global_dt) {
        REAL dt_min = 1E10;
        for (int i = 1; i <= L->IM - 1; i++)
            for (int j = 1; j <= L->JM - 1; j++)
                for (int k = 1; k <= L->KM - 1; k++) dt_min = MINV(dt_min, L->dt[IX(L, i, j, k)]);
        for (int i = 1; i <= L->IM - 1; i++)
            for (int j = 1; j <= L->JM - 1; j++)
                for (int k = 1; k <= L->KM - 1; k++) L->dt[IX(L, i, j, k)] = dt_min;
    }
    if (L->flag_low_dt > 0) L->flag_low_dt = L->flag_low_dt - 1;
}

/* source/Reconstruction.cpp:7-68 */
static void recon_cons(const orc_solver *s, cons_t FF, cons_t F, cons_t B, cons_t BB, cons_t *L_, cons_t *R_)
{
    REAL epsilon = 1E-6f, eta = 0.05f, k2c = 1.0f, k2u = -1.0f, Gamma = s->Gamma, lim_zero = 1E-20f;
    cons_t cl = {0, 0, 0, 0, 0}, cr = {0, 0, 0, 0, 0};
    int t = s->recon;
    if (t == 100) {
        cl = c_add(F, c_scl(c_minmod(c_sub(B, F), c_sub(F, FF)), 0.5f));
        cr = c_sub(B, c_scl(c_minmod(c_sub(B, F), c_sub(BB, B)), 0.5f));
    } else if (t == 200) {
        cl = c_add(F, c_scl(c_add(c_scl(c_minmod(c_scl(c_sub(B, F), 2.0f), c_sub(F, FF)), (1.0f - k2u)), c_scl(c_minmod(c_scl(c_sub(F, FF), 2.0f), c_sub(B, F)), (1.0f + k2u))), 0.25));
        cr = c_sub(B, c_scl(c_add(c_scl(c_minmod(c_scl(c_sub(B, F), 2.0f), c_sub(BB, B)), (1.0f - k2u)), c_scl(c_minmod(c_scl(c_sub(BB, B), 2.0f), c_sub(B, F)), (1.0f + k2u))), 0.25));
    } else if (t == 300) {
        cl = c_add(F, c_scl(c_add(c_scl(c_minmod(c_scl(c_sub(B, F), 2.0f), c_sub(F, FF)), (1.0f - k2c)), c_scl(c_minmod(c_sub(B, F), c_scl(c_sub(F, FF), 2.0f)), (1.0f + k2c))), 0.25));
        cr = c_sub(B, c_scl(c_add(c_scl(c_minmod(c_scl(c_sub(B, F), 2.0f), c_sub(BB, B)), (1.0f - k2c)), c_scl(c_minmod(c_sub(B, F), c_scl(c_sub(BB, B), 2.0f)), (1.0f + k2c))), 0.25));
    } else if (t == 400) {
        cons_t r1 = c_div(c_adds(c_sub(F, FF), epsilon), c_adds(c_sub(B, F), epsilon));
        cons_t r2 = c_div(c_adds(c_sub(B, F), epsilon), c_adds(c_sub(BB, B), epsilon));
        /* operator order of the reference: (1-eta) + A + B with scalar+vector adds */
        cons_t f1 = c_add(c_adds(c_sdiv((eta - 0.55f) / 2.0f, r2), 1.0f - eta), c_scl(r1, (eta + 0.55f) / 2.0f));
        cons_t f = {MAXV(0.0f, min3(2.0f, f1.d, 2.0f * r1.d)), MAXV(0.0f, min3(2.0f, f1.mx, 2.0f * r1.mx)), MAXV(0.0f, min3(2.0f, f1.my, 2.0f * r1.my)),
                    MAXV(0.0f, min3(2.0f, f1.mz, 2.0f * r1.mz)), MAXV(0.0f, min3(2.0f, f1.e, 2.0f * r1.e))};
        cl = c_add(F, c_mul(c_scl(f, 0.5f), c_sub(B, F)));
        r1 = c_div(c_adds(c_sub(BB, B), epsilon), c_adds(c_sub(B, F), epsilon));
        r2 = c_div(c_adds(c_sub(B, F), epsilon), c_adds(c_sub(F, FF), epsilon));
        f1 = c_add(c_adds(c_sdiv((eta - 0.55f) / 2.0f, r2), 1.0f - eta), c_scl(r1, (eta + 0.55f) / 2.0f));
        cons_t g = {MAXV(0.0f, min3(2.0f, f1.d, 2.0f * r1.d)), MAXV(0.0f, min3(2.0f, f1.mx, 2.0f * r1.mx)), MAXV(0.0f, min3(2.0f, f1.my, 2.0f * r1.my)),
                    MAXV(0.0f, min3(2.0f, f1.mz, 2.0f * r1.mz)), MAXV(0.0f, min3(2.0f, f1.e, 2.0f * r1.e))};
        cr = c_sub(B, c_mul(c_scl(g, 0.5f), c_sub(B, F)));
    } else if (t == 500) {
        cons_t a = c_sub(F, FF), b = c_sub(B, F), c = c_sub(BB, B);
        cons_t SL = c_div(c_adds(c_mul(c_scl(a, 2.0f), b), epsilon), c_adds(c_add(c_pow(a, 2.0f), c_pow(b, 2.0f)), epsilon));
        cons_t SR = c_div(c_adds(c_mul(c_scl(c, 2.0f), b), epsilon), c_adds(c_add(c_pow(c, 2.0f), c_pow(b, 2.0f)), epsilon));
        cl = c_add(F, c_mul(c_divs(SL, 4.0f), c_add(c_mul(c_rsub(1.0f, c_divs(SL, 3.0f)), a), c_mul(c_adds(c_divs(SL, 3.0f), 1.0f), b))));
        cr = c_sub(B, c_mul(c_divs(SR, 4.0f), c_add(c_mul(c_rsub(1.0f, c_divs(SR, 3.0f)), c), c_mul(c_adds(c_divs(SR, 3.0f), 1.0f), b))));
    }
    (void)k2c;
    REAL pL = (Gamma - 1.0f) * (cl.e - 0.5f * (cl.mx * cl.mx + cl.my * cl.my + cl.mz * cl.mz) / cl.d);
    REAL pR = (Gamma - 1.0f) * (cr.e - 0.5f * (cr.mx * cr.mx + cr.my * cr.my + cr.mz * cr.mz) / cr.d);
    if (cl.d <= lim_zero || pL <= lim_zero) cl = F;
    if (cr.d <= lim_zero || pR <= lim_zero) cr = B;
    *L_ = cl; *R_ = cr;
}

/* source/Reconstruction.cpp:70-265 */
static void recon_prim(const orc_solver *s, prim_t FF, prim_t F, prim_t B, prim_t BB, cons_t *L_, cons_t *R_)
{
    REAL epsilon = 1E-6f, eta = 0.2f, k2c = 1.0, k2u = -1.0, Gamma = s->Gamma, lim_zero = 1E-20f;
    prim_t pl = {0, 0, 0, 0, 0, 0}, pr = {0, 0, 0, 0, 0, 0};
    int t = s->recon;
    if (t == 100) {
        pl = p_add(F, p_scl(0.5, p_minmod(p_sub(B, F), p_sub(F, FF))));
        pr = p_sub(B, p_scl(0.5, p_minmod(p_sub(B, F), p_sub(BB, B))));
    } else if (t == 200) {
        pl = p_add(F, p_scl(0.25f, p_add(p_scl((1.0f - k2u), p_minmod(p_scl(2.0f, p_sub(B, F)), p_sub(F, FF))), p_scl((1.0f + k2u), p_minmod(p_scl(2.0f, p_sub(F, FF)), p_sub(B, F))))));
        pr = p_sub(B, p_scl(0.25f, p_add(p_scl((1.0f - k2u), p_minmod(p_scl(2.0f, p_sub(B, F)), p_sub(BB, B))), p_scl((1.0f + k2u), p_minmod(p_scl(2.0f, p_sub(BB, B)), p_sub(B, F))))));
    } else if (t == 300) {
        pl = p_add(F, p_scl(0.25f, p_add(p_scl((1.0f - k2c), p_minmod(p_scl(2.0f, p_sub(B, F)), p_sub(F, FF))), p_scl((1.0f + k2c), p_minmod(p_sub(B, F), p_scl(2.0, p_sub(F, FF)))))));
        pr = p_sub(B, p_scl(0.25f, p_add(p_scl((1.0f - k2c), p_minmod(p_scl(2.0f, p_sub(B, F)), p_sub(BB, B))), p_scl((1.0f + k2c), p_minmod(p_sub(B, F), p_scl(2.0, p_sub(BB, B)))))));
    } else if (t == 400) {
        prim_t r1 = p_div(p_adds(p_sub(F, FF), epsilon), p_adds(p_sub(B, F), epsilon));
        prim_t r2 = p_div(p_adds(p_sub(B, F), epsilon), p_adds(p_sub(BB, B), epsilon));
        prim_t f1 = p_add(p_adds(p_sdiv((eta - 0.55f) / 2.0f, r2), 1.0f - eta), p_scl((eta + 0.55f) / 2.0f, r1));
        prim_t f = {MAXV(0.0f, min3(2.0f, f1.d, 2.0f * r1.d)), MAXV(0.0f, min3(2.0f, f1.u, 2.0f * r1.u)), MAXV(0.0f, min3(2.0f, f1.v, 2.0f * r1.v)),
                    MAXV(0.0f, min3(2.0f, f1.w, 2.0f * r1.w)), MAXV(0.0f, min3(2.0f, f1.p, 2.0f * r1.p)), 0.0};
        pl = p_add(F, p_mul(p_scl(0.5f, f), p_sub(B, F)));
        r1 = p_div(p_adds(p_sub(BB, B), epsilon), p_adds(p_sub(B, F), epsilon));
        r2 = p_div(p_adds(p_sub(B, F), epsilon), p_adds(p_sub(F, FF), epsilon));
        f1 = p_add(p_adds(p_sdiv((eta - 0.55f) / 2.0f, r2), 1.0f - eta), p_scl((eta + 0.55f) / 2.0f, r1));
        prim_t g = {MAXV(0.0f, min3(2.0f, f1.d, 2.0f * r1.d)), MAXV(0.0f, min3(2.0f, f1.u, 2.0f * r1.u)), MAXV(0.0f, min3(2.0f, f1.v, 2.0f * r1.v)),
                    MAXV(0.0f, min3(2.0f, f1.w, 2.0f * r1.w)), MAXV(0.0f, min3(2.0f, f1.p, 2.0f * r1.p)), 0.0};
        pr = p_sub(B, p_mul(p_scl(0.5f, g), p_sub(B, F)));
    } else if (t == 500) {
        prim_t a = p_sub(F, FF), b = p_sub(B, F), c = p_sub(BB, B);
        prim_t SL = p_div(p_adds(p_mul(p_scl(2.0, a), b), epsilon), p_adds(p_add(p_pow(a, 2.0), p_pow(b, 2.0)), epsilon));
        prim_t SR = p_div(p_adds(p_mul(p_scl(2.0, c), b), epsilon), p_adds(p_add(p_pow(c, 2.0), p_pow(b, 2.0)), epsilon));
        pl = p_add(F, p_mul(p_divs(SL, 4.0), p_add(p_mul(p_rsub(1.0, p_divs(SL, 3.0)), a), p_mul(p_adds(p_divs(SL, 3.0), 1.0), b))));
        pr = p_sub(B, p_mul(p_divs(SR, 4.0), p_add(p_mul(p_rsub(1.0, p_divs(SR, 3.0)), c), p_mul(p_adds(p_divs(SR, 3.0), 1.0), b))));
    }
    if (pl.d <= lim_zero || pl.p <= lim_zero) pl = F;
    if (pr.d <= lim_zero || pr.p <= lim_zero) pr = B;
    cons_t cl = {pl.d, pl.d * pl.u, pl.d * pl.v, pl.d * pl.w, pl.p / (Gamma - 1.0f) + pl.d * (pl.u * pl.u + pl.v * pl.v + pl.w * pl.w) / 2.0f};
    cons_t cr = {pr.d, pr.d * pr.u, pr.d * pr.v, pr.d * pr.w, pr.p / (Gamma - 1.0f) + pr.d * (pr.u * pr.u + pr.v * pr.v + pr.w * pr.w) / 2.0f};
    *L_ = cl; *R_ = cr;
}

/* face frame (source/Flux_Split_Scheme.cpp:728-776): unit normal, tau1 from a node diagonal,
 * tau2 = n x tau1; normal entrainment speed of the rotating frame */
typedef struct { vec_t n, t1, t2; REAL s, qe; } frame_t;
static frame_t face_frame(const level_t *L, int f, int i, int j, int k)
{
    frame_t fr;
    size_t p = IX(L, i, j, k);
    vec_t S = fS(L, f, p), r;
    REAL s = L->fs[f][p];
    fr.n.x = S.x / s; fr.n.y = S.y / s; fr.n.z = S.z / s;
    if (f == 0) r = vsub(node(L, i, j + 1, k + 1), node(L, i, j, k));
    else if (f == 1) r = vsub(node(L, i + 1, j, k + 1), node(L, i, j, k));
    else r = vsub(node(L, i + 1, j + 1, k), node(L, i, j, k));
    REAL ue = -1.0f * L->fc[f][1][p] * L->w_rot;
    REAL ve = L->fc[f][0][p] * L->w_rot;
    REAL rl = sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
    fr.t1.x = r.x / rl; fr.t1.y = r.y / rl; fr.t1.z = r.z / rl;
    r.x = fr.n.y * fr.t1.z - fr.n.z * fr.t1.y;
    r.y = fr.n.z * fr.t1.x - fr.n.x * fr.t1.z;
    r.z = fr.n.x * fr.t1.y - fr.n.y * fr.t1.x;
    rl = sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
    fr.t2.x = r.x / rl; fr.t2.y = r.y / rl; fr.t2.z = r.z / rl;
    fr.s = s;
    fr.qe = ue * fr.n.x + ve * fr.n.y + 0.0f * fr.n.z;
    return fr;
}
static cons_t rotate_in(const frame_t *fr, cons_t c)
{
    cons_t q = {c.d,
                c.mx * fr->n.x + c.my * fr->n.y + c.mz * fr->n.z,
                c.mx * fr->t1.x + c.my * fr->t1.y + c.mz * fr->t1.z,
                c.mx * fr->t2.x + c.my * fr->t2.y + c.mz * fr->t2.z, c.e};
    return q;
}

static REAL entropy_corr(REAL z, REAL d) { if (z > d) return z; else return 0.5f * (z * z + d * d) / d; }

/* source/Flux_Split_Scheme.cpp:568-635 */
static cons_t roe_flux(const orc_solver *s, cons_t QL, cons_t QR, REAL Qe)
{
    REAL Gamma = s->Gamma;
    REAL dL = QL.d, uL = QL.mx / QL.d, vL = QL.my / QL.d, wL = QL.mz / QL.d, EL = QL.e / QL.d;
    REAL pL = (Gamma - 1.0f) * dL * (EL - 0.5f * (uL * uL + vL * vL + wL * wL));
    REAL HL = EL + pL / dL;
    REAL dR = QR.d, uR = QR.mx / QR.d, vR = QR.my / QR.d, wR = QR.mz / QR.d, ER = QR.e / QR.d;
    REAL pR = (Gamma - 1.0f) * dR * (ER - 0.5f * (uR * uR + vR * vR + wR * wR));
    REAL HR = ER + pR / dR;
    cons_t FL = {QL.d * (uL - Qe), QL.mx * (uL - Qe) + pL, QL.my * (uL - Qe), QL.mz * (uL - Qe), (QL.e + pL) * (uL - Qe) + Qe * pL};
    cons_t FR = {QR.d * (uR - Qe), QR.mx * (uR - Qe) + pR, QR.my * (uR - Qe), QR.mz * (uR - Qe), (QR.e + pR) * (uR - Qe) + Qe * pR};
    REAL tmpp = sqrt(dR / dL);
    REAL u_av = (uL + tmpp * uR) / (1.0f + tmpp);
    REAL v_av = (vL + tmpp * vR) / (1.0f + tmpp);
    REAL w_av = (wL + tmpp * wR) / (1.0f + tmpp);
    REAL H_av = (HL + tmpp * HR) / (1.0f + tmpp);
    REAL c_av = sqrt((Gamma - 1.0f) * (H_av - 0.5f * (u_av * u_av + v_av * v_av + w_av * w_av)));
    REAL l1 = fabs((u_av - Qe) - c_av), l2 = fabs((u_av - Qe)), l5 = fabs((u_av - Qe) + c_av);
    REAL delta = 0.5f;
    l1 = entropy_corr(l1, delta); l2 = entropy_corr(l2, delta); l5 = entropy_corr(l5, delta);
    REAL arr[6];
    arr[2] = (QR.my - QL.my) / (v_av + 1E-8f) - (dR - dL);
    arr[3] = (QR.mz - QL.mz) / (w_av + 1E-8f) - (dR - dL);
    arr[4] = (Gamma - 1.0f) * ((dR - dL) * (H_av - u_av * u_av - v_av * v_av - w_av * w_av) + u_av * (QR.mx - QL.mx) +
                               v_av * (QR.my - QL.my) + w_av * (QR.mz - QL.mz) - (QR.e - QL.e)) / (c_av * c_av);
    arr[1] = ((u_av + c_av) * (dR - dL) - (QR.mx - QL.mx) - c_av * arr[4]) / (2.0f * c_av);
    arr[5] = dR - dL - (arr[1] + arr[4]);
    cons_t F;
    F.d = 0.5f * (FL.d + FR.d) - 0.5f * (l1 * arr[1] + l2 * arr[4] + l5 * arr[5]);
    F.mx = 0.5f * (FL.mx + FR.mx) - 0.5f * (l1 * arr[1] * (u_av - c_av) + l2 * arr[4] * u_av + l5 * arr[5] * (u_av + c_av));
    F.my = 0.5f * (FL.my + FR.my) - 0.5f * (l1 * arr[1] * v_av + l2 * arr[2] * v_av + l2 * arr[4] * v_av + l5 * arr[5] * v_av);
    F.mz = 0.5f * (FL.mz + FR.mz) - 0.5f * (l1 * arr[1] * w_av + l2 * arr[3] * w_av + l2 * arr[4] * w_av + l5 * arr[5] * w_av);
    F.e = 0.5f * (FL.e + FR.e) - 0.5f * (l1 * arr[1] * (H_av - u_av * c_av) + l2 * arr[2] * v_av * v_av + l2 * arr[3] * w_av * w_av +
                                          l2 * arr[4] * 0.5f * (u_av * u_av + v_av * v_av + w_av * w_av) + l5 * arr[5] * (H_av + u_av * c_av));
    return F;
}

/* source/Flux_Split_Scheme.cpp:82-149 */
static cons_t sw_flux(const orc_solver *s, cons_t QL, cons_t QR, REAL Qe)
{
    REAL Gamma = s->Gamma, epsilon = 1E-6f;
    REAL lp[6], lm[6], fp[6], fm[6];
    REAL dL = QL.d, uL = QL.mx / QL.d, vL = QL.my / QL.d, wL = QL.mz / QL.d, eL = QL.e / QL.d;
    REAL tL = Gamma * (Gamma - 1.0f) * (eL - 0.5f * (uL * uL + vL * vL + wL * wL));
    tL = sqrt(tL * tL);
    REAL cL = sqrt(tL);
    lp[1] = 0.5f * ((uL - Qe) + sqrt((uL - Qe) * (uL - Qe) + epsilon * epsilon));
    lp[2] = lp[1]; lp[3] = lp[1];
    lp[4] = 0.5f * (((uL - Qe) - cL) + sqrt(((uL - Qe) - cL) * ((uL - Qe) - cL) + epsilon * epsilon));
    lp[5] = 0.5f * (((uL - Qe) + cL) + sqrt(((uL - Qe) + cL) * ((uL - Qe) + cL) + epsilon * epsilon));
    REAL W2 = (3.0f - Gamma) * (lp[4] + lp[5]) * cL * cL / 2.0f / (Gamma - 1.0f);
    REAL A = (uL - cL) * (uL - cL) + vL * vL + wL * wL;
    REAL B = (uL + cL) * (uL + cL) + vL * vL + wL * wL;
    fp[1] = dL / 2.0f / Gamma * (2.0f * (Gamma - 1.0f) * lp[1] + lp[4] + lp[5]);
    fp[2] = dL / 2.0f / Gamma * (2.0f * (Gamma - 1.0f) * lp[1] * uL + lp[4] * (uL - cL) + lp[5] * (uL + cL));
    fp[3] = dL / 2.0f / Gamma * (2.0f * (Gamma - 1.0f) * lp[1] * vL + lp[4] * vL + lp[5] * vL);
    fp[4] = dL / 2.0f / Gamma * (2.0f * (Gamma - 1.0f) * lp[1] * wL + lp[4] * wL + lp[5] * wL);
    fp[5] = dL / 2.0f / Gamma * ((Gamma - 1.0f) * lp[1] * (uL * uL + vL * vL + wL * wL) + 0.5f * lp[4] * A + 0.5f * lp[5] * B + W2);
    REAL dR = QR.d, uR = QR.mx / QR.d, vR = QR.my / QR.d, wR = QR.mz / QR.d, eR = QR.e / QR.d;
    REAL tR = Gamma * (Gamma - 1.0f) * (eR - 0.5f * (uR * uR + vR * vR + wR * wR));
    tR = sqrt(tR * tR);
    REAL cR = sqrt(tR);
    lm[1] = 0.5f * ((uR - Qe) - sqrt((uR - Qe) * (uR - Qe) + epsilon * epsilon));
    lm[2] = lm[1]; lm[3] = lm[1];
    lm[4] = 0.5f * (((uR - Qe) - cR) - sqrt(((uR - Qe) - cR) * ((uR - Qe) - cR) + epsilon * epsilon));
    lm[5] = 0.5f * (((uR - Qe) + cR) - sqrt(((uR - Qe) + cR) * ((uR - Qe) + cR) + epsilon * epsilon));
    W2 = (3.0f - Gamma) * (lm[4] + lm[5]) * cR * cR / 2.0f / (Gamma - 1.0f);
    A = (uR - cR) * (uR - cR) + vR * vR + wR * wR;
    B = (uR + cR) * (uR + cR) + vR * vR + wR * wR;
    fm[1] = dR / 2.0f / Gamma * (2.0f * (Gamma - 1.0f) * lm[1] + lm[4] + lm[5]);
    fm[2] = dR / 2.0f / Gamma * (2.0f * (Gamma - 1.0f) * lm[1] * uR + lm[4] * (uR - cR) + lm[5] * (uR + cR));
    fm[3] = dR / 2.0f / Gamma * (2.0f * (Gamma - 1.0f) * lm[1] * vR + lm[4] * vR + lm[5] * vR);
    fm[4] = dR / 2.0f / Gamma * (2.0f * (Gamma - 1.0f) * lm[1] * wR + lm[4] * wR + lm[5] * wR);
    fm[5] = dR / 2.0f / Gamma * ((Gamma - 1.0f) * lm[1] * (uR * uR + vR * vR + wR * wR) + 0.5f * lm[4] * A + 0.5f * lm[5] * B + W2);
    cons_t F = {fp[1] + fm[1], fp[2] + fm[2], fp[3] + fm[3], fp[4] + fm[4], fp[5] + fm[5]};
    return F;
}

/* index remap of the reconstruction stencil: logical cell c (may be a ghost) -> storage
 * index, skipping the first ghost layer in favour of the dummy layers
 * (source/Upwind_Convective.cpp:38-97) */
static int rmap(int c, int N) { return c <= 0 ? c - 1 : (c >= N ? c + 1 : c); }

/* source/Upwind_Convective.cpp:5-360 */
static void upwind_convective(orc_solver *s, level_t *L)
{
    int IM = L->IM, JM = L->JM, KM = L->KM;
    for (int f = 0; f < 3; f++) {
        int ie = f == 0 ? IM : IM - 1, je = f == 1 ? JM : JM - 1, ke = f == 2 ? KM : KM - 1;
        for (int i = 1; i <= ie; i++)
            for (int j = 1; j <= je; j++)
                for (int k = 1; k <= ke; k++) {
                    size_t pc[4];
                    for (int q = 0; q < 4; q++) {
                        int o = q - 2;
                        if (f == 0) pc[q] = IX(L, rmap(i + o, IM), j, k);
                        else if (f == 1) pc[q] = IX(L, i, rmap(j + o, JM), k);
                        else pc[q] = IX(L, i, j, rmap(k + o, KM));
                    }
                    cons_t cl, cr;
                    if (s->recon_var == 100) recon_cons(s, ld_cv(L->cv, pc[0]), ld_cv(L->cv, pc[1]), ld_cv(L->cv, pc[2]), ld_cv(L->cv, pc[3]), &cl, &cr);
                    else recon_prim(s, ld_pv(L->pv, pc[0]), ld_pv(L->pv, pc[1]), ld_pv(L->pv, pc[2]), ld_pv(L->pv, pc[3]), &cl, &cr);
                    frame_t fr = face_frame(L, f, i, j, k);
                    cons_t QL = rotate_in(&fr, cl), QR = rotate_in(&fr, cr);
                    cons_t F = s->scheme == 300 ? roe_flux(s, QL, QR, fr.qe) : sw_flux(s, QL, QR, fr.qe);
                    size_t p = IX(L, i, j, k);
                    L->Ff[f][0][p] = F.d * fr.s;
                    L->Ff[f][1][p] = (F.mx * fr.n.x + F.my * fr.t1.x + F.mz * fr.t2.x) * fr.s;
                    L->Ff[f][2][p] = (F.mx * fr.n.y + F.my * fr.t1.y + F.mz * fr.t2.y) * fr.s;
                    L->Ff[f][3][p] = (F.mx * fr.n.z + F.my * fr.t1.z + F.mz * fr.t2.z) * fr.s;
                    L->Ff[f][4][p] = F.e * fr.s;
                }
    }
}

/* source/WallFlux.cpp:70-175 */
static void wall_flux(orc_solver *s, level_t *L, const wall_t *w)
{
    REAL Gamma = s->Gamma;
    int f = (w->face - 1) / 2;
    for (int i = w->is; i <= w->ie; i++)
        for (int j = w->js; j <= w->je; j++)
            for (int k = w->ks; k <= w->ke; k++) {
                size_t p = IX(L, i, j, k);
                size_t m = f == 0 ? IX(L, i - 1, j, k) : (f == 1 ? IX(L, i, j - 1, k) : IX(L, i, j, k - 1));
                vec_t S = fS(L, f, p);
                prim_t fp = p_scl(0.5f, p_add(ld_pv(L->pv, p), ld_pv(L->pv, m)));
                REAL fue = -1.0f * L->fc[f][1][p] * w->rot;
                REAL fve = L->fc[f][0][p] * w->rot;
                cons_t fc = {fp.d, fp.d * fp.u, fp.d * fp.v, fp.d * fp.w, 0.0};
                REAL Vn_a = fp.u * S.x + fp.v * S.y + fp.w * S.z;
                REAL Vn_e = fue * S.x + fve * S.y + 0.0f * S.z;
                fc.e = fp.p / (Gamma - 1.0f) + fp.d * (fp.u * fp.u + fp.v * fp.v + fp.w * fp.w) / 2.0f;
                L->Ff[f][0][p] = fc.d * (Vn_a - Vn_e);
                L->Ff[f][1][p] = fc.mx * (Vn_a - Vn_e) + fp.p * S.x;
                L->Ff[f][2][p] = fc.my * (Vn_a - Vn_e) + fp.p * S.y;
                L->Ff[f][3][p] = fc.mz * (Vn_a - Vn_e) + fp.p * S.z;
                L->Ff[f][4][p] = (fc.e + fp.p) * (Vn_a - Vn_e) + fp.p * Vn_e;
                if (w->face % 2 == 1) L->mut[m] = -L->mut[p];
                else L->mut[p] = -L->mut[m];
            }
}

/* source/JST_Convective.cpp:5-95: the central flux of every face from the average of the two
 * cells' primitive variables (the first ghost layer at the block faces), in the block's frame */
static void jst_convective(orc_solver *s, level_t *L)
{
    REAL Gamma = s->Gamma;
    int IM = L->IM, JM = L->JM, KM = L->KM;
    for (int f = 0; f < 3; f++) {
        int ie = f == 0 ? IM : IM - 1, je = f == 1 ? JM : JM - 1, ke = f == 2 ? KM : KM - 1;
        for (int i = 1; i <= ie; i++)
            for (int j = 1; j <= je; j++)
                for (int k = 1; k <= ke; k++) {
                    size_t p = IX(L, i, j, k);
                    size_t m = f == 0 ? IX(L, i - 1, j, k) : (f == 1 ? IX(L, i, j - 1, k) : IX(L, i, j, k - 1));
                    vec_t S = fS(L, f, p);
                    prim_t fp = p_scl(0.5f, p_add(ld_pv(L->pv, p), ld_pv(L->pv, m)));
                    REAL fue = -1.0f * L->fc[f][1][p] * L->w_rot;
                    REAL fve = L->fc[f][0][p] * L->w_rot;
                    cons_t fc = {fp.d, fp.d * fp.u, fp.d * fp.v, fp.d * fp.w, 0.0};
                    REAL Vn_a = fp.u * S.x + fp.v * S.y + fp.w * S.z;
                    REAL Vn_e = fue * S.x + fve * S.y + 0.0f * S.z;
                    fc.e = fp.p / (Gamma - 1.0f) + fp.d * (fp.u * fp.u + fp.v * fp.v + fp.w * fp.w) / 2.0f;
                    L->Ff[f][0][p] = fc.d * (Vn_a - Vn_e);
                    L->Ff[f][1][p] = fc.mx * (Vn_a - Vn_e) + fp.p * S.x;
                    L->Ff[f][2][p] = fc.my * (Vn_a - Vn_e) + fp.p * S.y;
                    L->Ff[f][3][p] = fc.mz * (Vn_a - Vn_e) + fp.p * S.z;
                    L->Ff[f][4][p] = (fc.e + fp.p) * (Vn_a - Vn_e) + fp.p * Vn_e;
                }
    }
}

/* the JST pressure sensor |p(c+1) - 2 p(c) + p(c-1)| / (p(c+1) + 2 p(c) + p(c-1)) at position c
 * along direction f of the line through (i, j, k) (source/JST_Dissip.cpp:5-194): positions at or
 * below 0 and at or above N lie in the dummy layers (the remap of the reconstruction stencil). The
 * range checks are the reference's, including its k-direction test of j against KM. */
static REAL jst_sensor(const level_t *L, int f, int i, int j, int k)
{
    int IM = L->IM, JM = L->JM, KM = L->KM;
    if (f == 0 && (j < 1 || j > JM || k < 1 || k > KM)) return 0.0;
    if (f == 1 && (i < 1 || i > IM || k < 1 || k > KM)) return 0.0;
    if (f == 2 && (i < 1 || i > IM || j < 1 || j > KM)) return 0.0;
    int c = f == 0 ? i : (f == 1 ? j : k), N = f == 0 ? IM : (f == 1 ? JM : KM);
    size_t q[3];
    for (int o = -1; o <= 1; o++) {
        int r = rmap(c + o, N);
        q[o + 1] = f == 0 ? IX(L, r, j, k) : (f == 1 ? IX(L, i, r, k) : IX(L, i, j, r));
    }
    REAL PF = L->pv[PP][q[2]], PC = L->pv[PP][q[1]], PB = L->pv[PP][q[0]];
    return fabs((PF - 2.0f * PC + PB) / (PF + 2.0f * PC + PB));
}

static REAL max4(REAL a, REAL b, REAL c, REAL d)
{
    REAL m = a;
    if (b > m) m = b;
    if (c > m) m = c;
    if (d > m) m = d;
    return m;
}

/* 1 + (lam_a / lam_n)^0.4 + (lam_b / lam_n)^0.4, the anisotropy weight of direction f; the two
 * other directions in the reference's order (I: J, K; J: I, K; K: J, I) */
static REAL jst_phi(const level_t *L, int f, size_t p)
{
    int a = f == 0 ? 1 : (f == 1 ? 0 : 1), b = f == 0 ? 2 : (f == 1 ? 2 : 0);
    return 1.0f + pow_rt(L->lamc[a][p] / L->lamc[f][p], (double)0.4f) + pow_rt(L->lamc[b][p] / L->lamc[f][p], (double)0.4f);
}

/* source/JST_Dissip.cpp:196-423 and the cell sum :425-431 */
static void jst_dissip(orc_solver *s, level_t *L)
{
    int IM = L->IM, JM = L->JM, KM = L->KM;
    for (int f = 0; f < 3; f++) {
        int ie = f == 0 ? IM : IM - 1, je = f == 1 ? JM : JM - 1, ke = f == 2 ? KM : KM - 1;
        int N = f == 0 ? IM : (f == 1 ? JM : KM);
        for (int i = 1; i <= ie; i++)
            for (int j = 1; j <= je; j++)
                for (int k = 1; k <= ke; k++) {
                    int c = f == 0 ? i : (f == 1 ? j : k);
                    size_t p = IX(L, i, j, k);
                    size_t m = f == 0 ? IX(L, i - 1, j, k) : (f == 1 ? IX(L, i, j - 1, k) : IX(L, i, j, k - 1));
                    REAL alpha;
                    if (c == 1) alpha = jst_phi(L, f, p) * L->lamc[f][p];
                    else if (c == N) alpha = jst_phi(L, f, m) * L->lamc[f][m];
                    else {
                        REAL VA_1 = jst_phi(L, f, p) * L->lamc[f][p];
                        REAL VA_2 = jst_phi(L, f, m) * L->lamc[f][m];
                        alpha = 0.5f * (VA_1 + VA_2);
                    }
                    REAL sn[4];
                    for (int o = 1; o >= -2; o--) {
                        int ii = f == 0 ? i + o : i, jj = f == 1 ? j + o : j, kk = f == 2 ? k + o : k;
                        sn[1 - o] = jst_sensor(L, f, ii, jj, kk);
                    }
                    REAL eps2 = s->k2 * max4(sn[0], sn[1], sn[2], sn[3]);
                    REAL eps4 = (0.0f > s->k4 - eps2) ? 0.0f : s->k4 - eps2;
                    size_t q[4];                                  /* cv_1 .. cv_4: c+1, c, c-1, c-2 */
                    for (int o = 1; o >= -2; o--) {
                        int r = rmap(c + o, N);
                        q[1 - o] = f == 0 ? IX(L, r, j, k) : (f == 1 ? IX(L, i, r, k) : IX(L, i, j, r));
                    }
                    cons_t c1 = ld_cv(L->cv, q[0]), c2 = ld_cv(L->cv, q[1]), c3 = ld_cv(L->cv, q[2]), c4 = ld_cv(L->cv, q[3]);
                    cons_t d4 = c_sub(c_add(c_sub(c1, c_scl(c2, 3.0)), c_scl(c3, 3.0)), c4);
                    cons_t fd = c_scl(c_sub(c_scl(c_sub(c2, c3), eps2), c_scl(d4, eps4)), alpha);
                    st_cv(L->Fdf[f], p, fd);
                }
    }
    for (int i = 1; i <= IM - 1; i++)
        for (int j = 1; j <= JM - 1; j++)
            for (int k = 1; k <= KM - 1; k++) {
                size_t p = IX(L, i, j, k);
                size_t q[3] = {IX(L, i + 1, j, k), IX(L, i, j + 1, k), IX(L, i, j, k + 1)};
                cons_t a = c_sub(ld_cv(L->Fdf[0], q[0]), ld_cv(L->Fdf[0], p));
                a = c_add(a, ld_cv(L->Fdf[1], q[1]));
                a = c_sub(a, ld_cv(L->Fdf[1], p));
                a = c_add(a, ld_cv(L->Fdf[2], q[2]));
                a = c_sub(a, ld_cv(L->Fdf[2], p));
                st_cv(L->Fd, p, a);
            }
}

/* source/ComputeAllBlockVars.cpp:73-119 */
static void convective_flux(orc_solver *s, level_t *L)
{
    if (s->scheme == 100) jst_convective(s, L);
    else upwind_convective(s, L);
    for (int q = 1; q <= L->n_wall; q++) wall_flux(s, L, &L->wall[q]);
    REAL w_rot = L->w_rot;
    for (int i = 1; i <= L->IM - 1; i++)
        for (int j = 1; j <= L->JM - 1; j++)
            for (int k = 1; k <= L->KM - 1; k++) {
                size_t p = IX(L, i, j, k);
                REAL u = L->pv[PU][p], v = L->pv[PV][p];
                cons_t Qc = {0.0, L->pv[PD][p] * (w_rot * v) * L->vol[p], -1.0f * L->pv[PD][p] * (w_rot * u) * L->vol[p], 0.0, 0.0};
                size_t q[3] = {IX(L, i + 1, j, k), IX(L, i, j + 1, k), IX(L, i, j, k + 1)};
                cons_t a = c_sub(ld_cv(L->Ff[0], q[0]), ld_cv(L->Ff[0], p));
                a = c_add(a, ld_cv(L->Ff[1], q[1]));
                a = c_sub(a, ld_cv(L->Ff[1], p));
                a = c_add(a, ld_cv(L->Ff[2], q[2]));
                a = c_sub(a, ld_cv(L->Ff[2], p));
                a = c_sub(a, Qc);
                st_cv(L->Fc, p, a);
            }
}

/* source/ViscousFlux.cpp:9-283 */
static void viscous_flux(orc_solver *s, level_t *L)
{
    int IM = L->IM, JM = L->JM, KM = L->KM;
    REAL Gamma = s->Gamma, Pr_lam = s->Pr_lam, Pr_tur = s->Pr_tur, Rgas = s->Rgas;
    for (int f = 0; f < 3; f++) {
        int ie = f == 0 ? IM : IM - 1, je = f == 1 ? JM : JM - 1, ke = f == 2 ? KM : KM - 1;
        for (int i = 1; i <= ie; i++)
            for (int j = 1; j <= je; j++)
                for (int k = 1; k <= ke; k++) {
                    size_t p = IX(L, i, j, k);
                    size_t m = f == 0 ? IX(L, i - 1, j, k) : (f == 1 ? IX(L, i, j - 1, k) : IX(L, i, j, k - 1));
                    REAL g[3][4];
                    if (f == 0) grad_faceI(L, i, j, k, g);
                    else if (f == 1) grad_faceJ(L, i, j, k, g);
                    else grad_faceK(L, i, j, k, g);
                    REAL uf = 0.5f * (L->pv[PU][p] + L->pv[PU][m]);
                    REAL vf = 0.5f * (L->pv[PV][p] + L->pv[PV][m]);
                    REAL wf = 0.5f * (L->pv[PW][p] + L->pv[PW][m]);
                    REAL tf = 0.5f * (L->pv[PT][p] + L->pv[PT][m]);
                    REAL mue_lam = sutherland(s, tf);
                    REAL cond_lam = mue_lam * Gamma * Rgas / (Gamma - 1.0f) / Pr_lam;
                    REAL mue_tur, cond_tur;
                    if (s->turb_bl) {
                        mue_tur = (L->mut[m] + L->mut[p]) / 2.0f;
                        cond_tur = mue_tur * Gamma * Rgas / (Gamma - 1.0f) / Pr_tur;
                    } else { mue_tur = 0.0; cond_tur = 0.0; }
                    REAL mue = mue_lam + mue_tur, cond = cond_lam + cond_tur;
                    /* g[a][c]: a = x,y,z derivative, c = u,v,w,T */
                    REAL txx = mue * (4.0f / 3.0f * g[0][0] - 2.0f / 3.0f * (g[1][1] + g[2][2]));
                    REAL txy = mue * (g[1][0] + g[0][1]);
                    REAL txz = mue * (g[2][0] + g[0][2]);
                    REAL tyy = mue * (4.0f / 3.0f * g[1][1] - 2.0f / 3.0f * (g[0][0] + g[2][2]));
                    REAL tyz = mue * (g[2][1] + g[1][2]);
                    REAL tzz = mue * (4.0f / 3.0f * g[2][2] - 2.0f / 3.0f * (g[0][0] + g[1][1]));
                    vec_t F1 = {0.0, 0.0, 0.0}, F2 = {txx, txy, txz}, F3 = {txy, tyy, tyz}, F4 = {txz, tyz, tzz};
                    vec_t F5 = {uf * txx + vf * txy + wf * txz + cond * g[0][3], uf * txy + vf * tyy + wf * tyz + cond * g[1][3],
                                uf * txz + vf * tyz + wf * tzz + cond * g[2][3]};
                    vec_t S = fS(L, f, p);
                    L->Vf[f][0][p] = vdot(F1, S); L->Vf[f][1][p] = vdot(F2, S); L->Vf[f][2][p] = vdot(F3, S);
                    L->Vf[f][3][p] = vdot(F4, S); L->Vf[f][4][p] = vdot(F5, S);
                }
    }
    for (int i = 1; i <= IM - 1; i++)
        for (int j = 1; j <= JM - 1; j++)
            for (int k = 1; k <= KM - 1; k++) {
                size_t p = IX(L, i, j, k);
                size_t q[3] = {IX(L, i + 1, j, k), IX(L, i, j + 1, k), IX(L, i, j, k + 1)};
                cons_t a = c_sub(ld_cv(L->Vf[0], q[0]), ld_cv(L->Vf[0], p));
                a = c_add(a, ld_cv(L->Vf[1], q[1]));
                a = c_sub(a, ld_cv(L->Vf[1], p));
                a = c_add(a, ld_cv(L->Vf[2], q[2]));
                a = c_sub(a, ld_cv(L->Vf[2], p));
                st_cv(L->Fv, p, a);
            }
}

/* source/ComputeAllBlockVars.cpp:223-255 */
static void resflux(orc_solver *s, level_t *L)
{
    boundary_condition(s, L);
    spectral_radii(s, L);
    if (s->equation_ns) { curl(L); }
    if (L->id == 1 && s->turb_bl) bl_model(s, L);
    time_step(s, L);
    convective_flux(s, L);
    if (s->equation_ns) viscous_flux(s, L);
    else
        for (int c = 0; c < NQ; c++) memset(L->Fv[c], 0, L->n * sizeof(REAL));
    /* CMesh::Dissipation (:162-191): the JST dissipation, zero for the upwind schemes */
    if (s->scheme == 100) jst_dissip(s, L);
    else
        for (int c = 0; c < NQ; c++) memset(L->Fd[c], 0, L->n * sizeof(REAL));
    for (int i = 1; i <= L->IM - 1; i++)
        for (int j = 1; j <= L->JM - 1; j++)
            for (int k = 1; k <= L->KM - 1; k++) {
                size_t p = IX(L, i, j, k);
                st_cv(L->res, p, c_sub(c_sub(ld_cv(L->Fc, p), ld_cv(L->Fv, p)), ld_cv(L->Fd, p)));
            }
}

/* ====================================================================================
 * LU-SGS (source/LU_SGS_Marching.cpp)
 * ==================================================================================== */
/* :293-355 (lower neighbour, dir 0/1/2) and :357-419 (upper neighbour) */
static cons_t delt_fn(orc_solver *s, level_t *L, int i, int j, int k, int dir, int upper)
{
    vec_t nrm;
    size_t a, b;                   /* the two faces whose unit normals are averaged */
    int ni = i, nj = j, nk = k;    /* neighbour cell */
    if (!upper) {
        if (dir == 0) { a = IX(L, i, j, k); b = IX(L, i - 1, j, k); ni = i - 1; }
        else if (dir == 1) { a = IX(L, i, j, k); b = IX(L, i, j - 1, k); nj = j - 1; }
        else { a = IX(L, i, j, k); b = IX(L, i, j, k - 1); nk = k - 1; }
    } else {
        if (dir == 0) { a = IX(L, i + 2, j, k); b = IX(L, i + 1, j, k); ni = i + 1; }
        else if (dir == 1) { a = IX(L, i, j + 2, k); b = IX(L, i, j + 1, k); nj = j + 1; }
        else { a = IX(L, i, j, k + 2); b = IX(L, i, j, k + 1); nk = k + 1; }
    }
    int f = dir;
    nrm.x = (L->fS[f][0][a] / L->fs[f][a] + L->fS[f][0][b] / L->fs[f][b]) / 2.0f;
    nrm.y = (L->fS[f][1][a] / L->fs[f][a] + L->fS[f][1][b] / L->fs[f][b]) / 2.0f;
    nrm.z = (L->fS[f][2][a] / L->fs[f][a] + L->fS[f][2][b] / L->fs[f][b]) / 2.0f;
    size_t p = IX(L, ni, nj, nk);
    REAL ue = -1.0f * L->cc[1][p] * L->w_rot;
    REAL ve = L->cc[0][p] * L->w_rot;
    cons_t co = ld_cv(L->cv, p);
    cons_t cn = c_add(co, ld_cv(L->dq, p));
    REAL Gamma = s->Gamma;
    REAL dens = cn.d, u = cn.mx / cn.d, v = cn.my / cn.d, w = cn.mz / cn.d, E = cn.e / cn.d;
    REAL pn = (Gamma - 1.0f) * dens * (E - 0.5f * (u * u + v * v + w * w));
    REAL po = L->pv[PP][p];
    REAL Vo = co.mx / co.d * nrm.x + co.my / co.d * nrm.y + co.mz / co.d * nrm.z;
    REAL Vn = u * nrm.x + v * nrm.y + w * nrm.z;
    REAL Ve = ue * nrm.x + ve * nrm.y + 0.0f * nrm.z;
    cons_t d;
    d.d = cn.d * (Vn - Ve) - co.d * (Vo - Ve);
    d.mx = (cn.mx * (Vn - Ve) + pn * nrm.x) - (co.mx * (Vo - Ve) + po * nrm.x);
    d.my = (cn.my * (Vn - Ve) + pn * nrm.y) - (co.my * (Vo - Ve) + po * nrm.y);
    d.mz = (cn.mz * (Vn - Ve) + pn * nrm.z) - (co.mz * (Vo - Ve) + po * nrm.z);
    d.e = ((cn.e + pn) * (Vn - Ve) + pn * Ve) - ((co.e + po) * (Vo - Ve) + po * Ve);
    return d;
}

static void lusgs(orc_solver *s, level_t *L)
{
    int IM = L->IM, JM = L->JM, KM = L->KM;
    REAL relax = s->relax;
    cons_t zero = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int i = 1; i <= IM - 1; i++)
        for (int j = 1; j <= JM - 1; j++)
            for (int k = 1; k <= KM - 1; k++) {
                size_t p = IX(L, i, j, k);
                st_cv(L->cvold, p, ld_cv(L->cv, p));
            }
    if (!L->use_force) resflux(s, L);
    else {
        /* ComputeAllBlockVars.cpp:269-309 */
        for (int i = 1; i <= IM - 1; i++)
            for (int j = 1; j <= JM - 1; j++)
                for (int k = 1; k <= KM - 1; k++) {
                    size_t p = IX(L, i, j, k);
                    st_cv(L->qf2h, p, c_sub(ld_cv(L->res2h, p), ld_cv(L->res, p)));
                }
        if (L->id == 2)
            for (int i = 1; i <= IM - 1; i++)
                for (int j = 1; j <= JM - 1; j++)
                    for (int k = 1; k <= KM - 1; k++) {
                        size_t p = IX(L, i, j, k);
                        st_cv(L->res, p, c_add(ld_cv(L->res, p), ld_cv(L->qf2h, p)));
                    }
    }
    for (int plane = 3; plane <= IM + JM + KM - 3; plane++)
        for (int i = 1; i <= IM - 1; i++)
            for (int j = 1; j <= JM - 1; j++) {
                int k = plane - i - j;
                if (k < 1 || k > KM - 1) continue;
                size_t p = IX(L, i, j, k);
                REAL alpha = L->vol[p] / L->dt[p] + relax * (L->lamc[0][p] + L->lamc[1][p] + L->lamc[2][p]) + 2.0f * (L->lamv[0][p] + L->lamv[1][p] + L->lamv[2][p]);
                cons_t AW[3], VW[3];
                size_t nb[3] = {IX(L, i - 1, j, k), IX(L, i, j - 1, k), IX(L, i, j, k - 1)};
                size_t fa[3][2] = {{IX(L, i - 1, j, k), p}, {IX(L, i, j - 1, k), p}, {IX(L, i, j, k - 1), p}};
                int idx[3] = {i, j, k};
                for (int d = 0; d < 3; d++) {
                    if (idx[d] != 1) {
                        cons_t dF = delt_fn(s, L, i, j, k, d, 0);
                        REAL sd = 0.5f * (L->fs[d][fa[d][0]] + L->fs[d][fa[d][1]]);
                        AW[d] = c_scl(c_add(c_scl(dF, sd), c_scl(ld_cv(L->dq, nb[d]), relax * L->lamc[d][nb[d]])), 0.5f);
                        VW[d] = c_scl(ld_cv(L->dq, nb[d]), L->lamv[d][nb[d]]);
                    } else { AW[d] = zero; VW[d] = zero; }
                }
                cons_t r = c_scl(ld_cv(L->res, p), -1.0f);
                r = c_add(r, AW[0]); r = c_add(r, AW[1]); r = c_add(r, AW[2]);
                r = c_add(r, VW[0]); r = c_add(r, VW[1]); r = c_add(r, VW[2]);
                st_cv(L->dq, p, c_divs(r, alpha));
            }
    for (int plane = IM + JM + KM - 3; plane >= 3; plane--)
        for (int i = IM - 1; i >= 1; i--)
            for (int j = JM - 1; j >= 1; j--) {
                int k = plane - i - j;
                if (k < 1 || k > KM - 1) continue;
                size_t p = IX(L, i, j, k);
                REAL alpha = L->vol[p] / L->dt[p] + relax * (L->lamc[0][p] + L->lamc[1][p] + L->lamc[2][p]) + 2.0f * (L->lamv[0][p] + L->lamv[1][p] + L->lamv[2][p]);
                cons_t AW[3], VW[3];
                size_t nb[3] = {IX(L, i + 1, j, k), IX(L, i, j + 1, k), IX(L, i, j, k + 1)};
                size_t fa[3][2] = {{IX(L, i + 1, j, k), IX(L, i + 2, j, k)}, {IX(L, i, j + 1, k), IX(L, i, j + 2, k)}, {IX(L, i, j, k + 1), IX(L, i, j, k + 2)}};
                int idx[3] = {i, j, k}, top[3] = {IM - 1, JM - 1, KM - 1};
                for (int d = 0; d < 3; d++) {
                    if (idx[d] != top[d]) {
                        cons_t dF = delt_fn(s, L, i, j, k, d, 1);
                        REAL sd = 0.5f * (L->fs[d][fa[d][0]] + L->fs[d][fa[d][1]]);
                        AW[d] = c_scl(c_sub(c_scl(dF, sd), c_scl(ld_cv(L->dq, nb[d]), relax * L->lamc[d][nb[d]])), 0.5f);
                        VW[d] = c_scl(ld_cv(L->dq, nb[d]), L->lamv[d][nb[d]]);
                    } else { AW[d] = zero; VW[d] = zero; }
                }
                cons_t r = c_scl(ld_cv(L->dq, p), alpha);
                r = c_sub(r, AW[0]); r = c_sub(r, AW[1]); r = c_sub(r, AW[2]);
                r = c_add(r, VW[0]); r = c_add(r, VW[1]); r = c_add(r, VW[2]);
                st_cv(L->dq, p, c_divs(r, alpha));
            }
    for (int i = 1; i <= IM - 1; i++)
        for (int j = 1; j <= JM - 1; j++)
            for (int k = 1; k <= KM - 1; k++) {
                size_t p = IX(L, i, j, k);
                st_cv(L->cv, p, c_add(ld_cv(L->cv, p), ld_cv(L->dq, p)));
            }
    primitive_vars(s, L);
    if (s->limiter) limit_vars(s, L);
}

/* source/ComputeAllBlockVars.cpp:318-372 */
static void res_calculate(orc_solver *s, level_t *L)
{
    REAL acc[NQ] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int i = 1; i <= L->IM - 1; i++)
        for (int j = 1; j <= L->JM - 1; j++)
            for (int k = 1; k <= L->KM - 1; k++) {
                size_t p = IX(L, i, j, k);
                for (int c = 0; c < NQ; c++) {
                    REAL r = fabs((L->cvold[c][p] - L->cv[c][p]) / L->cvold[c][p]);
                    r = r * L->vol[p];
                    acc[c] = acc[c] + r;
                }
            }
    for (int c = 0; c < NQ; c++) s->res[c] = (0.0 + acc[c]) / L->totalvol;
}

/* ====================================================================================
 * multigrid transfer (source/Prolong_Interpolate.cpp, ComputeAllBlockVars.cpp:374-438)
 * ==================================================================================== */
static void mg_restrict(orc_solver *s, level_t *F, level_t *C)
{
    (void)s;
    for (int i = 1; i <= C->IM - 1; i++)
        for (int j = 1; j <= C->JM - 1; j++)
            for (int k = 1; k <= C->KM - 1; k++) {
                int i1 = 2 * i - 1, j1 = 2 * j - 1, k1 = 2 * k - 1, i2 = 2 * i, j2 = 2 * j, k2 = 2 * k;
                size_t f[8] = {IX(F, i1, j1, k1), IX(F, i1, j1, k2), IX(F, i1, j2, k1), IX(F, i1, j2, k2),
                               IX(F, i2, j1, k1), IX(F, i2, j1, k2), IX(F, i2, j2, k1), IX(F, i2, j2, k2)};
                cons_t sum = c_scl(ld_cv(F->cv, f[0]), F->vol[f[0]]);
                for (int q = 1; q < 8; q++) sum = c_add(sum, c_scl(ld_cv(F->cv, f[q]), F->vol[f[q]]));
                size_t p = IX(C, i, j, k);
                cons_t c2h = c_divs(sum, C->vol[p]);
                st_cv(C->cv2h, p, c2h);
                cons_t r = ld_cv(F->res, f[0]);
                for (int q = 1; q < 8; q++) r = c_add(r, ld_cv(F->res, f[q]));
                st_cv(C->res2h, p, r);
                st_cv(C->cv, p, c2h);
            }
}

static void mg_interpolate(orc_solver *s, level_t *F, level_t *C, int init_from_coarse)
{
    (void)s;
    REAL a1 = 27.0f / 64.0f, a2 = 9.0f / 64.0f, a3_ = 3.0f / 64.0f, a4_ = 1.0f / 64.0f;
    for (int i = 1; i <= F->IM - 1; i++)
        for (int j = 1; j <= F->JM - 1; j++)
            for (int k = 1; k <= F->KM - 1; k++) {
                int ia1 = (i % 2 == 0) ? i / 2 : i / 2 + 1, ia2 = (i % 2 == 0) ? i / 2 + 1 : i / 2;
                int ja1 = (j % 2 == 0) ? j / 2 : j / 2 + 1, ja2 = (j % 2 == 0) ? j / 2 + 1 : j / 2;
                int ka1 = (k % 2 == 0) ? k / 2 : k / 2 + 1, ka2 = (k % 2 == 0) ? k / 2 + 1 : k / 2;
                REAL *const *src = init_from_coarse ? C->cv : C->dq2h;
                cons_t t1 = c_scl(ld_cv(src, IX(C, ia1, ja1, ka1)), a1);
                cons_t t2 = c_scl(c_add(c_add(ld_cv(src, IX(C, ia1, ja1, ka2)), ld_cv(src, IX(C, ia1, ja2, ka1))), ld_cv(src, IX(C, ia2, ja1, ka1))), a2);
                cons_t t3 = c_scl(c_add(c_add(ld_cv(src, IX(C, ia2, ja2, ka1)), ld_cv(src, IX(C, ia1, ja2, ka2))), ld_cv(src, IX(C, ia2, ja1, ka2))), a3_);
                cons_t t4 = c_scl(ld_cv(src, IX(C, ia2, ja2, ka2)), a4_);
                cons_t d = c_add(c_add(c_add(t1, t2), t3), t4);
                size_t p = IX(F, i, j, k);
                if (init_from_coarse) st_cv(F->cv, p, d);
                else st_cv(F->cv, p, c_add(ld_cv(F->cv, p), d));
            }
}

static void mg_delta(level_t *C)
{
    for (int i = 1; i <= C->IM - 1; i++)
        for (int j = 1; j <= C->JM - 1; j++)
            for (int k = 1; k <= C->KM - 1; k++) {
                size_t p = IX(C, i, j, k);
                st_cv(C->dq2h, p, c_sub(ld_cv(C->cv, p), ld_cv(C->cv2h, p)));
            }
}

static void corner_fill(level_t *L, REAL *const a[NQ])
{
    int IM = L->IM, JM = L->JM, KM = L->KM;
#define G(i, j, k) ld_cv(a, IX(L, i, j, k))
#define E2(dst, x, y) st_cv(a, IX(L, dst), c_scl(c_add(x, y), 0.5f))
    for (int i = 1; i <= IM - 1; i++) {
        st_cv(a, IX(L, i, 0, 0), c_scl(c_add(G(i, 1, 0), G(i, 0, 1)), 0.5f));
        st_cv(a, IX(L, i, JM, 0), c_scl(c_add(G(i, JM - 1, 0), G(i, JM, 1)), 0.5f));
        st_cv(a, IX(L, i, 0, KM), c_scl(c_add(G(i, 0, KM - 1), G(i, 1, KM)), 0.5f));
        st_cv(a, IX(L, i, JM, KM), c_scl(c_add(G(i, JM - 1, KM), G(i, JM, KM - 1)), 0.5f));
    }
    for (int j = 1; j <= JM - 1; j++) {
        st_cv(a, IX(L, 0, j, 0), c_scl(c_add(G(1, j, 0), G(0, j, 1)), 0.5f));
        st_cv(a, IX(L, 0, j, KM), c_scl(c_add(G(1, j, KM), G(0, j, KM - 1)), 0.5f));
        st_cv(a, IX(L, IM, j, KM), c_scl(c_add(G(IM - 1, j, KM), G(IM, j, KM - 1)), 0.5f));
        st_cv(a, IX(L, IM, j, 0), c_scl(c_add(G(IM - 1, j, 0), G(IM, j, 1)), 0.5f));
    }
    for (int k = 1; k <= KM - 1; k++) {
        st_cv(a, IX(L, 0, 0, k), c_scl(c_add(G(1, 0, k), G(0, 1, k)), 0.5f));
        st_cv(a, IX(L, IM, 0, k), c_scl(c_add(G(IM, 1, k), G(IM - 1, 0, k)), 0.5f));
        st_cv(a, IX(L, 0, JM, k), c_scl(c_add(G(1, JM, k), G(0, JM - 1, k)), 0.5f));
        st_cv(a, IX(L, IM, JM, k), c_scl(c_add(G(IM - 1, JM, k), G(IM, JM - 1, k)), 0.5f));
    }
#define CORNER(ci, cj, ck, i1, j1, k1) st_cv(a, IX(L, ci, cj, ck), c_divs(c_sub(c_scl(c_add(c_add(G(i1, cj, ck), G(ci, j1, ck)), G(ci, cj, k1)), 2.0f), \
                                                   c_add(c_add(G(i1, j1, ck), G(i1, cj, k1)), G(ci, j1, k1))), 3.0f))
    CORNER(0, 0, 0, 1, 1, 1);
    CORNER(IM, 0, 0, IM - 1, 1, 1);
    CORNER(0, JM, 0, 1, JM - 1, 1);
    CORNER(IM, JM, 0, IM - 1, JM - 1, 1);
    CORNER(IM, 0, KM, IM - 1, 1, KM - 1);
    CORNER(0, 0, KM, 1, 1, KM - 1);
    CORNER(0, JM, KM, 1, JM - 1, KM - 1);
    CORNER(IM, JM, KM, IM - 1, JM - 1, KM - 1);
#undef CORNER
#undef E2
#undef G
}

/* ====================================================================================
 * driver (source/Solver.cpp:47-140, Ouput.cpp:9-107,282-300, Structured_FV3D.cpp:142-219)
 * ==================================================================================== */
static void section(orc_solver *s, level_t *L, int K, REAL *mass, REAL *pt, REAL *tt)
{
    REAL Gamma = s->Gamma, Rgas = s->Rgas;
    REAL m = 0.0, mp = 0.0, pmed = 0.0, mt = 0.0, tmed = 0.0;
    int k = K;
    for (int i = 1; i <= L->IM - 1; i++)
        for (int j = 1; j <= L->JM - 1; j++) {
            size_t p = IX(L, i, j, k), q = IX(L, i, j, k - 1);
            REAL dens = 0.5f * (L->pv[PD][p] + L->pv[PD][q]);
            REAL u = 0.5f * (L->pv[PU][p] + L->pv[PU][q]);
            REAL v = 0.5f * (L->pv[PV][p] + L->pv[PV][q]);
            REAL w = 0.5f * (L->pv[PW][p] + L->pv[PW][q]);
            vec_t S = fS(L, 2, p);
            m = m + dens * (u * S.x + v * S.y + w * S.z);
        }
    *mass = m * s->dens_ref * s->Vel_ref;
    for (int i = 1; i <= L->IM - 1; i++)
        for (int j = 1; j <= L->JM - 1; j++) {
            size_t p = IX(L, i, j, k), q = IX(L, i, j, k - 1);
            REAL dens = 0.5f * (L->pv[PD][p] + L->pv[PD][q]);
            REAL u = 0.5f * (L->pv[PU][p] + L->pv[PU][q]);
            REAL v = 0.5f * (L->pv[PV][p] + L->pv[PV][q]);
            REAL w = 0.5f * (L->pv[PW][p] + L->pv[PW][q]);
            vec_t S = fS(L, 2, p);
            REAL mc = dens * (u * S.x + v * S.y + w * S.z);
            REAL temp = 0.5f * (L->pv[PT][p] + L->pv[PT][q]);
            REAL Ma = sqrt(u * u + v * v + w * w) / sqrt(Gamma * Rgas * temp);
            REAL Ptc = L->pv[PP][p] * pow(1.0f + (Gamma - 1.0f) / 2.0f * Ma * Ma, Gamma / (Gamma - 1.0f));
            REAL PtG = pow(Ptc, (Gamma - 1.0f) / Gamma) * mc;
            pmed = pmed + PtG;
            mp = mp + mc;
        }
    *pt = pow(pmed / mp, Gamma / (Gamma - 1.0f)) * s->dens_ref * s->Vel_ref * s->Vel_ref;
    for (int i = 1; i <= L->IM - 1; i++)
        for (int j = 1; j <= L->JM - 1; j++) {
            size_t p = IX(L, i, j, k), q = IX(L, i, j, k - 1);
            REAL dens = 0.5f * (L->pv[PD][p] + L->pv[PD][q]);
            REAL u = 0.5f * (L->pv[PU][p] + L->pv[PU][q]);
            REAL v = 0.5f * (L->pv[PV][p] + L->pv[PV][q]);
            REAL w = 0.5f * (L->pv[PW][p] + L->pv[PW][q]);
            vec_t S = fS(L, 2, p);
            REAL mc = dens * (u * S.x + v * S.y + w * S.z);
            REAL temp = 0.5f * (L->pv[PT][p] + L->pv[PT][q]);
            REAL Ma = sqrt(u * u + v * v + w * w) / sqrt(Gamma * Rgas * temp);
            REAL Ttc = L->pv[PT][p] * pow(1 + (Gamma - 1.0f) / 2.0f * Ma * Ma, 1);
            tmed = tmed + Ttc * mc;
            mt = mt + mc;
        }
    *tt = tmed / mt * s->Temp_ref;
}

static void integrals(orc_solver *s, level_t *L)
{
    REAL mi, pti, tti, mo, pto, tto;
    section(s, L, L->in[1].ks, &mi, &pti, &tti);
    section(s, L, L->out[1].ks, &mo, &pto, &tto);
    s->m_in = mi * L->nblade;
    s->m_out = mo * L->nblade;
    REAL Gamma = s->Gamma, Rgas = s->Rgas;
    REAL PR = pto / pti;
    REAL L_adk = Gamma / (Gamma - 1.0f) * Rgas * tti * (pow(PR, (Gamma - 1.0f) / Gamma) - 1.0f);
    REAL L_k = Gamma / (Gamma - 1.0f) * Rgas * tti * (tto / tti - 1.0f);
    s->eff = L_adk / L_k;
    s->m_ratio = fabs((s->m_in - s->m_out) / s->m_in);
    s->pr = pto / pti;
}

static void solver_step(orc_solver *s)
{
    REAL CFL_amplify = 1.2f, CFL_MAX = 10.0f;
    if (s->iter > 1) {
        if (s->res[0] <= s->CFL_res) { s->CFL = s->CFL * CFL_amplify; s->CFL_res = s->CFL_res / 10.0f; }
        if (s->CFL > CFL_MAX) s->CFL = CFL_MAX;
    }
    level_t *F = &s->L[1], *C = &s->L[2];
    if (s->ng == 1) { lusgs(s, F); res_calculate(s, F); return; }
    if (s->iter < s->coarse_iter) { lusgs(s, C); res_calculate(s, C); }
    else if (s->iter == s->coarse_iter) {
        lusgs(s, C); res_calculate(s, C); corner_fill(C, C->cv); corner_fill(C, C->dq2h);
        mg_interpolate(s, F, C, 1);
        primitive_vars(s, F);
        if (s->limiter) limit_vars(s, F);
    } else {
        C->use_force = 1;
        lusgs(s, F); res_calculate(s, F);
        resflux(s, F);
        mg_restrict(s, F, C);
        primitive_vars(s, C);
        if (s->limiter) limit_vars(s, C);
        lusgs(s, C);
        mg_delta(C);
        corner_fill(C, C->cv); corner_fill(C, C->dq2h);
        mg_interpolate(s, F, C, 0);
        primitive_vars(s, F);
        if (s->limiter) limit_vars(s, F);
    }
}

/* ====================================================================================
 * API
 * ==================================================================================== */
orc_solver *orc_open(const char *dir, char *err, int errlen)
{
    orc_solver *s = (orc_solver *)calloc(1, sizeof(orc_solver));
    char grid[1024], bcf[1024];
    int IMb, JMb, KMb, nblade;
    REAL rpm;
    s->CFL_res = 1.0E-3f;
    if (read_config(s, dir, grid, bcf, err, errlen) ||
        read_bc(s, dir, bcf, &IMb, &JMb, &KMb, &nblade, &rpm, err, errlen) ||
        read_grid(s, dir, grid, IMb, JMb, KMb, err, errlen)) {
        orc_close(s);
        return NULL;
    }
    level_t *F = &s->L[1];
    F->id = 1;
    /* read_bc stored the patches in L[1] before the level was allocated; keep them */
    F->nblade = nblade;
    F->delta_th = 2.0f * PIF / nblade;
    F->w_rot = 2.0f * PIF * rpm / 60.0f;
    for (int q = 1; q <= F->n_wall; q++)
        if (s->turb_bl && (F->wall[q].face == 5 || F->wall[q].face == 6)) {
            seterr(err, errlen, "Baldwin-Lomax with k-face walls is not supported");
            orc_close(s);
            return NULL;
        }
    if (s->ng == 2) {
        if (make_coarse(s)) { seterr(err, errlen, "out of memory"); orc_close(s); return NULL; }
        s->L[2].id = 2;
    }
    /* source/UserInput.cpp:1070-1092 */
    s->Temp_ref = s->Ttin;
    s->Press_ref = s->Ptin;
    s->Vel_ref = sqrt(s->Gamma * s->Rgas * s->Temp_ref);
    s->mue_ref = 1.716e-5f * pow(s->Temp_ref / 288.15f, 3.0f / 2.0f) * (288.15f + 110.4f) / (s->Temp_ref + 110.4f);
    s->dens_ref = s->Press_ref / s->Rgas / s->Temp_ref;
    s->Re_ref = s->dens_ref * s->Vel_ref * s->Len_ref / s->mue_ref;
    s->Ma_ref = 1.0f;
    s->Pout = s->Pout / (s->dens_ref * s->Vel_ref * s->Vel_ref);
    s->Ttin = 1.0f;
    s->Ptin = 1.0f / s->Gamma;
    s->Rgas = 1.0f / (s->Ma_ref * s->Ma_ref * s->Gamma);
    for (int l = 1; l <= s->ng; l++) s->L[l].w_rot = s->L[l].w_rot / (s->Vel_ref / s->Len_ref);
    for (int l = 1; l <= s->ng; l++) { face_vector_volume(&s->L[l]); jacobi_convert(&s->L[l]); }
    initial_uniform(s, &s->L[s->ng == 1 ? 1 : 2]);
    return s;
}

void orc_close(orc_solver *s)
{
    if (!s) return;
    for (int l = 0; l < 3; l++) {
        if (s->L[l].x) free_level(&s->L[l]);
        else { free(s->L[l].in); free(s->L[l].out); free(s->L[l].wall); free(s->L[l].per); }
    }
    free(s);
}

int orc_iterate(orc_solver *s, double row[12])
{
    s->iter++;
    solver_step(s);
    level_t *M = &s->L[1];
    if (s->ng != 1 && s->iter <= s->coarse_iter) M = &s->L[2];
    integrals(s, M);
    if (row) {
        row[0] = s->iter;
        for (int c = 0; c < NQ; c++) row[1 + c] = s->res[c];
        row[6] = s->m_in; row[7] = s->m_out; row[8] = s->pr; row[9] = s->eff; row[10] = s->m_ratio; row[11] = s->CFL;
    }
    return (s->res[0] <= s->convtol) && (s->m_ratio <= 0.003);
}

void orc_resflux(orc_solver *s, int level) { resflux(s, &s->L[level]); }

void orc_dims(const orc_solver *s, int level, int out[4])
{
    out[0] = s->L[level].IM; out[1] = s->L[level].JM; out[2] = s->L[level].KM; out[3] = s->ng;
}
double orc_cfl(const orc_solver *s) { return s->CFL; }
int orc_iter(const orc_solver *s) { return s->iter; }

/* copy a box [i0,i1]x[j0,j1]x[k0,k1] of nc component arrays */
static long box(const level_t *L, REAL *const *arr, int nc, int i0, int i1, int j0, int j1, int k0, int k1, double *out, long cap)
{
    long n = (long)(i1 - i0 + 1) * (j1 - j0 + 1) * (k1 - k0 + 1) * nc;
    if (n > cap) return -1;
    long q = 0;
    for (int i = i0; i <= i1; i++)
        for (int j = j0; j <= j1; j++)
            for (int k = k0; k <= k1; k++) {
                size_t p = IX(L, i, j, k);
                for (int c = 0; c < nc; c++) out[q++] = arr[c][p];
            }
    return n;
}

long orc_get(const orc_solver *s, int level, const char *name, double *out, long cap)
{
    const level_t *L = &s->L[level];
    int IM = L->IM, JM = L->JM, KM = L->KM;
    REAL *tmp[18];
    if (!strcmp(name, "cv")) return box(L, L->cv, 5, 0, IM, 0, JM, 0, KM, out, cap);
    if (!strcmp(name, "pv")) return box(L, L->pv, 6, 0, IM, 0, JM, 0, KM, out, cap);
    if (!strcmp(name, "mut")) { tmp[0] = L->mut; return box(L, tmp, 1, 0, IM, 0, JM, 0, KM, out, cap); }
    if (!strcmp(name, "res")) return box(L, L->res, 5, 1, IM - 1, 1, JM - 1, 1, KM - 1, out, cap);
    if (!strcmp(name, "Fc")) return box(L, L->Fc, 5, 1, IM - 1, 1, JM - 1, 1, KM - 1, out, cap);
    if (!strcmp(name, "Fv")) return box(L, L->Fv, 5, 1, IM - 1, 1, JM - 1, 1, KM - 1, out, cap);
    if (!strcmp(name, "dt")) { tmp[0] = L->dt; return box(L, tmp, 1, 1, IM - 1, 1, JM - 1, 1, KM - 1, out, cap); }
    if (!strcmp(name, "omega")) { tmp[0] = L->omega; return box(L, tmp, 1, 1, IM - 1, 1, JM - 1, 1, KM - 1, out, cap); }
    const char *lam[6] = {"lamcI", "lamcJ", "lamcK", "lamvI", "lamvJ", "lamvK"};
    for (int q = 0; q < 6; q++)
        if (!strcmp(name, lam[q])) { tmp[0] = q < 3 ? L->lamc[q] : L->lamv[q - 3]; return box(L, tmp, 1, 1, IM - 1, 1, JM - 1, 1, KM - 1, out, cap); }
    const char *fcn[3] = {"FcI", "FcJ", "FcK"}, *fvn[3] = {"FvI", "FvJ", "FvK"}, *gn[3] = {"faceI", "faceJ", "faceK"};
    for (int f = 0; f < 3; f++) {
        int i1 = f == 0 ? IM : IM - 1, j1 = f == 1 ? JM : JM - 1, k1 = f == 2 ? KM : KM - 1;
        if (!strcmp(name, fcn[f])) return box(L, L->Ff[f], 5, 1, i1, 1, j1, 1, k1, out, cap);
        if (!strcmp(name, fvn[f])) return box(L, L->Vf[f], 5, 1, i1, 1, j1, 1, k1, out, cap);
        if (!strcmp(name, gn[f])) {
            tmp[0] = L->fS[f][0]; tmp[1] = L->fS[f][1]; tmp[2] = L->fS[f][2]; tmp[3] = L->fs[f];
            tmp[4] = L->fc[f][0]; tmp[5] = L->fc[f][1]; tmp[6] = L->fc[f][2]; tmp[7] = L->fr[f]; tmp[8] = L->fth[f];
            for (int c = 0; c < 9; c++) tmp[9 + c] = L->fm[f][c];
            return box(L, tmp, 18, 1, i1, 1, j1, 1, k1, out, cap);
        }
    }
    if (!strcmp(name, "cell")) {
        tmp[0] = L->vol; tmp[1] = L->cc[0]; tmp[2] = L->cc[1]; tmp[3] = L->cc[2];
        for (int c = 0; c < 9; c++) tmp[4 + c] = L->cm[c];
        return box(L, tmp, 13, 1, IM - 1, 1, JM - 1, 1, KM - 1, out, cap);
    }
    if (!strcmp(name, "totalvol")) { if (cap < 1) return -1; out[0] = L->totalvol; return 1; }
    /* reconstruction layers: [layer 1..2] along the face normal */
    const char *dn[6] = {"dIS", "dIP", "dJS", "dJP", "dKS", "dKP"};
    for (int q = 0; q < 6; q++) {
        char nc[16], np[16];
        snprintf(nc, sizeof nc, "%s_cv", dn[q]); snprintf(np, sizeof np, "%s_pv", dn[q]);
        int is_cv = !strcmp(name, nc), is_pv = !strcmp(name, np);
        if (!is_cv && !is_pv) continue;
        int dir = q / 2, hi = q % 2, nc_ = is_cv ? 5 : 6;
        REAL *const *arr = is_cv ? L->cv : L->pv;
        int N = dir == 0 ? IM : (dir == 1 ? JM : KM);
        int ext[3][2] = {{1, IM - 1}, {1, JM - 1}, {1, KM - 1}};
        long n = 2L * nc_;
        for (int d = 0; d < 3; d++) if (d != dir) n *= (ext[d][1] - ext[d][0] + 1);
        if (n > cap) return -1;
        long o = 0;
        int r0[3], r1[3];
        for (int d = 0; d < 3; d++) { r0[d] = ext[d][0]; r1[d] = ext[d][1]; }
        r0[dir] = 1; r1[dir] = 2;
        for (int a = r0[0]; a <= r1[0]; a++)
            for (int b = r0[1]; b <= r1[1]; b++)
                for (int c = r0[2]; c <= r1[2]; c++) {
                    int ii[3] = {a, b, c};
                    int nd = ii[dir];
                    ii[dir] = hi ? N + nd : -nd;
                    size_t p = IX(L, ii[0], ii[1], ii[2]);
                    for (int cc = 0; cc < nc_; cc++) out[o++] = arr[cc][p];
                }
        return n;
    }
    return -1;
}

int orc_set_cv(orc_solver *s, int level, const double *cv, long n)
{
    level_t *L = &s->L[level];
    long need = (long)(L->IM - 1) * (L->JM - 1) * (L->KM - 1) * 5;
    if (n != need) return -1;
    long q = 0;
    for (int i = 1; i <= L->IM - 1; i++)
        for (int j = 1; j <= L->JM - 1; j++)
            for (int k = 1; k <= L->KM - 1; k++)
                for (int c = 0; c < NQ; c++) L->cv[c][IX(L, i, j, k)] = cv[q++];
    primitive_vars(s, L);
    return 0;
}
