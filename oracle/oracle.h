/* CPU oracle for the residual-and-update hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, single-threaded, FP64 restatement of the reference solver's single-block
 * per-iteration path (boundary fill, primitive variables, spectral radii, curl, face
 * gradients, Baldwin-Lomax eddy viscosity, local time step, MUSCL/NND reconstruction,
 * Roe and Steger-Warming fluxes, wall flux, viscous flux, hyperplane LU-SGS, residual norm,
 * inlet/outlet integrals and the two-level multigrid transfer). Every function cites the
 * reference file:line it follows. The arithmetic keeps the reference's evaluation order and
 * float-literal types so that, built with -ffp-contract=off, it reproduces the reference's
 * FP64 build bit for bit; it is pinned against dumps of the reference itself
 * (tests/golden/, made by tests/golden/make_golden.py from oracle/_ref).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this library;
 * the GPU product never links or calls it.
 */
#ifndef GB_ORACLE_H
#define GB_ORACLE_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_solver orc_solver;

/* Reads <dir>/config.dat, the grid file it names and BoundaryDefinition.dat, computes the
 * geometry of every level and applies the uniform start (source/Structured_FV3D.cpp:36-103).
 * Returns NULL and writes a message to err (if given) on failure. */
orc_solver *orc_open(const char *dir, char *err, int errlen);
void orc_close(orc_solver *s);

/* one outer iteration of the reference driver: CSolver::Solver() followed by the integrals
 * (source/Structured_FV3D.cpp:146-157). row[12] = iter, Res(5), m_in, m_out, PR, eta,
 * m_ratio, CFL. Returns 1 when the reference's convergence test is met. */
int orc_iterate(orc_solver *s, double row[12]);

/* one CMesh::ResFlux() on a level (1 = fine) */
void orc_resflux(orc_solver *s, int level);

/* dimensions of a level: out[0..2] = IM, JM, KM; out[3] = NG */
void orc_dims(const orc_solver *s, int level, int out[4]);

/* Copies a named array of a level into out (double), in the layout of the reference dump:
 *   "cv" (IM+1,JM+1,KM+1,5), "pv" (..,6), "mut" (..,1)  -- with ghosts i in [0,IM]
 *   "res","Fc","Fv" (IM-1,JM-1,KM-1,5); "dt","omega","lamcI".."lamvK" (IM-1,JM-1,KM-1,1)
 *   "FcI","FvI" (IM,JM-1,KM-1,5); "FcJ","FvJ" (IM-1,JM,KM-1,5); "FcK","FvK" (IM-1,JM-1,KM,5)
 *   "faceI" (IM,JM-1,KM-1,18), "faceJ", "faceK", "cell" (IM-1,JM-1,KM-1,13)
 *   "dIS_cv","dIP_cv" (2,JM-1,KM-1,5) ... "dKP_pv" (IM-1,JM-1,2,6)
 * Returns the number of doubles written, or -1 for an unknown name / short buffer. */
long orc_get(const orc_solver *s, int level, const char *name, double *out, long cap);

/* Overwrites the interior conserved variables of a level (shape (IM-1,JM-1,KM-1,5)) and
 * recomputes the primitive variables; used to start the oracle from an arbitrary state. */
int orc_set_cv(orc_solver *s, int level, const double *cv, long n);

/* scalar state: CFL, iteration counter, Flag_low_dt of a level */
double orc_cfl(const orc_solver *s);
int orc_iter(const orc_solver *s);

#ifdef __cplusplus
}
#endif
#endif
