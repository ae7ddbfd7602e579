/* gbturbo: C-ABI of the GB300 residual-and-update path of the structured-grid turbomachinery
 * RANS solver (wuchuankang/3D-fluid-numerical-simulation-software).
 *
 * A handle owns one batch of operating points ("solves") on the current CUDA device; each solve
 * is configured from the reference's own case files (config.dat, BoundaryDefinition.dat and the
 * grid file named in config.dat) and all solves of a batch share the numerical options. A solve
 * may have several blocks joined by interfaces (source/BndCondInteriorPeriodic.cpp:8-34); every
 * block has its own slot in the handle, the blocks of solve 0 first, then those of solve 1, and
 * so on (gb_case_blocks). Calls that report per solve (norms, integrals, history, status, back
 * pressure, solution files) take or fill one entry per solve; calls that address one box (dims,
 * field access) take a slot, which equals the solve index when every solve has one block. The
 * entry points replace the reference's C++ member-function surface one for one (file:line of the
 * reference in each comment). All calls are asynchronous on the handle's stream unless they
 * return data to host buffers; all return 0 on success and a negative code on failure, with
 * the message available from gb_last_error(). The device owns all state; the caller passes
 * host buffers only.
 */
#ifndef GBTURBO_H
#define GBTURBO_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct gb_solver gb_solver;

#define GB_PRECISION_FP64 0   /* every field FP64: parity with the reference's FP64 build */
#define GB_PRECISION_MIXED 1  /* fluxes, residuals, sweeps, transfers FP32; Q, geometry, norms, integrals FP64 */

#define GB_OK 0
#define GB_ERR_ARG -1
#define GB_ERR_CASE -2
#define GB_ERR_CUDA -3

/* Reads n case directories and builds the batch: input reading of source/Structured_FV3D.cpp:36-56
 * (CUserInput::ReadConfig, NumberOfMultigrid, ReadGrids, ReadBndGrid, NonDimensionalization),
 * memory and geometry of :59-69 (CMesh::AllocateMemory, CMesh::Geometry). */
int gb_solver_create(const char *const *case_dirs, int n_solves, int precision, gb_solver **out);
/* gb_solver_create with the number of grid levels of multigrid cases: 2 follows the reference
 * (at most two levels, source/UserInput.cpp:1062); 3 selects the three-level V-cycle extension
 * (no counterpart in the reference): the fine step as in the two-level cycle, then FAS smoothing
 * on levels 2 and 3 with their residuals evaluated at the restricted states. Three levels need
 * node counts N with (N-1) a multiple of 4 and (N-1)/4 > 2 and patch ranges that stay odd-aligned
 * on the second level. */
int gb_solver_create_levels(const char *const *case_dirs, int n_solves, int precision, int max_levels, gb_solver **out);
int gb_solver_destroy(gb_solver *h);
/* message of the last failure on the calling thread */
const char *gb_last_error(void);

/* out[0..3] = IM, JM, KM (node counts) of a level of one slot (block), and the number of levels */
int gb_dims(gb_solver *h, int solve, int level, int out[4]);
/* number of solves (case directories) and of slots (blocks of all solves); either may be NULL */
int gb_num_blocks(gb_solver *h, int *n_cases, int *n_blocks);
/* out[0] = first slot of a solve, out[1] = its number of blocks (CMesh::NB) */
int gb_case_blocks(gb_solver *h, int solve, int out[2]);

/* CMesh::Initial, uniform start (source/Initialization.cpp:17-76) on the coarsest used level */
int gb_init_uniform(gb_solver *h);
/* CMesh::ResFlux (source/ComputeAllBlockVars.cpp:223-255): boundary fill, spectral radii, curl,
 * Baldwin-Lomax (fine level), time step, convective + wall + viscous flux, residual */
int gb_resflux(gb_solver *h, int level);
/* CMesh::Time_Marching -> LU_SGS_Marching (source/LU_SGS_Marching.cpp:10-291) */
int gb_time_marching(gb_solver *h, int level);
/* CMesh::Res_Calculate (source/ComputeAllBlockVars.cpp:318-372); out[5*n_solves] may be NULL */
int gb_res_calculate(gb_solver *h, int level, double *out);
/* CMesh::PrimitiveVars (source/PrimitiveVars.cpp:7-28) */
int gb_primitive_vars(gb_solver *h, int level);
/* CMesh::Limit_Vars (source/Limit_FlowVars.cpp:8-118) */
int gb_limit_vars(gb_solver *h, int level);
/* CMesh::CornerTreatment (source/ComputeAllBlockVars.cpp:374-438) */
int gb_corner_treatment(gb_solver *h, int level);
/* CSolver::Prolong: restriction fine -> coarse (source/Prolong_Interpolate.cpp:7-50) */
int gb_restrict(gb_solver *h);
/* CSolver::Interpolate: prolongation coarse -> fine (source/Prolong_Interpolate.cpp:52-156);
 * init = 1 interpolates Q itself (first fine-level iteration), 0 adds the coarse correction */
int gb_interpolate(gb_solver *h, int init);
/* CSolver::ComputeDeltConsVars (source/Prolong_Interpolate.cpp:159-176) */
int gb_delta_cons(gb_solver *h);
/* CMesh::UseForceFunction of a level (source/Solver.cpp:98) */
int gb_set_use_force(gb_solver *h, int level, int on);
/* CSolver::Solver (source/Solver.cpp:47-140): one iteration of the driver, CFL ramp included */
int gb_solver_step(gb_solver *h);
/* COutput::OutputGeneralParameters (source/Ouput.cpp:282-300) on a level; out[5*n_solves] =
 * mass flow in, mass flow out, total-pressure ratio, isentropic efficiency, |m_in - m_out|/m_in */
int gb_integrals(gb_solver *h, int level, double *out);
/* n iterations of the reference driver loop (source/Structured_FV3D.cpp:142-219: Solver() and
 * the integrals), replayed as CUDA graphs. hist (may be NULL) receives n * n_solves rows of 12:
 * iter, Res(dens,xmom,ymom,zmom,ener), m_in, m_out, PR, eta, m_ratio, CFL. */
int gb_iterate(gb_solver *h, int n, double *hist);
/* per-solve status words (bit 1: non-finite residual or integral, bit 2: limiter active in the
 * last step, bit 4: limiter list overflow); out[n_solves] */
int gb_get_status(gb_solver *h, int *out);

/* Copies a named array of one slot (block) and level to out (row-major, components fastest):
 * "cv" (IM+1,JM+1,KM+1,5) and "pv" (..,6), "mut" (..,1) including ghosts; "res","dq" and
 * "dt","omega","lamcI".."lamvK" over the cells; "FcI","FvI" (IM,JM-1,KM-1,5) and J, K;
 * "faceI" (IM,JM-1,KM-1,18), "faceJ", "faceK", "cell" (IM-1,JM-1,KM-1,13), "totalvol" (of the
 * slot's whole solve, CMesh::TotalVol);
 * "dIS_cv".."dKP_pv" reconstruction layers. Returns the count written (>= 0) or < 0. */
long gb_get_field(gb_solver *h, int solve, int level, const char *name, double *out, long cap);
/* overwrites the interior conserved variables (IM-1,JM-1,KM-1,5) and the primitive variables */
int gb_set_cv(gb_solver *h, int solve, int level, const double *cv, long n);

/* The reference's solution files for one solve, all its blocks in block order (fine level). A
 * NULL path means the file of that name in the solve's case directory.
 * gb_read_restart: CUserInput::ReadSolution (source/UserInput.cpp:1118-1159): reads
 *   RestartSolution.dat and sets Q and the primitive variables as read; it takes the place of
 *   gb_init_uniform for cases whose config asks for the previous solution, for which the driver
 *   runs full multigrid cycles from the first iteration (source/Solver.cpp:113-138).
 * gb_write_restart: COutput::OutputRestartSolution (source/Ouput.cpp:227-259).
 * gb_write_solution: COutput::OutputSolution (source/Ouput.cpp:109-225), RelativeSolution.plt. */
int gb_read_restart(gb_solver *h, int solve, const char *path);
int gb_write_restart(gb_solver *h, int solve, const char *path);
int gb_write_solution(gb_solver *h, int solve, const char *path);

/* Imposed mass flow (config "use flow mass outlet" and its line of imposed mass flow, relaxation,
 * iteration step and residual gate): CSolver::MassFlowImposed with the driver's conditions
 * (source/Solver.cpp:142-145, source/Structured_FV3D.cpp:186-193). gb_iterate applies it after
 * every iteration's integrals; gb_mass_flow_imposed applies it once, for callers that drive
 * gb_solver_step and gb_integrals themselves. gb_get_outlet_pressure: the current
 * nondimensional back pressure of every solve (CBndConds::Pout). */
int gb_mass_flow_imposed(gb_solver *h);
int gb_get_outlet_pressure(gb_solver *h, double *out);

/* waits for the handle's stream */
int gb_sync(gb_solver *h);
/* block shape of the LU-SGS sweep kernels on a level: out[0] cells per warp, out[1] warps per
 * block, chosen at create by timing the plane chains of each candidate shape; the choice changes
 * timing only, not results */
int gb_sweep_tuning(gb_solver *h, int level, int out[2]);
/* whether a level's face stage runs on tiles of faces staged in shared memory by the tensor memory
 * accelerator (*tma = 1; the mixed form's default scheme on meshes whose k extent KM is 4n + 1 and
 * at least 33) or reads its stencils straight from HBM (*tma = 0); the choice changes timing only,
 * the arithmetic is the same. The staged form is chosen at create by the environment variable
 * GBTURBO_FACE_TMA (1: the cell fields staged, the per-face geometry streamed; 2: both staged;
 * unset or 0: the plain kernel). No counterpart in the reference. */
int gb_face_staging(gb_solver *h, int level, int *tma);
/* 0 disables graph replay in gb_iterate (eager launches) */
int gb_set_graphs(gb_solver *h, int enable);
/* stage profiler: between the two calls iterations run without graphs and every stage of the
 * path is bracketed by CUDA events on the handle's stream; gb_profile_end writes
 * "stage:milliseconds:kernel launches:evaluations on level 1,2,3;..." totals into buf (an
 * evaluation is one bracketed group of the stage's launches, e.g. the three face families of one
 * residual, or one sweep over every plane of a level) */
int gb_profile_begin(gb_solver *h);
int gb_profile_end(gb_solver *h, char *buf, int buflen);
/* device time of everything enqueued between the two calls, in milliseconds (events on the
 * handle's stream) */
int gb_timer_start(gb_solver *h);
int gb_timer_stop(gb_solver *h, float *ms);
/* FP64 arithmetic rate of the current device in FLOP/s (two per FMA), from a device-timed loop of
 * independent FMA chains over every SM (best of five launches, about 0.1 s). No counterpart in the
 * reference: it is the roof against which the FP64 form's face-flux and sweep kernels are
 * reported, since on this GPU they are bound by the FP64 pipe rather than by HBM. */
int gb_fp64_rate(double *flop_per_s);
/* The FP64 form's Newton-refined reciprocal, quotient and square root (which replace the IEEE
 * division and root in its compute-bound kernels) evaluated on the device for n inputs, so that
 * they can be checked against the IEEE operations: op 0 x / y, 1 sqrt(x), 2 1 / x; op 3 and 4 are
 * the device's IEEE x / y and sqrt(x). Also the mixed form's integer operations: op 5 splits x into
 * a pair of FP32 numbers (returned as their FP64 sum), op 6 rounds x to FP32 and widens it back by
 * integer operations, op 7 does the same by the conversion instructions. x, y (y only for ops 0
 * and 3) and out are host arrays. No counterpart in the reference. */
int gb_fp64_arith_check(int op, const double *x, const double *y, long long n, double *out);

/* Residual norm of gb_res_calculate (same arguments, same values in out and in the solve states)
 * computed with no allocation on success: its scratch is a static device array of fixed size
 * inside the library. It has no counterpart in the reference; it exists for callers that may not
 * allocate between iterations (a convergence monitor of a batch whose device memory is committed
 * to the solve pools, a host thread under a no-heap rule). Batches of more than
 * GB_NOALLOC_MAX_SOLVES slots (blocks of all solves) are rejected with GB_ERR_ARG. All calls on a device share the one
 * array, so calls that overlap in time race and must be serialised by the caller. The first call
 * on a device looks the array up and zeroes it: make that call before any stream capture begins.
 * The looked-up address is kept for the life of the process, so do not call it again after a
 * cudaDeviceReset of that device.
 * Call it with the handle's device current. */
#define GB_NOALLOC_MAX_SOLVES 128
int gb_res_calculate_noalloc(gb_solver *h, int level, double *out);

/* Reads one case directory on the host only (no device, no handle): the reader of
 * gb_solver_create with its checks. info[0..8] = blocks, grid levels, inlets, outlets, walls,
 * periodic pairs, block interfaces, mixing planes, nodes of all blocks; nodes_out (may be NULL)
 * receives x, y, z of every node, block after block, i fastest (3 * info[8] doubles, cap the
 * buffer's length). It has no counterpart in the reference; it lets a caller (and the CPU tests)
 * check a case without a GPU. */
int gb_case_info(const char *case_dir, long long info[9], double *nodes_out, long long cap);

/* ---- Learned warm start. No counterpart in the reference: its solves start from the uniform
 * inlet state of CBlocks::Initialization (source/Initialization.cpp:34-68), which stays the
 * fallback here. A coordinate MLP (64 Fourier / parameter features, five hidden layers of 256
 * with SiLU, 16 outputs of which the first six are rho, rho u, rho v, rho w, rho E, mu_t,
 * normalised) is trained on fine-level fields of solves this library ran, in BF16 with FP32
 * accumulation on the tensor cores (tcgen05), and gives new cases their starting field.
 * Case parameters: GB_WS_PARAMS floats per case (the caller's operating-point descriptors, e.g.
 * back-pressure ratio, rotation-speed ratio, stagger offset), normalised by the training set.
 * gb_ws_add_solves: appends every fine interior cell of every case of h (its current state).
 * gb_ws_train: Adam steps on random minibatches of `batch` samples; *loss = mean loss of the last
 *   (up to) 20 steps. The first call fixes the normalisation from the training set.
 * gb_ws_apply: before the first iteration of h: evaluates the network on every fine cell, keeps
 *   it for a case when the case's sum of |R_rho| over its cells (one residual evaluation) is below
 *   the uniform start's (used[case] = 1), else puts the uniform start back (used = 0); the
 *   following iterations run full cycles from the fine field, as a restarted case does; when no
 *   case keeps the network's field, the plain start-up of gb_init_uniform runs. res_warm and
 *   res_uniform (may be NULL) receive the two residual sums per case.
 * gb_ws_get/set_params: the flat FP32 parameters, layer after layer the weights [N][K] (row-major)
 *   and the biases [N]; gb_ws_num_params() values. gb_ws_get/set_norm: GB_WS_NORM constants
 *   (coordinate min[3], max[3] of axial position, radius, pitch angle; parameter mean[3], std[3];
 *   target mean[6], std[6]).
 * gb_ws_forward / gb_ws_forward_backward: the network on given features (n x 64, FP32, rounded to
 *   BF16 on upload): outputs (n x 16); with targets (n x 6, normalised) the mean-squared loss and
 *   the gradient of every parameter (the layout of gb_ws_get_params). */
/* After gb_init_uniform and gb_set_cv of the fine level (level 1) of every slot, before the first
 * iteration: the iterations run full multigrid cycles from that fine field, as a restarted case
 * does, with the coarse levels' time steps and spectral radii evaluated once at the fine field
 * restricted to them. No counterpart in the reference (its start-up always begins on the coarse
 * level unless the config asks for the previous solution); gb_ws_apply uses it. */
int gb_start_from_fine_state(gb_solver *h);

#define GB_WS_PARAMS 3
#define GB_WS_NORM 24
typedef struct gb_warmstart gb_warmstart;
int gb_ws_create(unsigned seed, gb_warmstart **out);
int gb_ws_destroy(gb_warmstart *w);
long gb_ws_num_params(void);
int gb_ws_add_solves(gb_warmstart *w, gb_solver *h, const float *params);
long long gb_ws_samples(gb_warmstart *w);
int gb_ws_train(gb_warmstart *w, int steps, int batch, float lr, float *loss);
int gb_ws_apply(gb_warmstart *w, gb_solver *h, const float *params, int *used, double *res_warm, double *res_uniform);
int gb_ws_get_params(gb_warmstart *w, float *out);
int gb_ws_set_params(gb_warmstart *w, const float *in);
int gb_ws_get_norm(gb_warmstart *w, float *out);
int gb_ws_set_norm(gb_warmstart *w, const float *in);
int gb_ws_forward(gb_warmstart *w, const float *feat, int n, float *y);
int gb_ws_forward_backward(gb_warmstart *w, const float *feat, const float *target, int n, float *loss, float *grad);
/* device time per layer-by-layer forward pass, per forward-and-backward pass (loss and every
 * gradient) and per fused inference pass (every layer in one kernel, the activations kept on
 * chip; gb_ws_forward and gb_ws_apply use it) over n rows of device-resident random inputs, mean
 * of iters after one warm-up (CUDA events); max_diff (may be NULL) receives the largest difference
 * between the fused and the layer-by-layer outputs on those rows (the same arithmetic: 0) */
int gb_ws_benchmark(gb_warmstart *w, long long n, int iters, float *ms_forward, float *ms_step, float *ms_infer,
                    double *max_diff);

#ifdef __cplusplus
}
#endif
#endif
