// Host orchestration of a batch of operating points ("solves", one case directory each) on one GPU.
// Every block of every case has its own box ("slot"): the blocks of case 0 come first, then those
// of case 1, and so on; a single-block case has one slot, and then slot and case index agree. The class keeps the
// reference's call surface (CSolver::Solver, CMesh::ResFlux / Time_Marching / Res_Calculate /
// PrimitiveVars / Limit_Vars / CornerTreatment, CSolver::Prolong / Interpolate /
// ComputeDeltConsVars, COutput::OutputGeneralParameters) as methods that enqueue kernels on the
// handle's stream; the C-ABI in capi.cu forwards to them.
#pragma once
#include <memory>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "case_io.hpp"
#include "kernels.hpp"

namespace gbt {

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    ~DevBuf() { if (p) cudaFree(p); }
};

// Fine-level arrays of a batch as the warm start reads and writes them (device pointers into the
// level's pools, box layout of gbt_common.cuh)
struct FineView {
    int nslot = 0;
    std::vector<Lvl> lv;                         // per slot
    const Lvl *lv_dev = nullptr;
    double *cv[NQ] = {};
    const double *cc[3] = {};                    // cell centres
    const void *mut = nullptr;                   // eddy viscosity, in the working type
    bool fp32 = false;                           // working type float (mixed form)
};

class SolverBase {
public:
    virtual ~SolverBase() = default;
    int nsolve = 0, ng = 1, coarse_iter = 0, iter = 0, precision = 0;   // nsolve: slots (blocks of all cases)
    int ncase = 0;
    std::vector<int> case_first, case_nblk;      // per case: its first slot and its number of blocks
    std::vector<CaseSpec> cases;                 // per slot: the options, patches and grid of that block
    Phys P{};
    cudaStream_t stream = nullptr;
    bool use_graphs = true;

    virtual void init_uniform() = 0;
    virtual void resflux(int level) = 0;
    virtual void time_marching(int level) = 0;
    virtual void res_calculate(int level) = 0;
    // res_calculate with static scratch and no allocation; norms to host_out (5 per case) if given
    virtual void res_calculate_static(int level, double *host_out) = 0;
    virtual void primitive_vars(int level) = 0;
    virtual void limit_vars(int level) = 0;
    virtual void corner_treatment(int level) = 0;
    virtual void restrict_to_coarse() = 0;
    virtual void interpolate(int init) = 0;
    virtual void delta_cons() = 0;
    virtual void integrals(int level) = 0;
    virtual void solver_step() = 0;
    // one back-pressure update of the cases that impose their mass flow (after the integrals)
    virtual void mass_flow_imposed() = 0;
    // current nondimensional back pressure of every case
    virtual void outlet_pressure(double *out) = 0;
    // n driver iterations; hist (if not null) receives n * ncase rows of 12 values
    virtual void iterate(int n, double *hist) = 0;
    // box dimensions and field access address a slot (one block of one case)
    virtual void dims(int slot, int level, int out[4]) const = 0;
    virtual long get_field(int slot, int level, const std::string &name, double *out, long cap) = 0;
    virtual void set_cv(int slot, int level, const double *in, long n) = 0;
    // the reference's solution files for one case, all its blocks (fine level): RestartSolution.dat
    // in and out, RelativeSolution.plt out; an empty path means the file of that name in the case
    // directory
    virtual void read_restart(int solve, const std::string &path) = 0;
    virtual void write_restart(int solve, const std::string &path) = 0;
    virtual void write_solution(int solve, const std::string &path) = 0;
    // per case: the state of its first slot, with the status bits of all its blocks combined and
    // their limiter hits summed
    virtual void states(SolveState *out) = 0;
    virtual void set_use_force(int level, bool on) = 0;
    // block shape the sweep autotuner chose for a level: cells per warp, warps per block
    virtual void sweep_shape(int level, int out[2]) const = 0;
    // whether a level's face stage runs on tiles staged in shared memory by TMA (mixed form)
    virtual bool face_staged(int level) const = 0;
    // stage profiler: while on, iterations run eagerly and every stage is bracketed by events
    virtual void profile_begin() = 0;
    // "stage:milliseconds:launches;..." totals since profile_begin
    virtual std::string profile_end() = 0;

    // start from a given fine-level field (the warm start): the arrays it writes, the uniform
    // inlet state of init_uniform on the fine level's interior cells of the listed slots (every
    // slot for an empty list), the primitive variables from Q, per case the sum over its cells of
    // |R_rho| after one residual evaluation of the fine level, and the switch that makes the
    // following iterations run full cycles from the fine state (as a restarted case does)
    virtual FineView fine_view() = 0;
    virtual void fill_uniform_fine(const std::vector<int> &slots) = 0;
    virtual void fine_primitive() = 0;
    virtual void fine_residual(std::vector<double> &per_case) = 0;
    virtual void start_from_fine_state() = 0;
    // a device copy of the fine level's flow arrays and of the solve states, put back (or dropped)
    // after residual evaluations that must leave no trace
    virtual void save_fine_state() = 0;
    virtual void restore_fine_state(bool put_back) = 0;
};

// max_levels: 2 follows the reference (at most two grid levels); 3 enables the three-level
// V-cycle extension for multigrid cases whose grids coarsen twice
std::unique_ptr<SolverBase> make_solver(const std::vector<std::string> &dirs, int precision, int max_levels = 2);

// nondimensional constants exactly as the reference derives them (source/UserInput.cpp:1070-1092)
struct NonDim {
    double vel_ref, dens_ref, temp_ref, mue_ref, re_ref, pout, ptin, ttin, rgas, w_rot, delta_th;
};
NonDim nondimensionalise(const CaseSpec &c);

void check_cuda(cudaError_t e, const char *what);

}  // namespace gbt
