// Host-side readers and writers of the reference's solution files (restart_io.cpp).
#pragma once
#include <string>
#include <vector>

namespace gbt {

// nondimensional-to-dimensional scales of the Tecplot writer
struct SolutionScales {
    double gamma, rgas;                   // nondimensional gas constants as the solver uses them
    double len_ref, dens_ref, vel_ref, temp_ref, mue_ref, re_ref;
};

// one block's fine-level state: pv (IM+1, JM+1, KM+1, 6) rho u v w p T over cells 0..IM;
// cv (IM+1, JM+1, KM+1, 5); mut (IM+1, JM+1, KM+1); x, y, z nodes, i innermost
struct BlockField {
    int IM, JM, KM;
    const double *pv = nullptr, *cv = nullptr, *mut = nullptr;
    const double *ev = nullptr;           // Spalart-Allmaras variable (IM+1, JM+1, KM+1), or null
    const double *x = nullptr, *y = nullptr, *z = nullptr;
    double w_rot = 0, delta_th = 0;       // nondimensional rotation speed, pitch angle of the copy zone
};

// the blocks of one case, in block order
void write_restart_file(const std::string &path, const std::vector<BlockField> &blocks);
// per block b: cv[b] (IM-1, JM-1, KM-1, 5), pv[b] (IM-1, JM-1, KM-1, 6) of the interior, i outermost;
// with_ev: lines carry the Spalart-Allmaras variable as a twelfth value, returned in ev[b]
void read_restart_file(const std::string &path, const std::vector<BlockField> &blocks, std::vector<std::vector<double>> &cv,
                       std::vector<std::vector<double>> &pv, bool with_ev = false, std::vector<std::vector<double>> *ev = nullptr);
void write_solution_file(const std::string &path, const std::vector<BlockField> &blocks, const SolutionScales &sc);

}  // namespace gbt
