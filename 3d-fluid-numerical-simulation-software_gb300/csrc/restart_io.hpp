// Host-side readers and writers of the reference's solution files (restart_io.cpp).
#pragma once
#include <string>

namespace gbt {

// nondimensional-to-dimensional scales and per-solve frame data of the Tecplot writer
struct SolutionScales {
    double gamma, rgas;                   // nondimensional gas constants as the solver uses them
    double len_ref, dens_ref, vel_ref, temp_ref, mue_ref, re_ref;
    double w_rot, delta_th;               // nondimensional rotation speed, pitch angle of the copy zone
};

// pv: (IM+1, JM+1, KM+1, 6) rho u v w p T over cells 0..IM; cv: (IM+1, JM+1, KM+1, 5)
void write_restart_file(const std::string &path, int IM, int JM, int KM, const double *pv, const double *cv);
// cv: (IM-1, JM-1, KM-1, 5), pv: (IM-1, JM-1, KM-1, 6) of the interior, i outermost
void read_restart_file(const std::string &path, int IM, int JM, int KM, double *cv, double *pv);
// x, y, z: nodes, i innermost; pv, mut: as for write_restart_file (mut one component)
void write_solution_file(const std::string &path, int IM, int JM, int KM, const double *x, const double *y,
                         const double *z, const double *pv, const double *mut, const SolutionScales &sc);

}  // namespace gbt
