// Reader for the reference solver's case files: config.dat (positional option list),
// BoundaryDefinition.dat (patch list) and the text grid file. Host side of the drop-in boundary:
// the GPU solver is configured from exactly the files the reference reads.
#pragma once
#include <string>
#include <vector>
#include <stdexcept>

namespace gbt {

struct PatchIO {               // inlet / outlet (block: 1-based block of the case)
    int face, is, ie, js, je, ks, ke;
    int block = 1;
};
struct WallIO {
    int face, rotate, is, ie, js, je, ks, ke;
    int block = 1;
};
// periodic pair or block interface: side 1 (block b1, face type f1, node range r1) and side 2
struct PeriodicIO {
    int orient, f1, r1[6], f2, r2[6];
    int b1 = 1, b2 = 1;
};

// Everything the reference reads before its first iteration, with scalar options already
// rounded the way the reference parses them (std::stof -> float, then widened).
struct CaseSpec {
    std::string dir, grid_file, bc_file;
    // options (source/UserInput.cpp:17-239)
    bool turbo_axial = true, equation_ns = true, uniform_init = true;
    double Rgas = 0, Gamma = 0, Pr_lam = 0, Pr_tur = 0;
    double Ptin = 0, Ttin = 0, Pout = 0, P21 = 0, Ma0 = 0, Len_ref = 0, ev_ratio = 0;
    double inlet_dir[3] = {0, 0, 1};
    bool mass_imposed = false;
    double m_imposed = 0.0, relax_press = 0.0, resc_mass_imp = 0.0;   // imposed mass flow [kg/s], relaxation, residual gate
    int iter_mass_imp = 1;                                            // iterations between back-pressure updates
    int maxiter = 0, coarse_iter = 0, outstep = 0, nt = 1;
    double convtol = 0;
    bool use_mg = false, restart = false;
    double CFL = 0, C_timestep = 0, relax = 0, epsEntr = 0, k2 = 0, k4 = 0;
    bool irs = false, limiter = false, global_dt = false;
    int recon_var = 200, recon = 500, scheme = 300, time_scheme = 500, turb = 100;
    // boundary definition (source/UserInput.cpp:336-446). A case of several blocks is held as one
    // spec per block: inlets, outlets and walls are those of this block, in file order; periodic
    // pairs and block interfaces (which join two blocks) are the case's full lists, in file order
    std::vector<PatchIO> inlets, outlets;
    std::vector<WallIO> walls;
    std::vector<PeriodicIO> periodics, interiors, mixing;     // mixing: mixing planes (same line format)
    PatchIO first_inlet{}, first_outlet{};       // the case's Inlet[1] and Outlet[1] (the reported sections)
    int nblade = 1;
    double rpm = 0;
    int ng = 1;                                  // levels chosen as the reference does (<= 2)
    int block = 1, nblock = 1;                   // this spec's block and the case's block count
    // grid of this block
    int IM = 0, JM = 0, KM = 0;
    std::vector<double> x, y, z;                 // node coordinates, index ((k-1)*JM + (j-1))*IM + (i-1)
};

// Reads a case directory into one spec per block (block order of the files); throws
// std::runtime_error with a message naming the problem. `threads` host threads parse the node
// lines of large grids.
std::vector<CaseSpec> read_case(const std::string &dir, int threads = 1);

// One line of a reference input file: comment from '#' removed, leading and trailing blanks
// removed (tabs are kept, as the reference keeps them); a trailing carriage return is dropped.
std::string ref_read_line(std::FILE *f, bool *ok);

}  // namespace gbt
