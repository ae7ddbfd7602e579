// Test-infrastructure harness around the reference solver's own objects (oracle/_ref).
//
// Linked against the reference sources compiled unmodified from their original location
// (recipe: oracle/build_ref.sh). It replays the initialisation sequence of the reference driver
// (source/Structured_FV3D.cpp:36-103), runs the outer iteration loop exactly as that driver
// does (source/Structured_FV3D.cpp:142-219, minus the console output), and writes the arrays
// the hot path produces as .npy files so that the CPU oracle and the GPU path can be compared
// against the reference itself.
//
//   ref_harness <n_iter> <out_dir> [dump_resflux=1] [write_outputs=0]
//
// run from a directory holding config.dat, BoundaryDefinition.dat and the grid file.
// This file is compiled with -Dprivate=public to read members the reference keeps private.
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include <sys/stat.h>
#include <unistd.h>
#include "Solver.h"
#include "Output.h"
#include "BndConds.h"
#include "UserInput.h"

static std::string g_out;

static void npy_write(const std::string &name, const std::vector<double> &data,
                      const std::vector<size_t> &shape)
{
    std::string path = g_out + "/" + name + ".npy";
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) { perror(path.c_str()); exit(2); }
    std::string dict = "{'descr': '<f8', 'fortran_order': False, 'shape': (";
    for (size_t s : shape) dict += std::to_string(s) + ", ";
    dict += "), }";
    size_t hl = 10 + dict.size() + 1;
    size_t pad = (64 - hl % 64) % 64;
    dict += std::string(pad, ' ') + "\n";
    unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    fwrite(magic, 1, 8, f);
    uint16_t len = (uint16_t)dict.size();
    fwrite(&len, 2, 1, f);
    fwrite(dict.data(), 1, dict.size(), f);
    fwrite(data.data(), sizeof(double), data.size(), f);
    fclose(f);
}

// cell-centred array over i in [0,IM], j in [0,JM], k in [0,KM]
template <class T, class F>
static void dump_cells(const std::string &name, T ***a, int IM, int JM, int KM, int ncomp, F get)
{
    std::vector<double> v;
    v.reserve((size_t)(IM + 1) * (JM + 1) * (KM + 1) * ncomp);
    for (int i = 0; i <= IM; i++)
        for (int j = 0; j <= JM; j++)
            for (int k = 0; k <= KM; k++)
                for (int c = 0; c < ncomp; c++) v.push_back(get(a[i][j][k], c));
    npy_write(name, v, {(size_t)IM + 1, (size_t)JM + 1, (size_t)KM + 1, (size_t)ncomp});
}

template <class T, class F>
static void dump_box(const std::string &name, T ***a, int i0, int i1, int j0, int j1, int k0,
                     int k1, int ncomp, F get)
{
    std::vector<double> v;
    for (int i = i0; i <= i1; i++)
        for (int j = j0; j <= j1; j++)
            for (int k = k0; k <= k1; k++)
                for (int c = 0; c < ncomp; c++) v.push_back(get(a[i][j][k], c));
    npy_write(name, v, {(size_t)(i1 - i0 + 1), (size_t)(j1 - j0 + 1), (size_t)(k1 - k0 + 1),
                        (size_t)ncomp});
}

static double cv_c(const TConsVars &q, int c)
{
    switch (c) { case 0: return q.dens; case 1: return q.xmom; case 2: return q.ymom;
                 case 3: return q.zmom; default: return q.ener; }
}
static double pv_c(const TPrimVars &q, int c)
{
    switch (c) { case 0: return q.dens; case 1: return q.uvel; case 2: return q.vvel;
                 case 3: return q.wvel; case 4: return q.press; default: return q.temp; }
}
static double face_c(const TFace &f, int c)
{
    switch (c) {
    case 0: return f.S.x; case 1: return f.S.y; case 2: return f.S.z; case 3: return f.s;
    case 4: return f.coord.x; case 5: return f.coord.y; case 6: return f.coord.z;
    case 7: return f.r; case 8: return f.th;
    case 9: return f.gradx_kesi; case 10: return f.grady_kesi; case 11: return f.gradz_kesi;
    case 12: return f.gradx_yita; case 13: return f.grady_yita; case 14: return f.gradz_yita;
    case 15: return f.gradx_zita; case 16: return f.grady_zita; default: return f.gradz_zita;
    }
}
static double cell_c(const TCell &f, int c)
{
    switch (c) {
    case 0: return f.Vol; case 1: return f.coord.x; case 2: return f.coord.y;
    case 3: return f.coord.z;
    case 4: return f.gradx_kesi; case 5: return f.grady_kesi; case 6: return f.gradz_kesi;
    case 7: return f.gradx_yita; case 8: return f.grady_yita; case 9: return f.gradz_yita;
    case 10: return f.gradx_zita; case 11: return f.grady_zita; default: return f.gradz_zita;
    }
}

static void dump_geometry(CMesh &M, const std::string &p, int nb = 1)
{
    CGeometry &G = M.Block[nb].Geometry;
    int IM = G.IM, JM = G.JM, KM = G.KM;
    dump_box(p + "faceI", G.FaceI, 1, IM, 1, JM - 1, 1, KM - 1, 18, face_c);
    dump_box(p + "faceJ", G.FaceJ, 1, IM - 1, 1, JM, 1, KM - 1, 18, face_c);
    dump_box(p + "faceK", G.FaceK, 1, IM - 1, 1, JM - 1, 1, KM, 18, face_c);
    dump_box(p + "cell", G.Cell, 1, IM - 1, 1, JM - 1, 1, KM - 1, 13, cell_c);
    if (CFluidProps::turbulenceType == TurbulenceTypes::SA && M.Mesh_ID == 1)
        dump_box(p + "dwall", G.Cell, 1, IM - 1, 1, JM - 1, 1, KM - 1, 1, [](const TCell &c, int) { return (double)c.dis_Wall; });
    npy_write(p + "totalvol", {(double)M.TotalVol}, {1});
}

static void dump_state(CMesh &M, const std::string &p, int nb = 1)
{
    CBlocks &B = M.Block[nb];
    CFluidProps &F = B.FluidProp;
    int IM = B.Geometry.IM, JM = B.Geometry.JM, KM = B.Geometry.KM;
    dump_cells(p + "cv", F.Cell_cv, IM, JM, KM, 5, cv_c);
    dump_cells(p + "pv", F.Cell_pv, IM, JM, KM, 6, pv_c);
    dump_cells(p + "mut", F.Cell_tur, IM, JM, KM, 1,
               [](const TVisVars &v, int) { return (double)v.mue; });
    if (CFluidProps::turbulenceType == TurbulenceTypes::SA)
        dump_cells(p + "ev", F.Cell_ev, IM, JM, KM, 1, [](const TEddyVars &v, int) { return (double)v.ev; });
}

static void dump_resflux(CMesh &M, const std::string &p, int nb = 1)
{
    CBlocks &B = M.Block[nb];
    CFluidProps &F = B.FluidProp;
    CSpaceDiscr &S = B.SpaceDiscr;
    CTimeDiscr &T = B.TimeDiscr;
    int IM = B.Geometry.IM, JM = B.Geometry.JM, KM = B.Geometry.KM;
    dump_state(M, p, nb);
    auto cvg = cv_c;
    auto pvg = pv_c;
    // reconstruction dummies, stored as [layer 1..2] in the direction normal to the face
    dump_box(p + "dIS_cv", F.DummyIS_cv, 1, 2, 1, JM - 1, 1, KM - 1, 5, cvg);
    dump_box(p + "dIP_cv", F.DummyIP_cv, 1, 2, 1, JM - 1, 1, KM - 1, 5, cvg);
    dump_box(p + "dJS_cv", F.DummyJS_cv, 1, IM - 1, 1, 2, 1, KM - 1, 5, cvg);
    dump_box(p + "dJP_cv", F.DummyJP_cv, 1, IM - 1, 1, 2, 1, KM - 1, 5, cvg);
    dump_box(p + "dKS_cv", F.DummyKS_cv, 1, IM - 1, 1, JM - 1, 1, 2, 5, cvg);
    dump_box(p + "dKP_cv", F.DummyKP_cv, 1, IM - 1, 1, JM - 1, 1, 2, 5, cvg);
    dump_box(p + "dIS_pv", F.DummyIS_pv, 1, 2, 1, JM - 1, 1, KM - 1, 6, pvg);
    dump_box(p + "dIP_pv", F.DummyIP_pv, 1, 2, 1, JM - 1, 1, KM - 1, 6, pvg);
    dump_box(p + "dJS_pv", F.DummyJS_pv, 1, IM - 1, 1, 2, 1, KM - 1, 6, pvg);
    dump_box(p + "dJP_pv", F.DummyJP_pv, 1, IM - 1, 1, 2, 1, KM - 1, 6, pvg);
    dump_box(p + "dKS_pv", F.DummyKS_pv, 1, IM - 1, 1, JM - 1, 1, 2, 6, pvg);
    dump_box(p + "dKP_pv", F.DummyKP_pv, 1, IM - 1, 1, JM - 1, 1, 2, 6, pvg);
    auto sc = [](const REAL &v, int) { return (double)v; };
    dump_box(p + "omega", F.Omega, 1, IM - 1, 1, JM - 1, 1, KM - 1, 1, sc);
    dump_box(p + "lamcI", F.lambda_cI, 1, IM - 1, 1, JM - 1, 1, KM - 1, 1, sc);
    dump_box(p + "lamcJ", F.lambda_cJ, 1, IM - 1, 1, JM - 1, 1, KM - 1, 1, sc);
    dump_box(p + "lamcK", F.lambda_cK, 1, IM - 1, 1, JM - 1, 1, KM - 1, 1, sc);
    dump_box(p + "lamvI", F.lambda_vI, 1, IM - 1, 1, JM - 1, 1, KM - 1, 1, sc);
    dump_box(p + "lamvJ", F.lambda_vJ, 1, IM - 1, 1, JM - 1, 1, KM - 1, 1, sc);
    dump_box(p + "lamvK", F.lambda_vK, 1, IM - 1, 1, JM - 1, 1, KM - 1, 1, sc);
    dump_box(p + "dt", T.dt, 1, IM - 1, 1, JM - 1, 1, KM - 1, 1, sc);
    dump_box(p + "FcI", S.FaceI_Fc, 1, IM, 1, JM - 1, 1, KM - 1, 5, cvg);
    dump_box(p + "FcJ", S.FaceJ_Fc, 1, IM - 1, 1, JM, 1, KM - 1, 5, cvg);
    dump_box(p + "FcK", S.FaceK_Fc, 1, IM - 1, 1, JM - 1, 1, KM, 5, cvg);
    if (CFluidProps::equationType == EquationTypes::NavierStokes) {
        dump_box(p + "FvI", S.FaceI_Fv, 1, IM, 1, JM - 1, 1, KM - 1, 5, cvg);
        dump_box(p + "FvJ", S.FaceJ_Fv, 1, IM - 1, 1, JM, 1, KM - 1, 5, cvg);
        dump_box(p + "FvK", S.FaceK_Fv, 1, IM - 1, 1, JM - 1, 1, KM, 5, cvg);
    }
    dump_box(p + "Fc", S.Cell_Fc, 1, IM - 1, 1, JM - 1, 1, KM - 1, 5, cvg);
    dump_box(p + "Fv", S.Cell_Fv, 1, IM - 1, 1, JM - 1, 1, KM - 1, 5, cvg);
    dump_box(p + "res", S.Res_cv, 1, IM - 1, 1, JM - 1, 1, KM - 1, 5, cvg);
    if (CFluidProps::turbulenceType == TurbulenceTypes::SA)
        dump_box(p + "res_ev", S.Res_ev, 1, IM - 1, 1, JM - 1, 1, KM - 1, 1, [](const TEddyVars &v, int) { return (double)v.ev; });
}

int main(int argc, char **argv)
{
    if (argc < 3) { fprintf(stderr, "usage: ref_harness n_iter out_dir [dump_resflux] [write_outputs]\n"); return 2; }
    int n_iter = atoi(argv[1]);
    g_out = argv[2];
    int dump_rf = argc > 3 ? atoi(argv[3]) : 1;
    int write_out = argc > 4 ? atoi(argv[4]) : 0;      // the reference's solution and restart files
    mkdir(g_out.c_str(), 0755);

    CSolver Solver;
    CUserInput::ReadConfig(Solver);
    CUserInput::NumberOfMultigrid(Solver);
    CUserInput::ReadGrids(Solver);
    CUserInput::ReadBndGrid(Solver);
    CUserInput::NonDimensionalization(Solver);
    for (int i = 1; i <= Solver.NG; i++) Solver.Mesh[i].AllocateMemory();
    if (Solver.NG == 2) Solver.Mesh[2].AllocateMemory_Pro_Inter_Vars();
    for (int i = 1; i <= Solver.NG; i++) Solver.Mesh[i].Geometry();
    // Spalart-Allmaras wall distances of the fine mesh (source/Structured_FV3D.cpp:71-84)
    if (CFluidProps::turbulenceType == TurbulenceTypes::SA) {
        if (!Solver.reUseWallDistance) Solver.Mesh[1].WallDistanceSA();
        else CUserInput::ReadWallDistance(Solver.Mesh[1]);
    }
    // start: uniform field, or the reference's restart file when the case asks for it
    // (source/Structured_FV3D.cpp:86-102)
    if (Solver.reUseSolution) CUserInput::ReadSolution(Solver.Mesh[1]);
    else if (Solver.NG == 1) Solver.Mesh[1].Initial();
    else Solver.Mesh[2].Initial();

    // a case of several blocks gets every array once per block, prefixed "b<block>_"
    const int NB = CMesh::NB;
    auto bp = [&](int nb) { return NB > 1 ? "b" + std::to_string(nb) + "_" : std::string(); };
    for (int nb = 1; nb <= NB; nb++) {
        dump_geometry(Solver.Mesh[1], bp(nb) + "g1_", nb);
        if (Solver.NG == 2) dump_geometry(Solver.Mesh[2], bp(nb) + "g2_", nb);
    }
    npy_write("ng", {(double)Solver.NG}, {1});
    npy_write("nb", {(double)NB}, {1});

    // history rows: iter, Res.dens, Res.xmom..ener, m_in, m_out, PR, eta, m_ratio, CFL
    std::vector<double> hist;
    std::vector<double> pout_hist;          // nondimensional back pressure used in each iteration
    int done = 0;
    for (Solver.iter = 1; Solver.iter <= n_iter; Solver.iter++) {
        Solver.Solver();
        CMesh *Mo = &Solver.Mesh[1];
        if (Solver.NG != 1 && Solver.iter <= Solver.Coarse_iter) Mo = &Solver.Mesh[2];
        COutput::OutputGeneralParameters(Solver.MassFlow_in, Solver.MassFlow_out, Solver.Efficiency,
                                         Solver.MassFlow_ratio, Solver.Press_ratio, *Mo);
        double row[12] = {(double)Solver.iter, Solver.Res.dens, Solver.Res.xmom, Solver.Res.ymom,
                          Solver.Res.zmom, Solver.Res.ener, Solver.MassFlow_in, Solver.MassFlow_out,
                          Solver.Press_ratio, Solver.Efficiency, Solver.MassFlow_ratio,
                          (double)CTimeDiscr::CFL};
        hist.insert(hist.end(), row, row + 12);
        done++;
        pout_hist.push_back((double)CBndConds::Pout);
        // imposed mass flow, as the driver applies it after the output (source/Structured_FV3D.cpp:186-193)
        if (Solver.UseFlowMassImposed == 1 && Solver.Res.dens <= Solver.resc_mass_imp &&
            Solver.iter % Solver.iter_mass_imp == 0)
            Solver.MassFlowImposed();
        if (Solver.Res.dens <= Solver.ConvTol && Solver.MassFlow_ratio <= 0.003) break;
    }
    npy_write("history", hist, {(size_t)done, 12});
    npy_write("pout", pout_hist, {(size_t)done});
    if (write_out) {
        // RelativeSolution.plt and RestartSolution.dat in the working directory (source/Ouput.cpp:109-259)
        COutput::OutputSolution(Solver.Mesh[1]);
        COutput::OutputRestartSolution(Solver.Mesh[1]);
    }
    for (int nb = 1; nb <= NB; nb++) {
        dump_state(Solver.Mesh[1], bp(nb) + "s1_", nb);
        if (Solver.NG == 2) dump_state(Solver.Mesh[2], bp(nb) + "s2_", nb);
    }
    if (dump_rf) {
        // one more residual evaluation on the fine level at the final state, with every
        // intermediate array of the path
        Solver.Mesh[1].ResFlux();
        for (int nb = 1; nb <= NB; nb++) dump_resflux(Solver.Mesh[1], bp(nb) + "r1_", nb);
    }
    // the reference's destructors crash on the two-level mesh arrays; the dumps are complete
    fflush(nullptr);
    _exit(0);
}
