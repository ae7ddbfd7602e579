// The reference's solution files, written and read on the host from the device state:
//  - RestartSolution.dat (COutput::OutputRestartSolution, source/Ouput.cpp:227-259, read back by
//    CUserInput::ReadSolution, source/UserInput.cpp:1118-1159): one line per interior cell of the
//    fine level, block by block, k outermost, "nb i j k p u v w T rho rhoE" in the stream's default format (six
//    significant digits);
//  - RelativeSolution.plt (COutput::OutputSolution, source/Ouput.cpp:109-225): Tecplot ASCII,
//    node values as the mean of the eight surrounding cells (ghost layer included), dimensional,
//    per block one zone at the passage and one rotated by the pitch angle.
// The default stream format of a double is printf's "%g", which is what is written here, so the
// same state gives the same bytes.
#include "restart_io.hpp"
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace gbt {

namespace {

struct File {
    FILE *f;
    File(const std::string &path, const char *mode) : f(std::fopen(path.c_str(), mode))
    {
        if (!f) throw std::runtime_error("cannot open " + path);
    }
    ~File() { if (f) std::fclose(f); }
};

// index of cell (i,j,k), i,j,k in 0..N, of a box array shaped (IM+1, JM+1, KM+1, nc)
inline size_t bx(int i, int j, int k, int JM, int KM, int nc) { return (((size_t)i * (JM + 1) + j) * (KM + 1) + k) * nc; }

}  // namespace

void write_restart_file(const std::string &path, const std::vector<BlockField> &blocks)
{
    File out(path, "w");
    for (size_t nb = 0; nb < blocks.size(); nb++) {
        const BlockField &B = blocks[nb];
        const int IM = B.IM, JM = B.JM, KM = B.KM;
        for (int k = 1; k <= KM - 1; k++)
            for (int j = 1; j <= JM - 1; j++)
                for (int i = 1; i <= IM - 1; i++) {
                    const double *q = B.pv + bx(i, j, k, JM, KM, 6);
                    const double e = B.cv[bx(i, j, k, JM, KM, 5) + 4];
                    // p, u, v, w, T, rho, rhoE (pv holds rho u v w p T), and the SA variable if present
                    if (B.ev)
                        std::fprintf(out.f, "%d %d %d %d %g %g %g %g %g %g %g %g\n", (int)nb + 1, i, j, k, q[4], q[1], q[2],
                                     q[3], q[5], q[0], e, B.ev[bx(i, j, k, JM, KM, 1)]);
                    else
                        std::fprintf(out.f, "%d %d %d %d %g %g %g %g %g %g %g\n", (int)nb + 1, i, j, k, q[4], q[1], q[2], q[3],
                                     q[5], q[0], e);
                }
    }
}

void read_restart_file(const std::string &path, const std::vector<BlockField> &blocks, std::vector<std::vector<double>> &cvs,
                       std::vector<std::vector<double>> &pvs, bool with_ev, std::vector<std::vector<double>> *evs)
{
    File in(path, "r");
    cvs.resize(blocks.size());
    pvs.resize(blocks.size());
    if (with_ev) evs->resize(blocks.size());
    for (size_t nb = 0; nb < blocks.size(); nb++) {
        const int IM = blocks[nb].IM, JM = blocks[nb].JM, KM = blocks[nb].KM;
        // the reference reads the values in its own loop order and ignores the indices on each line
        const long n = (long)(IM - 1) * (JM - 1) * (KM - 1);
        std::vector<double> rows((size_t)n * 8);
        for (long r = 0; r < n; r++) {
            int b, i, j, k;
            double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            const int got = std::fscanf(in.f, "%d %d %d %d %lf %lf %lf %lf %lf %lf %lf", &b, &i, &j, &k, &v[0], &v[1], &v[2],
                                        &v[3], &v[4], &v[5], &v[6]);
            const bool ok = got == 11 && (!with_ev || std::fscanf(in.f, "%lf", &v[7]) == 1);
            if (!ok)
                throw std::runtime_error(path + ": block " + std::to_string(nb + 1) + " expects " + std::to_string(n) +
                                         (with_ev ? " lines of 12 values (with the SA variable)" : " lines of 11 values (no SA variable)") +
                                         "; its line " + std::to_string(r + 1) + " is short");
            std::memcpy(&rows[(size_t)r * 8], v, sizeof v);
        }
        if (with_ev) (*evs)[nb].assign((size_t)n, 0.0);
        std::vector<double> &cv = cvs[nb], &pv = pvs[nb];
        cv.assign((size_t)n * 5, 0.0);
        pv.assign((size_t)n * 6, 0.0);
        // file order: k outermost, i innermost; output order: i outermost, k innermost
        long r = 0;
        for (int k = 1; k <= KM - 1; k++)
            for (int j = 1; j <= JM - 1; j++)
                for (int i = 1; i <= IM - 1; i++, r++) {
                    const double *v = &rows[(size_t)r * 8];
                    const double press = v[0], u = v[1], vv = v[2], w = v[3], temp = v[4], dens = v[5], ener = v[6];
                    const size_t o = ((size_t)(i - 1) * (JM - 1) + (j - 1)) * (KM - 1) + (k - 1);
                    cv[o * 5 + 0] = dens; cv[o * 5 + 1] = dens * u; cv[o * 5 + 2] = dens * vv; cv[o * 5 + 3] = dens * w;
                    cv[o * 5 + 4] = ener;
                    pv[o * 6 + 0] = dens; pv[o * 6 + 1] = u; pv[o * 6 + 2] = vv; pv[o * 6 + 3] = w; pv[o * 6 + 4] = press;
                    pv[o * 6 + 5] = temp;
                    if (with_ev) (*evs)[nb][o] = v[7];
                }
    }
}

void write_solution_file(const std::string &path, const std::vector<BlockField> &blocks, const SolutionScales &sc)
{
    File out(path, "w");
    std::fprintf(out.f, "VARIABLES = x y z dens uvel vvel wvel temp press Ma Pt  miu_t \n");
    const double G = sc.gamma, R = sc.rgas;
    for (const BlockField &B : blocks)
    for (int zone = 0; zone < 2; zone++) {
        const int IM = B.IM, JM = B.JM, KM = B.KM;
        const double *pv = B.pv, *mut = B.mut, *x = B.x, *y = B.y, *z = B.z;
        const double cth = std::cos(B.delta_th), sth = std::sin(B.delta_th);
        std::fprintf(out.f, "ZONE i=%d j=%d k=%d f=point\n", IM, JM, KM);
        for (int k = 1; k <= KM; k++)
            for (int j = 1; j <= JM; j++)
                for (int i = 1; i <= IM; i++) {
                    // mean of the eight cells around node (i,j,k), summed in the reference's order
                    const int ci[8][3] = {{i, j, k}, {i - 1, j, k}, {i - 1, j, k - 1}, {i, j, k - 1},
                                          {i, j - 1, k}, {i - 1, j - 1, k}, {i - 1, j - 1, k - 1}, {i, j - 1, k - 1}};
                    double p[6], mue;
                    for (int c = 0; c < 6; c++) {
                        double s = pv[bx(ci[0][0], ci[0][1], ci[0][2], JM, KM, 6) + c];
                        for (int m = 1; m < 8; m++) s = s + pv[bx(ci[m][0], ci[m][1], ci[m][2], JM, KM, 6) + c];
                        p[c] = 0.125 * s;
                    }
                    {
                        double s = mut[bx(ci[0][0], ci[0][1], ci[0][2], JM, KM, 1)];
                        for (int m = 1; m < 8; m++) s = s + mut[bx(ci[m][0], ci[m][1], ci[m][2], JM, KM, 1)];
                        mue = 0.125 * s;
                    }
                    const size_t nq = ((size_t)(k - 1) * JM + (j - 1)) * IM + (i - 1);
                    const double cx = x[nq], cy = y[nq], cz = z[nq];
                    const double dens = p[0], u = p[1], v = p[2], w = p[3], press = p[4], temp = p[5];
                    const double ure = u + B.w_rot * cy;
                    const double vre = v - B.w_rot * cx;
                    const double ma_re = std::sqrt(ure * ure + vre * vre + w * w) / std::sqrt(G * R * temp);
                    const double ma_abs = std::sqrt(u * u + v * v + w * w) / std::sqrt(G * R * temp);
                    const double pt = press * std::pow(1 + (G - 1) / 2.0 * ma_abs * ma_abs, G / (G - 1));
                    double X, Y, U, V;
                    if (zone == 0) {
                        X = cx * sc.len_ref;
                        Y = cy * sc.len_ref;
                        U = ure;          // the relative velocity is written nondimensional in this zone
                        V = vre;
                    } else {
                        X = (cx * cth - cy * sth) * sc.len_ref;
                        Y = (cy * cth + cx * sth) * sc.len_ref;
                        U = (ure * cth - vre * sth) * sc.vel_ref;
                        V = (vre * cth + ure * sth) * sc.vel_ref;
                    }
                    const double Z = cz * sc.len_ref;
                    std::fprintf(out.f, "%g %g %g %g %g %g %g %g %g %g %g %g\n", X, Y, Z, dens * sc.dens_ref, U, V,
                                 w * sc.vel_ref, temp * sc.temp_ref, press * sc.dens_ref * sc.vel_ref * sc.vel_ref, ma_re,
                                 pt * sc.dens_ref * sc.vel_ref * sc.vel_ref, mue * sc.mue_ref * sc.re_ref);
                }
    }
}

}  // namespace gbt
