// Case-file reader. Follows the reference's positional parsing (source/UserInput.cpp:17-239,
// 241-334, 336-446, 799-1068; include/fstringIO.h:15-42) so the same files drive both solvers.
#include "case_io.hpp"
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <charconv>
#include <system_error>
#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

namespace gbt {

std::string ref_read_line(std::FILE *f, bool *ok)
{
    std::string s;
    int ch;
    bool any = false;
    while ((ch = std::fgetc(f)) != EOF) {
        any = true;
        if (ch == '\n') break;
        s.push_back((char)ch);
    }
    if (ok) *ok = any;
    if (!s.empty() && s.back() == '\r') s.pop_back();
    size_t h = s.find('#');
    if (h != std::string::npos) s.erase(h);
    size_t a = s.find_first_not_of(' ');
    if (a == std::string::npos) return std::string();
    s.erase(0, a);
    size_t b = s.find_last_not_of(' ');
    s.erase(b + 1);
    return s;
}

namespace {

struct LineReader {
    std::FILE *f = nullptr;
    std::string name;
    int lineno = 0;
    LineReader(const std::string &path, const std::string &nm) : name(nm)
    {
        f = std::fopen(path.c_str(), "r");
        if (!f) throw std::runtime_error("cannot open " + path);
    }
    ~LineReader() { if (f) std::fclose(f); }
    std::string next()
    {
        bool ok;
        std::string s = ref_read_line(f, &ok);
        lineno++;
        if (!ok) throw std::runtime_error(name + ": file ended at line " + std::to_string(lineno));
        return s;
    }
    void skip(int n) { for (int i = 0; i < n; i++) next(); }
};

// std::stof, then widened: the reference's REAL is double but its options pass through float
double as_float(const std::string &s, const std::string &what)
{
    char *e = nullptr;
    float v = std::strtof(s.c_str(), &e);
    if (e == s.c_str()) throw std::runtime_error("config.dat: cannot read " + what + " from '" + s + "'");
    return (double)v;
}
int as_int(const std::string &s, const std::string &what)
{
    char *e = nullptr;
    long v = std::strtol(s.c_str(), &e, 10);
    if (e == s.c_str()) throw std::runtime_error("cannot read " + what + " from '" + s + "'");
    return (int)v;
}
bool is_yes(const std::string &s) { return s == "y" || s == "Y"; }

std::vector<int> ints(const std::string &s)
{
    std::vector<int> v;
    const char *p = s.c_str();
    char *e;
    for (;;) {
        long x = std::strtol(p, &e, 10);
        if (e == p) break;
        v.push_back((int)x);
        p = e;
    }
    return v;
}

void read_config(CaseSpec &c)
{
    LineReader r(c.dir + "/config.dat", "config.dat");
    r.next(); c.grid_file = r.next();
    r.skip(2); c.bc_file = r.next();
    r.skip(3);
    std::string s = r.next(); c.turbo_axial = (s == "a" || s == "A");
    s = r.next(); c.equation_ns = !(s == "e" || s == "E");
    s = r.next(); c.uniform_init = (s == "u" || s == "U");
    c.Rgas = as_float(r.next(), "gas constant");
    c.Gamma = as_float(r.next(), "specific heat ratio");
    c.Pr_lam = as_float(r.next(), "laminar Prandtl number");
    c.Pr_tur = as_float(r.next(), "turbulent Prandtl number");
    r.skip(3);
    c.Ptin = as_float(r.next(), "inlet total pressure");
    c.Ttin = as_float(r.next(), "inlet total temperature");
    c.Pout = as_float(r.next(), "outlet static pressure");
    c.P21 = as_float(r.next(), "pressure ratio guess");
    c.Ma0 = as_float(r.next(), "initial Mach number");
    c.Len_ref = as_float(r.next(), "reference length");
    c.ev_ratio = as_float(r.next(), "eddy viscosity ratio");
    {
        std::istringstream is(r.next());
        is >> c.inlet_dir[0] >> c.inlet_dir[1] >> c.inlet_dir[2];
    }
    r.next();
    c.mass_imposed = is_yes(r.next());
    {
        // read with the stream as the reference does (source/UserInput.cpp:80), not through stof
        std::istringstream is(r.next());
        is >> c.m_imposed >> c.relax_press >> c.iter_mass_imp >> c.resc_mass_imp;
        if (c.mass_imposed && (!is || c.m_imposed <= 0.0 || c.iter_mass_imp < 1))
            throw std::runtime_error("config.dat: the imposed mass flow line needs a positive mass flow and an iteration step >= 1");
    }
    r.skip(3);
    c.maxiter = as_int(r.next(), "max iterations");
    c.coarse_iter = as_int(r.next(), "coarse iterations");
    c.outstep = as_int(r.next(), "output step");
    c.convtol = as_float(r.next(), "convergence tolerance");
    c.nt = as_int(r.next(), "thread count");
    c.use_mg = is_yes(r.next());
    c.restart = is_yes(r.next());
    r.next();
    r.skip(3);
    c.CFL = as_float(r.next(), "CFL");
    c.C_timestep = as_float(r.next(), "time step coefficient");
    c.relax = as_float(r.next(), "LU-SGS relaxation");
    c.epsEntr = as_float(r.next(), "entropy correction");
    c.k2 = as_float(r.next(), "k2");
    c.k4 = as_float(r.next(), "k4");
    c.k4 = (double)(1.0f / c.k4);
    c.irs = is_yes(r.next());
    c.limiter = is_yes(r.next());
    s = r.next(); c.global_dt = !(s == "l" || s == "L");
    c.recon_var = as_int(r.next(), "reconstruction variables");
    c.recon = as_int(r.next(), "reconstruction scheme");
    c.scheme = as_int(r.next(), "space scheme");
    c.time_scheme = as_int(r.next(), "time scheme");
    c.turb = as_int(r.next(), "turbulence model");
}

void ng_check(int is, int ie, int js, int je, int ks, int ke, int &NG)
{
    if (is != ie) ie = ie + 1;
    if (js != je) je = je + 1;
    if (ks != ke) ke = ke + 1;
    int num = 1;
    if ((is - 1) % 2 == 0 && (ie - 1) % 2 == 0 && (js - 1) % 2 == 0 && (je - 1) % 2 == 0 &&
        (ks - 1) % 2 == 0 && (ke - 1) % 2 == 0)
        num = 2;
    NG = std::min(num, NG);
}

struct BlockRow { int IM, JM, KM, nblade; double rpm; };

void read_bc(CaseSpec &c, std::vector<BlockRow> &blocks)
{
    LineReader r(c.dir + "/" + c.bc_file, c.bc_file);
    int NG = 4;
    auto count = [&](const char *what) { return as_int(r.next(), what); };
    r.skip(4);
    int n = count("inlet count");
    r.next();
    for (int q = 0; q < n; q++) {
        auto v = ints(r.next());
        if (v.size() < 9) throw std::runtime_error(c.bc_file + ": bad inlet line");
        c.inlets.push_back({v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[1]});
        ng_check(v[3], v[4], v[5], v[6], v[7], v[8], NG);
    }
    r.skip(3);
    n = count("outlet count");
    r.next();
    for (int q = 0; q < n; q++) {
        auto v = ints(r.next());
        if (v.size() < 9) throw std::runtime_error(c.bc_file + ": bad outlet line");
        c.outlets.push_back({v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[1]});
        ng_check(v[3], v[4], v[5], v[6], v[7], v[8], NG);
    }
    r.skip(3);
    n = count("wall count");
    r.next();
    for (int q = 0; q < n; q++) {
        auto v = ints(r.next());
        if (v.size() < 10) throw std::runtime_error(c.bc_file + ": bad wall line");
        c.walls.push_back({v[2], v[3] != 0, v[4], v[5], v[6], v[7], v[8], v[9], v[1]});
        ng_check(v[4], v[5], v[6], v[7], v[8], v[9], NG);
    }
    // periodic pairs and block interfaces share one line format
    // (ID orient BID1 FT1 range1 BID2 FT2 range2; source/UserInput.cpp:380-420)
    auto pair_line = [&](const char *what) {
        auto v = ints(r.next());
        if (v.size() < 18) throw std::runtime_error(c.bc_file + ": bad " + what + " line");
        PeriodicIO p;
        p.orient = v[1]; p.b1 = v[2]; p.f1 = v[3]; p.b2 = v[10]; p.f2 = v[11];
        for (int d = 0; d < 6; d++) { p.r1[d] = v[4 + d]; p.r2[d] = v[12 + d]; }
        ng_check(v[4], v[5], v[6], v[7], v[8], v[9], NG);
        return p;
    };
    r.skip(3);
    n = count("periodic count");
    r.next();
    for (int q = 0; q < n; q++) c.periodics.push_back(pair_line("periodic"));
    r.skip(3);
    n = count("interior count");
    r.next();
    for (int q = 0; q < n; q++) c.interiors.push_back(pair_line("interior"));
    r.skip(3);
    n = count("mixing-plane count");
    r.next();
    for (int q = 0; q < n; q++) c.mixing.push_back(pair_line("mixing plane"));
    r.skip(3);
    const int nb = count("block count");
    if (nb < 1) throw std::runtime_error(c.bc_file + ": the case needs at least one block");
    r.next();
    for (int b = 0; b < nb; b++) {
        // BID IM JM KM NBlade rpm (rpm read by a stream into a REAL: exact decimal parse)
        std::string s = r.next();
        const char *p = s.c_str();
        char *e;
        int v[5];
        for (int q = 0; q < 5; q++) { v[q] = (int)std::strtol(p, &e, 10); p = e; }
        BlockRow br;
        br.rpm = std::strtod(p, &e);
        br.IM = v[1]; br.JM = v[2]; br.KM = v[3]; br.nblade = v[4];
        blocks.push_back(br);
        int IM = br.IM, JM = br.JM, KM = br.KM;
        for (int j = 1; j <= std::min(std::min(IM, JM), KM); j++) {
            int nn = 2 * j;
            if ((IM - 1) % nn == 0 && (JM - 1) % nn == 0 && (KM - 1) % nn == 0 && (IM - 1) / nn > 2 &&
                (JM - 1) / nn > 2 && (KM - 1) / nn > 2)
                NG = std::min(j + 1, NG);
            else
                break;
        }
    }
    c.ng = c.use_mg ? std::min(NG, 2) : 1;
    c.nblock = nb;
    auto in_range = [&](int b, const char *what) {
        if (b < 1 || b > nb) throw std::runtime_error(c.bc_file + ": " + what + " names block " + std::to_string(b) + " of " + std::to_string(nb));
    };
    for (auto &p : c.inlets) in_range(p.block, "an inlet");
    for (auto &p : c.outlets) in_range(p.block, "an outlet");
    for (auto &w : c.walls) in_range(w.block, "a wall");
    for (auto &p : c.periodics) { in_range(p.b1, "a periodic pair"); in_range(p.b2, "a periodic pair"); }
    for (auto &p : c.interiors) { in_range(p.b1, "an interface"); in_range(p.b2, "an interface"); }
    for (auto &p : c.mixing) {
        in_range(p.b1, "a mixing plane"); in_range(p.b2, "a mixing plane");
        // CMesh::BndCondMixingPlane averages the k = KM cells of block 1 and the k = 1 cells of
        // block 2 over the pitch, row by row of block 1's i range (source/BndCondMixingPlane.cpp:287-520)
        if (p.f1 != 6 || p.f2 != 5)
            throw std::runtime_error(c.bc_file + ": a mixing plane joins the k+ face (6) of its first block to the k- face (5) of its second");
    }
}

// The grid file in memory, line by line, with the reference's line rule (ReadLine: '#' starts a
// comment, surrounding blanks dropped, a trailing carriage return dropped). Text grids of large
// cases hold millions of numbers, so the file is read with one fread and the numbers are parsed
// in place (std::from_chars, correctly rounded like the stream the reference reads with).
struct GridText {
    std::string buf;
    size_t pos = 0;
    int lineno = 0;
    std::string name;
    GridText(const std::string &path, const std::string &nm) : name(nm)
    {
        std::FILE *f = std::fopen(path.c_str(), "rb");
        if (!f) throw std::runtime_error("cannot open " + path);
        std::fseek(f, 0, SEEK_END);
        const long n = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        buf.resize(n > 0 ? (size_t)n : 0);
        const size_t got = n > 0 ? std::fread(&buf[0], 1, (size_t)n, f) : 0;
        std::fclose(f);
        if (got != buf.size()) throw std::runtime_error("cannot read " + path);
    }
    // [b, e) of the next line's content
    void next(const char *&b, const char *&e)
    {
        if (pos >= buf.size()) throw std::runtime_error(name + ": file ended at line " + std::to_string(lineno + 1));
        const char *s0 = buf.data() + pos, *end = buf.data() + buf.size();
        const char *nl = (const char *)std::memchr(s0, '\n', (size_t)(end - s0));
        const char *le = nl ? nl : end;
        pos = (size_t)(le - buf.data()) + (nl ? 1 : 0);
        lineno++;
        if (le > s0 && le[-1] == '\r') le--;
        const char *h = (const char *)std::memchr(s0, '#', (size_t)(le - s0));
        if (h) le = h;
        while (s0 < le && *s0 == ' ') s0++;
        while (le > s0 && le[-1] == ' ') le--;
        b = s0;
        e = le;
    }
    std::string next_string()
    {
        const char *b, *e;
        next(b, e);
        return std::string(b, e);
    }
};

// three numbers of a node line
inline bool parse3(const char *b, const char *e, double &x, double &y, double &z)
{
    double *v[3] = {&x, &y, &z};
    for (int q = 0; q < 3; q++) {
        while (b < e && (*b == ' ' || *b == '\t')) b++;
        if (b < e && *b == '+') b++;
        auto r = std::from_chars(b, e, *v[q]);
        if (r.ec != std::errc()) return false;
        b = r.ptr;
    }
    return true;
}

// the grid file: block count, then per block its id line, "IM JM KM" and the nodes, i fastest
// (source/UserInput.cpp:241-290). A block's node lines are split in one pass, then parsed by
// `threads` host threads (each line is one node, so a line's index is its node's).
void read_grid(const CaseSpec &c, const std::vector<BlockRow> &rows, std::vector<CaseSpec> &out, int threads)
{
    std::string path = c.dir + "/" + c.grid_file;
    GridText r(path, c.grid_file);
    const int nb = as_int(r.next_string(), "block count");
    if (nb != (int)rows.size()) throw std::runtime_error("grid and boundary file disagree on the number of blocks");
    for (int b = 1; b <= nb; b++) {
        if (as_int(r.next_string(), "block id") != b)
            throw std::runtime_error(c.grid_file + ": blocks must be numbered 1, 2, ... in file order");
        int IM, JM, KM;
        {
            std::istringstream is(r.next_string());
            if (!(is >> IM >> JM >> KM)) throw std::runtime_error(c.grid_file + ": bad block size line");
        }
        const BlockRow &br = rows[b - 1];
        if (IM != br.IM || JM != br.JM || KM != br.KM)
            throw std::runtime_error("grid and boundary file disagree on the size of block " + std::to_string(b));
        CaseSpec bs;
        // options and the case-wide lists, then this block's own patches and grid
        bs = c;
        bs.inlets.clear(); bs.outlets.clear(); bs.walls.clear();
        for (auto &p : c.inlets) if (p.block == b) bs.inlets.push_back(p);
        for (auto &p : c.outlets) if (p.block == b) bs.outlets.push_back(p);
        for (auto &w : c.walls) if (w.block == b) bs.walls.push_back(w);
        bs.block = b;
        bs.IM = IM; bs.JM = JM; bs.KM = KM; bs.nblade = br.nblade; bs.rpm = br.rpm;
        size_t n = (size_t)IM * JM * KM;
        bs.x.resize(n); bs.y.resize(n); bs.z.resize(n);
        const int line0 = r.lineno;                       // the line before the block's first node
        // The node lines [pos0, ...): line q starts at pos0 (q = 0) or right after the q-th newline.
        // The buffer is cut into `nt` byte ranges; each thread counts the newlines of its range,
        // and after a prefix sum parses the lines that start in its range (parse3 stops at a
        // comment, a carriage return or the line end the way the one-line reader's trimming does).
        const char *base = r.buf.data();
        const size_t pos0 = r.pos, end = r.buf.size();
        const size_t nt = (threads > 1 && n >= 65536) ? (size_t)threads : 1;
        std::vector<size_t> cut(nt + 1), nl_count(nt + 1, 0);
        for (size_t t = 0; t <= nt; t++) cut[t] = pos0 + (end - pos0) * t / nt;
        std::atomic<size_t> bad{n};                       // first node line that does not parse
        std::atomic<size_t> next_pos{end};                // start of the line after the block's nodes
        auto note_bad = [&](size_t q) {
            size_t cur = bad.load();
            while (q < cur && !bad.compare_exchange_weak(cur, q)) {}
        };
        auto count_range = [&](size_t t) {
            nl_count[t + 1] = (size_t)std::count(base + cut[t], base + cut[t + 1], '\n');
        };
        auto parse_range = [&](size_t t) {
            size_t q = 0;
            for (size_t u = 0; u <= t; u++) q += nl_count[u];  // newlines before this range
            const char *p = base + cut[t], *e = base + cut[t + 1];
            const char *ls;                               // start of the next line to parse
            if (t == 0) ls = base + pos0;
            else {
                // the first line starting in this range follows the first newline at or after cut[t] - 1
                const char *nl = (const char *)std::memchr(p - 1, '\n', (size_t)(e - (p - 1)));
                if (!nl || nl + 1 >= e) return;
                q += (nl >= p) ? 1 : 0;                   // a newline at cut[t] - 1 was counted by the range before
                ls = nl + 1;
            }
            while (ls < e) {
                if (q >= n) {
                    if (q == n) next_pos.store((size_t)(ls - base));
                    return;
                }
                const char *nl = (const char *)std::memchr(ls, '\n', (size_t)(base + end - ls));
                const char *le = nl ? nl : base + end;
                if (!parse3(ls, le, bs.x[q], bs.y[q], bs.z[q])) note_bad(q);
                q++;
                if (!nl) break;
                ls = nl + 1;
            }
        };
        if (nt == 1) {
            count_range(0);
            parse_range(0);
        } else {
            std::vector<std::thread> pool;
            for (size_t t = 0; t < nt; t++) pool.emplace_back(count_range, t);
            for (auto &th : pool) th.join();
            pool.clear();
            for (size_t t = 0; t < nt; t++) pool.emplace_back(parse_range, t);
            for (auto &th : pool) th.join();
        }
        size_t total_nl = 0;
        for (size_t t = 1; t <= nt; t++) total_nl += nl_count[t];
        const size_t lines = total_nl + ((end > pos0 && base[end - 1] != '\n') ? 1 : 0);
        if (lines < n) throw std::runtime_error(c.grid_file + ": file ended at line " + std::to_string(line0 + (int)lines + 1));
        if (bad.load() < n)
            throw std::runtime_error(c.grid_file + ": bad node line " + std::to_string(line0 + 1 + (int)bad.load()));
        r.pos = next_pos.load();
        r.lineno = line0 + (int)n;
        out.push_back(std::move(bs));
    }
}

void validate_block(const CaseSpec &c)
{
    const std::string b = c.nblock > 1 ? "block " + std::to_string(c.block) + ": " : "";
    if (c.IM < 4 || c.JM < 4 || c.KM < 4) throw std::runtime_error(b + "each direction needs at least 4 nodes");
    for (auto &p : c.inlets)
        if (p.ks != p.ke || (p.ks != 1 && p.ks != c.KM)) throw std::runtime_error(b + "inlets must be k-faces (k = 1 or KM)");
    for (auto &p : c.outlets)
        if (p.ks != p.ke || p.ke != c.KM) throw std::runtime_error(b + "the axial outlet must be the k = KM face");
    for (auto &w : c.walls)
        if (c.turb == 100 && (w.face == 5 || w.face == 6))
            throw std::runtime_error(b + "Baldwin-Lomax with k-face walls is not supported");
}

void validate(const CaseSpec &c)
{
    if (c.scheme != 100 && c.scheme != 200 && c.scheme != 300)
        throw std::runtime_error("space scheme " + std::to_string(c.scheme) + " is not on this path (JST 100, Steger-Warming 200, Roe 300)");
    if (c.recon_var != 100 && c.recon_var != 200)
        throw std::runtime_error("reconstruction variables " + std::to_string(c.recon_var) + " are not supported (100, 200)");
    if (c.time_scheme >= 100 && c.time_scheme <= 400)
        throw std::runtime_error("Runge-Kutta marching is not on this path (LU-SGS only)");
    if (c.turb != 0 && c.turb != 100 && c.turb != 200)
        throw std::runtime_error("turbulence model " + std::to_string(c.turb) + " is not on this path (none 0, Baldwin-Lomax 100, Spalart-Allmaras 200)");
    if (c.turb == 200 && c.use_mg)
        throw std::runtime_error("Spalart-Allmaras runs on a single grid level here: under multigrid the reference starts on the coarse "
                                 "level and never initialises or transfers the fine level's variable");
    if (c.turb == 200 && c.walls.empty()) throw std::runtime_error("Spalart-Allmaras needs at least one wall (wall distances)");
    if (c.irs) throw std::runtime_error("implicit residual smoothing is not on this path");
    if (!c.turbo_axial) throw std::runtime_error("only the axial outlet is on this path");
    if (c.use_mg && c.coarse_iter < 1)
        throw std::runtime_error("multigrid needs at least one coarse-grid iteration (the fine level is initialised from it)");
    if (c.inlets.empty() || c.outlets.empty()) throw std::runtime_error("the case needs an inlet and an outlet");
}

}  // namespace

std::vector<CaseSpec> read_case(const std::string &dir, int threads)
{
    CaseSpec c;
    c.dir = dir;
    read_config(c);
    std::vector<BlockRow> rows;
    read_bc(c, rows);
    validate(c);
    c.first_inlet = c.inlets[0];
    c.first_outlet = c.outlets[0];
    std::vector<CaseSpec> blocks;
    read_grid(c, rows, blocks, threads);
    for (auto &b : blocks) validate_block(b);
    return blocks;
}

}  // namespace gbt
