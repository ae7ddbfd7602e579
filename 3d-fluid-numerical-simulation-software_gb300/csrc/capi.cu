// extern "C" boundary: forwards to gbt::SolverBase and turns exceptions into error codes.
#include "../../include/gbturbo.h"
#include "solver.hpp"
#include "warmstart.hpp"
#include <cstring>
#include <string>
#include <thread>
#include <algorithm>

struct gb_solver {
    std::unique_ptr<gbt::SolverBase> s;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
};
struct gb_warmstart {
    std::unique_ptr<gbt::WarmStart> w;
};

static thread_local std::string g_err;

template <class F>
static int guard(F &&f)
{
    try {
        f();
        return GB_OK;
    } catch (const std::exception &e) {
        g_err = e.what();
        std::string m = e.what();
        if (m.find("cuda") != std::string::npos || m.find("CUDA") != std::string::npos) return GB_ERR_CUDA;
        return GB_ERR_CASE;
    } catch (...) {
        g_err = "unknown error";
        return GB_ERR_CASE;
    }
}
#define NEED(h) do { if (!(h) || !(h)->s) { g_err = "null handle"; return GB_ERR_ARG; } } while (0)
#define LEVEL(h, l) do { if ((l) < 1 || (l) > (h)->s->ng) { g_err = "level out of range"; return GB_ERR_ARG; } } while (0)

extern "C" {

const char *gb_last_error(void) { return g_err.c_str(); }

int gb_case_info(const char *case_dir, long long info[9], double *nodes_out, long long cap)
{
    if (!case_dir || !info) { g_err = "bad arguments"; return GB_ERR_ARG; }
    return guard([&] {
        std::vector<gbt::CaseSpec> b = gbt::read_case(case_dir, (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency())));
        const gbt::CaseSpec &c = b[0];
        long long nodes = 0, nin = 0, nout = 0, nwall = 0;
        for (auto &s : b) {
            nodes += (long long)s.IM * s.JM * s.KM;
            nin += (long long)s.inlets.size(); nout += (long long)s.outlets.size(); nwall += (long long)s.walls.size();
        }
        const long long v[9] = {(long long)b.size(), c.ng, nin, nout, nwall, (long long)c.periodics.size(),
                                (long long)c.interiors.size(), (long long)c.mixing.size(), nodes};
        for (int q = 0; q < 9; q++) info[q] = v[q];
        if (nodes_out) {
            if (cap < 3 * nodes) throw std::invalid_argument("node buffer too short");
            long long o = 0;
            for (auto &s : b)
                for (size_t q = 0; q < s.x.size(); q++) {
                    nodes_out[o++] = s.x[q]; nodes_out[o++] = s.y[q]; nodes_out[o++] = s.z[q];
                }
        }
    });
}

int gb_solver_create_levels(const char *const *case_dirs, int n_solves, int precision, int max_levels, gb_solver **out)
{
    if (!case_dirs || n_solves < 1 || !out) { g_err = "bad arguments"; return GB_ERR_ARG; }
    *out = nullptr;
    return guard([&] {
        std::vector<std::string> d;
        for (int i = 0; i < n_solves; i++) d.push_back(case_dirs[i] ? case_dirs[i] : "");
        auto h = new gb_solver;
        try {
            h->s = gbt::make_solver(d, precision, max_levels);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

int gb_solver_create(const char *const *case_dirs, int n_solves, int precision, gb_solver **out)
{
    return gb_solver_create_levels(case_dirs, n_solves, precision, 2, out);
}

int gb_solver_destroy(gb_solver *h)
{
    if (!h) return GB_OK;
    if (h->t0) cudaEventDestroy(h->t0);
    if (h->t1) cudaEventDestroy(h->t1);
    delete h;
    return GB_OK;
}

int gb_dims(gb_solver *h, int solve, int level, int out[4])
{
    NEED(h); LEVEL(h, level);
    if (solve < 0 || solve >= h->s->nsolve) { g_err = "solve out of range"; return GB_ERR_ARG; }
    return guard([&] { h->s->dims(solve, level, out); });
}

int gb_num_blocks(gb_solver *h, int *n_cases, int *n_blocks)
{
    NEED(h);
    if (n_cases) *n_cases = h->s->ncase;
    if (n_blocks) *n_blocks = h->s->nsolve;
    return GB_OK;
}

int gb_case_blocks(gb_solver *h, int solve, int out[2])
{
    NEED(h);
    if (!out) { g_err = "null buffer"; return GB_ERR_ARG; }
    if (solve < 0 || solve >= h->s->ncase) { g_err = "solve out of range"; return GB_ERR_ARG; }
    out[0] = h->s->case_first[solve];
    out[1] = h->s->case_nblk[solve];
    return GB_OK;
}

int gb_init_uniform(gb_solver *h) { NEED(h); return guard([&] { h->s->init_uniform(); }); }
int gb_resflux(gb_solver *h, int level) { NEED(h); LEVEL(h, level); return guard([&] { h->s->resflux(level); }); }
int gb_time_marching(gb_solver *h, int level) { NEED(h); LEVEL(h, level); return guard([&] { h->s->time_marching(level); }); }
int gb_primitive_vars(gb_solver *h, int level) { NEED(h); LEVEL(h, level); return guard([&] { h->s->primitive_vars(level); }); }
int gb_limit_vars(gb_solver *h, int level) { NEED(h); LEVEL(h, level); return guard([&] { h->s->limit_vars(level); }); }
int gb_corner_treatment(gb_solver *h, int level) { NEED(h); LEVEL(h, level); return guard([&] { h->s->corner_treatment(level); }); }
int gb_restrict(gb_solver *h) { NEED(h); return guard([&] { h->s->restrict_to_coarse(); }); }
int gb_interpolate(gb_solver *h, int init) { NEED(h); return guard([&] { h->s->interpolate(init); }); }
int gb_delta_cons(gb_solver *h) { NEED(h); return guard([&] { h->s->delta_cons(); }); }
int gb_set_use_force(gb_solver *h, int level, int on) { NEED(h); LEVEL(h, level); return guard([&] { h->s->set_use_force(level, on != 0); }); }
int gb_solver_step(gb_solver *h) { NEED(h); return guard([&] { h->s->solver_step(); }); }

int gb_res_calculate(gb_solver *h, int level, double *out)
{
    NEED(h); LEVEL(h, level);
    return guard([&] {
        h->s->res_calculate(level);
        if (out) {
            std::vector<gbt::SolveState> st(h->s->ncase);
            h->s->states(st.data());
            for (int s = 0; s < h->s->ncase; s++)
                for (int c = 0; c < 5; c++) out[s * 5 + c] = st[s].res[c];
        }
    });
}

int gb_res_calculate_noalloc(gb_solver *h, int level, double *out)
{
    NEED(h); LEVEL(h, level);
    if (h->s->nsolve > GB_NOALLOC_MAX_SOLVES) {
        g_err = "gb_res_calculate_noalloc: the batch has more blocks than the static scratch holds (GB_NOALLOC_MAX_SOLVES)";
        return GB_ERR_ARG;
    }
    return guard([&] { h->s->res_calculate_static(level, out); });
}

int gb_integrals(gb_solver *h, int level, double *out)
{
    NEED(h); LEVEL(h, level);
    return guard([&] {
        h->s->integrals(level);
        if (out) {
            std::vector<gbt::SolveState> st(h->s->ncase);
            h->s->states(st.data());
            for (int s = 0; s < h->s->ncase; s++) {
                out[s * 5 + 0] = st[s].m_in; out[s * 5 + 1] = st[s].m_out; out[s * 5 + 2] = st[s].pr;
                out[s * 5 + 3] = st[s].eff; out[s * 5 + 4] = st[s].m_ratio;
            }
        }
    });
}

int gb_mass_flow_imposed(gb_solver *h) { NEED(h); return guard([&] { h->s->mass_flow_imposed(); }); }

int gb_get_outlet_pressure(gb_solver *h, double *out)
{
    NEED(h);
    if (!out) { g_err = "null buffer"; return GB_ERR_ARG; }
    return guard([&] { h->s->outlet_pressure(out); });
}

int gb_iterate(gb_solver *h, int n, double *hist)
{
    NEED(h);
    if (n < 0) { g_err = "negative iteration count"; return GB_ERR_ARG; }
    return guard([&] { h->s->iterate(n, hist); });
}

int gb_get_status(gb_solver *h, int *out)
{
    NEED(h);
    if (!out) { g_err = "null buffer"; return GB_ERR_ARG; }
    return guard([&] {
        std::vector<gbt::SolveState> st(h->s->ncase);
        h->s->states(st.data());
        for (int s = 0; s < h->s->ncase; s++) out[s] = st[s].status;
    });
}

long gb_get_field(gb_solver *h, int solve, int level, const char *name, double *out, long cap)
{
    NEED(h);
    if (!name || !out) { g_err = "null argument"; return GB_ERR_ARG; }
    long r = -1;
    int rc = guard([&] { r = h->s->get_field(solve, level, name, out, cap); });
    if (rc) return rc;
    if (r < 0) { g_err = std::string("unknown field, level, solve or short buffer: ") + name; return GB_ERR_ARG; }
    return r;
}

int gb_set_cv(gb_solver *h, int solve, int level, const double *cv, long n)
{
    NEED(h);
    if (!cv) { g_err = "null buffer"; return GB_ERR_ARG; }
    return guard([&] { h->s->set_cv(solve, level, cv, n); });
}

static std::string path_or_empty(const char *p) { return p ? std::string(p) : std::string(); }
int gb_read_restart(gb_solver *h, int solve, const char *path)
{
    NEED(h);
    return guard([&] { h->s->read_restart(solve, path_or_empty(path)); });
}
int gb_write_restart(gb_solver *h, int solve, const char *path)
{
    NEED(h);
    return guard([&] { h->s->write_restart(solve, path_or_empty(path)); });
}
int gb_write_solution(gb_solver *h, int solve, const char *path)
{
    NEED(h);
    return guard([&] { h->s->write_solution(solve, path_or_empty(path)); });
}

int gb_sync(gb_solver *h)
{
    NEED(h);
    return guard([&] { gbt::check_cuda(cudaStreamSynchronize(h->s->stream), "cudaStreamSynchronize"); });
}

int gb_profile_begin(gb_solver *h) { NEED(h); return guard([&] { h->s->profile_begin(); }); }

int gb_profile_end(gb_solver *h, char *buf, int buflen)
{
    NEED(h);
    if (!buf || buflen < 1) { g_err = "null buffer"; return GB_ERR_ARG; }
    return guard([&] {
        std::string r = h->s->profile_end();
        std::strncpy(buf, r.c_str(), (size_t)buflen - 1);
        buf[buflen - 1] = 0;
    });
}

int gb_sweep_tuning(gb_solver *h, int level, int out[2])
{
    NEED(h); LEVEL(h, level);
    if (!out) { g_err = "null buffer"; return GB_ERR_ARG; }
    h->s->sweep_shape(level, out);
    return GB_OK;
}

int gb_face_staging(gb_solver *h, int level, int *tma)
{
    NEED(h); LEVEL(h, level);
    if (!tma) { g_err = "null buffer"; return GB_ERR_ARG; }
    *tma = h->s->face_staged(level) ? 1 : 0;
    return GB_OK;
}

int gb_set_graphs(gb_solver *h, int enable) { NEED(h); h->s->use_graphs = enable != 0; return GB_OK; }

int gb_timer_start(gb_solver *h)
{
    NEED(h);
    return guard([&] {
        if (!h->t0) { gbt::check_cuda(cudaEventCreate(&h->t0), "cudaEventCreate"); gbt::check_cuda(cudaEventCreate(&h->t1), "cudaEventCreate"); }
        gbt::check_cuda(cudaEventRecord(h->t0, h->s->stream), "cudaEventRecord");
    });
}

int gb_timer_stop(gb_solver *h, float *ms)
{
    NEED(h);
    if (!h->t0) { g_err = "timer not started"; return GB_ERR_ARG; }
    return guard([&] {
        gbt::check_cuda(cudaEventRecord(h->t1, h->s->stream), "cudaEventRecord");
        gbt::check_cuda(cudaEventSynchronize(h->t1), "cudaEventSynchronize");
        gbt::check_cuda(cudaEventElapsedTime(ms, h->t0, h->t1), "cudaEventElapsedTime");
    });
}

int gb_start_from_fine_state(gb_solver *h)
{
    NEED(h);
    return guard([&] { h->s->start_from_fine_state(); });
}

#define NEEDW(x) do { if (!(x) || !(x)->w) { g_err = "null warm-start handle"; return GB_ERR_ARG; } } while (0)

int gb_ws_create(unsigned seed, gb_warmstart **out)
{
    if (!out) { g_err = "null out"; return GB_ERR_ARG; }
    *out = nullptr;
    return guard([&] {
        std::unique_ptr<gb_warmstart> p(new gb_warmstart);
        p->w.reset(new gbt::WarmStart(seed));
        *out = p.release();
    });
}
int gb_ws_destroy(gb_warmstart *w)
{
    delete w;
    return GB_OK;
}
long gb_ws_num_params(void) { return (long)gbt::WarmStart::n_params(); }
int gb_ws_add_solves(gb_warmstart *w, gb_solver *h, const float *params)
{
    NEEDW(w); NEED(h);
    if (!params) { g_err = "null parameters"; return GB_ERR_ARG; }
    return guard([&] { w->w->add_solves(*h->s, params); });
}
long long gb_ws_samples(gb_warmstart *w) { return (w && w->w) ? w->w->samples() : -1; }
int gb_ws_train(gb_warmstart *w, int steps, int batch, float lr, float *loss)
{
    NEEDW(w);
    if (steps < 0 || batch <= 0) { g_err = "bad steps or batch"; return GB_ERR_ARG; }
    return guard([&] {
        const float l = w->w->train(steps, batch, lr);
        if (loss) *loss = l;
    });
}
int gb_ws_apply(gb_warmstart *w, gb_solver *h, const float *params, int *used, double *res_warm, double *res_uniform)
{
    NEEDW(w); NEED(h);
    if (!params || !used) { g_err = "null buffer"; return GB_ERR_ARG; }
    return guard([&] { w->w->apply(*h->s, params, used, res_warm, res_uniform); });
}
int gb_ws_get_params(gb_warmstart *w, float *out)
{
    NEEDW(w);
    if (!out) { g_err = "null buffer"; return GB_ERR_ARG; }
    return guard([&] { w->w->get_params(out); });
}
int gb_ws_set_params(gb_warmstart *w, const float *in)
{
    NEEDW(w);
    if (!in) { g_err = "null buffer"; return GB_ERR_ARG; }
    return guard([&] { w->w->set_params(in); });
}
int gb_ws_get_norm(gb_warmstart *w, float *out)
{
    NEEDW(w);
    if (!out) { g_err = "null buffer"; return GB_ERR_ARG; }
    w->w->get_norm(out);
    return GB_OK;
}
int gb_ws_set_norm(gb_warmstart *w, const float *in)
{
    NEEDW(w);
    if (!in) { g_err = "null buffer"; return GB_ERR_ARG; }
    return guard([&] { w->w->set_norm(in); });
}
int gb_ws_forward(gb_warmstart *w, const float *feat, int n, float *y)
{
    NEEDW(w);
    if (!feat || !y || n <= 0) { g_err = "bad arguments"; return GB_ERR_ARG; }
    return guard([&] { w->w->forward(feat, n, y); });
}
int gb_ws_forward_backward(gb_warmstart *w, const float *feat, const float *target, int n, float *loss, float *grad)
{
    NEEDW(w);
    if (!feat || !target || !grad || n <= 0) { g_err = "bad arguments"; return GB_ERR_ARG; }
    return guard([&] {
        const float l = w->w->forward_backward(feat, target, n, grad);
        if (loss) *loss = l;
    });
}
int gb_ws_benchmark(gb_warmstart *w, long long n, int iters, float *ms_forward, float *ms_step, float *ms_infer,
                    double *max_diff)
{
    NEEDW(w);
    if (!ms_forward || !ms_step || !ms_infer) { g_err = "null buffer"; return GB_ERR_ARG; }
    return guard([&] { w->w->benchmark(n, iters, ms_forward, ms_step, ms_infer, max_diff); });
}

}  // extern "C"
