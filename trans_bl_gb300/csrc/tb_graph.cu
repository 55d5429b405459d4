// RK4 steps replayed as CUDA graphs, and ensembles of independent runs.
//
// The reference advances one run per MPI job and synchronises the ranks
// after every V-cycle of its Poisson solve (poisson_par.f:31-55, the
// allreduce of verifica_poi).  Here a whole step, the four stages of
// main_par.f:165-254, is recorded once into a CUDA graph and replayed:
//   - each stage's Poisson correction loop is a conditional WHILE node whose
//     body (V-cycles, correction, FP64 defect, per-mode test) decides on the
//     device whether to run again, so no host round trip remains in a step;
//   - the values that change from step to step are read from device memory
//     that the host refreshes before each replay: the wall-forcing amplitudes
//     of stages 1 and 3 (ts2d_pert, main_par.f:1613-1650) and the validity of
//     each stage's warm-start history;
//   - the per-solve statistics are copied aside inside the graph and read
//     once after the step.
// An ensemble records the steps of several contexts, of any sizes, as
// parallel branches of one graph, so one launch advances every run and the
// small runs fill the device together.
#include "tb_internal.h"
#include <algorithm>
#include <cstring>
#include <new>

namespace {

int prepare(tb_ctx* c) {
    int r;
    if ((r = tb_spectral_prepare(c))) return r;
    const int K = c->g.K;
    if (!c->d_fct) TB_CUDA(cudaMalloc(&c->d_fct, 8 * sizeof(double)));
    if (!c->gsnap) TB_CUDA(cudaMalloc(&c->gsnap, (size_t)8 * K * sizeof(int)));
    if (!c->gerr) TB_CUDA(cudaMalloc(&c->gerr, (size_t)4 * K * sizeof(double)));
    if (!c->body_stream) TB_CUDA(cudaStreamCreateWithFlags(&c->body_stream, cudaStreamNonBlocking));
    return TB_OK;
}

bool graph_form(const tb_ctx* c) { return c->cfg.precision == TB_FORM_MIXED && c->mixed; }

// Record the four stages of c onto c->stream, which is capturing; the
// launch counter keeps only executed launches, so the recorded ones are
// taken back out and split into those outside and inside the WHILE bodies.
int record(tb_ctx* c) {
    const long long l0 = c->launches;
    for (long long& b : c->g_body) b = 0;
    for (long long& b : c->g_learn) b = 0;
    c->capturing = true;
    int r = tb_graph_record_step(c);
    c->capturing = false;
    const long long body = c->g_body[0] + c->g_body[1] + c->g_body[2] + c->g_body[3] + c->g_learn[0] + c->g_learn[1] +
                           c->g_learn[2] + c->g_learn[3];
    c->g_outer = (c->launches - l0) - body;
    c->launches = l0;
    return r;
}

int end_capture(cudaStream_t s, cudaGraph_t* g, int r) {
    cudaError_t e = cudaStreamEndCapture(s, g);
    if (r) {
        if (*g) cudaGraphDestroy(*g);
        *g = nullptr;
        (void)cudaGetLastError();
        return r;
    }
    if (e != cudaSuccess) {
        if (*g) cudaGraphDestroy(*g);
        *g = nullptr;
        tb_set_error("step graph: recording failed: %s", cudaGetErrorString(e));
        return TB_ERR_CUDA;
    }
    return TB_OK;
}

int capture_one(tb_ctx* c) {
    int r;
    if ((r = prepare(c))) return r;
    TB_CUDA(cudaStreamSynchronize(c->stream));
    TB_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
    r = record(c);
    cudaGraph_t g = nullptr;
    if ((r = end_capture(c->stream, &g, r))) return r;
    cudaError_t e = cudaGraphInstantiate(&c->gexec, g, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        c->gexec = nullptr;
        tb_set_error("step graph: instantiate: %s", cudaGetErrorString(e));
        return TB_ERR_CUDA;
    }
    c->graph = g;
    return TB_OK;
}

// Statistics of one replayed step: the four solves in stage order, as the
// host-launched step records them, and the kernels that ran (the WHILE body
// of a solve runs as often as its slowest mode needed corrections).
int read_back(tb_ctx* c, const int* hs, const double* he) {
    const int K = c->g.K;
    int rc = TB_OK;
    long long n = c->g_outer;
    for (int s = 0; s < 4; s++) {
        const int* h = hs + (size_t)2 * K * s;
        int iters = 0;
        for (int k = 0; k < K; k++) {
            int vc = h[2 * k + 1];
            if (vc < 0) vc = -vc - 1;
            iters = std::max(iters, vc);
        }
        n += c->g_body[s] * iters;
        int r = tb_mixed_absorb_stats(c, h, he + (size_t)K * s);
        if (r && !rc) rc = r;
    }
    // the learned correction's kernels ran in the replays whose gate opened
    LearnSolve* L = tb_learn_solve(c);
    if (L && L->gated && L->gate) {
        int g[32];
        if (cudaMemcpy(g, L->gate, sizeof g, cudaMemcpyDeviceToHost) == cudaSuccess)
            for (int s = 0; s < 4; s++) {
                n += c->g_learn[s] * (g[8 * s + 2] - c->g_learn_seen[s]);
                c->g_learn_seen[s] = g[8 * s + 2];
            }
    }
    c->launches += n;
    return rc;
}

}  // namespace

int tb_graph_record_step(tb_ctx* c) {
    // the step index only reaches the forcing amplitudes and the warm-start
    // bookkeeping, both of which a replay takes from device memory
    for (int s = 1; s <= 4; s++) {
        int r = tb_rk_stage(c, s, 0);
        if (r) return r;
    }
    return TB_OK;
}

int tb_graph_pre(tb_ctx* c, int t, cudaStream_t s) {
    double f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    tb_ts_pert_fct(c, t, 0.5, f);
    tb_ts_pert_fct(c, t, 1.0, f + 4);
    // from pageable memory: the source is staged before the call returns
    TB_CUDA(cudaMemcpyAsync(c->d_fct, f, sizeof f, cudaMemcpyHostToDevice, s));
    return c->cfg.warm_start ? tb_mixed_graph_pre(c, t, s) : TB_OK;
}

int tb_graph_post(tb_ctx* c, const int* hs, const double* he) { return read_back(c, hs, he); }

void tb_graph_reset(tb_ctx* c) {
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    if (c->graph) cudaGraphDestroy(c->graph);
    c->gexec = nullptr;
    c->graph = nullptr;
    c->graph_gen++;
}

void tb_graph_free(tb_ctx* c) {
    tb_graph_reset(c);
    if (c->d_fct) cudaFree(c->d_fct);
    if (c->gsnap) cudaFree(c->gsnap);
    if (c->gerr) cudaFree(c->gerr);
    if (c->body_stream) cudaStreamDestroy(c->body_stream);
    c->d_fct = nullptr; c->gsnap = nullptr; c->gerr = nullptr; c->body_stream = nullptr;
}

bool tb_graph_usable(const tb_ctx* c) {
    // collecting training crops draws crop positions on the host per solve
    LearnSolve* L = tb_learn_solve(const_cast<tb_ctx*>(c));
    return c->cfg.step_graph && graph_form(c) && !c->prof && !(L && L->sample);
}

int tb_graph_step(tb_ctx* c, int t) {
    int r;
    if (!c->gexec && (r = capture_one(c))) return r;
    if ((r = tb_graph_pre(c, t, c->stream))) return r;
    TB_CUDA(cudaGraphLaunch(c->gexec, c->stream));
    const int K = c->g.K;
    std::vector<int> hs((size_t)8 * K);
    std::vector<double> he((size_t)4 * K);
    TB_CUDA(cudaMemcpyAsync(hs.data(), c->gsnap, hs.size() * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TB_CUDA(cudaMemcpyAsync(he.data(), c->gerr, he.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    TB_CUDA(cudaStreamSynchronize(c->stream));
    tb_mixed_graph_post(c, t);
    if ((r = tb_tc_check(c))) return r;
    return tb_graph_post(c, hs.data(), he.data());
}

// ---- ensembles ------------------------------------------------------------
struct tb_ensemble {
    std::vector<tb_ctx*> m;
    std::vector<long long> gen;     // members' graph generation at recording
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t x = nullptr;
    std::vector<std::vector<int>> hs;
    std::vector<std::vector<double>> he;
};

namespace {

void ens_drop(tb_ensemble* e) {
    if (e->x) cudaGraphExecDestroy(e->x);
    if (e->g) cudaGraphDestroy(e->g);
    e->x = nullptr;
    e->g = nullptr;
}

// Every member's step as a branch forked from and joined back into the
// ensemble's stream.  A member that fails to record is still joined, so the
// capture can be closed before the error is returned.
int ens_capture(tb_ensemble* e) {
    int r;
    for (tb_ctx* c : e->m)
        if ((r = prepare(c))) return r;
    TB_CUDA(cudaDeviceSynchronize());
    TB_CUDA(cudaStreamBeginCapture(e->s, cudaStreamCaptureModeRelaxed));
    int rc = TB_OK;
    cudaError_t ce = cudaEventRecord(e->fork, e->s);
    for (size_t i = 0; i < e->m.size() && ce == cudaSuccess; i++) {
        tb_ctx* c = e->m[i];
        ce = cudaStreamWaitEvent(c->stream, e->fork, 0);
        if (ce != cudaSuccess) break;
        if (!rc) rc = record(c);
        ce = cudaEventRecord(e->join[i], c->stream);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(e->s, e->join[i], 0);
    }
    if (!rc && ce != cudaSuccess) {
        tb_set_error("ensemble: recording: %s", cudaGetErrorString(ce));
        rc = TB_ERR_CUDA;
    }
    cudaGraph_t g = nullptr;
    if ((r = end_capture(e->s, &g, rc))) return r;
    cudaError_t ie = cudaGraphInstantiate(&e->x, g, 0);
    if (ie != cudaSuccess) {
        cudaGraphDestroy(g);
        e->x = nullptr;
        tb_set_error("ensemble: instantiate: %s", cudaGetErrorString(ie));
        return TB_ERR_CUDA;
    }
    e->g = g;
    for (size_t i = 0; i < e->m.size(); i++) e->gen[i] = e->m[i]->graph_gen;
    return TB_OK;
}

}  // namespace

extern "C" {

int tb_ensemble_create(tb_ctx* const* members, int n, tb_ensemble** out) {
    if (!out) { tb_set_error("null output pointer"); return TB_ERR_ARG; }
    *out = nullptr;
    if (!members || n < 1) { tb_set_error("ensemble needs at least one member"); return TB_ERR_ARG; }
    for (int i = 0; i < n; i++) {
        tb_ctx* c = members[i];
        if (!c) { tb_set_error("ensemble member %d is null", i); return TB_ERR_ARG; }
        for (int j = 0; j < i; j++)
            if (members[j] == c) { tb_set_error("ensemble member %d repeats member %d", i, j); return TB_ERR_ARG; }
        if (!c->have_coefs) { tb_set_error("ensemble member %d: coefficients not set", i); return TB_ERR_STATE; }
        if (!graph_form(c)) { tb_set_error("ensemble member %d: the mixed form is required", i); return TB_ERR_ARG; }
    }
    tb_ensemble* e = new (std::nothrow) tb_ensemble();
    if (!e) return TB_ERR_NOMEM;
    e->m.assign(members, members + n);
    e->gen.assign(n, -1);
    e->join.assign(n, nullptr);
    e->hs.resize(n);
    e->he.resize(n);
    for (int i = 0; i < n; i++) {
        e->hs[i].resize((size_t)8 * members[i]->g.K);
        e->he[i].resize((size_t)4 * members[i]->g.K);
    }
    cudaError_t ce = cudaStreamCreateWithFlags(&e->s, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
    for (int i = 0; i < n && ce == cudaSuccess; i++) ce = cudaEventCreateWithFlags(&e->join[i], cudaEventDisableTiming);
    if (ce != cudaSuccess) {
        tb_set_error("ensemble: %s", cudaGetErrorString(ce));
        tb_ensemble_destroy(e);
        return TB_ERR_CUDA;
    }
    *out = e;
    return TB_OK;
}

int tb_ensemble_step(tb_ensemble* e, const int* t) {
    if (!e || !t) { tb_set_error("null argument"); return TB_ERR_ARG; }
    int r;
    bool stale = !e->x;
    for (size_t i = 0; i < e->m.size(); i++) {
        if (e->m[i]->prof) { tb_set_error("ensemble member %zu is profiling", i); return TB_ERR_STATE; }
        LearnSolve* L = tb_learn_solve(e->m[i]);
        if (L && L->sample) { tb_set_error("ensemble member %zu is collecting training crops", i); return TB_ERR_STATE; }
        stale = stale || e->gen[i] != e->m[i]->graph_gen;
    }
    if (stale) {
        ens_drop(e);
        if ((r = ens_capture(e))) return r;
    }
    // members' own streams may still hold work from single steps
    for (size_t i = 0; i < e->m.size(); i++) TB_CUDA(cudaStreamSynchronize(e->m[i]->stream));
    for (size_t i = 0; i < e->m.size(); i++)
        if ((r = tb_graph_pre(e->m[i], t[i], e->s))) return r;
    TB_CUDA(cudaGraphLaunch(e->x, e->s));
    for (size_t i = 0; i < e->m.size(); i++) {
        tb_ctx* c = e->m[i];
        TB_CUDA(cudaMemcpyAsync(e->hs[i].data(), c->gsnap, e->hs[i].size() * sizeof(int), cudaMemcpyDeviceToHost, e->s));
        TB_CUDA(cudaMemcpyAsync(e->he[i].data(), c->gerr, e->he[i].size() * sizeof(double), cudaMemcpyDeviceToHost, e->s));
    }
    TB_CUDA(cudaStreamSynchronize(e->s));
    int rc = TB_OK;
    for (size_t i = 0; i < e->m.size(); i++) {
        r = tb_tc_check(e->m[i]);
        if (r && !rc) rc = r;
        tb_mixed_graph_post(e->m[i], t[i]);
        r = tb_graph_post(e->m[i], e->hs[i].data(), e->he[i].data());
        if (r && !rc) rc = r;
    }
    return rc;
}

int tb_ensemble_destroy(tb_ensemble* e) {
    if (!e) return TB_OK;
    if (e->s) cudaStreamSynchronize(e->s);
    ens_drop(e);
    for (cudaEvent_t ev : e->join)
        if (ev) cudaEventDestroy(ev);
    if (e->fork) cudaEventDestroy(e->fork);
    if (e->s) cudaStreamDestroy(e->s);
    delete e;
    return TB_OK;
}

}  // extern "C"
