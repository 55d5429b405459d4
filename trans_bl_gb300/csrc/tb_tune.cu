// Launch shapes of the stage's batched kernels, picked per context by
// timing the candidates on the context's own grid (CUDA events on its
// stream): warps per block of the x-line solves, threads per block of the
// y-line solves, and resident blocks per SM of the tensor-core passes of the
// nonlinear terms.  The timed launches write only the stage's scratch fields
// (tmp), so the state is untouched.  Recorded step graphs are dropped, since
// they hold the previous shapes.
#include "tb_internal.h"
#include <cstring>

namespace {

template <class F>
int time_ms(tb_ctx* c, F&& launch, float* ms) {
    cudaEvent_t a, b;
    TB_CUDA(cudaEventCreate(&a));
    TB_CUDA(cudaEventCreate(&b));
    int r = TB_OK;
    for (int w = 0; w < 2 && !r; w++) r = launch();   // warm-up
    if (!r) {
        const int n = 5;
        cudaEventRecord(a, c->stream);
        for (int q = 0; q < n && !r; q++) r = launch();
        cudaEventRecord(b, c->stream);
        if (!r && cudaEventSynchronize(b) == cudaSuccess) {
            cudaEventElapsedTime(ms, a, b);
            *ms /= n;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (!r) TB_CUDA(cudaGetLastError());
    return r;
}

// The candidate of `vals` with the smallest time of `launch` after `set`.
template <class S, class F>
int pick(tb_ctx* c, const int* vals, int n, S&& set, F&& launch, int* best, float* best_ms) {
    *best = vals[0];
    *best_ms = 1e30f;
    for (int q = 0; q < n; q++) {
        set(vals[q]);
        float ms = 0.f;
        int r = time_ms(c, launch, &ms);
        if (r) return r;
        if (ms < *best_ms) { *best_ms = ms; *best = vals[q]; }
    }
    set(*best);
    return TB_OK;
}

}  // namespace

extern "C" int tb_autotune(tb_ctx* c, tb_tune_result* out) {
    if (!c || !out) { tb_set_error("null argument"); return TB_ERR_ARG; }
    if (!c->have_coefs) { tb_set_error("coefficients not set (tb_set_coefs)"); return TB_ERR_STATE; }
    std::memset(out, 0, sizeof *out);
    int r;
    if ((r = tb_spectral_prepare(c))) return r;
    TB_CUDA(cudaStreamSynchronize(c->stream));
    const long long l0 = c->launches;
    cplx** t = c->tmp;
    XJob xj[3] = {{c->ux, t[20], XOP_D1}, {c->uy, t[21], XOP_D1}, {c->wz, t[22], XOP_D2}};
    const int xv[2] = {1, 2};
    if ((r = pick(c, xv, 2, [&](int v) { c->tune_xw = v; }, [&]() { return tb_launch_xlines(c, xj, 3); },
                  &out->xline_warps, &out->xline_ms)))
        return r;
    YJob yj[3] = {{c->ux, t[20], YOP_D1}, {c->uy, t[21], YOP_D1FV}, {c->wz, t[22], YOP_D2}};
    const int yv[3] = {32, 64, 128};
    if ((r = pick(c, yv, 3, [&](int v) { c->tune_yt = v; }, [&]() { return tb_launch_ylines(c, yj, 3); },
                  &out->yline_threads, &out->yline_ms)))
        return r;
    if (c->cfg.precision == TB_FORM_MIXED && c->nl_tensor && c->g.P >= 16 && c->g.P <= 128) {
        const int nv[4] = {1, 2, 4, 8};   // capped by each shape's resource limit inside the launcher
        if ((r = pick(c, nv, 4, [&](int v) { c->tune_nl = v; }, [&]() { return tb_launch_nlterms(c, t[20], t[21], t[22]); },
                      &out->nl_blocks_per_sm, &out->nl_ms)))
            return r;
    }
    if (c->cfg.precision == TB_FORM_PLAIN_FP64 && c->pl_fc) {
        // warps per line of the plain form's fine-level sweeps (the solve
        // rebuilds its work arrays from uy, so the timed sweeps change nothing)
        const int multi[3] = {0, 1, 2}, single[2] = {1, 2};
        int b3 = 0, b1 = 0;
        if ((r = tb_plain_tune(c, 0, 3, multi, 3, &b3, &out->plain_multi_ms))) return r;
        if ((r = tb_plain_tune(c, 0, 1, single, 2, &b1, &out->plain_single_ms))) return r;
        out->plain_line_warps_multi = 1 << b3;
        out->plain_line_warps_single = 1 << b1;
    }
    c->launches = l0;   // tuning launches are not the run's work
    tb_graph_reset(c);
    TB_CUDA(cudaStreamSynchronize(c->stream));
    return tb_tc_check(c);
}

// ---------------------------------------------------------------------------
// FP64 throughput of this GPU, measured: the denominator of the FP64-pipe
// rooflines of the stage's FP64 kernels.  Every thread runs 8 independent
// FMA chains (x = x * a + b, a fused multiply-add, counted as 2 flops) over
// a grid of 8 blocks of 256 threads per SM; the time is taken with CUDA events.
namespace {
__global__ void k_fp64_peak(double* out, int iters, double a, double b) {
    double x[8];
#pragma unroll
    for (int q = 0; q < 8; q++) x[q] = 1.0 + 1e-3 * (threadIdx.x + q);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int q = 0; q < 8; q++) x[q] = fma(x[q], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 8; q++) s += x[q];
    out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = s;
}
}  // namespace

extern "C" int tb_fp64_peak(double* tflops) {
    if (!tflops) { tb_set_error("null argument"); return TB_ERR_ARG; }
    int dev = 0, sms = 0;
    TB_CUDA(cudaGetDevice(&dev));
    TB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = 8 * sms, threads = 256, iters = 4096;
    double* buf = nullptr;
    TB_CUDA(cudaMalloc(&buf, (size_t)blocks * threads * sizeof(double)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fp64_peak<<<blocks, threads>>>(buf, iters, 0.999999, 1e-7);   // warm-up
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(e0);
        k_fp64_peak<<<blocks, threads>>>(buf, iters, 0.999999, 1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    if (e != cudaSuccess) { tb_set_error("tb_fp64_peak: %s", cudaGetErrorString(e)); return TB_ERR_CUDA; }
    *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
    return TB_OK;
}
