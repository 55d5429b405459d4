// tb_api.cu -- the C ABI of the library (include/transbl.h): context life
// cycle, state transfer, the RK4 stage and the per-subroutine mirrors.
#include "tb_internal.h"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

static const double PI = 3.141592653589793;

namespace {

int check_cfg(const tb_config* c) {
    if (!c) { tb_set_error("null config"); return TB_ERR_ARG; }
    int msh = c->msh;
    if (msh < 2 || msh > TB_MAX_MSH) { tb_set_error("msh must be in [2, %d]", TB_MAX_MSH); return TB_ERR_ARG; }
    int step = 1 << (msh - 1);
    if (c->nx < 16 || (c->nx - 1) % step) { tb_set_error("nx-1 must be a multiple of 2^(msh-1) and nx >= 16 (main_par.f:90)"); return TB_ERR_ARG; }
    if (c->ny < (1 << msh) || c->ny < 16 || (c->ny - 1) % step) { tb_set_error("ny-1 must be a multiple of 2^(msh-1) and ny >= 2^msh (main_par.f:114-124)"); return TB_ERR_ARG; }
    if (c->ny > 512) { tb_set_error("ny > 512 not supported"); return TB_ERR_ARG; }
    // the coarsest level's stencils reach 4 points in from each x-border and
    // 3 rows up from the wall (coef_border, poisson_par.f:229-540)
    if ((c->nx - 1) / step + 1 < 6 || (c->ny - 1) / step + 1 < 5) {
        tb_set_error("the coarsest multigrid level needs >= 6 points in x and >= 5 in y; lower msh");
        return TB_ERR_ARG;
    }
    int P = c->kphys;
    if (P < 2 || P > 128 || (P & (P - 1))) { tb_set_error("kphys must be a power of two in [2, 128]"); return TB_ERR_ARG; }
    if (c->kfour < 1 || c->kfour > P / 2 || c->kfour > TB_MAX_K) { tb_set_error("kfour must be in [1, kphys/2]"); return TB_ERR_ARG; }
    if (c->i0 < 2 || c->i0 > c->i3 || c->i3 > c->i4 || c->i4 > c->nx) { tb_set_error("need 2 <= i0 <= i3 <= i4 <= nx"); return TB_ERR_ARG; }
    if (c->i1 < 1 || c->i2 <= c->i1 + 1 || c->i2 > c->nx) { tb_set_error("need 1 <= i1 < i2-1, i2 <= nx"); return TB_ERR_ARG; }
    if (c->stpp < 1 || c->omega == 0.0 || c->Re <= 0.0 || c->dx <= 0.0 || c->dy <= 0.0 || c->stf <= 0.0 || c->fac_y <= 0.0) {
        tb_set_error("non-positive physical parameter"); return TB_ERR_ARG;
    }
    if (c->max_vcycles < 1) { tb_set_error("max_vcycles must be >= 1"); return TB_ERR_ARG; }
    if (c->n_forced < 0 || c->n_forced > 4) { tb_set_error("n_forced must be in [0, 4]"); return TB_ERR_ARG; }
    if (c->precision != TB_FORM_PLAIN_FP64 && c->precision != TB_FORM_MIXED) { tb_set_error("unknown precision form"); return TB_ERR_ARG; }
    if (c->my_form < 0 || c->my_form > 4 || c->my_form == 3) { tb_set_error("my_form must be 0, 1, 2 or 4"); return TB_ERR_ARG; }
    if ((c->my_form == 1 || c->my_form == 2) && c->ibm) {
        tb_set_error("my_form %d (drv_gv/drv_gvth) has no immersed-boundary term", c->my_form);
        return TB_ERR_ARG;
    }
    if (c->my_form == 2 && !(c->Pr > 0.0)) { tb_set_error("my_form 2 needs Pr > 0"); return TB_ERR_ARG; }
    if (c->les_damping < 0 || c->les_damping > 3) { tb_set_error("les_damping must be 0..3"); return TB_ERR_ARG; }
    return TB_OK;
}

template <class T>
int dalloc(T** p, size_t n) {
    TB_CUDA(cudaMalloc((void**)p, n * sizeof(T)));
    TB_CUDA(cudaMemset(*p, 0, n * sizeof(T)));
    return TB_OK;
}

// Host <-> device copies of state fields, queued on the context's stream;
// readers wait once after all fields (tb_get_state, tb_get_wall).  Measured
// on a GB300 host with page-locked buffers (config 2, 608 MB per state):
// the copy engines move ~208 GB/s host to device and ~78 GB/s device to
// host (three streams instead of one changed neither); the SMs, loading
// and storing 16 bytes a thread over NVLink-C2C, ~208 and ~190 GB/s.  So a
// state whose host buffers the device can address moves by k_copy_state.
int copy_field(tb_ctx* c, void* dst, const void* src, size_t bytes, bool to_device) {
    TB_CUDA(cudaMemcpyAsync(dst, src, bytes, to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, c->stream));
    return TB_OK;
}
int up(tb_ctx* c, cplx* d, const double* h, size_t n) { return copy_field(c, d, h, n * sizeof(cplx), true); }
// Device -> host, complete on return (the mirrors hand the buffer back at once).
int down(tb_ctx* c, double* h, const cplx* d, size_t n) {
    int r = copy_field(c, h, d, n * sizeof(cplx), false);
    if (r) return r;
    TB_CUDA(cudaStreamSynchronize(c->stream));
    return TB_OK;
}
// Device -> host, queued only: the caller waits once after its last copy.
int down_async(tb_ctx* c, double* h, const cplx* d, size_t n) { return copy_field(c, h, d, n * sizeof(cplx), false); }
int finish(tb_ctx* c) {
    TB_CUDA(cudaGetLastError());
    TB_CUDA(cudaStreamSynchronize(c->stream));
    return tb_tc_check(c);
}
bool ready(tb_ctx* c) {
    if (!c) { tb_set_error("null context"); return false; }
    if (!c->have_coefs) { tb_set_error("coefficients not set (tb_set_coefs)"); return false; }
    return true;
}

}  // namespace

// Device staging of one physical-space field for the tb_f_to_p / tb_p_to_f
// mirrors: owned by the context (allocated on the context's device at first
// use, freed by tb_destroy).
static int phys_buf(tb_ctx* c, double** out) {
    if (!c->phys_stage) TB_CUDA(cudaMalloc(&c->phys_stage, tb_n2(c) * c->g.P * sizeof(double)));
    *out = c->phys_stage;
    return TB_OK;
}

extern "C" {

int tb_create(const tb_config* cfg, tb_ctx** out) {
    if (!out) { tb_set_error("null output pointer"); return TB_ERR_ARG; }
    *out = nullptr;
    int r = check_cfg(cfg);
    if (r) return r;
    tb_ctx* c = new (std::nothrow) tb_ctx();
    if (!c) return TB_ERR_NOMEM;
    std::memset(&c->stats, 0, sizeof c->stats);
    c->cfg = *cfg;
    TbGrid& g = c->g;
    g.nx = cfg->nx; g.ny = cfg->ny; g.K = cfg->kfour; g.P = cfg->kphys; g.msh = cfg->msh;
    g.ptsx[0] = g.nx; g.ptsy[0] = g.ny;
    for (int l = 1; l < g.msh; l++) { g.ptsx[l] = (g.ptsx[l - 1] + 1) / 2; g.ptsy[l] = (g.ptsy[l - 1] + 1) / 2; }
    size_t off = 0;
    for (int l = 0; l < g.msh; l++) { g.lvl_off[l] = off; off += (size_t)g.ptsx[l] * g.ptsy[l]; }
    g.lvl_elems = off;
    c->dt = (2.0 * PI) / cfg->omega / (double)cfg->stpp;
    c->dt2 = 0.5 * c->dt; c->dt6 = c->dt / 6.0;
    c->dz = (2.0 * PI) / ((double)g.P * cfg->beta);
    cudaGetDevice(&c->device);
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        tb_set_error("cudaStreamCreate failed: %s", cudaGetErrorString(cudaGetLastError()));
        delete c;
        return TB_ERR_CUDA;
    }
    size_t n3 = tb_n3(c);
    cplx** fields[] = {&c->ux, &c->uy, &c->uz, &c->wx, &c->wy, &c->wz, &c->wx1, &c->wy1, &c->wz1,
                       &c->dv1x, &c->dv1y, &c->dv1z, &c->dv2x, &c->dv2y, &c->dv2z};
    for (cplx** f : fields)
        if ((r = dalloc(f, n3))) { tb_destroy(c); return r == TB_ERR_CUDA ? TB_ERR_NOMEM : r; }
    for (int q = 0; q < 24; q++)
        if ((r = dalloc(&c->tmp[q], n3))) { tb_destroy(c); return TB_ERR_NOMEM; }
    if (cfg->my_form == 2) {   // the temperature, its RK storage, thb and nlterms_th's planes
        if ((r = dalloc(&c->th, n3)) || (r = dalloc(&c->th1, n3)) || (r = dalloc(&c->dv1t, n3)) ||
            (r = dalloc(&c->dv2t, n3)) || (r = dalloc(&c->thb, tb_n2(c))) ||
            (r = dalloc(&c->th_phys, (size_t)7 * g.P * tb_n2(c)))) {
            tb_destroy(c);
            return TB_ERR_NOMEM;
        }
    }
    if ((r = dalloc(&c->d2uydx2, (size_t)g.nx * g.K)) || (r = dalloc(&c->lapv, (size_t)g.nx * g.K))) { tb_destroy(c); return TB_ERR_NOMEM; }
    size_t n2 = tb_n2(c);
    c->h_uxb.assign(n2, 0.0); c->h_uyb.assign(n2, 0.0); c->h_wzb.assign(n2, 0.0);
    *out = c;
    return TB_OK;
}

int tb_destroy(tb_ctx* c) {
    if (!c) return TB_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    tb_mixed_free(c);
    void* ptrs[] = {c->ux, c->uy, c->uz, c->wx, c->wy, c->wz, c->wx1, c->wy1, c->wz1, c->dv1x, c->dv1y, c->dv1z, c->dv2x,
                    c->dv2y, c->dv2z, c->d2uydx2, c->lapv, c->uxb, c->uyb, c->wzb, c->duexmdx, c->bdfc, c->fcx, c->fcllx,
                    c->fcx2, c->fcllx2, c->th, c->th1, c->dv1t, c->dv2t, c->thb, c->th_phys, c->gibbs, c->delta_no, c->k2b2, c->tx1.a, c->tx1.g, c->tx1.ib, c->tx2.a, c->tx2.g, c->tx2.ib,
                    c->tfil.a, c->tfil.g, c->tfil.ib,
                    c->tx1.hf, c->tx1.hb, c->tx1.pf, c->tx1.pb, c->tx2.hf, c->tx2.hb, c->tx2.pf, c->tx2.pb,
                    c->tfil.hf, c->tfil.hb, c->tfil.pf, c->tfil.pb,
                    c->tx1.af, c->tx1.gf, c->tx1.ibf, c->tx1.hff, c->tx1.hbf, c->tx1.pff, c->tx1.pbf,
                    c->tx2.af, c->tx2.gf, c->tx2.ibf, c->tx2.hff, c->tx2.hbf, c->tx2.pff, c->tx2.pbf,
                    c->tfil.af, c->tfil.gf, c->tfil.ibf, c->tfil.hff, c->tfil.hbf, c->tfil.pff, c->tfil.pbf, c->ty1.a, c->ty1.g, c->ty1.ib, c->tyfv.a, c->tyfv.g, c->tyfv.ib,
                    c->ty2.a, c->ty2.g, c->ty2.ib, c->ry1.w, c->ry1.off, c->ry1.cnt, c->ryfv.w, c->ryfv.off, c->ryfv.cnt,
                    c->ry2.w, c->ry2.off, c->ry2.cnt, c->px.lu, c->pfc, c->psc, c->pfct, c->pdef,
                    c->pl_fc, c->pl_sc, c->pl_fct, c->pl_def, c->pl_tab, c->pl_maxsq, c->pstate, c->perr, c->pqdy2, c->pcoef, c->wcoef};
    for (void* p : ptrs) if (p) cudaFree(p);
    tb_graph_free(c);
    tb_learn_free(c);
    if (c->nl_phys) cudaFree(c->nl_phys);
    if (c->phys_stage) cudaFree(c->phys_stage);
    if (c->dft_tc) cudaFree(c->dft_tc);
    if (c->tc_err) cudaFree(c->tc_err);
    for (int q = 0; q < 24; q++) if (c->tmp[q]) cudaFree(c->tmp[q]);
    for (auto& r : c->prof_open) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    for (auto e : c->prof_pool) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return TB_OK;
}

int tb_set_coefs(tb_ctx* c, const double* blob) {
    if (!c || !blob) { tb_set_error("null argument"); return TB_ERR_ARG; }
    c->coefs.assign(blob, blob + tb_coef_count(c->g.msh));
    tb_graph_reset(c);
    tb_learn_free(c);   // its operator tables follow the coefficients
    int r;
    if ((r = tb_host_build_tables(c))) return r;
    if ((r = tb_poisson_setup(c))) return r;
    if (c->cfg.precision == TB_FORM_PLAIN_FP64 && (r = tb_plain_setup(c))) return r;
    if ((r = tb_delta_setup(c))) return r;
    if (c->cfg.precision == TB_FORM_MIXED && (r = tb_mixed_setup(c))) return r;
    c->have_coefs = true;
    return finish(c);
}

int tb_set_baseflow(tb_ctx* c, const double* uxb, const double* uyb, const double* wzb) {
    if (!c || !uxb || !uyb || !wzb) { tb_set_error("null argument"); return TB_ERR_ARG; }
    size_t n2 = tb_n2(c);
    c->h_uxb.assign(uxb, uxb + n2); c->h_uyb.assign(uyb, uyb + n2); c->h_wzb.assign(wzb, wzb + n2);
    tb_graph_reset(c);
    int r = tb_host_upload_baseflow(c);
    if (r) return r;
    c->have_base = true;
    return TB_OK;
}

__global__ static void k_init_mode0(cplx* ux, cplx* uy, cplx* wz, const double* uxb, const double* uyb, const double* wzb, size_t n2) {
    size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= n2) return;
    ux[q] = make_double2(uxb[q], 0.0);
    uy[q] = make_double2(uyb[q], 0.0);
    wz[q] = make_double2(wzb[q], 0.0);
}

int tb_init_fields(tb_ctx* c) {  // main_par.f:601-641
    if (!ready(c)) return TB_ERR_STATE;
    if (!c->have_base) { tb_set_error("base flow not set (tb_set_baseflow)"); return TB_ERR_STATE; }
    size_t n3 = tb_n3(c);
    tb_mixed_invalidate(c);
    cplx* fields[] = {c->ux, c->uy, c->uz, c->wx, c->wy, c->wz, c->wx1, c->wy1, c->wz1, c->dv1x, c->dv1y, c->dv1z, c->dv2x, c->dv2y, c->dv2z};
    for (cplx* f : fields) TB_CUDA(cudaMemsetAsync(f, 0, n3 * sizeof(cplx), c->stream));
    TB_CUDA(cudaMemsetAsync(c->d2uydx2, 0, (size_t)c->g.nx * c->g.K * sizeof(cplx), c->stream));
    size_t n2 = tb_n2(c);
    // forms 0 and 4 carry the base flow in mode 0; in the Goertler and
    // thermal forms every mode is a disturbance about it (init_gv and
    // init_gvth zero every field, the temperature too)
    if (c->cfg.my_form == 2)
        for (cplx* f : {c->th, c->th1, c->dv1t, c->dv2t}) TB_CUDA(cudaMemsetAsync(f, 0, n3 * sizeof(cplx), c->stream));
    if (c->cfg.my_form != 1 && c->cfg.my_form != 2) {
        k_init_mode0<<<tb_blocks(n2, 256), 256, 0, c->stream>>>(c->ux, c->uy, c->wz, c->uxb, c->uyb, c->wzb, n2);
        TB_CHECK_LAUNCH(c);
    }
    c->inited = true;
    return finish(c);
}

namespace {
__global__ void k_copy_state(const double2* __restrict__ src, double2* __restrict__ dst, size_t n) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        dst[q] = src[q];
}
// Device addresses of six page-locked host buffers, if the device can
// address all of them.
bool state_mapped(const double* const h[6], void* dv[6]) {
    for (int f = 0; f < 6; f++) {
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, h[f]) != cudaSuccess || at.type != cudaMemoryTypeHost || !at.devicePointer) {
            cudaGetLastError();   // a pageable pointer is not an error here
            return false;
        }
        dv[f] = at.devicePointer;
    }
    return true;
}
int copy_state_sm(tb_ctx* c, void* const dv[6], bool to_device) {
    cplx* const dev[6] = {c->ux, c->uy, c->uz, c->wx, c->wy, c->wz};
    const size_t n3 = tb_n3(c);
    for (int f = 0; f < 6; f++) {
        const double2* src = to_device ? static_cast<const double2*>(dv[f]) : dev[f];
        double2* dst = to_device ? dev[f] : static_cast<double2*>(dv[f]);
        k_copy_state<<<4 * c->sm_count, 256, 0, c->stream>>>(src, dst, n3);
        TB_CHECK_LAUNCH(c);
    }
    return TB_OK;
}
}  // namespace

int tb_put_state(tb_ctx* c, const double* ux, const double* uy, const double* uz, const double* wx, const double* wy, const double* wz) {
    if (!c || !ux || !uy || !uz || !wx || !wy || !wz) { tb_set_error("null argument"); return TB_ERR_ARG; }
    size_t n3 = tb_n3(c);
    int r;
    const double* const h[6] = {ux, uy, uz, wx, wy, wz};
    void* dv[6];
    if (state_mapped(h, dv)) {
        if ((r = copy_state_sm(c, dv, true))) return r;
        return finish(c);
    }
    if ((r = up(c, c->ux, ux, n3)) || (r = up(c, c->uy, uy, n3)) || (r = up(c, c->uz, uz, n3)) ||
        (r = up(c, c->wx, wx, n3)) || (r = up(c, c->wy, wy, n3)) || (r = up(c, c->wz, wz, n3)))
        return r;
    return finish(c);
}
int tb_get_state(tb_ctx* c, double* ux, double* uy, double* uz, double* wx, double* wy, double* wz) {
    if (!c || !ux || !uy || !uz || !wx || !wy || !wz) { tb_set_error("null argument"); return TB_ERR_ARG; }
    size_t n3 = tb_n3(c);
    int r;
    const double* const h[6] = {ux, uy, uz, wx, wy, wz};
    void* dv[6];
    if (state_mapped(h, dv)) {
        if ((r = copy_state_sm(c, dv, false))) return r;
        return finish(c);
    }
    if ((r = down_async(c, ux, c->ux, n3)) || (r = down_async(c, uy, c->uy, n3)) || (r = down_async(c, uz, c->uz, n3)) ||
        (r = down_async(c, wx, c->wx, n3)) || (r = down_async(c, wy, c->wy, n3)) || (r = down_async(c, wz, c->wz, n3)))
        return r;
    return finish(c);
}
int tb_set_baseflow_th(tb_ctx* c, const double* thb) {
    if (!c || !thb) { tb_set_error("null argument"); return TB_ERR_ARG; }
    if (!c->thb) { tb_set_error("the base temperature exists in my_form 2 only"); return TB_ERR_STATE; }
    TB_CUDA(cudaMemcpyAsync(c->thb, thb, tb_n2(c) * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    tb_graph_reset(c);
    return finish(c);
}
int tb_put_th(tb_ctx* c, const double* th) {
    if (!c || !th) { tb_set_error("null argument"); return TB_ERR_ARG; }
    if (!c->th) { tb_set_error("the temperature exists in my_form 2 only"); return TB_ERR_STATE; }
    int r = up(c, c->th, th, tb_n3(c));
    return r ? r : finish(c);
}
int tb_get_th(tb_ctx* c, double* th) {
    if (!c || !th) { tb_set_error("null argument"); return TB_ERR_ARG; }
    if (!c->th) { tb_set_error("the temperature exists in my_form 2 only"); return TB_ERR_STATE; }
    int r = down_async(c, th, c->th, tb_n3(c));
    return r ? r : finish(c);
}
int tb_put_wall(tb_ctx* c, const double* d) {
    if (!c || !d) { tb_set_error("null argument"); return TB_ERR_ARG; }
    int r = up(c, c->d2uydx2, d, (size_t)c->g.nx * c->g.K);
    return r ? r : finish(c);
}
int tb_get_wall(tb_ctx* c, double* d) {
    if (!c || !d) { tb_set_error("null argument"); return TB_ERR_ARG; }
    int r = down_async(c, d, c->d2uydx2, (size_t)c->g.nx * c->g.K);
    return r ? r : finish(c);
}

int tb_synchronize(tb_ctx* c) { return c ? finish(c) : TB_ERR_ARG; }

// ---- time stepping ------------------------------------------------------
int tb_rk_stage(tb_ctx* c, int stage, int t) {
    if (!ready(c)) return TB_ERR_STATE;
    if (stage < 1 || stage > 4) { tb_set_error("stage must be 1..4"); return TB_ERR_ARG; }
    int r;
    cudaEvent_t ps = nullptr;
    if ((r = tb_prof_begin(c, PROF_STAGE, &ps))) return r;
    if (stage == 1) r = tb_drv_k(c, c->dv1x, c->dv1y, c->dv1z);
    else r = tb_drv_k(c, c->dv2x, c->dv2y, c->dv2z);
    if (r) return r;
    if ((r = tb_rk_update(c, stage))) return r;
    if (stage == 1 && (r = tb_ts_pert_k(c, t, 0.5))) return r;
    if (stage == 3 && (r = tb_ts_pert_k(c, t, 1.0))) return r;
    c->ws_stage = stage; c->ws_t = t; c->g_stage = stage;
    if (stage < 4) r = tb_loop_impl(c, c->cfg.tol_stage, false);
    else r = tb_loop_impl(c, c->cfg.tol_final, true);
    c->ws_stage = 0;
    if (r) return r;
    if ((r = tb_prof_end(c, PROF_STAGE, ps))) return r;
    TB_CUDA(cudaGetLastError());
    return TB_OK;
}
int tb_step(tb_ctx* c, int t) {
    if (!ready(c)) return TB_ERR_STATE;
    if (tb_graph_usable(c)) return tb_graph_step(c, t);
    for (int s = 1; s <= 4; s++) {
        int r = tb_rk_stage(c, s, t);
        if (r) return r;
    }
    return TB_OK;
}
int tb_steps(tb_ctx* c, int t0, int n) {
    for (int t = t0; t < t0 + n; t++) {
        int r = tb_step(c, t);
        if (r) return r;
    }
    return TB_OK;
}
int tb_mixed_fp32_lines(tb_ctx* c, int on) {
    if (!c) { tb_set_error("null context"); return TB_ERR_ARG; }
    TB_CUDA(cudaStreamSynchronize(c->stream));
    c->fp32_lines = on != 0;
    tb_graph_reset(c);
    return TB_OK;
}
int tb_tc_timeout_test(tb_ctx* c, int on) {
    if (!c) { tb_set_error("null context"); return TB_ERR_ARG; }
    TB_CUDA(cudaStreamSynchronize(c->stream));
    c->tc_timeout_test = on != 0;
    tb_graph_reset(c);
    return TB_OK;
}
int tb_nl_tensor_cores(tb_ctx* c, int on) {
    if (!c) { tb_set_error("null context"); return TB_ERR_ARG; }
    TB_CUDA(cudaStreamSynchronize(c->stream));
    c->nl_tensor = on != 0;
    tb_graph_reset(c);
    return TB_OK;
}
int tb_get_poisson_stats(tb_ctx* c, tb_poisson_stats* st) {
    if (!c || !st) { tb_set_error("null argument"); return TB_ERR_ARG; }
    *st = c->stats;
    return TB_OK;
}

// ---- per-subroutine mirrors ---------------------------------------------
static int xmirror(tb_ctx* c, double* out, const double* in, int op) {
    if (!ready(c)) return TB_ERR_STATE;
    size_t n3 = tb_n3(c);
    int r;
    if ((r = up(c, c->tmp[20], in, n3))) return r;
    XJob j[1] = {{c->tmp[20], c->tmp[21], op}};
    if ((r = tb_launch_xlines(c, j, 1))) return r;
    return down(c, out, c->tmp[21], n3);
}
static int ymirror(tb_ctx* c, double* out, const double* in, int op) {
    if (!ready(c)) return TB_ERR_STATE;
    size_t n3 = tb_n3(c);
    int r;
    if ((r = up(c, c->tmp[20], in, n3))) return r;
    YJob j[1] = {{c->tmp[20], c->tmp[21], op}};
    if ((r = tb_launch_ylines(c, j, 1))) return r;
    return down(c, out, c->tmp[21], n3);
}
int tb_derparx(tb_ctx* c, double* d, const double* f) { return xmirror(c, d, f, XOP_D1); }
int tb_derparxx(tb_ctx* c, double* d, const double* f) { return xmirror(c, d, f, XOP_D2); }
int tb_dery(tb_ctx* c, double* d, const double* f) { return ymirror(c, d, f, YOP_D1); }
int tb_deryfv(tb_ctx* c, double* d, const double* f) { return ymirror(c, d, f, YOP_D1FV); }
int tb_deryy(tb_ctx* c, double* d, const double* f) { return ymirror(c, d, f, YOP_D2); }

int tb_nlterms(tb_ctx* c, double* a, double* b, double* cc) {
    if (!ready(c)) return TB_ERR_STATE;
    int r;
    if ((r = tb_launch_nlterms(c, c->tmp[0], c->tmp[1], c->tmp[2]))) return r;
    size_t n3 = tb_n3(c);
    if ((r = down(c, a, c->tmp[0], n3)) || (r = down(c, b, c->tmp[1], n3)) || (r = down(c, cc, c->tmp[2], n3))) return r;
    return tb_tc_check(c);
}
int tb_drv(tb_ctx* c, double* x, double* y, double* z) {
    if (!ready(c)) return TB_ERR_STATE;
    int r;
    if ((r = tb_drv_k(c, c->tmp[13], c->tmp[14], c->tmp[15]))) return r;
    size_t n3 = tb_n3(c);
    if ((r = down(c, x, c->tmp[13], n3)) || (r = down(c, y, c->tmp[14], n3)) || (r = down(c, z, c->tmp[15], n3))) return r;
    return TB_OK;
}
int tb_loop(tb_ctx* c, double erro) {
    if (!ready(c)) return TB_ERR_STATE;
    int r = tb_loop_impl(c, erro, erro < 1.0e-5);
    return r ? r : finish(c);
}
int tb_filter_trid(tb_ctx* c) { if (!ready(c)) return TB_ERR_STATE; int r = tb_filter(c); return r ? r : finish(c); }
int tb_bzone(tb_ctx* c) { if (!ready(c)) return TB_ERR_STATE; int r = tb_bzone_k(c); return r ? r : finish(c); }
int tb_bzonew(tb_ctx* c) { if (!ready(c)) return TB_ERR_STATE; int r = tb_bzonew_k(c); return r ? r : finish(c); }
int tb_outuy(tb_ctx* c, double* dwzdx) {
    if (!ready(c)) return TB_ERR_STATE;
    int r = tb_outuy_k(c, c->tmp[0]);
    return r ? r : down(c, dwzdx, c->tmp[0], tb_n3(c));
}
int tb_poi_uy(tb_ctx* c, const double* dwzdx, double erro) {
    if (!ready(c)) return TB_ERR_STATE;
    int r;
    if ((r = up(c, c->tmp[23], dwzdx, tb_n3(c)))) return r;
    r = (c->cfg.precision == TB_FORM_MIXED) ? tb_poi_uy_mixed(c, c->tmp[23], erro) : tb_poi_uy_k(c, c->tmp[23], erro);
    return r ? r : finish(c);
}
int tb_poi_ux(tb_ctx* c, double* duydy) {
    if (!ready(c)) return TB_ERR_STATE;
    int r = tb_poi_ux_k(c, c->tmp[1]);
    return r ? r : down(c, duydy, c->tmp[1], tb_n3(c));
}
int tb_poi_uz(tb_ctx* c, const double* duydy) {
    if (!ready(c)) return TB_ERR_STATE;
    int r;
    if ((r = up(c, c->tmp[23], duydy, tb_n3(c)))) return r;
    r = tb_poi_uz_k(c, c->tmp[23]);
    return r ? r : finish(c);
}
int tb_wx_wall(tb_ctx* c, double* lapv) {
    if (!ready(c)) return TB_ERR_STATE;
    int r = tb_wx_wall_k(c, c->lapv);
    return r ? r : down(c, lapv, c->lapv, (size_t)c->g.nx * c->g.K);
}
int tb_wz_wall(tb_ctx* c, const double* lapv) {
    if (!ready(c)) return TB_ERR_STATE;
    int r;
    if ((r = up(c, c->lapv, lapv, (size_t)c->g.nx * c->g.K))) return r;
    r = tb_wz_wall_k(c, c->lapv);
    return r ? r : finish(c);
}
int tb_ts_pert(tb_ctx* c, int t, double tempt) {
    if (!ready(c)) return TB_ERR_STATE;
    int r = tb_ts_pert_k(c, t, tempt);
    return r ? r : finish(c);
}
int tb_les_terms(tb_ctx* c, double* fx, double* fy, double* fz) {
    if (!ready(c)) return TB_ERR_STATE;
    int r;
    if ((r = tb_launch_les(c, c->tmp[16], c->tmp[17], c->tmp[18]))) return r;
    size_t n3 = tb_n3(c);
    if ((r = down(c, fx, c->tmp[16], n3)) || (r = down(c, fy, c->tmp[17], n3)) || (r = down(c, fz, c->tmp[18], n3))) return r;
    return TB_OK;
}
int tb_cvirt(tb_ctx* c, double* fx, double* fy, double* fz) {
    if (!ready(c)) return TB_ERR_STATE;
    int r;
    if ((r = tb_launch_cvirt(c, c->tmp[16], c->tmp[17], c->tmp[18], false))) return r;
    size_t n3 = tb_n3(c);
    if ((r = down(c, fx, c->tmp[16], n3)) || (r = down(c, fy, c->tmp[17], n3)) || (r = down(c, fz, c->tmp[18], n3))) return r;
    return TB_OK;
}
int tb_f_to_p(tb_ctx* c, double* phys, const double* four) {
    if (!ready(c)) return TB_ERR_STATE;
    double* pb;
    int r;
    if ((r = phys_buf(c, &pb))) return r;
    if ((r = up(c, c->tmp[23], four, tb_n3(c)))) return r;
    if ((r = tb_launch_f_to_p(c, pb, c->tmp[23]))) return r;
    size_t n = tb_n2(c) * c->g.P;
    TB_CUDA(cudaMemcpyAsync(phys, pb, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    return finish(c);
}
int tb_p_to_f(tb_ctx* c, double* four, const double* phys) {
    if (!ready(c)) return TB_ERR_STATE;
    double* pb;
    int r;
    if ((r = phys_buf(c, &pb))) return r;
    size_t n = tb_n2(c) * c->g.P;
    TB_CUDA(cudaMemcpyAsync(pb, phys, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if ((r = tb_launch_p_to_f(c, c->tmp[23], pb))) return r;
    return down(c, four, c->tmp[23], tb_n3(c));
}

int tb_device_field(tb_ctx* c, int which, void** p) {
    if (!c || !p || which < 0 || which > 5) { tb_set_error("bad argument"); return TB_ERR_ARG; }
    cplx* f[6] = {c->ux, c->uy, c->uz, c->wx, c->wy, c->wz};
    *p = f[which];
    return TB_OK;
}
int tb_stream(tb_ctx* c, void** s) {
    if (!c || !s) { tb_set_error("bad argument"); return TB_ERR_ARG; }
    *s = (void*)c->stream;
    return TB_OK;
}
long long tb_launch_count(tb_ctx* c) { return c ? c->launches : -1; }

int tb_profile(tb_ctx* c, int enable) {
    if (!c) { tb_set_error("null context"); return TB_ERR_ARG; }
    TB_CUDA(cudaStreamSynchronize(c->stream));
    for (auto& r : c->prof_open) { c->prof_pool.push_back(r.a); c->prof_pool.push_back(r.b); }
    c->prof_open.clear();
    for (int i = 0; i < 16; i++) { c->prof_ms[i] = 0; c->prof_n[i] = 0; }
    c->prof = enable != 0;
    return TB_OK;
}
int tb_profile_read(tb_ctx* c, int family, double* ms, long long* n) {
    if (!c || family < 0 || family >= 16 || !ms || !n) { tb_set_error("bad argument"); return TB_ERR_ARG; }
    TB_CUDA(cudaStreamSynchronize(c->stream));
    for (auto& r : c->prof_open) {
        float t = 0.f;
        TB_CUDA(cudaEventElapsedTime(&t, r.a, r.b));
        c->prof_ms[r.id] += t;
        c->prof_n[r.id] += 1;
        c->prof_pool.push_back(r.a);
        c->prof_pool.push_back(r.b);
    }
    c->prof_open.clear();
    *ms = c->prof_ms[family];
    *n = c->prof_n[family];
    return TB_OK;
}

}  // extern "C"
