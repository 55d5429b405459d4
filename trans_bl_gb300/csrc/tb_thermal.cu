// tb_thermal.cu -- the thermal form (my_form 2): drv_gvth with nlterms_th
// (main_par.f:1404-1484, nlterms_par.f:216-300), the temperature's RK update
// (main_par.f:354-445) and its buffer zone (loop_par.f:36-39).
//
// The disturbance (every Fourier mode, no base flow in mode 0) is advanced
// with its full nonlinear products: the seven fields go to physical space,
// the seven products a, b, c, d, ux th, uy th, uz th are formed pointwise in
// place, and come back; the products with the 2D base flow (uxb, uyb, wzb,
// thb) are added in Fourier space.  The temperature is a passive scalar: it
// does not act on the momentum equations.
#include "tb_internal.h"
#include <cmath>
#include <cstring>

namespace {

__device__ __forceinline__ cplx cm(double s, cplx a) { return make_double2(s * a.x, s * a.y); }
__device__ __forceinline__ cplx ca(cplx a, cplx b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ cplx cs_(cplx a, cplx b) { return make_double2(a.x - b.x, a.y - b.y); }
// v_kb(k) * a with v_kb = -i k beta (0-based k)
__device__ __forceinline__ cplx ikb(double kb, cplx a) { return make_double2(kb * a.y, -kb * a.x); }

// Physical-space products, in place over the seven planes (ux, uy, uz, wx,
// wy, wz, th) -> (a, b, c, d, uth, vth, wth), nlterms_par.f:255-267.
__global__ void k_th_products(double* ph, size_t plane) {
    const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= plane) return;
    const double ux = ph[q], uy = ph[plane + q], uz = ph[2 * plane + q];
    const double wx = ph[3 * plane + q], wy = ph[4 * plane + q], wz = ph[5 * plane + q], th = ph[6 * plane + q];
    ph[q] = uy * wx - ux * wy;
    ph[plane + q] = ux * wz - uz * wx;
    ph[2 * plane + q] = uz * wy - uy * wz;
    ph[3 * plane + q] = ux * ux;
    ph[4 * plane + q] = ux * th;
    ph[5 * plane + q] = uy * th;
    ph[6 * plane + q] = uz * th;
}

// The base-flow products added to the transformed ones, nlterms_par.f:279-293.
struct ThBase {
    const cplx *ux, *uy, *uz, *wx, *wy, *wz, *th;
    const double *uxb, *uyb, *wzb, *thb;
    cplx *a, *b, *c, *d, *uth, *vth, *wth;
    size_t n2, n3;
};
__global__ void k_th_base(ThBase A) {
    const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= A.n3) return;
    const size_t p = q % A.n2;
    const double U = A.uxb[p], V = A.uyb[p], W = A.wzb[p], T = A.thb[p];
    const cplx ux = A.ux[q], uy = A.uy[q], uz = A.uz[q], wx = A.wx[q], wy = A.wy[q], wz = A.wz[q], th = A.th[q];
    A.a[q] = ca(cs_(cm(V, wx), cm(U, wy)), A.a[q]);
    A.b[q] = ca(ca(cm(U, wz), cm(W, ux)), A.b[q]);
    A.c[q] = ca(cs_(cm(-V, wz), cm(W, uy)), A.c[q]);
    A.d[q] = ca(cm(2.0 * U, ux), A.d[q]);
    A.uth[q] = ca(ca(cm(U, th), cm(T, ux)), A.uth[q]);
    A.vth[q] = ca(ca(cm(V, th), cm(T, uy)), A.vth[q]);
    A.wth[q] = ca(cm(T, uz), A.wth[q]);
}

// dvt of drv_gvth (main_par.f:1474-1477), rows j >= 2:
// - d(uth)/dx - d(vth)/dy - v_kb wth + (d2th/dx2 + d2th/dy2 + k^2 beta^2 th) / (Re Pr).
struct ThComb {
    const cplx *duthdx, *dvthdy, *wth, *thxx, *thyy, *th;
    cplx* dvt;
    const double* k2b2;
    int nx, ny, K;
    double beta, invRePr;
};
__global__ void k_combine_th(ThComb A) {
    const size_t n = (size_t)A.nx * A.ny * A.K;
    const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int j = (int)((q / A.nx) % A.ny);
    if (j < 1) return;
    const int k = (int)(q / ((size_t)A.nx * A.ny));
    const double kb = (double)k * A.beta, k2 = A.k2b2[k];
    const cplx vis = cm(A.invRePr, ca(ca(A.thxx[q], A.thyy[q]), cm(k2, A.th[q])));
    A.dvt[q] = ca(cs_(cs_(make_double2(-A.duthdx[q].x, -A.duthdx[q].y), A.dvthdy[q]), ikb(kb, A.wth[q])), vis);
}

// RK4 update of th (main_par.f:366-440): j = 2..jmax-1, i = 3..ptsx (1-based).
__global__ void k_rk_th(cplx* th, cplx* th1, cplx* d1, const cplx* d2, int nx, int ny, int K, int stage, double dt,
                        double dt2, double dt6) {
    const size_t n = (size_t)nx * ny * K;
    const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int i = (int)(q % nx), j = (int)((q / nx) % ny);
    if (j < 1 || j > ny - 2 || i < 2) return;
    if (stage == 1) {
        const cplx x = th[q];
        th1[q] = x;
        th[q] = ca(x, cm(dt2, d1[q]));
    } else if (stage == 2 || stage == 3) {
        const double h = (stage == 2) ? dt2 : dt;
        const cplx e = d2[q];
        th[q] = ca(th1[q], cm(h, e));
        d1[q] = ca(d1[q], cm(2.0, e));
    } else {
        th[q] = ca(th1[q], cm(dt6, ca(d1[q], d2[q])));
    }
}

// bzone for th (loop_par.f:36-39): j >= 2, the second ramp row for the third mode.
__global__ void k_bzone_th(cplx* th, const double* bdfc, int nx, int ny, int K) {
    const size_t n = (size_t)nx * ny * K;
    const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int i = (int)(q % nx), j = (int)((q / nx) % ny), k = (int)(q / ((size_t)nx * ny));
    if (j < 1) return;
    th[q] = cm(bdfc[(k == 2 ? (size_t)nx : 0) + i], th[q]);
}

}  // namespace

int tb_drv_gvth(tb_ctx* c, cplx* dvx, cplx* dvy, cplx* dvz, cplx* dvt) {
    cplx** t = c->tmp;
    const size_t n2 = tb_n2(c), n3 = tb_n3(c), plane = (size_t)c->g.P * n2;
    int r;
    // nlterms_th: seven fields to physical space, products in place, back
    const cplx* in[7] = {c->ux, c->uy, c->uz, c->wx, c->wy, c->wz, c->th};
    cplx* out[7] = {t[0], t[1], t[2], t[16], t[17], t[18], t[19]};   // a b c d uth vth wth
    for (int f = 0; f < 7; f++)
        if ((r = tb_launch_f_to_p(c, c->th_phys + f * plane, in[f]))) return r;
    k_th_products<<<tb_blocks(plane, 256), 256, 0, c->stream>>>(c->th_phys, plane);
    TB_CHECK_LAUNCH(c);
    for (int f = 0; f < 7; f++)
        if ((r = tb_launch_p_to_f(c, out[f], c->th_phys + f * plane))) return r;
    ThBase B{c->ux, c->uy, c->uz, c->wx, c->wy, c->wz, c->th, c->uxb, c->uyb, c->wzb, c->thb,
             out[0], out[1], out[2], out[3], out[4], out[5], out[6], n2, n3};
    k_th_base<<<tb_blocks(n3, 256), 256, 0, c->stream>>>(B);
    TB_CHECK_LAUNCH(c);
    // derivatives (drv_gvth, main_par.f:1434-1456)
    XJob xj[8] = {{t[0], t[3], XOP_D1}, {t[1], t[4], XOP_D1}, {t[16], t[20], XOP_D1}, {t[17], t[21], XOP_D1},
                  {c->wx, t[5], XOP_D2}, {c->wy, t[6], XOP_D2}, {c->wz, t[7], XOP_D2}, {c->th, t[22], XOP_D2}};
    YJob yj[7] = {{t[0], t[8], YOP_D1}, {t[2], t[9], YOP_D1}, {t[18], t[14], YOP_D1},
                  {c->wx, t[10], YOP_D2}, {c->wy, t[11], YOP_D2}, {c->wz, t[12], YOP_D2}, {c->th, t[13], YOP_D2}};
    if ((r = tb_launch_xlines(c, xj, 8))) return r;
    if ((r = tb_launch_ylines(c, yj, 7))) return r;
    // the temperature first: its inputs t[13], t[14] may be the momentum outputs
    ThComb T{t[21], t[14], t[19], t[22], t[13], c->th, dvt, c->k2b2, c->g.nx, c->g.ny, c->g.K, c->cfg.beta,
             1.0 / (c->cfg.Re * c->cfg.Pr)};
    k_combine_th<<<tb_blocks(n3, 256), 256, 0, c->stream>>>(T);
    TB_CHECK_LAUNCH(c);
    const double varg = c->cfg.go_number * c->cfg.go_number / std::sqrt(c->cfg.Re);
    return tb_combine_gv(c, t[3], t[8], t[1], t[5], t[10], t[2], t[6], t[11], t[4], t[9], t[7], t[12], t[16], t[20],
                         varg, dvx, dvy, dvz);
}

int tb_rk_update_th(tb_ctx* c, int stage) {
    k_rk_th<<<tb_blocks(tb_n3(c), 256), 256, 0, c->stream>>>(c->th, c->th1, c->dv1t, c->dv2t, c->g.nx, c->g.ny, c->g.K,
                                                              stage, c->dt, c->dt2, c->dt6);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}

int tb_bzone_th(tb_ctx* c) {
    k_bzone_th<<<tb_blocks(tb_n3(c), 256), 256, 0, c->stream>>>(c->th, c->bdfc, c->g.nx, c->g.ny, c->g.K);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}
