// tb_loop.cu -- the stage driver (drv_fi/drv_les, RK4 update, wall forcing)
// and the velocity recovery of loop() except the v-Poisson solve.
#include "tb_internal.h"
#include <cmath>
#include <cstring>

namespace {

__device__ __forceinline__ cplx cm(double s, cplx a) { return make_double2(s * a.x, s * a.y); }
__device__ __forceinline__ cplx ca(cplx a, cplx b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ cplx cs_(cplx a, cplx b) { return make_double2(a.x - b.x, a.y - b.y); }
// v_kb(k) * a with v_kb = -i (k-1) beta  (main_par.f:1888)
__device__ __forceinline__ cplx ikb(double kb, cplx a) { return make_double2(kb * a.y, -kb * a.x); }

// ---------------------------------------------------------------------------
// drv_fi / drv_les combine (main_par.f:1312-1333, 1550-1571), rows j >= 2.
struct CombArgs {
    const cplx *dady, *b, *xx0, *yy0, *wx;
    const cplx *c, *dadx, *xx1, *yy1, *wy;
    const cplx *dbdx, *dcdy, *xx2, *yy2, *wz;
    const cplx *fx, *fy, *dfzdy, *dfzdx, *dfxdy, *dfydx;  // force terms, null if none
    cplx *dvx, *dvy, *dvz;
    const double* k2b2;
    int nx, ny, K;
    double beta, invRe, fac_y;
};
__global__ void k_combine(CombArgs A) {
    size_t n = (size_t)A.nx * A.ny * A.K;
    size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    int j = (int)((q / A.nx) % A.ny);
    if (j < 1) return;
    int k = (int)(q / ((size_t)A.nx * A.ny));
    double kb = (double)k * A.beta, k2 = A.k2b2[k], fy = A.fac_y;
    cplx vx = ca(cs_(ikb(kb, A.b[q]), A.dady[q]), cm(A.invRe, ca(ca(A.xx0[q], cm(fy, A.yy0[q])), cm(k2, A.wx[q]))));
    cplx vy = ca(cs_(A.dadx[q], ikb(kb, A.c[q])), cm(A.invRe, ca(ca(A.xx1[q], cm(fy, A.yy1[q])), cm(k2, A.wy[q]))));
    cplx vz = ca(cs_(A.dcdy[q], A.dbdx[q]), cm(A.invRe, ca(ca(A.xx2[q], cm(fy, A.yy2[q])), cm(k2, A.wz[q]))));
    if (A.fx) {
        vx = cs_(ca(vx, cm(1.0 / fy, ikb(kb, A.fy[q]))), A.dfzdy[q]);
        vy = cs_(ca(vy, A.dfzdx[q]), ikb(kb, A.fx[q]));
        vz = cs_(ca(vz, A.dfxdy[q]), cm(1.0 / fy, A.dfydx[q]));
    }
    A.dvx[q] = vx; A.dvy[q] = vy; A.dvz[q] = vz;
}

// RK4 update (main_par.f:170-246): j = 2..jmax-1, i = 3..ptsx.
struct RkArgs {
    cplx *wx, *wy, *wz, *wx1, *wy1, *wz1, *d1x, *d1y, *d1z;
    const cplx *d2x, *d2y, *d2z;
    int nx, ny, K, stage;
    double dt, dt2, dt6;
};
__global__ void k_rk(RkArgs A) {
    size_t n = (size_t)A.nx * A.ny * A.K;
    size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    int i = (int)(q % A.nx), j = (int)((q / A.nx) % A.ny);
    if (j < 1 || j > A.ny - 2 || i < 2) return;
    if (A.stage == 1) {
        cplx x = A.wx[q], y = A.wy[q], z = A.wz[q];
        A.wx1[q] = x; A.wy1[q] = y; A.wz1[q] = z;
        A.wx[q] = ca(x, cm(A.dt2, A.d1x[q]));
        A.wy[q] = ca(y, cm(A.dt2, A.d1y[q]));
        A.wz[q] = ca(z, cm(A.dt2, A.d1z[q]));
    } else if (A.stage == 2 || A.stage == 3) {
        double h = (A.stage == 2) ? A.dt2 : A.dt;
        cplx ex = A.d2x[q], ey = A.d2y[q], ez = A.d2z[q];
        A.wx[q] = ca(A.wx1[q], cm(h, ex));
        A.wy[q] = ca(A.wy1[q], cm(h, ey));
        A.wz[q] = ca(A.wz1[q], cm(h, ez));
        A.d1x[q] = ca(A.d1x[q], cm(2.0, ex));
        A.d1y[q] = ca(A.d1y[q], cm(2.0, ey));
        A.d1z[q] = ca(A.d1z[q], cm(2.0, ez));
    } else {
        A.wx[q] = ca(A.wx1[q], cm(A.dt6, ca(A.d1x[q], A.d2x[q])));
        A.wy[q] = ca(A.wy1[q], cm(A.dt6, ca(A.d1y[q], A.d2y[q])));
        A.wz[q] = ca(A.wz1[q], cm(A.dt6, ca(A.d1z[q], A.d2z[q])));
    }
}

// bzone (loop_par.f:6-45) for j >= 2 and bzonew (691-725) for j = 1.
__global__ void k_bzone(cplx* wx, cplx* wy, cplx* wz, const double* bdfc, const double* wzb, int nx, int ny, int K,
                        int wall, int form) {
    size_t n = (size_t)nx * (wall ? 1 : ny) * K;
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i, j, k;
    if (wall) { i = (int)(t % nx); k = (int)(t / nx); j = 0; }
    else { i = (int)(t % nx); j = (int)((t / nx) % ny); k = (int)(t / ((size_t)nx * ny)); if (j < 1) return; }
    size_t q = (size_t)i + (size_t)nx * (j + (size_t)ny * k);
    double bd = bdfc[i];
    wx[q] = cm(bd, wx[q]);
    wy[q] = cm(bd, wy[q]);
    if ((form == 0 || form == 4) && k == 0) {
        double b = wzb[i + (size_t)nx * j];
        cplx v = wz[q];
        wz[q] = make_double2((v.x - b) * bd + b, v.y * bd);
    } else {
        wz[q] = cm(bd, wz[q]);
    }
}

// outuy tail (loop_par.f:96-114): Dirichlet uy at the outflow column, j >= 2.
__global__ void k_outuy_bc(cplx* uy, const double* uyb, int nx, int ny, int K, int form) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ny * K) return;
    int j = t % ny, k = t / ny;
    if (j < 1) return;
    size_t q = (size_t)(nx - 1) + (size_t)nx * (j + (size_t)ny * k);
    uy[q] = ((form == 0 || form == 4) && k == 0) ? make_double2(uyb[(nx - 1) + (size_t)nx * j], 0.0) : make_double2(0.0, 0.0);
}

// filter_trid copy-back (filter_par.f:166-174): i >= 2, j >= 2.
__global__ void k_copy_inner(cplx* dst, const cplx* src, int nx, int ny, int K) {
    size_t n = (size_t)nx * ny * K;
    size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    int i = (int)(q % nx), j = (int)((q / nx) % ny);
    if (i < 1 || j < 1) return;
    dst[q] = src[q];
}

// poi_ux, fundamental mode (loop_par.f:452-499): ux from continuity by the
// 4th-order implicit x integration, one thread per row j = 2..jmax-1.
__global__ void k_ux_mode0(cplx* ux, const cplx* duydy, int nx, int ny, double dx) {
    int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (j > ny - 2) return;
    cplx* U = ux + (size_t)nx * j;
    const cplx* D = duydy + (size_t)nx * j;
    const double i720 = 1.0 / 720.0, i27 = 1.0 / 27.0, i90 = 1.0 / 90.0, i57 = 1.0 / 57.0;
    auto rr = [&](double a0, cplx d0, double a1, cplx d1, double a2, cplx d2, double a3, cplx d3, double a4, cplx d4) {
        return make_double2(a0 * d0.x + a1 * d1.x + a2 * d2.x + a3 * d3.x + a4 * d4.x,
                            a0 * d0.y + a1 * d1.y + a2 * d2.y + a3 * d3.y + a4 * d4.y);
    };
    cplx u0 = U[0];
    cplx s = rr(251.0, D[0], 646.0, D[1], -264.0, D[2], 106.0, D[3], -19.0, D[4]);
    cplx u1 = make_double2((-dx * s.x + 720.0 * u0.x) * i720, (-dx * s.y + 720.0 * u0.y) * i720);
    U[1] = u1;
    cplx um2 = u0, um1 = u1;
    cplx d0 = D[0], d1 = D[1], d2 = D[2], d3 = D[3];
    for (int i = 2; i <= nx - 3; i++) {
        cplx d4 = D[i + 2];
        cplx t = rr(281.0, d0, 2056.0, d1, 1176.0, d2, -104.0, d3, 11.0, d4);
        cplx u = make_double2((-dx * t.x * i90 + 11.0 * um2.x + 16.0 * um1.x) * i27,
                              (-dx * t.y * i90 + 11.0 * um2.y + 16.0 * um1.y) * i27);
        U[i] = u;
        um2 = um1; um1 = u;
        d0 = d1; d1 = d2; d2 = d3; d3 = d4;
    }
    int i = nx - 2;
    {
        cplx a = D[i - 2], b = D[i - 1], c0 = D[i], d = D[i + 1];
        cplx t = make_double2(10.0 * a.x + 57.0 * b.x + 24.0 * c0.x - d.x, 10.0 * a.y + 57.0 * b.y + 24.0 * c0.y - d.y);
        cplx u = make_double2((-dx * t.x + 33.0 * um2.x + 24.0 * um1.x) * i57, (-dx * t.y + 33.0 * um2.y + 24.0 * um1.y) * i57);
        U[i] = u; um2 = um1; um1 = u;
    }
    i = nx - 1;
    {
        cplx t = rr(251.0, D[i], 646.0, D[i - 1], -264.0, D[i - 2], 106.0, D[i - 3], -19.0, D[i - 4]);
        U[i] = make_double2((-dx * t.x + 720.0 * um1.x) * i720, (-dx * t.y + 720.0 * um1.y) * i720);
    }
}

// x-penta Poisson of poi_ux / poi_uz (loop_par.f:519-563, 641-685): one thread
// per line (j >= 2, k >= 2); rhs formed on the fly, lusolver (penta_par.f:130-208).
// sgn_d multiplies the derivative term, sgn_w the i k beta term; for poi_ux
// rhs = -(D + vkb W) weights, for poi_uz rhs = (D - vkb W) weights.
struct PentaArgs {
    const cplx* D;   // d2uydxdy or dwydx
    const cplx* W;   // wy or duydy
    cplx* out;       // ux or uz
    const double* lu;
    int nx, ny, K, uz;
    double dxx, beta;
};
__global__ void k_penta_x(PentaArgs A) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int nl = (A.ny - 1) * (A.K - 1);
    if (t >= nl) return;
    int j = 1 + t % (A.ny - 1);
    int k = 1 + t / (A.ny - 1);
    int n = A.nx;
    size_t base = (size_t)n * (j + (size_t)A.ny * k);
    const cplx* D = A.D + base;
    const cplx* W = A.W + base;
    cplx* O = A.out + base;
    const double* L1 = A.lu + (size_t)k * 5 * n;  // lu(:,1)
    const double* L2 = L1 + n;                    // lu(:,2)
    const double* IU3 = L1 + 2 * n;               // 1/lu(:,3)
    const double* U4 = L1 + 3 * n;
    const double* U5 = L1 + 4 * n;
    double kb = (double)k * A.beta;
    double den = 1.0 / ((double)k * (double)k * A.beta * A.beta);
    // combination D + s * vkb W, s = +1 (ux) or -1 (uz); overall sign g = -1 (ux) or +1 (uz)
    double s = A.uz ? -1.0 : 1.0, g = A.uz ? 1.0 : -1.0;
    auto comb = [&](cplx d, cplx w) { cplx v = ikb(kb, w); return make_double2(d.x + s * v.x, d.y + s * v.y); };
    const double c12 = A.dxx / 12.0, c8 = 8.0 * A.dxx;
    // forward: y(1) = rhs(1), y(2) = rhs(2) - l2 y(1), y(i) = rhs(i) - l1 y(i-2) - l2 y(i-1)
    cplx y0 = O[0];  // rhs(1) = ux(1,j,k) / uz(1,j,k)
    O[0] = y0;
    cplx e0 = comb(D[0], W[0]), e1 = comb(D[1], W[1]), e2 = comb(D[2], W[2]);
    cplx r1 = make_double2(g * c12 * (e0.x + 10.0 * e1.x + e2.x), g * c12 * (e0.y + 10.0 * e1.y + e2.y));
    cplx y1 = make_double2(r1.x - L2[1] * y0.x, r1.y - L2[1] * y0.y);
    O[1] = y1;
    cplx ym2 = y0, ym1 = y1;
    for (int i = 2; i <= n - 3; i++) {
        cplx e3 = comb(D[i + 1], W[i + 1]);
        cplx r = make_double2(g * c8 * (e1.x + 5.5 * e2.x + e3.x), g * c8 * (e1.y + 5.5 * e2.y + e3.y));
        cplx y = make_double2(r.x - L1[i] * ym2.x - L2[i] * ym1.x, r.y - L1[i] * ym2.y - L2[i] * ym1.y);
        O[i] = y;
        ym2 = ym1; ym1 = y;
        e1 = e2; e2 = e3;
    }
    {
        int i = n - 2;
        cplx a = comb(D[n - 1], W[n - 1]);  // e1=comb(i-1), e2 = comb(i)
        cplx r = make_double2(g * c12 * (a.x + 10.0 * e2.x + e1.x), g * c12 * (a.y + 10.0 * e2.y + e1.y));
        cplx y = make_double2(r.x - L1[i] * ym2.x - L2[i] * ym1.x, r.y - L1[i] * ym2.y - L2[i] * ym1.y);
        O[i] = y;
        ym2 = ym1; ym1 = y;
        i = n - 1;
        cplx v = ikb(kb, W[n - 1]);
        cplx dn = D[n - 1];
        cplx rn = A.uz ? make_double2((-dn.x + v.x) * den, (-dn.y + v.y) * den)
                       : make_double2((v.x + dn.x) * den, (v.y + dn.y) * den);
        cplx yn = make_double2(rn.x - L1[i] * ym2.x - L2[i] * ym1.x, rn.y - L1[i] * ym2.y - L2[i] * ym1.y);
        // backward: x(n) = y(n)/lu3, x(n-1) = (y - lu4 x(n))/lu3, x(i) = (y - lu4 x(i+1) - lu5 x(i+2))/lu3
        cplx xn = make_double2(yn.x * IU3[n - 1], yn.y * IU3[n - 1]);
        cplx xm = make_double2((y.x - U4[n - 2] * xn.x) * IU3[n - 2], (y.y - U4[n - 2] * xn.y) * IU3[n - 2]);
        O[n - 1] = xn; O[n - 2] = xm;
        cplx xp2 = xn, xp1 = xm;
        for (int ii = n - 3; ii >= 1; ii--) {
            cplx yy = O[ii];
            cplx x = make_double2((yy.x - U4[ii] * xp1.x - U5[ii] * xp2.x) * IU3[ii],
                                  (yy.y - U4[ii] * xp1.y - U5[ii] * xp2.y) * IU3[ii]);
            O[ii] = x;
            xp2 = xp1; xp1 = x;
        }
        // i = 1 keeps ux(1) (lu(1,3) = 1, upper entries 0)
    }
}

// lapv (loop_par.f:194-205) for every (i, k).
__global__ void k_lapv(cplx* lapv, const cplx* uy, const cplx* d2uydx2, const double* k2b2, const double* w, int nx, int ny,
                       int K, double inv_dyyw1) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nx * K) return;
    int i = t % nx, k = t / nx;
    const cplx* U = uy + (size_t)i + (size_t)nx * ny * k;
    size_t s = nx;
    cplx acc = make_double2(0, 0);
#pragma unroll
    for (int m = 0; m < 7; m++) { cplx v = U[m * s]; acc.x += w[2 + m] * v.x; acc.y += w[2 + m] * v.y; }
    cplx d = d2uydx2[t];
    cplx u1 = U[0];
    lapv[t] = make_double2(d.x + acc.x * inv_dyyw1 + k2b2[k] * u1.x, d.y + acc.y * inv_dyyw1 + k2b2[k] * u1.y);
}

// wall dwy/dy (der2wydxdy first loop, loop_par.f:313-321) per (i, k).
__global__ void k_dwydy_wall(cplx* out, const cplx* wy, const double* w, int nx, int ny, int K, double invdy) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nx * K) return;
    int i = t % nx, k = t / nx;
    const cplx* W = wy + (size_t)i + (size_t)nx * ny * k;
    size_t s = nx;
    cplx acc = make_double2(0, 0);
#pragma unroll
    for (int m = 0; m < 7; m++) { cplx v = W[m * s]; acc.x += w[1 + m] * v.x; acc.y += w[1 + m] * v.y; }
    out[t] = make_double2(invdy * acc.x, invdy * acc.y);
}

// wx_wall (loop_par.f:174-255): per mode k >= 2, d2wy/dxdy by explicit
// stencils, then the x-penta solve with lusolver_1 (penta_par.f:53-127).
// One thread per mode.
__global__ void k_wx_wall(cplx* wx, const cplx* dwdy, const cplx* lapv, const double* lu_all, int nx, int ny, int K,
                          double dx, double dxx, double beta) {
    int k = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const int n = nx;
    const cplx* dw = dwdy + (size_t)nx * k;
    const cplx* LV = lapv + (size_t)nx * k;
    cplx* WX = wx + (size_t)nx * ny * k;  // row j = 1
    const double* L1 = lu_all + (size_t)k * 5 * n;
    const double* L2 = L1 + n;
    const double* IU3 = L1 + 2 * n;
    const double* U4 = L1 + 3 * n;
    const double* U5 = L1 + 4 * n;
    double kb = (double)k * beta;
    double idx6 = 1.0 / 6.0 / dx, idx60 = 1.0 / 60.0 / dx, idx12 = 1.0 / 12.0 / dx, idx2 = 1.0 / 2.0 / dx;
    auto d2 = [&](int i) -> cplx {  // d2wydxdy(i), 0-based i
        if (i >= 3 && i <= n - 4) {
            cplx a = dw[i + 1], b = dw[i - 1], c = dw[i - 2], d = dw[i + 2], e = dw[i + 3], f = dw[i - 3];
            return make_double2((45.0 * (a.x - b.x) + 9.0 * (c.x - d.x) + e.x - f.x) * idx60,
                                (45.0 * (a.y - b.y) + 9.0 * (c.y - d.y) + e.y - f.y) * idx60);
        }
        const double* cw; int b0, e; double sc;
        static const double W0[7] = {-14.7, 36.0, -45.0, 40.0, -22.5, 7.2, -1.0};
        static const double W1[7] = {-1.0, -7.7, 15.0, -10.0, 5.0, -1.5, 0.2};
        static const double W2[7] = {0.2, -2.4, -3.5, 8.0, -3.0, 0.8, -0.1};
        if (i == 0) { cw = W0; b0 = 0; e = 7; sc = idx6; }
        else if (i == 1) { cw = W1; b0 = 0; e = 7; sc = idx6; }
        else if (i == 2) { cw = W2; b0 = 0; e = 7; sc = idx6; }
        else if (i == n - 3) {
            cplx a = dw[n - 5], b = dw[n - 4], c = dw[n - 2], d = dw[n - 1];
            return make_double2((a.x - 8.0 * b.x + 8.0 * c.x - d.x) * idx12, (a.y - 8.0 * b.y + 8.0 * c.y - d.y) * idx12);
        } else if (i == n - 2) {
            cplx a = dw[n - 1], b = dw[n - 2], c = dw[n - 3], d = dw[n - 4];
            return make_double2((2.0 * a.x + 3.0 * b.x - 6.0 * c.x + d.x) * idx6, (2.0 * a.y + 3.0 * b.y - 6.0 * c.y + d.y) * idx6);
        } else {
            cplx a = dw[n - 1], b = dw[n - 2], c = dw[n - 3];
            return make_double2((3.0 * a.x - 4.0 * b.x + c.x) * idx2, (3.0 * a.y - 4.0 * b.y + c.y) * idx2);
        }
        cplx acc = make_double2(0, 0);
        for (int m = 0; m < e; m++) { acc.x += cw[m] * dw[b0 + m].x; acc.y += cw[m] * dw[b0 + m].y; }
        return make_double2(acc.x * sc, acc.y * sc);
    };
    // combination -d2 + vkb lapv
    auto comb = [&](int i) { cplx a = d2(i); cplx v = ikb(kb, LV[i]); return make_double2(-a.x + v.x, -a.y + v.y); };
    const double c12 = dxx / 12.0, c8 = 8.0 * dxx;
    // forward (lusolver_1 order: - l2 y(i-1) - l1 y(i-2))
    cplx y0 = WX[0];
    WX[0] = y0;
    cplx e0 = comb(0), e1 = comb(1), e2 = comb(2);
    cplx r1 = make_double2(c12 * (e0.x + 10.0 * e1.x + e2.x), c12 * (e0.y + 10.0 * e1.y + e2.y));
    cplx y1 = make_double2(r1.x - L2[1] * y0.x, r1.y - L2[1] * y0.y);
    WX[1] = y1;
    cplx ym2 = y0, ym1 = y1;
    for (int i = 2; i <= n - 3; i++) {
        cplx e3 = comb(i + 1);
        cplx r = make_double2(c8 * (e1.x + 5.5 * e2.x + e3.x), c8 * (e1.y + 5.5 * e2.y + e3.y));
        cplx y = make_double2(r.x - L2[i] * ym1.x - L1[i] * ym2.x, r.y - L2[i] * ym1.y - L1[i] * ym2.y);
        WX[i] = y;
        ym2 = ym1; ym1 = y;
        e1 = e2; e2 = e3;
    }
    int i = n - 2;
    cplx a = comb(n - 1);
    cplx r = make_double2(c12 * (a.x + 10.0 * e2.x + e1.x), c12 * (a.y + 10.0 * e2.y + e1.y));
    cplx y = make_double2(r.x - L2[i] * ym1.x - L1[i] * ym2.x, r.y - L2[i] * ym1.y - L1[i] * ym2.y);
    WX[i] = y; ym2 = ym1; ym1 = y;
    i = n - 1;
    cplx dd = d2(n - 1), vv = ikb(kb, LV[n - 1]);
    double den = 1.0 / ((double)k * (double)k * beta * beta);
    cplx rn = make_double2((dd.x - vv.x) * den, (dd.y - vv.y) * den);
    cplx yn = make_double2(rn.x - L2[i] * ym1.x - L1[i] * ym2.x, rn.y - L2[i] * ym1.y - L1[i] * ym2.y);
    cplx xn = make_double2(yn.x * IU3[n - 1], yn.y * IU3[n - 1]);
    cplx xm = make_double2((y.x - U4[n - 2] * xn.x) * IU3[n - 2], (y.y - U4[n - 2] * xn.y) * IU3[n - 2]);
    WX[n - 1] = xn; WX[n - 2] = xm;
    cplx xp2 = xn, xp1 = xm;
    for (int ii = n - 3; ii >= 1; ii--) {
        cplx yy = WX[ii];
        cplx x = make_double2((yy.x - U4[ii] * xp1.x - U5[ii] * xp2.x) * IU3[ii], (yy.y - U4[ii] * xp1.y - U5[ii] * xp2.y) * IU3[ii]);
        WX[ii] = x;
        xp2 = xp1; xp1 = x;
    }
}

// wz_wall (loop_par.f:361-425): wall wz by implicit x integration, one thread per mode.
__global__ void k_wz_wall(cplx* wz, const cplx* wx, const cplx* lapv, int nx, int ny, int K, double dx, double beta) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    double kb = (double)k * beta;
    const cplx* WX = wx + (size_t)nx * ny * k;
    const cplx* LV = lapv + (size_t)nx * k;
    cplx* W = wz + (size_t)nx * ny * k;
    auto R = [&](int i) { cplx v = ikb(kb, WX[i]); cplx l = LV[i]; return make_double2(v.x - l.x, v.y - l.y); };
    const double i720 = 1.0 / 720.0, i27 = 1.0 / 27.0, i90 = 1.0 / 90.0, i57 = 1.0 / 57.0;
    cplx r0 = R(0), r1 = R(1), r2 = R(2), r3 = R(3), r4 = R(4);
    cplx w0 = W[0];
    cplx w1 = make_double2((dx * (251.0 * r0.x + 646.0 * r1.x - 264.0 * r2.x + 106.0 * r3.x - 19.0 * r4.x) + 720.0 * w0.x) * i720,
                           (dx * (251.0 * r0.y + 646.0 * r1.y - 264.0 * r2.y + 106.0 * r3.y - 19.0 * r4.y) + 720.0 * w0.y) * i720);
    W[1] = w1;
    cplx wm2 = w0, wm1 = w1;
    cplx a0 = r0, a1 = r1, a2 = r2, a3 = r3;
    for (int i = 2; i <= nx - 3; i++) {
        cplx a4 = R(i + 2);
        cplx w = make_double2((dx * (281.0 * a0.x + 2056.0 * a1.x + 1176.0 * a2.x - 104.0 * a3.x + 11.0 * a4.x) * i90 +
                               11.0 * wm2.x + 16.0 * wm1.x) * i27,
                              (dx * (281.0 * a0.y + 2056.0 * a1.y + 1176.0 * a2.y - 104.0 * a3.y + 11.0 * a4.y) * i90 +
                               11.0 * wm2.y + 16.0 * wm1.y) * i27);
        W[i] = w;
        wm2 = wm1; wm1 = w;
        a0 = a1; a1 = a2; a2 = a3; a3 = a4;
    }
    int i = nx - 2;
    cplx b0 = R(i - 2), b1 = R(i - 1), b2 = R(i), b3 = R(i + 1);
    cplx w = make_double2((dx * (10.0 * b0.x + 57.0 * b1.x + 24.0 * b2.x - b3.x) + 33.0 * wm2.x + 24.0 * wm1.x) * i57,
                          (dx * (10.0 * b0.y + 57.0 * b1.y + 24.0 * b2.y - b3.y) + 33.0 * wm2.y + 24.0 * wm1.y) * i57);
    W[i] = w; wm2 = wm1; wm1 = w;
    i = nx - 1;
    cplx c0 = R(i), c1 = R(i - 1), c2 = R(i - 2), c3 = R(i - 3), c4 = R(i - 4);
    W[i] = make_double2((dx * (251.0 * c0.x + 646.0 * c1.x - 264.0 * c2.x + 106.0 * c3.x - 19.0 * c4.x) + 720.0 * wm1.x) * i720,
                        (dx * (251.0 * c0.y + 646.0 * c1.y - 264.0 * c2.y + 106.0 * c3.y - 19.0 * c4.y) + 720.0 * wm1.y) * i720);
}

// ts2d_pert / ts3d_pert (main_par.f:1613-1685) for each forced mode.
struct PertArgs {
    cplx *uy, *d2uydx2;
    const double *fcx, *fcllx;
    int nx, ny, i1, i2, nf;
    int mode[4];
    double fct[4];
};
__global__ void k_ts_pert(PertArgs A) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;  // 0-based
    if (i < A.i1 || i > A.i2 - 2) return;          // 1-based i1+1 .. i2-1
    for (int m = 0; m < A.nf; m++) {
        int k = A.mode[m];
        A.uy[(size_t)i + (size_t)A.nx * A.ny * k] = make_double2(A.fcx[i] * A.fct[m], 0.0);
        A.d2uydx2[(size_t)i + (size_t)A.nx * k] = make_double2(A.fcllx[i] * A.fct[m], 0.0);
    }
}

}  // namespace

// ===========================================================================
int tb_drv_k(tb_ctx* c, cplx* dvx, cplx* dvy, cplx* dvz) {
    cplx** t = c->tmp;
    int r;
    if (c->cfg.my_form == 4 || c->cfg.ibm) {
        cplx* f[3] = {t[16], t[17], t[18]};
        cplx* df[4] = {t[19], t[20], t[21], t[22]};
        return tb_drv_forced(c, dvx, dvy, dvz, f, df);
    }
    // nonlinear terms a, b, c -> t[0..2]
    if ((r = tb_launch_nlterms(c, t[0], t[1], t[2]))) return r;
    XJob xj[5] = {{t[0], t[3], XOP_D1}, {t[1], t[4], XOP_D1},
                  {c->wx, t[5], XOP_D2}, {c->wy, t[6], XOP_D2}, {c->wz, t[7], XOP_D2}};
    YJob yj[5] = {{t[0], t[8], YOP_D1}, {t[2], t[9], YOP_D1},
                  {c->wx, t[10], YOP_D2}, {c->wy, t[11], YOP_D2}, {c->wz, t[12], YOP_D2}};
    if ((r = tb_launch_xlines(c, xj, 5))) return r;
    if ((r = tb_launch_ylines(c, yj, 5))) return r;
    CombArgs A;
    std::memset(&A, 0, sizeof A);
    A.dady = t[8]; A.b = t[1]; A.xx0 = t[5]; A.yy0 = t[10]; A.wx = c->wx;
    A.c = t[2]; A.dadx = t[3]; A.xx1 = t[6]; A.yy1 = t[11]; A.wy = c->wy;
    A.dbdx = t[4]; A.dcdy = t[9]; A.xx2 = t[7]; A.yy2 = t[12]; A.wz = c->wz;
    A.dvx = dvx; A.dvy = dvy; A.dvz = dvz; A.k2b2 = c->k2b2;
    A.nx = c->g.nx; A.ny = c->g.ny; A.K = c->g.K; A.beta = c->cfg.beta; A.invRe = 1.0 / c->cfg.Re; A.fac_y = c->cfg.fac_y;
    k_combine<<<tb_blocks(tb_n3(c), 256), 256, 0, c->stream>>>(A);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}

// drv with LES and/or IBM forcing: forces first (they use tmp[0..11] as
// scratch), the force curl terms, then the standard terms.
int tb_drv_forced(tb_ctx* c, cplx* dvx, cplx* dvy, cplx* dvz, cplx* f[3], cplx* df[4]) {
    int r;
    bool les = c->cfg.my_form == 4, ibm = c->cfg.ibm != 0;
    if (les) { if ((r = tb_launch_les(c, f[0], f[1], f[2]))) return r; }
    if (ibm) { if ((r = tb_launch_cvirt(c, f[0], f[1], f[2], les))) return r; }
    XJob fx[2] = {{f[1], df[0], XOP_D1}, {f[2], df[1], XOP_D1}};   // dfydx, dfzdx
    YJob fy[2] = {{f[0], df[2], YOP_D1}, {f[2], df[3], YOP_D1}};   // dfxdy, dfzdy
    if ((r = tb_launch_xlines(c, fx, 2))) return r;
    if ((r = tb_launch_ylines(c, fy, 2))) return r;
    cplx** t = c->tmp;
    if ((r = tb_launch_nlterms(c, t[0], t[1], t[2]))) return r;
    XJob xj[5] = {{t[0], t[3], XOP_D1}, {t[1], t[4], XOP_D1},
                  {c->wx, t[5], XOP_D2}, {c->wy, t[6], XOP_D2}, {c->wz, t[7], XOP_D2}};
    YJob yj[5] = {{t[0], t[8], YOP_D1}, {t[2], t[9], YOP_D1},
                  {c->wx, t[10], YOP_D2}, {c->wy, t[11], YOP_D2}, {c->wz, t[12], YOP_D2}};
    if ((r = tb_launch_xlines(c, xj, 5))) return r;
    if ((r = tb_launch_ylines(c, yj, 5))) return r;
    CombArgs A;
    std::memset(&A, 0, sizeof A);
    A.dady = t[8]; A.b = t[1]; A.xx0 = t[5]; A.yy0 = t[10]; A.wx = c->wx;
    A.c = t[2]; A.dadx = t[3]; A.xx1 = t[6]; A.yy1 = t[11]; A.wy = c->wy;
    A.dbdx = t[4]; A.dcdy = t[9]; A.xx2 = t[7]; A.yy2 = t[12]; A.wz = c->wz;
    A.fx = f[0]; A.fy = f[1]; A.dfydx = df[0]; A.dfzdx = df[1]; A.dfxdy = df[2]; A.dfzdy = df[3];
    A.dvx = dvx; A.dvy = dvy; A.dvz = dvz; A.k2b2 = c->k2b2;
    A.nx = c->g.nx; A.ny = c->g.ny; A.K = c->g.K; A.beta = c->cfg.beta; A.invRe = 1.0 / c->cfg.Re; A.fac_y = c->cfg.fac_y;
    k_combine<<<tb_blocks(tb_n3(c), 256), 256, 0, c->stream>>>(A);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}

int tb_rk_update(tb_ctx* c, int stage) {
    RkArgs A{c->wx, c->wy, c->wz, c->wx1, c->wy1, c->wz1, c->dv1x, c->dv1y, c->dv1z, c->dv2x, c->dv2y, c->dv2z,
             c->g.nx, c->g.ny, c->g.K, stage, c->dt, c->dt2, c->dt6};
    k_rk<<<tb_blocks(tb_n3(c), 256), 256, 0, c->stream>>>(A);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}

int tb_filter(tb_ctx* c) {
    cplx** t = c->tmp;
    XJob xj[3] = {{c->wx, t[0], XOP_FILTER}, {c->wy, t[1], XOP_FILTER}, {c->wz, t[2], XOP_FILTER}};
    int r;
    if ((r = tb_launch_xlines(c, xj, 3))) return r;
    unsigned nb = tb_blocks(tb_n3(c), 256);
    k_copy_inner<<<nb, 256, 0, c->stream>>>(c->wx, t[0], c->g.nx, c->g.ny, c->g.K); TB_CHECK_LAUNCH(c);
    k_copy_inner<<<nb, 256, 0, c->stream>>>(c->wy, t[1], c->g.nx, c->g.ny, c->g.K); TB_CHECK_LAUNCH(c);
    k_copy_inner<<<nb, 256, 0, c->stream>>>(c->wz, t[2], c->g.nx, c->g.ny, c->g.K); TB_CHECK_LAUNCH(c);
    return TB_OK;
}

int tb_bzone_k(tb_ctx* c) {
    k_bzone<<<tb_blocks(tb_n3(c), 256), 256, 0, c->stream>>>(c->wx, c->wy, c->wz, c->bdfc, c->wzb, c->g.nx, c->g.ny, c->g.K, 0,
                                                              c->cfg.my_form);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}
int tb_bzonew_k(tb_ctx* c) {
    k_bzone<<<tb_blocks((size_t)c->g.nx * c->g.K, 256), 256, 0, c->stream>>>(c->wx, c->wy, c->wz, c->bdfc, c->wzb, c->g.nx,
                                                                              c->g.ny, c->g.K, 1, c->cfg.my_form);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}
int tb_outuy_k(tb_ctx* c, cplx* dwzdx) {
    XJob xj[1] = {{c->wz, dwzdx, XOP_D1}};
    int r;
    if ((r = tb_launch_xlines(c, xj, 1))) return r;
    k_outuy_bc<<<tb_blocks((size_t)c->g.ny * c->g.K, 128), 128, 0, c->stream>>>(c->uy, c->uyb, c->g.nx, c->g.ny, c->g.K,
                                                                                 c->cfg.my_form);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}
int tb_poi_ux_k(tb_ctx* c, cplx* duydy) {
    int r;
    YJob yj[1] = {{c->uy, duydy, YOP_D1FV}};
    if ((r = tb_launch_ylines(c, yj, 1))) return r;
    k_ux_mode0<<<tb_blocks(c->g.ny, 64), 64, 0, c->stream>>>(c->ux, duydy, c->g.nx, c->g.ny, c->cfg.dx);
    TB_CHECK_LAUNCH(c);
    if (c->g.K < 2) return TB_OK;
    cplx* d2 = c->tmp[13];
    XJob xj[1] = {{duydy, d2, XOP_D1}};
    if ((r = tb_launch_xlines(c, xj, 1))) return r;
    PentaArgs A{d2, c->wy, c->ux, c->px.lu, c->g.nx, c->g.ny, c->g.K, 0, c->cfg.dx * c->cfg.dx, c->cfg.beta};
    cudaEvent_t ps = nullptr;
    if ((r = tb_prof_begin(c, PROF_PENTA, &ps))) return r;
    k_penta_x<<<tb_blocks((size_t)(c->g.ny - 1) * (c->g.K - 1), 128), 128, 0, c->stream>>>(A);
    TB_CHECK_LAUNCH(c);
    return tb_prof_end(c, PROF_PENTA, ps);
}
int tb_poi_uz_k(tb_ctx* c, const cplx* duydy) {
    if (c->g.K < 2) return TB_OK;
    int r;
    cplx* dwydx = c->tmp[14];
    XJob xj[1] = {{c->wy, dwydx, XOP_D1}};
    if ((r = tb_launch_xlines(c, xj, 1))) return r;
    PentaArgs A{dwydx, duydy, c->uz, c->px.lu, c->g.nx, c->g.ny, c->g.K, 1, c->cfg.dx * c->cfg.dx, c->cfg.beta};
    k_penta_x<<<tb_blocks((size_t)(c->g.ny - 1) * (c->g.K - 1), 128), 128, 0, c->stream>>>(A);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}
int tb_wx_wall_k(tb_ctx* c, cplx* lapv) {
    const double* wat = c->coefs.data() + 100 + 24 * c->g.msh - 17;  // w_at_w_coef(9)
    const double* dwy = wat + 9;                                       // dwydy_coef(8)
    // coefficients live on the host; stage them through a small device buffer
    static thread_local double* dcoef = nullptr;
    static thread_local int dcoef_dev = -1;
    if (!dcoef || dcoef_dev != c->device) {
        TB_CUDA(cudaMalloc(&dcoef, 17 * sizeof(double)));
        dcoef_dev = c->device;
    }
    TB_CUDA(cudaMemcpyAsync(dcoef, wat, 17 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    double dyy = c->cfg.dy * c->cfg.dy;
    unsigned nb = tb_blocks((size_t)c->g.nx * c->g.K, 128);
    k_lapv<<<nb, 128, 0, c->stream>>>(lapv, c->uy, c->d2uydx2, c->k2b2, dcoef, c->g.nx, c->g.ny, c->g.K,
                                       1.0 / (dyy * wat[0]));
    TB_CHECK_LAUNCH(c);
    if (c->g.K < 2) return TB_OK;
    cplx* dw = c->tmp[15];
    k_dwydy_wall<<<nb, 128, 0, c->stream>>>(dw, c->wy, dcoef + 9, c->g.nx, c->g.ny, c->g.K, 1.0 / c->cfg.dy);
    TB_CHECK_LAUNCH(c);
    k_wx_wall<<<tb_blocks(c->g.K - 1, 32), 32, 0, c->stream>>>(c->wx, dw, lapv, c->px.lu, c->g.nx, c->g.ny, c->g.K, c->cfg.dx,
                                                               c->cfg.dx * c->cfg.dx, c->cfg.beta);
    TB_CHECK_LAUNCH(c);
    (void)dwy;
    return TB_OK;
}
int tb_wz_wall_k(tb_ctx* c, const cplx* lapv) {
    k_wz_wall<<<tb_blocks(c->g.K, 32), 32, 0, c->stream>>>(c->wz, c->wx, lapv, c->g.nx, c->g.ny, c->g.K, c->cfg.dx, c->cfg.beta);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}
int tb_ts_pert_k(tb_ctx* c, int t, double tempt) {
    const tb_config& cf = c->cfg;
    PertArgs A;
    std::memset(&A, 0, sizeof A);
    A.uy = c->uy; A.d2uydx2 = c->d2uydx2; A.fcx = c->fcx; A.fcllx = c->fcllx;
    A.nx = c->g.nx; A.ny = c->g.ny; A.i1 = cf.i1; A.i2 = cf.i2;
    for (int m = 0; m < cf.n_forced && m < 4; m++) {
        int k = cf.forced_mode[m];
        if (k < 0 || k >= c->g.K) continue;
        double Aamp = cf.forced_amp[m] * std::sqrt(cf.fac_y);
        double H = 1.0;
        double arg = H * ((double)t + tempt) * cf.omega * c->dt;
        if (cf.forced_phase[m] != 0.0) arg = arg + cf.forced_phase[m];
        double fct = Aamp * std::sin(arg);
        if (t < cf.stpp) {
            double ept = (double)t / (double)cf.stpp;
            fct = fct * ((6.0 * ept - 15.0) * ept + 10.0) * tb_powi(ept, 3);
        }
        A.mode[A.nf] = k; A.fct[A.nf] = fct; A.nf++;
    }
    if (A.nf == 0) return TB_OK;
    k_ts_pert<<<tb_blocks(c->g.nx, 128), 128, 0, c->stream>>>(A);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}

// loop(erro) (main_par.f:1762-1785)
int tb_loop_impl(tb_ctx* c, double erro, bool filter) {
    int r;
    if (filter && (r = tb_filter(c))) return r;
    if ((r = tb_bzone_k(c))) return r;
    cplx* dwzdx = c->tmp[0];
    cplx* duydy = c->tmp[1];
    if ((r = tb_outuy_k(c, dwzdx))) return r;
    if (c->cfg.precision == TB_FORM_MIXED) r = tb_poi_uy_mixed(c, dwzdx, erro);
    else r = tb_poi_uy_k(c, dwzdx, erro);
    if (r) return r;
    if ((r = tb_poi_ux_k(c, duydy))) return r;
    if ((r = tb_poi_uz_k(c, duydy))) return r;
    if ((r = tb_wx_wall_k(c, c->lapv))) return r;
    if ((r = tb_wz_wall_k(c, c->lapv))) return r;
    return tb_bzonew_k(c);
}
