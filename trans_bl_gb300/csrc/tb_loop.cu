// tb_loop.cu -- the stage driver (drv_fi/drv_les, RK4 update, wall forcing)
// and the velocity recovery of loop() except the v-Poisson solve.
#include "tb_internal.h"
#include "tb_warp.cuh"
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
    const cplx *gd, *gdddx;                               // drv_gv's d and dd/dx, null if none
    cplx *dvx, *dvy, *dvz;
    const double* k2b2;
    int nx, ny, K;
    double beta, invRe, fac_y, varg;
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
    if (A.gd) {   // drv_gv (main_par.f:1382-1396): - v_kb d varg, + varg dd/dx
        vx = cs_(vx, cm(A.varg, ikb(kb, A.gd[q])));
        vz = ca(vz, cm(A.varg, A.gdddx[q]));
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

// bzone (loop_par.f:6-45) for j >= 2 and bzonew (691-725) for j = 1; bdfc
// holds the two ramp rows bdfc(1,:), bdfc(2,:) one after the other.
__global__ void k_bzone(cplx* wx, cplx* wy, cplx* wz, const double* bdfc, const double* wzb, int nx, int ny, int K,
                        int wall, int form) {
    size_t n = (size_t)nx * (wall ? 1 : ny) * K;
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i, j, k;
    if (wall) { i = (int)(t % nx); k = (int)(t / nx); j = 0; }
    else { i = (int)(t % nx); j = (int)((t / nx) % ny); k = (int)(t / ((size_t)nx * ny)); if (j < 1) return; }
    size_t q = (size_t)i + (size_t)nx * (j + (size_t)ny * k);
    double bd = bdfc[(k == 2 ? (size_t)nx : 0) + i];   // bdt = 2 for the third mode (loop_par.f:19-20)
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

// ---------------------------------------------------------------------------
// x-direction recurrences, one warp per line (tb_warp.cuh).  Shared memory
// per warp: two line buffers of 32 x Sp complex (inputs E, rows V).

// The 4th-order implicit x integration of poi_ux mode 0 (loop_par.f:452-499)
// and of wz_wall (loop_par.f:361-425): w_0 given,
//   w_1     = (sg dx (251 r0 + 646 r1 - 264 r2 + 106 r3 - 19 r4) + 720 w_0) / 720
//   w_i     = (sg dx (281 r_{i-2} + 2056 r_{i-1} + 1176 r_i - 104 r_{i+1} + 11 r_{i+2}) / 90
//              + 11 w_{i-2} + 16 w_{i-1}) / 27                       2 <= i <= n-3
//   w_{n-2} = (sg dx (10 r_{n-4} + 57 r_{n-3} + 24 r_{n-2} - r_{n-1}) + 33 w_{n-4} + 24 w_{n-3}) / 57
//   w_{n-1} = (sg dx (251 r_{n-1} + 646 r_{n-2} - 264 r_{n-3} + 106 r_{n-4} - 19 r_{n-5}) + 720 w_{n-2}) / 720
// with r in E (lane chunks), w_0 = w0; the result (rows 1..n-1) goes to out.
__device__ void xint_line(const cplx* E, cplx* V, const WarpLine& L, int lane, cplx w0, double sgdx, cplx* out) {
    const int n = L.n, r0 = lane * L.S, r1 = min(n, r0 + L.S);
    const double i720 = 1.0 / 720.0, i27 = 1.0 / 27.0, i90 = 1.0 / 90.0, i57 = 1.0 / 57.0;
    auto e = [&](int i) { return E[L.slot(i)]; };
    cplx* Vl = V + lane * L.Sp;
    for (int i = r0; i < r1; i++) {
        cplx v;
        if (i == 0) v = w0;
        else if (i == 1) {
            cplx a = e(0), b = e(1), c = e(2), d = e(3), f = e(4);
            v = make_double2(sgdx * (251.0 * a.x + 646.0 * b.x - 264.0 * c.x + 106.0 * d.x - 19.0 * f.x) * i720,
                             sgdx * (251.0 * a.y + 646.0 * b.y - 264.0 * c.y + 106.0 * d.y - 19.0 * f.y) * i720);
        } else if (i <= n - 3) {
            cplx a = e(i - 2), b = e(i - 1), c = e(i), d = e(i + 1), f = e(i + 2);
            v = make_double2(sgdx * (281.0 * a.x + 2056.0 * b.x + 1176.0 * c.x - 104.0 * d.x + 11.0 * f.x) * i90 * i27,
                             sgdx * (281.0 * a.y + 2056.0 * b.y + 1176.0 * c.y - 104.0 * d.y + 11.0 * f.y) * i90 * i27);
        } else if (i == n - 2) {
            cplx a = e(i - 2), b = e(i - 1), c = e(i), d = e(i + 1);
            v = make_double2(sgdx * (10.0 * a.x + 57.0 * b.x + 24.0 * c.x - d.x) * i57,
                             sgdx * (10.0 * a.y + 57.0 * b.y + 24.0 * c.y - d.y) * i57);
        } else {
            cplx a = e(i), b = e(i - 1), c = e(i - 2), d = e(i - 3), f = e(i - 4);
            v = make_double2(sgdx * (251.0 * a.x + 646.0 * b.x - 264.0 * c.x + 106.0 * d.x - 19.0 * f.x) * i720,
                             sgdx * (251.0 * a.y + 646.0 * b.y - 264.0 * c.y + 106.0 * d.y - 19.0 * f.y) * i720);
        }
        Vl[i - r0] = v;
    }
    auto ca_ = [=](int i) -> double {
        if (i == 0) return 0.0;
        if (i == 1 || i == n - 1) return -720.0 * i720;
        if (i == n - 2) return -24.0 * i57;
        return -16.0 * i27;
    };
    auto cb_ = [=](int i) -> double {
        if (i <= 1 || i == n - 1) return 0.0;
        if (i == n - 2) return -33.0 * i57;
        return -11.0 * i27;
    };
    warp_rec2_fwd(Vl, r0, r1, lane, ca_, cb_);
    __syncwarp();
    for (int i = lane; i < n; i += 32)
        if (i >= 1) out[i] = V[L.slot(i)];
}

// poi_ux mode 0: ux(:, j, 0) from duydy by x integration, one warp per row j = 1..ny-2.
__global__ void __launch_bounds__(64) k_ux_mode0(cplx* ux, const cplx* duydy, int nx, int ny, double dx) {
    extern __shared__ cplx wsm[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int j = 1 + blockIdx.x * (blockDim.x >> 5) + wib;
    if (j > ny - 2) return;
    const WarpLine L{nx, WarpLine::chunk(nx), WarpLine::padded(nx)};
    cplx* E = wsm + (size_t)wib * 64 * L.Sp;
    cplx* V = E + 32 * L.Sp;
    const cplx* D = duydy + (size_t)nx * j;
    for (int i = lane; i < nx; i += 32) E[L.slot(i)] = D[i];
    __syncwarp();
    cplx* U = ux + (size_t)nx * j;
    xint_line(E, V, L, lane, U[0], -dx, U);
}

// wz_wall: wall wz of mode k from r = v_kb wx - lapv by x integration, one warp per mode.
__global__ void __launch_bounds__(64) k_wz_wall(cplx* wz, const cplx* wx, const cplx* lapv, int nx, int ny, int K, double dx,
                                                double beta) {
    extern __shared__ cplx wsm[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int k = blockIdx.x * (blockDim.x >> 5) + wib;
    if (k >= K) return;
    const WarpLine L{nx, WarpLine::chunk(nx), WarpLine::padded(nx)};
    cplx* E = wsm + (size_t)wib * 64 * L.Sp;
    cplx* V = E + 32 * L.Sp;
    const double kb = (double)k * beta;
    const cplx* WX = wx + (size_t)nx * ny * k;
    const cplx* LV = lapv + (size_t)nx * k;
    for (int i = lane; i < nx; i += 32) { cplx v = ikb(kb, WX[i]); cplx l = LV[i]; E[L.slot(i)] = make_double2(v.x - l.x, v.y - l.y); }
    __syncwarp();
    cplx* W = wz + (size_t)nx * ny * k;
    xint_line(E, V, L, lane, W[0], dx, W);
}

// Pentadiagonal x solve with the LU of lhs5 (lusolver / lusolver_1,
// penta_par.f:53-208) of mode k, rhs rows
//   r_0 = boundary value, r_1 = c12 (e_0 + 10 e_1 + e_2),
//   r_i = c8 (e_{i-1} + 5.5 e_i + e_{i+1}),  r_{n-2} = c12 (e_{n-1} + 10 e_{n-2} + e_{n-3}),
//   r_{n-1} = rn,
// with e in E (overwritten); the solution (rows 1..n-1) goes to out.
__device__ void penta_line(cplx* E, const WarpLine& L, int lane, const double* lu, cplx r0v, cplx rn, double c12,
                           double c8, cplx* out) {
    const int n = L.n, r0 = lane * L.S, r1 = min(n, r0 + L.S);
    auto e = [&](int i) { return E[L.slot(i)]; };
    cplx* Vl = E + lane * L.Sp;   // the rhs and the solution overwrite this lane's rows of e in place
    // what the stencils read outside the lane's rows (e(r0-1), e(r1)) and the
    // rhs of rows 1 and n-2, taken before any lane overwrites its rows
    const cplx z = make_double2(0.0, 0.0);
    cplx ep = (r0 >= 1 && r0 < r1) ? e(r0 - 1) : z;
    const cplx en = (r1 < n && r0 < r1) ? e(r1) : z;
    cplx v1 = z, vn2 = z;
    if (1 >= r0 && 1 < r1) { cplx a = e(0), b = e(1), c = e(2); v1 = make_double2(c12 * (a.x + 10.0 * b.x + c.x), c12 * (a.y + 10.0 * b.y + c.y)); }
    if (n - 2 >= r0 && n - 2 < r1) { cplx a = e(n - 1), b = e(n - 2), c = e(n - 3); vn2 = make_double2(c12 * (a.x + 10.0 * b.x + c.x), c12 * (a.y + 10.0 * b.y + c.y)); }
    __syncwarp();
    for (int i = r0; i < r1; i++) {
        const cplx b = Vl[i - r0];   // e(i), not yet overwritten
        cplx v;
        if (i == 0) v = r0v;
        else if (i == 1) v = v1;
        else if (i <= n - 3) {
            const cplx a = ep, c = (i + 1 < r1) ? Vl[i + 1 - r0] : en;
            v = make_double2(c8 * (a.x + 5.5 * b.x + c.x), c8 * (a.y + 5.5 * b.y + c.y));
        } else if (i == n - 2) v = vn2;
        else v = rn;
        ep = b;
        Vl[i - r0] = v;
    }
    const double *L1 = lu, *L2 = lu + n, *IU3 = lu + 2 * n, *U4 = lu + 3 * n, *U5 = lu + 4 * n;
    // forward y_i = r_i - l2_i y_{i-1} - l1_i y_{i-2}; row 0 is the boundary row
    warp_rec2_fwd(Vl, r0, r1, lane, [=](int i) { return i == 0 ? 0.0 : L2[i]; }, [=](int i) { return i <= 1 ? 0.0 : L1[i]; });
    // backward x_i = (y_i - u4_i x_{i+1} - u5_i x_{i+2}) / u3_i; row 0 keeps its value
    warp_rec2_bwd(Vl, r0, r1, lane, [=](int i) { return i == 0 ? 0.0 : U4[i]; }, [=](int i) { return i == 0 ? 0.0 : U5[i]; },
                  [=](int i) { return i == 0 ? 1.0 : IU3[i]; });
    __syncwarp();
    for (int i = lane; i < n; i += 32)
        if (i >= 1) out[i] = E[L.slot(i)];
}

// x-penta Poisson of poi_ux / poi_uz (loop_par.f:519-563, 641-685), one warp
// per line (j >= 1, k >= 1): e = D + s v_kb W, rhs scaled by g (ux: s = +1,
// g = -1; uz: s = -1, g = +1); the last row is (g' D + v_kb W) / (k beta)^2.
struct PentaArgs {
    const cplx* D;   // d2uydxdy or dwydx
    const cplx* W;   // wy or duydy
    cplx* out;       // ux or uz
    const double* lu;
    int nx, ny, K, uz;
    double dxx, beta;
};
__global__ void __launch_bounds__(64) k_penta_x(PentaArgs A) {
    extern __shared__ cplx wsm[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int t = blockIdx.x * (blockDim.x >> 5) + wib;
    if (t >= (A.ny - 1) * (A.K - 1)) return;
    const int j = 1 + t % (A.ny - 1), k = 1 + t / (A.ny - 1);
    const int n = A.nx;
    const WarpLine L{n, WarpLine::chunk(n), WarpLine::padded(n)};
    cplx* E = wsm + (size_t)wib * 32 * L.Sp;
    size_t base = (size_t)n * (j + (size_t)A.ny * k);
    const cplx* D = A.D + base;
    const cplx* W = A.W + base;
    cplx* O = A.out + base;
    const double kb = (double)k * A.beta;
    const double s = A.uz ? -1.0 : 1.0, g = A.uz ? 1.0 : -1.0;
    for (int i = lane; i < n; i += 32) {
        cplx v = ikb(kb, W[i]), d = D[i];
        E[L.slot(i)] = make_double2(d.x + s * v.x, d.y + s * v.y);
    }
    __syncwarp();
    const double den = 1.0 / ((double)k * (double)k * A.beta * A.beta);
    cplx v = ikb(kb, W[n - 1]), dn = D[n - 1];
    cplx rn = A.uz ? make_double2((-dn.x + v.x) * den, (-dn.y + v.y) * den) : make_double2((v.x + dn.x) * den, (v.y + dn.y) * den);
    penta_line(E, L, lane, A.lu + (size_t)k * 5 * n, O[0], rn, g * (A.dxx / 12.0), g * (8.0 * A.dxx), O);
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

// wx_wall (loop_par.f:174-255): per mode k >= 1, d2wy/dxdy by explicit
// stencils, then the x-penta solve with the LU of lhs5 (lusolver_1,
// penta_par.f:53-127); one warp per mode.
__global__ void __launch_bounds__(64) k_wx_wall(cplx* wx, const cplx* dwdy, const cplx* lapv, const double* lu_all, int nx,
                                                int ny, int K, double dx, double dxx, double beta) {
    extern __shared__ cplx wsm[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int k = 1 + blockIdx.x * (blockDim.x >> 5) + wib;
    if (k >= K) return;
    const int n = nx;
    const WarpLine L{n, WarpLine::chunk(n), WarpLine::padded(n)};
    cplx* E = wsm + (size_t)wib * 32 * L.Sp;
    const cplx* dw = dwdy + (size_t)nx * k;
    const cplx* LV = lapv + (size_t)nx * k;
    cplx* WX = wx + (size_t)nx * ny * k;  // row j = 1
    const double kb = (double)k * beta;
    const double idx6 = 1.0 / 6.0 / dx, idx60 = 1.0 / 60.0 / dx, idx12 = 1.0 / 12.0 / dx, idx2 = 1.0 / 2.0 / dx;
    auto d2 = [&](int i) -> cplx {  // d2wydxdy(i), 0-based i
        if (i >= 3 && i <= n - 4) {
            cplx a = dw[i + 1], b = dw[i - 1], c = dw[i - 2], d = dw[i + 2], e = dw[i + 3], f = dw[i - 3];
            return make_double2((45.0 * (a.x - b.x) + 9.0 * (c.x - d.x) + e.x - f.x) * idx60,
                                (45.0 * (a.y - b.y) + 9.0 * (c.y - d.y) + e.y - f.y) * idx60);
        }
        if (i == n - 3) {
            cplx a = dw[n - 5], b = dw[n - 4], c = dw[n - 2], d = dw[n - 1];
            return make_double2((a.x - 8.0 * b.x + 8.0 * c.x - d.x) * idx12, (a.y - 8.0 * b.y + 8.0 * c.y - d.y) * idx12);
        }
        if (i == n - 2) {
            cplx a = dw[n - 1], b = dw[n - 2], c = dw[n - 3], d = dw[n - 4];
            return make_double2((2.0 * a.x + 3.0 * b.x - 6.0 * c.x + d.x) * idx6, (2.0 * a.y + 3.0 * b.y - 6.0 * c.y + d.y) * idx6);
        }
        if (i == n - 1) {
            cplx a = dw[n - 1], b = dw[n - 2], c = dw[n - 3];
            return make_double2((3.0 * a.x - 4.0 * b.x + c.x) * idx2, (3.0 * a.y - 4.0 * b.y + c.y) * idx2);
        }
        const double W0[7] = {-14.7, 36.0, -45.0, 40.0, -22.5, 7.2, -1.0};
        const double W1[7] = {-1.0, -7.7, 15.0, -10.0, 5.0, -1.5, 0.2};
        const double W2[7] = {0.2, -2.4, -3.5, 8.0, -3.0, 0.8, -0.1};
        const double* cw = (i == 0) ? W0 : (i == 1) ? W1 : W2;
        cplx acc = make_double2(0, 0);
        for (int m = 0; m < 7; m++) { acc.x += cw[m] * dw[m].x; acc.y += cw[m] * dw[m].y; }
        return make_double2(acc.x * idx6, acc.y * idx6);
    };
    for (int i = lane; i < n; i += 32) {
        cplx a = d2(i), v = ikb(kb, LV[i]);
        E[L.slot(i)] = make_double2(-a.x + v.x, -a.y + v.y);
    }
    __syncwarp();
    const double den = 1.0 / ((double)k * (double)k * beta * beta);
    cplx dd = d2(n - 1), vv = ikb(kb, LV[n - 1]);
    cplx rn = make_double2((dd.x - vv.x) * den, (dd.y - vv.y) * den);
    penta_line(E, L, lane, lu_all + (size_t)k * 5 * n, WX[0], rn, dxx / 12.0, 8.0 * dxx, WX);
}

// Shared memory of the warp-per-line x kernels (two line buffers per warp).
constexpr int XW_WARPS = 2;
size_t xw_smem(int nx) { return (size_t)XW_WARPS * 64 * WarpLine::padded(nx) * sizeof(cplx); }
size_t xw_smem1(int nx) { return (size_t)XW_WARPS * 32 * WarpLine::padded(nx) * sizeof(cplx); }   // in-place lines

// ts2d_pert / ts3d_pert (main_par.f:1613-1685) for each forced mode.
struct PertArgs {
    cplx *uy, *d2uydx2;
    const double *fcx, *fcllx;
    int nx, ny, i1, i2, nf;
    int mode[4];
    double fct[4];
    const double* fct_dev;   // when set, the amplitudes are read here (a recorded step graph)
};
__global__ void k_ts_pert(PertArgs A) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;  // 0-based
    if (i < A.i1 || i > A.i2 - 2) return;          // 1-based i1+1 .. i2-1
    for (int m = 0; m < A.nf; m++) {
        int k = A.mode[m];
        double f = A.fct_dev ? A.fct_dev[m] : A.fct[m];
        A.uy[(size_t)i + (size_t)A.nx * A.ny * k] = make_double2(A.fcx[i] * f, 0.0);
        A.d2uydx2[(size_t)i + (size_t)A.nx * k] = make_double2(A.fcllx[i] * f, 0.0);
    }
}

// lterms_gv (nlterms_par.f:89-112): the disturbance times the 2D base flow,
// pointwise in every mode.
__global__ void k_lterms_gv(const cplx* ux, const cplx* uy, const cplx* wx, const cplx* wy, const cplx* wz,
                            const double* uxb, const double* uyb, const double* wzb, cplx* a, cplx* b, cplx* c,
                            cplx* d, int nx, int ny, int K) {
    const size_t n2 = (size_t)nx * ny;
    const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= n2 * K) return;
    const size_t p = q % n2;
    const double U = uxb[p], V = uyb[p], W = wzb[p];
    const cplx ex = wx[q], ey = wy[q], ez = wz[q], u = ux[q], v = uy[q];
    a[q] = cs_(cm(V, ex), cm(U, ey));
    b[q] = ca(cm(U, ez), cm(W, u));
    c[q] = cs_(cm(-V, ez), cm(W, v));
    d[q] = cm(2.0 * U, u);
}

// gv_pert (main_par.f:1577-1610): the steady Goertler strip in every mode
// k >= 1 (0-based), wall row, 1-based i1+1 .. i2-1; amplitude a (or *a_dev
// in a recorded step).
__global__ void k_gv_pert(cplx* uy, cplx* d2uydx2, const double* fcx2, const double* fcllx2, int nx, int ny, int K,
                          int i1, int i2, double a, const double* a_dev) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t % nx, k = 1 + t / nx;
    if (k >= K || i < i1 || i > i2 - 2) return;
    const double A = a_dev ? *a_dev : a;
    uy[(size_t)i + (size_t)nx * ny * k] = make_double2(A * fcx2[i], 0.0);
    d2uydx2[(size_t)i + (size_t)nx * k] = make_double2(A * fcllx2[i], 0.0);
}

}  // namespace

// drv_gv (main_par.f:1338-1401): linear terms about the base flow, their
// derivatives, the viscous terms and the curvature terms with varg =
// Go^2 / sqrt(Re) at every point (init_gv, main_par.f:944-970); dvargdx, the
// compact x-derivative of the constant varg, is zero and left out.
int tb_drv_gv(tb_ctx* c, cplx* dvx, cplx* dvy, cplx* dvz) {
    cplx** t = c->tmp;
    int r;
    k_lterms_gv<<<tb_blocks(tb_n3(c), 256), 256, 0, c->stream>>>(c->ux, c->uy, c->wx, c->wy, c->wz, c->uxb, c->uyb,
                                                                  c->wzb, t[0], t[1], t[2], t[13], c->g.nx, c->g.ny,
                                                                  c->g.K);
    TB_CHECK_LAUNCH(c);
    XJob xj[6] = {{t[0], t[3], XOP_D1}, {t[1], t[4], XOP_D1}, {t[13], t[14], XOP_D1},
                  {c->wx, t[5], XOP_D2}, {c->wy, t[6], XOP_D2}, {c->wz, t[7], XOP_D2}};
    YJob yj[5] = {{t[0], t[8], YOP_D1}, {t[2], t[9], YOP_D1},
                  {c->wx, t[10], YOP_D2}, {c->wy, t[11], YOP_D2}, {c->wz, t[12], YOP_D2}};
    if ((r = tb_launch_xlines(c, xj, 6))) return r;
    if ((r = tb_launch_ylines(c, yj, 5))) return r;
    return tb_combine_gv(c, t[3], t[8], t[1], t[5], t[10], t[2], t[6], t[11], t[4], t[9], t[7], t[12], t[13], t[14],
                         c->cfg.go_number * c->cfg.go_number / std::sqrt(c->cfg.Re), dvx, dvy, dvz);
}

// The momentum part of drv_gv / drv_gvth from its derivative fields.
int tb_combine_gv(tb_ctx* c, const cplx* dadx, const cplx* dady, const cplx* b, const cplx* xx0, const cplx* yy0,
                  const cplx* cc, const cplx* xx1, const cplx* yy1, const cplx* dbdx, const cplx* dcdy,
                  const cplx* xx2, const cplx* yy2, const cplx* d, const cplx* dddx, double varg, cplx* dvx, cplx* dvy,
                  cplx* dvz) {
    CombArgs A;
    std::memset(&A, 0, sizeof A);
    A.dady = dady; A.b = b; A.xx0 = xx0; A.yy0 = yy0; A.wx = c->wx;
    A.c = cc; A.dadx = dadx; A.xx1 = xx1; A.yy1 = yy1; A.wy = c->wy;
    A.dbdx = dbdx; A.dcdy = dcdy; A.xx2 = xx2; A.yy2 = yy2; A.wz = c->wz;
    A.gd = d; A.gdddx = dddx; A.varg = varg;
    A.dvx = dvx; A.dvy = dvy; A.dvz = dvz; A.k2b2 = c->k2b2;
    A.nx = c->g.nx; A.ny = c->g.ny; A.K = c->g.K; A.beta = c->cfg.beta; A.invRe = 1.0 / c->cfg.Re; A.fac_y = c->cfg.fac_y;
    k_combine<<<tb_blocks(tb_n3(c), 256), 256, 0, c->stream>>>(A);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}

// ===========================================================================
int tb_drv_k(tb_ctx* c, cplx* dvx, cplx* dvy, cplx* dvz) {
    cplx** t = c->tmp;
    int r;
    if (c->cfg.my_form == 1) return tb_drv_gv(c, dvx, dvy, dvz);
    if (c->cfg.my_form == 2) return tb_drv_gvth(c, dvx, dvy, dvz, dvx == c->dv1x ? c->dv1t : c->dv2t);
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
    return c->cfg.my_form == 2 ? tb_rk_update_th(c, stage) : TB_OK;
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
    return c->cfg.my_form == 2 ? tb_bzone_th(c) : TB_OK;
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
    size_t sm = xw_smem(c->g.nx);
    TB_CUDA(cudaFuncSetAttribute(k_ux_mode0, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_ux_mode0<<<tb_blocks(c->g.ny - 2, XW_WARPS), 32 * XW_WARPS, sm, c->stream>>>(c->ux, duydy, c->g.nx, c->g.ny, c->cfg.dx);
    TB_CHECK_LAUNCH(c);
    if (c->g.K < 2) return TB_OK;
    cplx* d2 = c->tmp[13];
    XJob xj[1] = {{duydy, d2, XOP_D1}};
    if ((r = tb_launch_xlines(c, xj, 1))) return r;
    PentaArgs A{d2, c->wy, c->ux, c->px.lu, c->g.nx, c->g.ny, c->g.K, 0, c->cfg.dx * c->cfg.dx, c->cfg.beta};
    cudaEvent_t ps = nullptr;
    if ((r = tb_prof_begin(c, PROF_PENTA, &ps))) return r;
    const size_t sp = xw_smem1(c->g.nx);
    TB_CUDA(cudaFuncSetAttribute(k_penta_x, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp));
    k_penta_x<<<tb_blocks((size_t)(c->g.ny - 1) * (c->g.K - 1), XW_WARPS), 32 * XW_WARPS, sp, c->stream>>>(A);
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
    cudaEvent_t ps = nullptr;
    if ((r = tb_prof_begin(c, PROF_PENTA, &ps))) return r;
    const size_t sp = xw_smem1(c->g.nx);
    TB_CUDA(cudaFuncSetAttribute(k_penta_x, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp));
    k_penta_x<<<tb_blocks((size_t)(c->g.ny - 1) * (c->g.K - 1), XW_WARPS), 32 * XW_WARPS, sp, c->stream>>>(A);
    TB_CHECK_LAUNCH(c);
    return tb_prof_end(c, PROF_PENTA, ps);
}
int tb_wx_wall_k(tb_ctx* c, cplx* lapv) {
    const double* wat = c->coefs.data() + 100 + 24 * c->g.msh - 17;  // w_at_w_coef(9) on the host
    const double* dcoef = c->wcoef;   // device copy of w_at_w_coef(9), dwydy_coef(8)
    double dyy = c->cfg.dy * c->cfg.dy;
    unsigned nb = tb_blocks((size_t)c->g.nx * c->g.K, 128);
    k_lapv<<<nb, 128, 0, c->stream>>>(lapv, c->uy, c->d2uydx2, c->k2b2, dcoef, c->g.nx, c->g.ny, c->g.K,
                                       1.0 / (dyy * wat[0]));
    TB_CHECK_LAUNCH(c);
    if (c->g.K < 2) return TB_OK;
    cplx* dw = c->tmp[15];
    k_dwydy_wall<<<nb, 128, 0, c->stream>>>(dw, c->wy, dcoef + 9, c->g.nx, c->g.ny, c->g.K, 1.0 / c->cfg.dy);
    TB_CHECK_LAUNCH(c);
    size_t sm = xw_smem1(c->g.nx);
    TB_CUDA(cudaFuncSetAttribute(k_wx_wall, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_wx_wall<<<tb_blocks(c->g.K - 1, XW_WARPS), 32 * XW_WARPS, sm, c->stream>>>(c->wx, dw, lapv, c->px.lu, c->g.nx, c->g.ny,
                                                                                 c->g.K, c->cfg.dx, c->cfg.dx * c->cfg.dx,
                                                                                 c->cfg.beta);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}
int tb_wz_wall_k(tb_ctx* c, const cplx* lapv) {
    size_t sm = xw_smem(c->g.nx);
    TB_CUDA(cudaFuncSetAttribute(k_wz_wall, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_wz_wall<<<tb_blocks(c->g.K, XW_WARPS), 32 * XW_WARPS, sm, c->stream>>>(c->wz, c->wx, lapv, c->g.nx, c->g.ny, c->g.K,
                                                                             c->cfg.dx, c->cfg.beta);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}
// Wall-forcing amplitude of each forced mode at step t + tempt, in the order
// of the forced modes that exist on this grid; returns their number.
int tb_ts_pert_fct(tb_ctx* c, int t, double tempt, double* out) {
    const tb_config& cf = c->cfg;
    if (cf.my_form == 1) {   // gv_pert (main_par.f:1577-1600): steady after the ramp
        double A = 1e-6 * std::sqrt(cf.fac_y);
        if (t < cf.stpp) {
            double ep = (double)t / (double)cf.stpp;
            A = A * ((6.0 * ep - 15.0) * ep + 10.0) * tb_powi(ep, 3);
        }
        out[0] = A;
        return 1;
    }
    int nf = 0;
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
        out[nf++] = fct;
    }
    return nf;
}

int tb_ts_pert_k(tb_ctx* c, int t, double tempt) {
    const tb_config& cf = c->cfg;
    if (cf.my_form == 1) {
        double a = 0.0;
        tb_ts_pert_fct(c, t, tempt, &a);
        const double* a_dev = c->capturing ? c->d_fct + (tempt < 0.75 ? 0 : 4) : nullptr;
        if (c->g.K < 2) return TB_OK;
        k_gv_pert<<<tb_blocks((size_t)c->g.nx * (c->g.K - 1), 128), 128, 0, c->stream>>>(
            c->uy, c->d2uydx2, c->fcx2, c->fcllx2, c->g.nx, c->g.ny, c->g.K, cf.i1, cf.i2, a, a_dev);
        TB_CHECK_LAUNCH(c);
        return TB_OK;
    }
    PertArgs A;
    std::memset(&A, 0, sizeof A);
    A.uy = c->uy; A.d2uydx2 = c->d2uydx2; A.fcx = c->fcx; A.fcllx = c->fcllx;
    A.nx = c->g.nx; A.ny = c->g.ny; A.i1 = cf.i1; A.i2 = cf.i2;
    for (int m = 0; m < cf.n_forced && m < 4; m++) {
        int k = cf.forced_mode[m];
        if (k < 0 || k >= c->g.K) continue;
        A.mode[A.nf++] = k;
    }
    tb_ts_pert_fct(c, t, tempt, A.fct);
    // in a recorded step the amplitudes of stage 1 (tempt 0.5) and stage 3
    // (tempt 1) are uploaded before each replay
    if (c->capturing) A.fct_dev = c->d_fct + (tempt < 0.75 ? 0 : 4);
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
