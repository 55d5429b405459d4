// tb_oracle.cpp -- CPU restatement of the trans_bl per-RK4-stage hot path.
//
// TEST INFRASTRUCTURE ONLY (the checker of the GPU library; see tb_oracle.h
// for what pins it).  Each function restates one reference subroutine, in its
// loop order and operation order, with MPI collapsed to a single rank.  The
// build (oracle/Makefile) disables floating-point contraction so that the
// arithmetic is the same on x86-64 and aarch64 hosts.
#include "tb_oracle.h"
#ifdef _OPENMP
#include <omp.h>
#endif
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>

namespace {

struct C { double re, im; };
inline C mk(double r, double i) { C c; c.re = r; c.im = i; return c; }
inline C operator+(C a, C b) { return mk(a.re + b.re, a.im + b.im); }
inline C operator-(C a, C b) { return mk(a.re - b.re, a.im - b.im); }
inline C operator-(C a) { return mk(-a.re, -a.im); }
inline C operator*(double s, C a) { return mk(s * a.re, s * a.im); }
inline C operator*(C a, double s) { return mk(a.re * s, a.im * s); }
inline C operator/(C a, double s) { return mk(a.re / s, a.im / s); }
// Fortran complex*complex (gfortran expands it inline without NaN recovery).
inline C operator*(C a, C b) { return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
inline double cabs_(C a) { return std::hypot(a.re, a.im); }

// real ** integer as libgcc's __powidf2 (binary exponentiation).
double powi(double x, int m) {
    unsigned n = m < 0 ? -m : m;
    double y = (n % 2) ? x : 1.0;
    while (n >>= 1) { x = x * x; if (n % 2) y = y * x; }
    return m < 0 ? 1.0 / y : y;
}

const double PI = 3.141592653589793;      // par.for:49
const double TWOPI_NR = 6.28318530717959;  // nlterms_par.f:316,377,460

}  // namespace

struct ora_ctx {
    tb_config cfg;
    int nx, ny, K, P, msh;
    double dx, dxx, dy, dyy, stf, Re, fac_y, alpha, omega, beta, dt, dt2, dt6, dz;
    // coefficients (comm.coef)
    double fp_fd_e[6], sp_fd[9], cp_fd[8], pp_fd[9], lp_fd[7];
    double fp_sd[8], sp_sd[10], cp_sd[8], pp_sd[10], lp_sd[8];
    std::vector<double> sp_poi, cp_poi, pp_poi, lp_poi;  // (7|8|4|5, msh) column-major
    double w_at_w[9], dwydy[8];
    bool have_coefs = false, have_base = false;
    // comm.multi / comm.fourier
    std::vector<int> v_ptsx, v_ptsy;
    std::vector<double> v_dy0, v_stf, v_dx2, v_qdy, v_qdy2;  // v_qdy2(jmax, msh)
    std::vector<double> v_k2b2;
    std::vector<C> v_kb;
    // LHS of the compact schemes (derivs_par.f:6-29)
    std::vector<double> a1x, b1x, c1x, a2x, b2x, c2x, a1y, b1y, c1y, a2y, b2y, c2y, a1fv, b1fv, c1fv;
    std::vector<double> afil, bfil, cfil;
    std::vector<double> bdfc, bdfc2;     // (imax) ramps bdfc(1,:), bdfc(2,:) (equal but for form 1)
    std::vector<double> fcx, fcllx;      // (i2)
    std::vector<double> fcx2, fcllx2;    // (nx) Goertler strip (var_gv)
    std::vector<double> gibbs;           // (kfour)
    std::vector<double> delta_no;        // (nx, ny, kphys)
    std::vector<double> uxb, uyb, wzb, duexmdx;
    // state (comm.var) and RK storage
    std::vector<C> ux, uy, uz, wx, wy, wz;
    std::vector<C> wx1, wy1, wz1, dv1x, dv1y, dv1z, dv2x, dv2y, dv2z;
    std::vector<C> d2uydx2;              // (nx, kfour)
    std::vector<C> fx, fy, fz;           // common /force/
    std::vector<C> th, th1, dv1t, dv2t;  // thermal form: temperature and its RK storage
    std::vector<double> thb;             // common /blast/ (nx, ny)
    // Poisson statistics of the last poi_uy
    std::vector<int> pv; std::vector<double> pres;

    size_t N3() const { return (size_t)nx * ny * K; }
    size_t id(int i, int j, int k) const { return (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (k - 1)); }
    size_t id2(int i, int j) const { return (size_t)(i - 1) + (size_t)nx * (j - 1); }
    double& QDY2(int j, int l) { return v_qdy2[(size_t)(j - 1) + (size_t)ny * (l - 1)]; }
    double SP(int c, int l) const { return sp_poi[(c - 1) + 7 * (l - 1)]; }
    double CP(int c, int l) const { return cp_poi[(c - 1) + 8 * (l - 1)]; }
    double PP(int c, int l) const { return pp_poi[(c - 1) + 4 * (l - 1)]; }
    double LP(int c, int l) const { return lp_poi[(c - 1) + 5 * (l - 1)]; }
};

namespace {

// ---------------------------------------------------------------------------
// Tridiagonal Thomas sweep along a strided line (tridparx with one rank,
// derivs_par.f:775-858; tridy derivs_par.f:947-975; tridseqx 1009-1037).
// The single-rank path of tridparx recomputes bet at i_ini-1 with the same
// value, so all three reduce to this recurrence.
void thomas(const double* a, const double* b, const double* c, C* r, int n, size_t stride,
            std::vector<double>& gam, std::vector<C>& u) {
    double bet = b[0];
    u[0] = r[0] / bet;
    for (int i = 1; i < n; i++) {
        gam[i] = c[i - 1] / bet;
        bet = b[i] - a[i] * gam[i];
        u[i] = (r[(size_t)i * stride] - a[i] * u[i - 1]) / bet;
    }
    for (int i = n - 2; i >= 0; i--) u[i] = u[i] - gam[i + 1] * u[i + 1];
    for (int i = 0; i < n; i++) r[(size_t)i * stride] = u[i];
}
void thomas_r(const double* a, const double* b, const double* c, double* r, int n, size_t stride,
              std::vector<double>& gam, std::vector<double>& u) {
    double bet = b[0];
    u[0] = r[0] / bet;
    for (int i = 1; i < n; i++) {
        gam[i] = c[i - 1] / bet;
        bet = b[i] - a[i] * gam[i];
        u[i] = (r[(size_t)i * stride] - a[i] * u[i - 1]) / bet;
    }
    for (int i = n - 2; i >= 0; i--) u[i] = u[i] - gam[i + 1] * u[i + 1];
    for (int i = 0; i < n; i++) r[(size_t)i * stride] = u[i];
}

// RHS of the x first derivative (derivs_par.f:259-302; rhsxue 180-219).
template <class T>
void rhsx_line(const T* f, T* r, int n, double dx) {
    r[0] = (-(25.0 * f[0]) + 48.0 * f[1] - 36.0 * f[2] + 16.0 * f[3] - 3.0 * f[4]) / (12.0 * dx);
    r[1] = (-(406.0 * f[0]) - 300.0 * f[1] + 760.0 * f[2] - 80.0 * f[3] + 30.0 * f[4] - 4.0 * f[5]) / (120.0 * dx);
    for (int i = 2; i < n - 2; i++) r[i] = (f[i + 2] - f[i - 2] + 28.0 * (f[i + 1] - f[i - 1])) / (12.0 * dx);
    int m = n - 1;
    r[m - 1] = (-(406.0 * f[m]) - 300.0 * f[m - 1] + 760.0 * f[m - 2] - 80.0 * f[m - 3] + 30.0 * f[m - 4]
                - 4.0 * f[m - 5]) / (-(120.0 * dx));
    r[m] = (-(74.0 * f[m]) + 16.0 * f[m - 1] + 72.0 * f[m - 2] - 16.0 * f[m - 3] + 2.0 * f[m - 4]) / (-(24.0 * dx));
}
// RHS of the x second derivative (derivs_par.f:351-397).
void rhsxx_line(const C* f, C* r, int n, double dxx) {
    r[0] = (9775.0 * f[0] - 20285.0 * f[1] + 11170.0 * f[2] - 550.0 * f[3] - 145.0 * f[4] + 35.0 * f[5]) / (60.0 * dxx);
    r[1] = (4834.0 * f[0] - 8424.0 * f[1] + 1890.0 * f[2] + 2320.0 * f[3] - 810.0 * f[4] + 216.0 * f[5]
            - 26.0 * f[6]) / (360.0 * dxx);
    for (int i = 2; i < n - 2; i++)
        r[i] = (3.0 * (f[i + 2] + f[i - 2]) + 48.0 * (f[i + 1] + f[i - 1]) - 102.0 * f[i]) / (4.0 * dxx);
    int m = n - 1;
    r[m - 1] = (4834.0 * f[m] - 8424.0 * f[m - 1] + 1890.0 * f[m - 2] + 2320.0 * f[m - 3] - 810.0 * f[m - 4]
                + 216.0 * f[m - 5] - 26.0 * f[m - 6]) / (360.0 * dxx);
    r[m] = (9775.0 * f[m] - 20285.0 * f[m - 1] + 11170.0 * f[m - 2] - 550.0 * f[m - 3] - 145.0 * f[m - 4]
            + 35.0 * f[m - 5]) / (60.0 * dxx);
}

void derparx_impl(ora_ctx* o, C* ddx, const C* fc) {  // derivs_par.f:80-95
    int n = o->nx;
#pragma omp parallel for schedule(static)
    for (int q = 0; q < o->K * o->ny; q++) {
            std::vector<double> gam(n); std::vector<C> u(n);
            int k = 1 + q / o->ny, j = 1 + q % o->ny;
            size_t base = o->id(1, j, k);
            rhsx_line(fc + base, ddx + base, n, o->dx);
            thomas(o->a1x.data(), o->b1x.data(), o->c1x.data(), ddx + base, n, 1, gam, u);
        }
}
void derparxx_impl(ora_ctx* o, C* d2, const C* fc) {  // derivs_par.f:98-113
    int n = o->nx;
#pragma omp parallel for schedule(static)
    for (int q = 0; q < o->K * o->ny; q++) {
            std::vector<double> gam(n); std::vector<C> u(n);
            int k = 1 + q / o->ny, j = 1 + q % o->ny;
            size_t base = o->id(1, j, k);
            rhsxx_line(fc + base, d2 + base, n, o->dxx);
            thomas(o->a2x.data(), o->b2x.data(), o->c2x.data(), d2 + base, n, 1, gam, u);
        }
}
// y first derivative RHS (rhsy derivs_par.f:400-449, rhsyfv 504-549).
void rhsy_line(ora_ctx* o, const C* f, C* r, size_t s, bool fv) {
    int J = o->ny;
    auto F = [&](int j) -> C { return f[(size_t)(j - 1) * s]; };
    auto R = [&](int j) -> C& { return r[(size_t)(j - 1) * s]; };
    const double* q = o->v_qdy.data() - 1;  // 1-based
    if (fv) {
        R(1) = mk(0.0, 0.0);
    } else {
        R(1) = q[1] * (o->fp_fd_e[1] * F(1) + o->fp_fd_e[2] * F(2) + o->fp_fd_e[3] * F(3) + o->fp_fd_e[4] * F(4)
                       + o->fp_fd_e[5] * F(5));
    }
    R(2) = q[1] * (o->sp_fd[3] * F(1) + o->sp_fd[4] * F(2) + o->sp_fd[5] * F(3) + o->sp_fd[6] * F(4)
                   + o->sp_fd[7] * F(5) + o->sp_fd[8] * F(6));
    for (int j = 3; j <= J - 2; j++)
        R(j) = q[j - 2] * (o->cp_fd[3] * F(j - 2) + o->cp_fd[4] * F(j - 1) + o->cp_fd[5] * F(j) + o->cp_fd[6] * F(j + 1)
                           + o->cp_fd[7] * F(j + 2));
    R(J - 1) = q[J - 5] * (o->pp_fd[3] * F(J) + o->pp_fd[4] * F(J - 1) + o->pp_fd[5] * F(J - 2) + o->pp_fd[6] * F(J - 3)
                           + o->pp_fd[7] * F(J - 4) + o->pp_fd[8] * F(J - 5));
    R(J) = q[J - 4] * (o->lp_fd[2] * F(J) + o->lp_fd[3] * F(J - 1) + o->lp_fd[4] * F(J - 2) + o->lp_fd[5] * F(J - 3)
                       + o->lp_fd[6] * F(J - 4));
}
// y second derivative RHS (derivs_par.f:552-611).
void rhsyy_line(ora_ctx* o, const C* f, C* r, size_t s) {
    int J = o->ny;
    auto F = [&](int j) -> C { return f[(size_t)(j - 1) * s]; };
    auto R = [&](int j) -> C& { return r[(size_t)(j - 1) * s]; };
    R(1) = (o->fp_sd[2] * F(1) + o->fp_sd[3] * F(2) + o->fp_sd[4] * F(3) + o->fp_sd[5] * F(4) + o->fp_sd[6] * F(5)
            + o->fp_sd[7] * F(6)) * o->QDY2(1, 1);
    R(2) = (o->sp_sd[3] * F(1) + o->sp_sd[4] * F(2) + o->sp_sd[5] * F(3) + o->sp_sd[6] * F(4) + o->sp_sd[7] * F(5)
            + o->sp_sd[8] * F(6) + o->sp_sd[9] * F(7)) * o->QDY2(1, 1);
    for (int j = 3; j <= J - 2; j++)
        R(j) = (o->cp_sd[3] * F(j - 2) + o->cp_sd[4] * F(j - 1) + o->cp_sd[5] * F(j) + o->cp_sd[6] * F(j + 1)
                + o->cp_sd[7] * F(j + 2)) * o->QDY2(j - 2, 1);
    R(J - 1) = (o->pp_sd[3] * F(J) + o->pp_sd[4] * F(J - 1) + o->pp_sd[5] * F(J - 2) + o->pp_sd[6] * F(J - 3)
                + o->pp_sd[7] * F(J - 4) + o->pp_sd[8] * F(J - 5) + o->pp_sd[9] * F(J - 6)) * o->QDY2(J - 6, 1);
    R(J) = (o->lp_sd[2] * F(J) + o->lp_sd[3] * F(J - 1) + o->lp_sd[4] * F(J - 2) + o->lp_sd[5] * F(J - 3)
            + o->lp_sd[6] * F(J - 4) + o->lp_sd[7] * F(J - 5)) * o->QDY2(J - 5, 1);
}
void dery_impl(ora_ctx* o, C* ddy, const C* fc, int kind) {  // 0 dery, 1 deryfv, 2 deryy
    int J = o->ny;
    size_t s = o->nx;
    const double *a, *b, *c;
    if (kind == 0) { a = o->a1y.data(); b = o->b1y.data(); c = o->c1y.data(); }
    else if (kind == 1) { a = o->a1fv.data(); b = o->b1fv.data(); c = o->c1fv.data(); }
    else { a = o->a2y.data(); b = o->b2y.data(); c = o->c2y.data(); }
#pragma omp parallel for schedule(static)
    for (int q = 0; q < o->K * o->nx; q++) {
            std::vector<double> gam(J); std::vector<C> u(J);
            int k = 1 + q / o->nx, i = 1 + q % o->nx;
            size_t base = o->id(i, 1, k);
            if (kind == 2) rhsyy_line(o, fc + base, ddy + base, s);
            else rhsy_line(o, fc + base, ddy + base, s, kind == 1);
            thomas(a, b, c, ddy + base, J, s, gam, u);
        }
}

// ---------------------------------------------------------------------------
// Spanwise transforms (nlterms_par.f:303-484).
void four1(double* d /*1-based*/, int n, int isig) {  // nlterms_par.f:431-484
    int z = 1;
    for (int i = 1; i <= n; i += 2) {
        if (z > i) {
            double tr = d[z], ti = d[z + 1];
            d[z] = d[i]; d[z + 1] = d[i + 1];
            d[i] = tr; d[i + 1] = ti;
        }
        int mm = n / 2;
        while (mm >= 2 && z > mm) { z -= mm; mm /= 2; }
        z += mm;
    }
    int mmax = 2;
    while (n > mmax) {
        int istep = 2 * mmax;
        double theta = TWOPI_NR / (double)(isig * mmax);
        double s = std::sin(0.5 * theta);
        double wpr = -(2.0 * (s * s));
        double wpi = std::sin(theta);
        double wr = 1.0, wi = 0.0;
        for (int mm = 1; mm <= mmax; mm += 2) {
            for (int i = mm; i <= n; i += istep) {
                int zz = i + mmax;
                double tr = wr * d[zz] - wi * d[zz + 1];
                double ti = wr * d[zz + 1] + wi * d[zz];
                d[zz] = d[i] - tr; d[zz + 1] = d[i + 1] - ti;
                d[i] = d[i] + tr; d[i + 1] = d[i + 1] + ti;
            }
            double wt = wr;
            wr = wr * wpr - wi * wpi + wr;
            wi = wi * wpr + wt * wpi + wi;
        }
        mmax = istep;
    }
}
// Fourier -> physical for one (i,j) line (nlterms_par.f:323-356).
void f_to_p_line(int K, int P, const C* cf, size_t cs, double* dp /*1-based, P*/) {
    double theta = -TWOPI_NR / (double)P, c1 = 0.5;
    double s = std::sin(0.5 * theta);
    double wpr = -(2.0 * (s * s)), wpi = std::sin(theta);
    for (int k = 0; k < K; k++) { dp[2 * k + 1] = cf[k * cs].re; dp[2 * k + 2] = cf[k * cs].im; }
    for (int k = 2 * K + 1; k <= P; k++) dp[k] = 0.0;
    dp[1] = dp[1] * 2.0;
    double wr = 1.0 + wpr, wi = wpi;
    int n2p3 = P + 3;
    for (int p = 2; p <= P / 4; p++) {
        int p1 = 2 * p - 1, p2 = p1 + 1, p3 = n2p3 - p2, p4 = p3 + 1;
        double wrs = wr, wis = wi;
        double h1r = c1 * (dp[p1] + dp[p3]);
        double h1i = c1 * (dp[p2] - dp[p4]);
        double h2r = -c1 * (dp[p2] + dp[p4]);
        double h2i = c1 * (dp[p1] - dp[p3]);
        dp[p1] = h1r + wrs * h2r - wis * h2i;
        dp[p2] = h1i + wrs * h2i + wis * h2r;
        dp[p3] = h1r - wrs * h2r + wis * h2i;
        dp[p4] = -h1i + wrs * h2i + wis * h2r;
        double wt = wr;
        wr = wr * wpr - wi * wpi + wr;
        wi = wi * wpr + wt * wpi + wi;
    }
    double h1r = dp[1];
    dp[1] = c1 * (h1r + dp[2]);
    dp[2] = c1 * (h1r - dp[2]);
    four1(dp, P, -1);
}
// Physical -> Fourier for one (i,j) line (nlterms_par.f:384-423).
void p_to_f_line(int K, int P, double* dp /*1-based*/, C* cf, size_t cs) {
    double theta = TWOPI_NR / (double)P, c1 = 0.5;
    double s = std::sin(0.5 * theta);
    double wpr = -(2.0 * (s * s)), wpi = std::sin(theta);
    four1(dp, P, +1);
    double wr = 1.0 + wpr, wi = wpi;
    int n2p3 = P + 3;
    for (int p = 2; p <= P / 4; p++) {
        int p1 = 2 * p - 1, p2 = p1 + 1, p3 = n2p3 - p2, p4 = p3 + 1;
        double wrs = wr, wis = wi;
        double h1r = c1 * (dp[p1] + dp[p3]);
        double h1i = c1 * (dp[p2] - dp[p4]);
        double h2r = c1 * (dp[p2] + dp[p4]);
        double h2i = -c1 * (dp[p1] - dp[p3]);
        dp[p1] = h1r + wrs * h2r - wis * h2i;
        dp[p2] = h1i + wrs * h2i + wis * h2r;
        dp[p3] = h1r - wrs * h2r + wis * h2i;
        dp[p4] = -h1i + wrs * h2i + wis * h2r;
        double wt = wr;
        wr = wr * wpr - wi * wpi + wr;
        wi = wi * wpr + wt * wpi + wi;
    }
    double h1r = dp[1];
    dp[1] = (h1r + dp[2]) / (double)P;
    dp[2] = h1r - dp[2];
    for (int k = 2; k <= P; k++) dp[k] = 2.0 * dp[k] / (double)P;
    for (int k = 0; k < K; k++) {
        if (std::fabs(dp[2 * k + 1]) < 1e-14) dp[2 * k + 1] = 0.0;
        if (std::fabs(dp[2 * k + 2]) < 1e-14) dp[2 * k + 2] = 0.0;
        cf[k * cs] = mk(dp[2 * k + 1], dp[2 * k + 2]);
    }
    cf[0] = mk(cf[0].re, 0.0);
}
void f_to_p_impl(ora_ctx* o, double* phys, const C* four) {  // nlterms_par.f:303
    size_t n2 = (size_t)o->nx * o->ny;
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= o->ny; j++)
        for (int i = 1; i <= o->nx; i++) {
            std::vector<double> d(o->P + 2);
            size_t p = o->id2(i, j);
            f_to_p_line(o->K, o->P, four + p, n2, d.data());
            for (int z = 1; z <= o->P; z++) phys[p + n2 * (z - 1)] = d[z];
        }
}
void p_to_f_impl(ora_ctx* o, C* four, double* phys) {  // nlterms_par.f:364
    size_t n2 = (size_t)o->nx * o->ny;
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= o->ny; j++)
        for (int i = 1; i <= o->nx; i++) {
            std::vector<double> d(o->P + 2);
            size_t p = o->id2(i, j);
            for (int z = 1; z <= o->P; z++) d[z] = phys[p + n2 * (z - 1)];
            p_to_f_line(o->K, o->P, d.data(), four + p, n2);
            for (int z = 2 * o->K + 1; z <= o->P; z++) phys[p + n2 * (z - 1)] = 0.0;
        }
}

// nlterms_fi (nlterms_par.f:41-86)
void nlterms_impl(ora_ctx* o, C* a, C* b, C* c) {
    size_t n2 = (size_t)o->nx * o->ny, NP = n2 * o->P;
    std::vector<double> uxp(NP), uyp(NP), uzp(NP), wxp(NP), wyp(NP), wzp(NP), ap(NP), bp(NP), cp(NP);
    f_to_p_impl(o, uxp.data(), o->ux.data());
    f_to_p_impl(o, uyp.data(), o->uy.data());
    f_to_p_impl(o, uzp.data(), o->uz.data());
    f_to_p_impl(o, wxp.data(), o->wx.data());
    f_to_p_impl(o, wyp.data(), o->wy.data());
    f_to_p_impl(o, wzp.data(), o->wz.data());
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < NP; q++) {
        ap[q] = uyp[q] * wxp[q] - uxp[q] * wyp[q];
        bp[q] = uxp[q] * wzp[q] - uzp[q] * wxp[q];
        cp[q] = uzp[q] * wyp[q] - uyp[q] * wzp[q];
    }
    p_to_f_impl(o, a, ap.data());
    p_to_f_impl(o, b, bp.data());
    p_to_f_impl(o, c, cp.data());
}

// ---------------------------------------------------------------------------
// Pentadiagonal LU without pivoting (penta_par.f:6-50) and solves (53-208).
void lhs5(const ora_ctx* o, std::vector<double>& a, double k2b2) {  // loop_par.f:258-299
    int n = o->nx;
    auto A = [&](int i, int c) -> double& { return a[(size_t)(i - 1) + (size_t)n * (c - 1)]; };
    A(1, 1) = 0; A(1, 2) = 0; A(1, 3) = 1; A(1, 4) = 0; A(1, 5) = 0;
    A(2, 1) = 0; A(2, 2) = 1.0 + k2b2 / 12.0; A(2, 3) = -2.0 + k2b2 / 1.2; A(2, 4) = 1.0 + k2b2 / 12.0; A(2, 5) = 0;
    for (int i = 3; i <= n - 2; i++) {
        A(i, 1) = 3.0; A(i, 2) = 48.0 + 8.0 * k2b2; A(i, 3) = -102.0 + 44.0 * k2b2; A(i, 4) = 48.0 + 8.0 * k2b2;
        A(i, 5) = 3.0;
    }
    A(n - 1, 1) = 0; A(n - 1, 2) = 1.0 + k2b2 / 12.0; A(n - 1, 3) = -2.0 + k2b2 / 1.2; A(n - 1, 4) = 1.0 + k2b2 / 12.0;
    A(n - 1, 5) = 0;
    A(n, 1) = 0; A(n, 2) = 0; A(n, 3) = 1; A(n, 4) = 0; A(n, 5) = 0;
}
void ludecomp(int n, const std::vector<double>& a, std::vector<double>& lu) {  // penta_par.f:6-50
    auto A = [&](int i, int c) -> double { return a[(size_t)(i - 1) + (size_t)n * (c - 1)]; };
    auto L = [&](int i, int c) -> double& { return lu[(size_t)(i - 1) + (size_t)n * (c - 1)]; };
    for (int i = 1; i <= n - 2; i++) {
        int jj = i - 1; if (jj > 2) jj = 2;
        for (int j = 3; j <= 5; j++) {
            int kk = 2; double soma = 0.0;
            for (int k = 1; k <= jj; k++) { soma = soma + L(i, kk) * L(i - k, j + k); kk = kk - 1; }
            jj = jj - 1;
            L(i, j) = A(i, j) - soma;
        }
        int j = 2, ii = i - 1; if (ii > 1) ii = 1;
        for (int it = i + 1; it <= i + 2; it++) {
            double soma = 0.0;
            for (int k = 1; k <= ii; k++) soma = L(it, k) * L(i - 1, j + 2);
            L(it, j) = (A(it, j) - soma) / L(i, 3);
            ii = ii - 1; j = j - 1;
        }
    }
    int i = n - 1;
    L(i, 3) = A(i, 3) - L(i, 2) * L(i - 1, 4) - L(i, 1) * L(i - 2, 5);
    L(i, 4) = A(i, 4) - L(i, 2) * L(i - 1, 5);
    L(i + 1, 2) = (A(i + 1, 2) - L(i + 1, 1) * L(i - 1, 4)) / L(i, 3);
    i = n;
    L(i, 3) = A(i, 3) - L(i, 2) * L(i - 1, 4) - L(i, 1) * L(i - 2, 5);
}
// lusolver_1 (penta_par.f:53-127): Ly order "- l2 y(i-1) - l1 y(i-2)".
void lusolver_1(int n, const std::vector<double>& lu, C* rhs, std::vector<C>& y) {
    auto L = [&](int i, int c) -> double { return lu[(size_t)(i - 1) + (size_t)n * (c - 1)]; };
    y[1] = rhs[0];
    y[2] = rhs[1] - L(2, 2) * y[1];
    for (int i = 3; i <= n; i++) y[i] = rhs[i - 1] - L(i, 2) * y[i - 1] - L(i, 1) * y[i - 2];
    rhs[n - 1] = y[n] / L(n, 3);
    rhs[n - 2] = (y[n - 1] - L(n - 1, 4) * rhs[n - 1]) / L(n - 1, 3);
    for (int i = n - 2; i >= 1; i--)
        rhs[i - 1] = (y[i] - L(i, 4) * rhs[i] - L(i, 5) * rhs[i + 1]) / L(i, 3);
}
// lusolver (penta_par.f:130-208): Ly order "- l1 y(i-2) - l2 y(i-1)", lines j = 2..jmax.
void lusolver(int n, const std::vector<double>& lu, C* rhs /*line start*/, size_t s, std::vector<C>& y) {
    auto L = [&](int i, int c) -> double { return lu[(size_t)(i - 1) + (size_t)n * (c - 1)]; };
    auto R = [&](int i) -> C& { return rhs[(size_t)(i - 1) * s]; };
    y[1] = R(1);
    y[2] = R(2) - L(2, 2) * y[1];
    for (int i = 3; i <= n; i++) y[i] = R(i) - L(i, 1) * y[i - 2] - L(i, 2) * y[i - 1];
    R(n) = y[n] / L(n, 3);
    R(n - 1) = (y[n - 1] - L(n - 1, 4) * R(n)) / L(n - 1, 3);
    for (int i = n - 2; i >= 1; i--) R(i) = (y[i] - L(i, 4) * R(i + 1) - L(i, 5) * R(i + 2)) / L(i, 3);
}
// band5_poi / banbk5_poi: NR banded LU with m1 = m2 = 2, pivoting disabled
// (penta_par.f:308-404).  a and al are (jmax, 5) column-major, n = rows used.
void band5_poi(int J, std::vector<double>& a, int n, std::vector<double>& al) {
    auto A = [&](int i, int c) -> double& { return a[(size_t)(i - 1) + (size_t)J * (c - 1)]; };
    auto AL = [&](int i, int c) -> double& { return al[(size_t)(i - 1) + (size_t)J * (c - 1)]; };
    const double TINY = (double)1.e-20f;  // REAL literal in the reference
    int m1 = 2, mm = 5, l = m1;
    for (int i = 1; i <= m1; i++) {
        for (int j = m1 + 2 - i; j <= mm; j++) A(i, j - l) = A(i, j);
        l = l - 1;
        for (int j = mm - l; j <= mm; j++) A(i, j) = 0.0;
    }
    l = m1;
    for (int k = 1; k <= n; k++) {
        double dum = A(k, 1);
        if (l < n) l = l + 1;
        if (dum == 0.0) A(k, 1) = TINY;
        for (int i = k + 1; i <= l; i++) {
            dum = A(i, 1) / A(k, 1);
            AL(k, i - k) = dum;
            for (int j = 2; j <= mm; j++) A(i, j - 1) = A(i, j) - dum * A(k, j);
            A(i, mm) = 0.0;
        }
    }
}
void banbk5_poi(int J, const std::vector<double>& a, int n, const std::vector<double>& al, C* rhs /*1..n at [j-1]*/) {
    auto A = [&](int i, int c) -> double { return a[(size_t)(i - 1) + (size_t)J * (c - 1)]; };
    auto AL = [&](int i, int c) -> double { return al[(size_t)(i - 1) + (size_t)J * (c - 1)]; };
    int l = 2;
    for (int k = 1; k <= n; k++) {
        if (l < n) l = l + 1;
        for (int i = k + 1; i <= l; i++) rhs[i - 1] = rhs[i - 1] - AL(k, i - k) * rhs[k - 1];
    }
    l = 1;
    for (int i = n; i >= 1; i--) {
        C dum = rhs[i - 1];
        for (int k = 2; k <= l; k++) dum = dum - A(i, k) * rhs[k + i - 2];
        rhs[i - 1] = dum / A(i, 1);
        if (l < 5) l = l + 1;
    }
}

// ---------------------------------------------------------------------------
// Multigrid v-Poisson (poisson_par.f).
struct Poi {
    ora_ctx* o;
    int X, Y, M;            // ptsx, jmax, msh of the work arrays
    std::vector<C> fc, sc, fct;
    std::vector<double> ac, alc, acb, alcb;
    std::vector<C> rhs;
    C& FC(int i, int j, int m) { return fc[(size_t)(i - 1) + (size_t)X * ((size_t)(j - 1) + (size_t)Y * (m - 1))]; }
    C& SC(int i, int j, int m) { return sc[(size_t)(i - 1) + (size_t)X * ((size_t)(j - 1) + (size_t)Y * (m - 1))]; }
    C& FT(int i, int j, int m) { return fct[(size_t)(i - 1) + (size_t)X * ((size_t)(j - 1) + (size_t)Y * (m - 1))]; }
    explicit Poi(ora_ctx* oo) : o(oo), X(oo->nx), Y(oo->ny), M(oo->msh) {
        size_t n = (size_t)X * Y * M;
        fc.assign(n, mk(0, 0)); sc.assign(n, mk(0, 0)); fct.assign(n, mk(0, 0));
        ac.assign((size_t)Y * 5, 0.0); alc.assign((size_t)Y * 5, 0.0);
        acb.assign((size_t)Y * 5, 0.0); alcb.assign((size_t)Y * 5, 0.0);
        rhs.assign(Y, mk(0, 0));
    }
    // coef_center / coef_border (poisson_par.f:229-340); qn = -30 or -15.
    void coef(std::vector<double>& a, double k2b2, int mesh, double qn) {
        auto A = [&](int j, int c) -> double& { return a[(size_t)(j - 1) + (size_t)Y * (c - 1)]; };
        double qx = qn / (12.0 * o->v_dx2[mesh - 1]);
        double add = (qx + k2b2) / o->fac_y;
        int n = o->v_ptsy[mesh - 1];
        A(1, 1) = 0; A(1, 2) = 0; A(1, 3) = 1; A(1, 4) = 0; A(1, 5) = 0;
        A(2, 1) = 0;
        A(2, 2) = o->SP(4, mesh) * o->QDY2(1, mesh);
        A(2, 3) = o->SP(5, mesh) * o->QDY2(1, mesh) + o->SP(2, mesh) * add;
        A(2, 4) = o->SP(6, mesh) * o->QDY2(1, mesh) + o->SP(3, mesh) * add;
        A(2, 5) = o->SP(7, mesh) * o->QDY2(1, mesh);
        for (int j = 3; j <= n - 2; j++) {
            double q = o->QDY2(j - 2, mesh);
            A(j, 1) = o->CP(4, mesh) * q;
            A(j, 2) = o->CP(5, mesh) * q + o->CP(1, mesh) * add;
            A(j, 3) = o->CP(6, mesh) * q + o->CP(2, mesh) * add;
            A(j, 4) = o->CP(7, mesh) * q + o->CP(3, mesh) * add;
            A(j, 5) = o->CP(8, mesh) * q;
        }
        int j = n;
        double q = o->QDY2(j - 2, mesh);
        A(j - 1, 1) = 0;
        A(j - 1, 2) = o->PP(2, mesh) * q;
        A(j - 1, 3) = o->PP(3, mesh) * q + add;
        A(j - 1, 4) = o->PP(4, mesh) * q;
        A(j - 1, 5) = 0;
        A(j, 1) = o->LP(5, mesh) * q;
        A(j, 2) = o->LP(4, mesh) * q;
        A(j, 3) = o->LP(3, mesh) * q + add - o->LP(2, mesh) * std::sqrt(q) * std::sqrt((o->alpha * o->alpha - k2b2) / o->fac_y);
        A(j, 4) = 0; A(j, 5) = 0;
    }
    // rhs_border1 (poisson_par.f:343-409)
    void rhs_border1(int i, int mesh) {
        int n = o->v_ptsy[mesh - 1];
        double qx = 1.0 / (12.0 * o->v_dx2[mesh - 1] * o->fac_y);
        auto g = [&](int jj) -> C {
            return 10.0 * FC(i - 1, jj, mesh) - 4.0 * FC(i + 1, jj, mesh) + 14.0 * FC(i + 2, jj, mesh)
                   - 6.0 * FC(i + 3, jj, mesh) + FC(i + 4, jj, mesh);
        };
        rhs[0] = FC(i, 1, mesh);
        int j = 2;
        rhs[j - 1] = SC(i, j, mesh) - qx * (o->SP(3, mesh) * g(j + 1) + o->SP(2, mesh) * g(j));
        for (j = 3; j <= n - 2; j++)
            rhs[j - 1] = SC(i, j, mesh) - qx * (o->CP(1, mesh) * g(j - 1) + o->CP(2, mesh) * g(j) + o->CP(3, mesh) * g(j + 1));
        j = n - 1; rhs[j - 1] = SC(i, j, mesh) - qx * g(j);
        j = n;     rhs[j - 1] = SC(i, j, mesh) - qx * g(j);
    }
    // rhs_border2 (poisson_par.f:412-478)
    void rhs_border2(int i, int mesh) {
        int n = o->v_ptsy[mesh - 1];
        double qx = 1.0 / (12.0 * o->v_dx2[mesh - 1] * o->fac_y);
        auto g = [&](int jj) -> C {
            return 10.0 * FC(i + 1, jj, mesh) - 4.0 * FC(i - 1, jj, mesh) + 14.0 * FC(i - 2, jj, mesh)
                   - 6.0 * FC(i - 3, jj, mesh) + FC(i - 4, jj, mesh);
        };
        rhs[0] = FC(i, 1, mesh);
        int j = 2;
        rhs[j - 1] = SC(i, j, mesh) - qx * (o->SP(3, mesh) * g(j + 1) + o->SP(2, mesh) * g(j));
        for (j = 3; j <= n - 2; j++)
            rhs[j - 1] = SC(i, j, mesh) - qx * (o->CP(1, mesh) * g(j - 1) + o->CP(2, mesh) * g(j) + o->CP(3, mesh) * g(j + 1));
        j = n - 1; rhs[j - 1] = SC(i, j, mesh) - qx * g(j);
        j = n;     rhs[j - 1] = SC(i, j, mesh) - qx * g(j);
    }
    // rhs_center (poisson_par.f:481-540)
    void rhs_center(int i, int mesh) {
        int n = o->v_ptsy[mesh - 1];
        double qx = 1.0 / (12.0 * o->v_dx2[mesh - 1] * o->fac_y);
        auto g = [&](int jj) -> C {
            return -(1.0 * FC(i - 2, jj, mesh)) + 16.0 * FC(i - 1, jj, mesh) + 16.0 * FC(i + 1, jj, mesh)
                   - 1.0 * FC(i + 2, jj, mesh);
        };
        auto g2 = [&](int jj) -> C {
            return -(FC(i + 2, jj, mesh) + FC(i - 2, jj, mesh)) + 16.0 * (FC(i + 1, jj, mesh) + FC(i - 1, jj, mesh));
        };
        rhs[0] = FC(i, 1, mesh);
        int j = 2;
        rhs[j - 1] = SC(i, j, mesh) - qx * (o->SP(3, mesh) * g(j + 1) + o->SP(2, mesh) * g(j));
        for (j = 3; j <= n - 2; j++)
            rhs[j - 1] = SC(i, j, mesh) - qx * (o->CP(1, mesh) * g(j - 1) + o->CP(2, mesh) * g(j) + o->CP(3, mesh) * g(j + 1));
        j = n - 1; rhs[j - 1] = SC(i, j, mesh) - qx * g2(j);
        j = n;     rhs[j - 1] = SC(i, j, mesh) - qx * g2(j);
    }
    // sor (poisson_par.f:167-226)
    void sor(int k, int itera, int mesh) {
        double rf = 1.2;
        if (itera == 1) rf = 1.0;
        int n = o->v_ptsy[mesh - 1], nxm = o->v_ptsx[mesh - 1];
        coef(ac, o->v_k2b2[k - 1], mesh, -30.0); band5_poi(Y, ac, n, alc);
        coef(acb, o->v_k2b2[k - 1], mesh, -15.0); band5_poi(Y, acb, n, alcb);
        for (int it = 1; it <= itera; it++) {
            int i = 2;
            rhs_border1(i, mesh); banbk5_poi(Y, acb, n, alcb, rhs.data());
            for (int j = 2; j <= n; j++) FC(i, j, mesh) = FC(i, j, mesh) + rf * (rhs[j - 1] - FC(i, j, mesh));
            i = nxm - 1;
            rhs_border2(i, mesh); banbk5_poi(Y, acb, n, alcb, rhs.data());
            for (int j = 2; j <= n; j++) FC(i, j, mesh) = FC(i, j, mesh) + rf * (rhs[j - 1] - FC(i, j, mesh));
            for (i = 3; i <= nxm - 2; i++) {
                rhs_center(i, mesh); banbk5_poi(Y, ac, n, alc, rhs.data());
                for (int j = 2; j <= n; j++) FC(i, j, mesh) = FC(i, j, mesh) + rf * (rhs[j - 1] - FC(i, j, mesh));
            }
        }
    }
    // defect (poisson_par.f:543-793)
    void defect(double si, int k, int mesh) {
        int n = o->v_ptsy[mesh - 1], nxm = o->v_ptsx[mesh - 1];
        double k2b2 = o->v_k2b2[k - 1];
        double alpha2 = std::sqrt((o->alpha * o->alpha - k2b2) / o->fac_y);
        double den = 12.0 * o->v_dx2[mesh - 1] * o->fac_y;
        double fy = o->fac_y;
        // one-sided x operator at the two border columns; e = +1 left, -1 right
        auto bx = [&](int i, int jj, int e) -> C {
            return 10.0 * FC(i - e, jj, mesh) - 15.0 * FC(i, jj, mesh) - 4.0 * FC(i + e, jj, mesh)
                   + 14.0 * FC(i + 2 * e, jj, mesh) - 6.0 * FC(i + 3 * e, jj, mesh) + FC(i + 4 * e, jj, mesh);
        };
        auto border = [&](int i, int e) {
            int j = 2;
            C b = o->SP(3, mesh) * bx(i, j + 1, e) + o->SP(2, mesh) * bx(i, j, e);
            C c = o->SP(4, mesh) * FC(i, j - 1, mesh) + o->SP(5, mesh) * FC(i, j, mesh) + o->SP(6, mesh) * FC(i, j + 1, mesh)
                  + o->SP(7, mesh) * FC(i, j + 2, mesh);
            C d = k2b2 * (o->SP(2, mesh) * FC(i, j, mesh) + o->SP(3, mesh) * FC(i, j + 1, mesh));
            FT(i, j, 1) = SC(i, j, mesh) + si * (b / den + c * o->QDY2(1, mesh) + d / fy);
            for (j = 3; j <= n - 2; j++) {
                b = o->CP(1, mesh) * bx(i, j - 1, e) + o->CP(2, mesh) * bx(i, j, e) + o->CP(3, mesh) * bx(i, j + 1, e);
                c = o->CP(4, mesh) * FC(i, j - 2, mesh) + o->CP(5, mesh) * FC(i, j - 1, mesh) + o->CP(6, mesh) * FC(i, j, mesh)
                    + o->CP(7, mesh) * FC(i, j + 1, mesh) + o->CP(8, mesh) * FC(i, j + 2, mesh);
                d = k2b2 * (o->CP(1, mesh) * FC(i, j - 1, mesh) + o->CP(2, mesh) * FC(i, j, mesh) + o->CP(3, mesh) * FC(i, j + 1, mesh));
                FT(i, j, 1) = SC(i, j, mesh) + si * (b / den + c * o->QDY2(j - 2, mesh) + d / fy);
            }
            j = n - 1;
            b = bx(i, j, e);
            c = o->PP(4, mesh) * FC(i, j + 1, mesh) + o->PP(3, mesh) * FC(i, j, mesh) + o->PP(2, mesh) * FC(i, j - 1, mesh);
            d = k2b2 * FC(i, j, mesh);
            FT(i, j, 1) = SC(i, j, mesh) + si * (b / den + c * o->QDY2(j - 1, mesh) + d / fy);
            j = n;
            b = bx(i, j, e);
            c = o->LP(3, mesh) * FC(i, j, mesh) + o->LP(4, mesh) * FC(i, j - 1, mesh) + o->LP(5, mesh) * FC(i, j - 2, mesh);
            d = k2b2 * FC(i, j, mesh);
            FT(i, j, 1) = SC(i, j, mesh) + si * (b / den + c * o->QDY2(j - 2, mesh) + d / fy
                                                 - o->LP(2, mesh) * alpha2 * FC(i, j, mesh) * std::sqrt(o->QDY2(j - 2, mesh)));
        };
        border(2, +1);
        border(nxm - 1, -1);
        auto cx = [&](int i, int jj) -> C {
            return -(1.0 * FC(i - 2, jj, mesh)) + 16.0 * FC(i - 1, jj, mesh) - 30.0 * FC(i, jj, mesh)
                   + 16.0 * FC(i + 1, jj, mesh) - 1.0 * FC(i + 2, jj, mesh);
        };
        auto cx2 = [&](int i, int jj) -> C {
            return -(1.0 * (FC(i - 2, jj, mesh) + FC(i + 2, jj, mesh))) + 16.0 * (FC(i - 1, jj, mesh) + FC(i + 1, jj, mesh))
                   - 30.0 * FC(i, jj, mesh);
        };
        for (int i = 3; i <= nxm - 2; i++) {
            int j = 2;
            C b = o->SP(3, mesh) * cx(i, j + 1) + o->SP(2, mesh) * cx(i, j);
            C c = o->SP(4, mesh) * FC(i, j - 1, mesh) + o->SP(5, mesh) * FC(i, j, mesh) + o->SP(6, mesh) * FC(i, j + 1, mesh)
                  + o->SP(7, mesh) * FC(i, j + 2, mesh);
            C d = k2b2 * (o->SP(2, mesh) * FC(i, j, mesh) + o->SP(3, mesh) * FC(i, j + 1, mesh));
            FT(i, j, 1) = SC(i, j, mesh) + si * (b / den + c * o->QDY2(1, mesh) + d / fy);
            for (j = 3; j <= n - 2; j++) {
                b = o->CP(1, mesh) * cx(i, j - 1) + o->CP(2, mesh) * cx(i, j) + o->CP(3, mesh) * cx(i, j + 1);
                c = o->CP(4, mesh) * FC(i, j - 2, mesh) + o->CP(5, mesh) * FC(i, j - 1, mesh) + o->CP(6, mesh) * FC(i, j, mesh)
                    + o->CP(7, mesh) * FC(i, j + 1, mesh) + o->CP(8, mesh) * FC(i, j + 2, mesh);
                d = k2b2 * (o->CP(1, mesh) * FC(i, j - 1, mesh) + o->CP(2, mesh) * FC(i, j, mesh) + o->CP(3, mesh) * FC(i, j + 1, mesh));
                FT(i, j, 1) = SC(i, j, mesh) + si * (b / den + c * o->QDY2(j - 2, mesh) + d / fy);
            }
            j = n - 1;
            b = cx2(i, j);
            c = o->PP(4, mesh) * FC(i, j + 1, mesh) + o->PP(3, mesh) * FC(i, j, mesh) + o->PP(2, mesh) * FC(i, j - 1, mesh);
            d = k2b2 * FC(i, j, mesh);
            FT(i, j, 1) = SC(i, j, mesh) + si * (b / den + c * o->QDY2(j - 1, mesh) + d / fy);
            j = n;
            b = cx2(i, j);
            c = o->LP(3, mesh) * FC(i, j, mesh) + o->LP(4, mesh) * FC(i, j - 1, mesh) + o->LP(5, mesh) * FC(i, j - 2, mesh);
            d = k2b2 * FC(i, j, mesh);
            FT(i, j, 1) = SC(i, j, mesh) + si * (b / den + c * o->QDY2(j - 2, mesh) + d / fy
                                                 - o->LP(2, mesh) * alpha2 * FC(i, j, mesh) * std::sqrt(o->QDY2(j - 2, mesh)));
        }
        if (si < 0) return;
        for (int j = 2; j <= n; j++)
            for (int i = 2; i <= nxm - 1; i++) SC(i, j, mesh) = FT(i, j, 1);
    }
    // restrict (poisson_par.f:796-874)
    void restrict_(int mesh) {
        int nyc = o->v_ptsy[mesh], nxc = o->v_ptsx[mesh], nyf = o->v_ptsy[mesh - 1];
        int m2 = mesh + 1;
        int fj = 3;
        for (int j = 2; j <= nyc - 1; j++) {
            int fi = 3;
            for (int i = 2; i <= nxc - 1; i++) {
                FC(i, j, m2) = FC(fi, fj, mesh);
                FT(i, j, m2) = FC(i, j, m2);
                SC(i, j, m2) = 6.25e-2 * (2.0 * (FT(fi - 1, fj, 1) + FT(fi + 1, fj, 1) + FT(fi, fj - 1, 1) + FT(fi, fj + 1, 1))
                                          + 4.0 * FT(fi, fj, 1) + FT(fi + 1, fj + 1, 1) + FT(fi + 1, fj - 1, 1)
                                          + FT(fi - 1, fj + 1, 1) + FT(fi - 1, fj - 1, 1));
                fi += 2;
            }
            fj += 2;
        }
        int fi = 3;
        for (int i = 2; i <= nxc - 1; i++) {
            int j = 1;
            FC(i, j, m2) = FC(fi, j, mesh);
            FT(i, j, m2) = FC(i, j, m2);
            j = nyc;
            int fjj = 2 * j - 1;
            FC(i, j, m2) = FC(fi, fjj, mesh);
            FT(i, j, m2) = FC(i, j, m2);
            SC(i, j, m2) = 0.25 * (FT(fi - 1, fjj, 1) + 2.0 * FT(fi, fjj, 1) + FT(fi + 1, fjj, 1));
            fi += 2;
        }
        {   // first column (rank 0)
            int i = 1;
            FC(i, 1, m2) = FC(i, 1, mesh);
            FT(i, 1, m2) = FC(i, 1, m2);
            int fjj = 3;
            for (int j = 2; j <= nyc - 1; j++) {
                FC(i, j, m2) = FC(i, fjj, mesh);
                FT(i, j, m2) = FC(i, j, m2);
                fjj += 2;
            }
            FC(i, nyc, m2) = FC(i, nyf, mesh);
            FT(i, nyc, m2) = FC(i, nyc, m2);
        }
        {   // last column (last rank)
            int i = nxc, fi2 = 2 * i - 1;
            FC(i, 1, m2) = FC(fi2, 1, mesh);
            FT(i, 1, m2) = FC(i, 1, m2);
            int fjj = 3;
            for (int j = 2; j <= nyc - 1; j++) {
                FC(i, j, m2) = FC(fi2, fjj, mesh);
                FT(i, j, m2) = FC(i, j, m2);
                fjj += 2;
            }
            FC(i, nyc, m2) = FC(fi2, nyf, mesh);
            FT(i, nyc, m2) = FC(i, nyc, m2);
        }
    }
    // intpol (poisson_par.f:877-920): mesh = coarse level
    void intpol(int mesh) {
        int nxc = o->v_ptsx[mesh - 1], nyc = o->v_ptsy[mesh - 1];
        int nxf = o->v_ptsx[mesh - 2], nyf = o->v_ptsy[mesh - 2];
        std::vector<C> temp((size_t)X * Y, mk(0, 0));
        auto T = [&](int i, int j) -> C& { return temp[(size_t)(i - 1) + (size_t)X * (j - 1)]; };
        int fj = 1;
        for (int j = 1; j <= nyc; j++) {
            int fi = 1;
            for (int i = 1; i <= nxc; i++) { T(fi, fj) = FC(i, j, mesh); fi += 2; }
            fj += 2;
        }
        for (int j = 1; j <= nyf; j += 2)
            for (int i = 2; i <= nxf - 1; i += 2) T(i, j) = 0.5 * (T(i - 1, j) + T(i + 1, j));
        for (int j = 2; j <= nyf - 1; j += 2)
            for (int i = 1; i <= nxf; i++) T(i, j) = 0.5 * (T(i, j + 1) + T(i, j - 1));
        for (int j = 1; j <= nyf; j++)
            for (int i = 2; i <= nxf - 1; i++) FC(i, j, mesh - 1) = FC(i, j, mesh - 1) + T(i, j);
    }
    // correction (poisson_par.f:923-942)
    void correction(int mesh) {
        int n = o->v_ptsy[mesh - 1], nxm = o->v_ptsx[mesh - 1];
        for (int j = 1; j <= n; j++)
            for (int i = 2; i <= nxm - 1; i++) FC(i, j, mesh) = FC(i, j, mesh) - FT(i, j, mesh);
    }
    // get_max_value (poisson_par.f:945-963)
    double max_defect() {
        double e = 0.0;
        for (int j = 2; j <= o->ny; j++)
            for (int i = 2; i <= o->nx - 1; i++) e = std::max(e, cabs_(FT(i, j, 1)));
        return e;
    }
    // function_source (poisson_par.f:111-164)
    void function_source(const C* dwzdx, int k) {
        int J = o->ny;
        C vkb = o->v_kb[k - 1];
        auto S = [&](int i, int j) -> C { return vkb * o->wx[o->id(i, j, k)] - dwzdx[o->id(i, j, k)]; };
        for (int i = 1; i <= o->nx; i++) {
            SC(i, 1, 1) = mk(0, 0);
            SC(i, 2, 1) = o->SP(2, 1) * S(i, 2) + o->SP(3, 1) * S(i, 3);
            for (int j = 3; j <= J - 2; j++) SC(i, j, 1) = o->CP(1, 1) * S(i, j - 1) + o->CP(2, 1) * S(i, j) + o->CP(3, 1) * S(i, j + 1);
            SC(i, J - 1, 1) = S(i, J - 1);
            SC(i, J, 1) = mk(0, 0);
            if (o->cfg.my_form == 0 || o->cfg.my_form == 4) {
                if (k == 1) {
                    double dya = o->dy * powi(o->stf, J - 3);
                    SC(i, J, 1) = -(o->LP(1, 1) * dwzdx[o->id(i, J, k)]) + mk(o->LP(2, 1) * o->duexmdx[i - 1] / dya, 0.0)
                                  - mk(o->LP(2, 1) * o->alpha * o->uyb[o->id2(i, J)] / dya / std::sqrt(o->fac_y), 0.0);
                }
            }
        }
        for (int j = 1; j <= J; j++)
            for (int i = 1; i <= o->nx; i++) FC(i, j, 1) = o->uy[o->id(i, j, k)];
    }
};

void poi_uy_impl(ora_ctx* o, const C* dwzdx, double erromax) {  // poisson_par.f:6-64
    int msh = o->msh;
    o->pv.assign(o->K, 0); o->pres.assign(o->K, 0.0);
    // modes are independent problems (one work set per thread)
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 1; k <= o->K; k++) {
        Poi p(o);
        p.function_source(dwzdx, k);
        double sum_err = 0.0;
        int vcycles, done = 0;
        for (vcycles = 1; vcycles <= o->cfg.max_vcycles; vcycles++) {
            for (int mesh = 1; mesh <= msh - 1; mesh++) {
                p.sor(k, 3, mesh);
                p.defect(-1.0, k, mesh);
                if (mesh == 1) {
                    sum_err = p.max_defect();
                    if (sum_err < erromax) { done = 1; break; }
                }
                p.restrict_(mesh);
                p.defect(1.0, k, mesh + 1);
            }
            if (done) break;
            p.sor(k, 20 * 3, msh);
            for (int mesh = msh; mesh >= 2; mesh--) {
                p.correction(mesh);
                p.intpol(mesh);
                p.sor(k, 1, mesh - 1);
            }
        }
        for (int j = 2; j <= o->ny; j++)
            for (int i = 2; i <= o->nx - 1; i++) o->uy[o->id(i, j, k)] = p.FC(i, j, 1);
        o->pv[k - 1] = vcycles - 1;
        o->pres[k - 1] = sum_err;
    }
}

// ---------------------------------------------------------------------------
// loop_par.f
void bzone_impl(ora_ctx* o) {  // loop_par.f:6-45
    for (int k = 1; k <= o->K; k++)
        for (int j = 2; j <= o->ny; j++)
            for (int i = 1; i <= o->nx; i++) {
                size_t q = o->id(i, j, k);
                double bd = (k == 3) ? o->bdfc2[i - 1] : o->bdfc[i - 1];   // bdt = 2 for k = 3
                if (o->cfg.my_form == 2) o->th[q] = o->th[q] * bd;         // loop_par.f:36-39
                o->wx[q] = o->wx[q] * bd;
                o->wy[q] = o->wy[q] * bd;
                if ((o->cfg.my_form == 0 || o->cfg.my_form == 4) && k == 1) {
                    C wzb = mk(o->wzb[o->id2(i, j)], 0.0);
                    o->wz[q] = (o->wz[q] - wzb) * bd + wzb;
                } else {
                    o->wz[q] = o->wz[q] * bd;
                }
            }
}
void bzonew_impl(ora_ctx* o) {  // loop_par.f:691-725
    for (int k = 1; k <= o->K; k++)
        for (int i = 1; i <= o->nx; i++) {
            size_t q = o->id(i, 1, k);
            double bd = (k == 3) ? o->bdfc2[i - 1] : o->bdfc[i - 1];
            o->wx[q] = o->wx[q] * bd;
            o->wy[q] = o->wy[q] * bd;
            if ((o->cfg.my_form == 0 || o->cfg.my_form == 4) && k == 1) {
                C wzb = mk(o->wzb[o->id2(i, 1)], 0.0);
                o->wz[q] = (o->wz[q] - wzb) * bd + wzb;
            } else {
                o->wz[q] = o->wz[q] * bd;
            }
        }
}
void outuy_impl(ora_ctx* o, C* dwzdx) {  // loop_par.f:48-119
    derparx_impl(o, dwzdx, o->wz.data());
    for (int k = 1; k <= o->K; k++)
        for (int j = 2; j <= o->ny; j++) {
            size_t q = o->id(o->nx, j, k);
            if ((o->cfg.my_form == 0 || o->cfg.my_form == 4) && k == 1) o->uy[q] = mk(o->uyb[o->id2(o->nx, j)], 0.0);
            else o->uy[q] = mk(0.0, 0.0);
        }
}
void poi_ux_impl(ora_ctx* o, C* duydy) {  // loop_par.f:428-566
    int n = o->nx;
    dery_impl(o, duydy, o->uy.data(), 1);
    int k = 1;
    double dx = o->dx;
    for (int j = 2; j <= o->ny - 1; j++) {
        auto D = [&](int i) -> C { return duydy[o->id(i, j, k)]; };
        auto U = [&](int i) -> C& { return o->ux[o->id(i, j, k)]; };
        U(2) = (-(dx * (251.0 * D(1) + 646.0 * D(2) - 264.0 * D(3) + 106.0 * D(4) - 19.0 * D(5))) + 720.0 * U(1)) / 720.0;
        for (int i = 3; i <= n - 2; i++)
            U(i) = (-(dx * (281.0 * D(i - 2) + 2056.0 * D(i - 1) + 1176.0 * D(i) - 104.0 * D(i + 1) + 11.0 * D(i + 2)) / 90.0)
                    + 11.0 * U(i - 2) + 16.0 * U(i - 1)) / 27.0;
        int i = n - 1;
        U(i) = (-(dx * (10.0 * D(i - 2) + 57.0 * D(i - 1) + 24.0 * D(i) - D(i + 1))) + 33.0 * U(i - 2) + 24.0 * U(i - 1)) / 57.0;
        i = n;
        U(i) = (-(dx * (251.0 * D(i) + 646.0 * D(i - 1) - 264.0 * D(i - 2) + 106.0 * D(i - 3) - 19.0 * D(i - 4)))
                + 720.0 * U(i - 1)) / 720.0;
    }
    std::vector<C> d2uydxdy(o->N3());
    derparx_impl(o, d2uydxdy.data(), duydy);
    std::vector<double> a((size_t)n * 5), lu((size_t)n * 5, 0.0);
    std::vector<C> rhs((size_t)n * o->ny), y(n + 1);
    double dxx = o->dxx, beta = o->beta;
    for (k = 2; k <= o->K; k++) {
        double k2b2 = dxx * o->v_k2b2[k - 1];
        lhs5(o, a, k2b2);
        ludecomp(n, a, lu);
        C vkb = o->v_kb[k - 1];
        for (int j = 2; j <= o->ny; j++) {
            auto D = [&](int i) -> C { return d2uydxdy[o->id(i, j, k)]; };
            auto W = [&](int i) -> C { return o->wy[o->id(i, j, k)]; };
            auto R = [&](int i) -> C& { return rhs[(size_t)(i - 1) + (size_t)n * (j - 1)]; };
            R(1) = o->ux[o->id(1, j, k)];
            R(2) = -(dxx * (D(1) + 10.0 * D(2) + D(3) + vkb * (W(1) + 10.0 * W(2) + W(3)))) / 12.0;
            for (int i = 3; i <= n - 2; i++)
                R(i) = -(8.0 * dxx * (D(i - 1) + 5.5 * D(i) + D(i + 1) + vkb * (W(i - 1) + 5.5 * W(i) + W(i + 1))));
            R(n - 1) = -(dxx * (D(n) + 10.0 * D(n - 1) + D(n - 2) + vkb * (W(n) + 10.0 * W(n - 1) + W(n - 2)))) / 12.0;
            R(n) = (vkb * W(n) + D(n)) / ((double)(k - 1) * (double)(k - 1) * beta * beta);
        }
        for (int j = 2; j <= o->ny; j++) lusolver(n, lu, &rhs[(size_t)n * (j - 1)], 1, y);
        for (int j = 2; j <= o->ny; j++)
            for (int i = 2; i <= n; i++) o->ux[o->id(i, j, k)] = rhs[(size_t)(i - 1) + (size_t)n * (j - 1)];
    }
}
void poi_uz_impl(ora_ctx* o, const C* duydy) {  // loop_par.f:569-688
    int n = o->nx;
    std::vector<C> dwydx(o->N3());
    derparx_impl(o, dwydx.data(), o->wy.data());
    std::vector<double> a((size_t)n * 5), lu((size_t)n * 5, 0.0);
    std::vector<C> rhs((size_t)n * o->ny), y(n + 1);
    double dxx = o->dxx, beta = o->beta;
    for (int k = 2; k <= o->K; k++) {
        double k2b2 = dxx * o->v_k2b2[k - 1];
        lhs5(o, a, k2b2);
        ludecomp(n, a, lu);
        C vkb = o->v_kb[k - 1];
        for (int j = 2; j <= o->ny; j++) {
            auto D = [&](int i) -> C { return dwydx[o->id(i, j, k)]; };
            auto V = [&](int i) -> C { return duydy[o->id(i, j, k)]; };
            auto R = [&](int i) -> C& { return rhs[(size_t)(i - 1) + (size_t)n * (j - 1)]; };
            R(1) = o->uz[o->id(1, j, k)];
            R(2) = dxx * (D(1) + 10.0 * D(2) + D(3) - vkb * (V(1) + 10.0 * V(2) + V(3))) / 12.0;
            for (int i = 3; i <= n - 2; i++)
                R(i) = 8.0 * dxx * (D(i - 1) + 5.5 * D(i) + D(i + 1) - vkb * (V(i - 1) + 5.5 * V(i) + V(i + 1)));
            R(n - 1) = dxx * (D(n) + 10.0 * D(n - 1) + D(n - 2) - vkb * (V(n) + 10.0 * V(n - 1) + V(n - 2))) / 12.0;
            R(n) = (-D(n) + vkb * V(n)) / ((double)(k - 1) * (double)(k - 1) * beta * beta);
        }
        for (int j = 2; j <= o->ny; j++) lusolver(n, lu, &rhs[(size_t)n * (j - 1)], 1, y);
        for (int j = 2; j <= o->ny; j++)
            for (int i = 2; i <= n; i++) o->uz[o->id(i, j, k)] = rhs[(size_t)(i - 1) + (size_t)n * (j - 1)];
    }
}
void der2wydxdy(ora_ctx* o, std::vector<C>& d2, int k) {  // loop_par.f:302-358
    int n = o->nx;
    std::vector<C> dw(n + 1);
    double dy = o->dy, dx = o->dx;
    for (int i = 1; i <= n; i++) {
        auto W = [&](int j) -> C { return o->wy[o->id(i, j, k)]; };
        dw[i] = (1.0 / dy) * (o->dwydy[1] * W(1) + o->dwydy[2] * W(2) + o->dwydy[3] * W(3) + o->dwydy[4] * W(4)
                              + o->dwydy[5] * W(5) + o->dwydy[6] * W(6) + o->dwydy[7] * W(7));
    }
    d2[1] = (-(14.7 * dw[1]) + 36.0 * dw[2] - 45.0 * dw[3] + 40.0 * dw[4] - 22.5 * dw[5] + 7.2 * dw[6] - dw[7]) / 6.0 / dx;
    d2[2] = (-dw[1] - 7.7 * dw[2] + 15.0 * dw[3] - 10.0 * dw[4] + 5.0 * dw[5] - 1.5 * dw[6] + 0.2 * dw[7]) / 6.0 / dx;
    d2[3] = (0.2 * dw[1] - 2.4 * dw[2] - 3.5 * dw[3] + 8.0 * dw[4] - 3.0 * dw[5] + 0.8 * dw[6] - 0.1 * dw[7]) / 6.0 / dx;
    for (int i = 4; i <= n - 3; i++)
        d2[i] = (45.0 * (dw[i + 1] - dw[i - 1]) + 9.0 * (dw[i - 2] - dw[i + 2]) + dw[i + 3] - dw[i - 3]) / 60.0 / dx;
    d2[n - 2] = (dw[n - 4] - 8.0 * dw[n - 3] + 8.0 * dw[n - 1] - dw[n]) / 12.0 / dx;
    d2[n - 1] = (2.0 * dw[n] + 3.0 * dw[n - 1] - 6.0 * dw[n - 2] + dw[n - 3]) / 6.0 / dx;
    d2[n] = (3.0 * dw[n] - 4.0 * dw[n - 1] + dw[n - 2]) / 2.0 / dx;
}
void wx_wall_impl(ora_ctx* o, C* lapv) {  // loop_par.f:174-255
    int n = o->nx;
    double dyy = o->dyy, dxx = o->dxx, beta = o->beta;
    for (int k = 1; k <= o->K; k++)
        for (int i = 1; i <= n; i++) {
            auto U = [&](int j) -> C { return o->uy[o->id(i, j, k)]; };
            lapv[(size_t)(i - 1) + (size_t)n * (k - 1)] =
                o->d2uydx2[(size_t)(i - 1) + (size_t)n * (k - 1)]
                + (o->w_at_w[2] * U(1) + o->w_at_w[3] * U(2) + o->w_at_w[4] * U(3) + o->w_at_w[5] * U(4)
                   + o->w_at_w[6] * U(5) + o->w_at_w[7] * U(6) + o->w_at_w[8] * U(7)) / (dyy * o->w_at_w[0])
                + o->v_k2b2[k - 1] * U(1);
        }
    std::vector<double> a((size_t)n * 5), lu((size_t)n * 5, 0.0);
    std::vector<C> d2(n + 1), rhs(n), y(n + 1);
    for (int k = 2; k <= o->K; k++) {
        double k2b2 = dxx * o->v_k2b2[k - 1];
        lhs5(o, a, k2b2);
        ludecomp(n, a, lu);
        der2wydxdy(o, d2, k);
        C vkb = o->v_kb[k - 1];
        auto LV = [&](int i) -> C { return lapv[(size_t)(i - 1) + (size_t)n * (k - 1)]; };
        rhs[0] = o->wx[o->id(1, 1, k)];
        rhs[1] = dxx * (-d2[1] - 10.0 * d2[2] - d2[3] + vkb * (LV(1) + 10.0 * LV(2) + LV(3))) / 12.0;
        for (int i = 3; i <= n - 2; i++)
            rhs[i - 1] = 8.0 * dxx * (-d2[i - 1] - 5.5 * d2[i] - d2[i + 1] + vkb * (LV(i - 1) + 5.5 * LV(i) + LV(i + 1)));
        rhs[n - 2] = dxx * (-d2[n] - 10.0 * d2[n - 1] - d2[n - 2] + vkb * (LV(n) + 10.0 * LV(n - 1) + LV(n - 2))) / 12.0;
        rhs[n - 1] = (d2[n] - vkb * LV(n)) / ((double)(k - 1) * (double)(k - 1) * beta * beta);
        lusolver_1(n, lu, rhs.data(), y);
        for (int i = 2; i <= n; i++) o->wx[o->id(i, 1, k)] = rhs[i - 1];
    }
}
void wz_wall_impl(ora_ctx* o, const C* lapv) {  // loop_par.f:361-425
    int n = o->nx;
    double dx = o->dx;
    std::vector<C> rhs(n + 1);
    for (int k = 1; k <= o->K; k++) {
        for (int i = 1; i <= n; i++)
            rhs[i] = o->v_kb[k - 1] * o->wx[o->id(i, 1, k)] - lapv[(size_t)(i - 1) + (size_t)n * (k - 1)];
        auto W = [&](int i) -> C& { return o->wz[o->id(i, 1, k)]; };
        W(2) = (dx * (251.0 * rhs[1] + 646.0 * rhs[2] - 264.0 * rhs[3] + 106.0 * rhs[4] - 19.0 * rhs[5]) + 720.0 * W(1)) / 720.0;
        for (int i = 3; i <= n - 2; i++)
            W(i) = (dx * (281.0 * rhs[i - 2] + 2056.0 * rhs[i - 1] + 1176.0 * rhs[i] - 104.0 * rhs[i + 1] + 11.0 * rhs[i + 2]) / 90.0
                    + 11.0 * W(i - 2) + 16.0 * W(i - 1)) / 27.0;
        int i = n - 1;
        W(i) = (dx * (10.0 * rhs[i - 2] + 57.0 * rhs[i - 1] + 24.0 * rhs[i] - rhs[i + 1]) + 33.0 * W(i - 2) + 24.0 * W(i - 1)) / 57.0;
        i = n;
        W(i) = (dx * (251.0 * rhs[i] + 646.0 * rhs[i - 1] - 264.0 * rhs[i - 2] + 106.0 * rhs[i - 3] - 19.0 * rhs[i - 4])
                + 720.0 * W(i - 1)) / 720.0;
    }
}
void filter_trid_impl(ora_ctx* o) {  // filter_par.f:144-177, rhsf_trid 222-332
    int n = o->nx;
    double alphaf = o->cfg.alphaf;
    double af = (11.0 + 10.0 * alphaf) / 16.0, bf = (15.0 + 34.0 * alphaf) / 64.0;
    double cf = (-3.0 + 6.0 * alphaf) / 32.0, df = (1.0 - 2.0 * alphaf) / 64.0;
    std::vector<double> gam(n); std::vector<C> u(n), r(n);
    std::vector<C>* fields[3] = {&o->wx, &o->wy, &o->wz};
    std::vector<std::vector<C>> out(3, std::vector<C>(o->N3()));
    for (int f = 0; f < 3; f++) {
        std::vector<C>& w = *fields[f];
        for (int k = 1; k <= o->K; k++)
            for (int j = 1; j <= o->ny; j++) {
                const C* W = &w[o->id(1, j, k)] - 1;  // 1-based
                r[0] = (15.0 * W[1] + 4.0 * W[2] - 6.0 * W[3] + 4.0 * W[4] - W[5]) / 16.0;
                r[1] = (W[1] + 12.0 * W[2] + 6.0 * W[3] - 4.0 * W[4] + W[5]) / 16.0;
                r[2] = (-W[1] + 4.0 * W[2] + 10.0 * W[3] + 4.0 * W[4] - W[5]) / 16.0;
                for (int i = 4; i <= n - 3; i++)
                    r[i - 1] = af * W[i] + bf * (W[i + 1] + W[i - 1]) + cf * (W[i + 2] + W[i - 2]) + df * (W[i + 3] + W[i - 3]);
                r[n - 3] = (-W[n] + 4.0 * W[n - 1] + 10.0 * W[n - 2] + 4.0 * W[n - 3] - W[n - 4]) / 16.0;
                r[n - 2] = (W[n] + 12.0 * W[n - 1] + 6.0 * W[n - 2] - 4.0 * W[n - 3] + W[n - 4]) / 16.0;
                r[n - 1] = (15.0 * W[n] + 4.0 * W[n - 1] - 6.0 * W[n - 2] + 4.0 * W[n - 3] - W[n - 4]) / 16.0;
                thomas(o->afil.data(), o->bfil.data(), o->cfil.data(), r.data(), n, 1, gam, u);
                for (int i = 0; i < n; i++) out[f][o->id(1, j, k) + i] = r[i];
            }
    }
    for (int f = 0; f < 3; f++) {
        std::vector<C>& w = *fields[f];
        for (int k = 1; k <= o->K; k++)
            for (int j = 2; j <= o->ny; j++)
                for (int i = 2; i <= n; i++) w[o->id(i, j, k)] = out[f][o->id(i, j, k)];
    }
}
void ts_pert_impl(ora_ctx* o, int t, double tempt) {  // main_par.f:1613-1685
    const tb_config& c = o->cfg;
    for (int m = 0; m < c.n_forced; m++) {
        int kk = c.forced_mode[m] + 1;
        if (kk < 1 || kk > o->K) continue;
        double A = c.forced_amp[m] * std::sqrt(o->fac_y);
        double H = 1.0;
        double arg = H * ((double)t + tempt) * o->omega * o->dt;
        if (c.forced_phase[m] != 0.0) arg = arg + c.forced_phase[m];
        double fct = A * std::sin(arg);
        if (t < c.stpp) {
            double ept = (double)t / (double)c.stpp;
            fct = fct * ((6.0 * ept - 15.0) * ept + 10.0) * powi(ept, 3);
        }
        for (int i = c.i1 + 1; i <= c.i2 - 1; i++) {
            o->uy[o->id(i, 1, kk)] = mk(o->fcx[i - 1] * fct, 0.0);
            o->d2uydx2[(size_t)(i - 1) + (size_t)o->nx * (kk - 1)] = mk(o->fcllx[i - 1] * fct, 0.0);
        }
    }
}

void gv_pert_impl(ora_ctx* o, int t) {  // main_par.f:1577-1610
    const tb_config& c = o->cfg;
    double A = 1e-6 * std::sqrt(o->fac_y);
    if (t < c.stpp) {
        double ep = (double)t / (double)c.stpp;
        A = A * ((6.0 * ep - 15.0) * ep + 10.0) * powi(ep, 3);
    }
    for (int i = c.i1 + 1; i <= c.i2 - 1; i++)
        for (int k = 2; k <= o->K; k++) {
            o->uy[o->id(i, 1, k)] = mk(A * o->fcx2[i - 1], 0.0);
            o->d2uydx2[(size_t)(i - 1) + (size_t)o->nx * (k - 1)] = mk(A * o->fcllx2[i - 1], 0.0);
        }
}

// lterms_gv (nlterms_par.f:89-112) and drv_gv (main_par.f:1338-1401): the
// linearised terms about the 2D base flow and the curvature terms, with
// varg = Go^2 / sqrt(Re) at every point; dvargdx, its compact x-derivative,
// is zero for the constant varg and is left out.
void drv_gv_impl(ora_ctx* o, C* dvx, C* dvy, C* dvz) {
    size_t N3 = o->N3();
    std::vector<C> a(N3), b(N3), c(N3), d(N3), dadx(N3), dbdx(N3), dddx(N3), dady(N3), dcdy(N3);
    std::vector<C> xx[3] = {std::vector<C>(N3), std::vector<C>(N3), std::vector<C>(N3)};
    std::vector<C> yy[3] = {std::vector<C>(N3), std::vector<C>(N3), std::vector<C>(N3)};
    for (int k = 1; k <= o->K; k++)
        for (int j = 1; j <= o->ny; j++)
            for (int i = 1; i <= o->nx; i++) {
                size_t q = o->id(i, j, k), p = o->id2(i, j);
                double U = o->uxb[p], V = o->uyb[p], W = o->wzb[p];
                a[q] = V * o->wx[q] - o->wy[q] * U;
                b[q] = U * o->wz[q] + o->ux[q] * W;
                c[q] = -V * o->wz[q] - o->uy[q] * W;
                d[q] = 2.0 * U * o->ux[q];
            }
    derparx_impl(o, dadx.data(), a.data());
    derparx_impl(o, dbdx.data(), b.data());
    derparx_impl(o, dddx.data(), d.data());
    dery_impl(o, dady.data(), a.data(), 0);
    dery_impl(o, dcdy.data(), c.data(), 0);
    derparxx_impl(o, xx[0].data(), o->wx.data());
    derparxx_impl(o, xx[1].data(), o->wy.data());
    derparxx_impl(o, xx[2].data(), o->wz.data());
    dery_impl(o, yy[0].data(), o->wx.data(), 2);
    dery_impl(o, yy[1].data(), o->wy.data(), 2);
    dery_impl(o, yy[2].data(), o->wz.data(), 2);
    const double Re = o->Re, fy = o->fac_y, varg = o->cfg.go_number * o->cfg.go_number / std::sqrt(Re);
    for (int k = 1; k <= o->K; k++) {
        C vkb = o->v_kb[k - 1];
        double k2 = o->v_k2b2[k - 1];
        for (int j = 2; j <= o->ny; j++)
            for (int i = 1; i <= o->nx; i++) {
                size_t q = o->id(i, j, k);
                dvx[q] = -dady[q] + vkb * b[q] - vkb * d[q] * varg + (xx[0][q] + yy[0][q] * fy + k2 * o->wx[q]) / Re;
                dvy[q] = -(vkb * c[q]) + dadx[q] + (xx[1][q] + yy[1][q] * fy + k2 * o->wy[q]) / Re;
                dvz[q] = -dbdx[q] + dcdy[q] + varg * dddx[q] + (xx[2][q] + yy[2][q] * fy + k2 * o->wz[q]) / Re;
            }
    }
}

// nlterms_th (nlterms_par.f:216-300) and drv_gvth (main_par.f:1404-1484):
// the disturbance's full nonlinear products and those with the 2D base flow
// and base temperature, the momentum terms of drv_gv (without its d dvarg/dx
// term, commented out there) and the temperature equation.
void drv_gvth_impl(ora_ctx* o, C* dvx, C* dvy, C* dvz, C* dvt) {
    const size_t N3 = o->N3(), NP = (size_t)o->nx * o->ny * o->P;
    std::vector<double> ph[7];
    const std::vector<C>* in[7] = {&o->ux, &o->uy, &o->uz, &o->wx, &o->wy, &o->wz, &o->th};
    for (int f = 0; f < 7; f++) { ph[f].assign(NP, 0.0); f_to_p_impl(o, ph[f].data(), in[f]->data()); }
    for (size_t q = 0; q < NP; q++) {
        const double ux = ph[0][q], uy = ph[1][q], uz = ph[2][q], wx = ph[3][q], wy = ph[4][q], wz = ph[5][q], th = ph[6][q];
        ph[0][q] = uy * wx - ux * wy;
        ph[1][q] = ux * wz - uz * wx;
        ph[2][q] = uz * wy - uy * wz;
        ph[3][q] = ux * ux;
        ph[4][q] = ux * th;
        ph[5][q] = uy * th;
        ph[6][q] = uz * th;
    }
    std::vector<C> a(N3), b(N3), c(N3), d(N3), uth(N3), vth(N3), wth(N3);
    std::vector<C>* out[7] = {&a, &b, &c, &d, &uth, &vth, &wth};
    for (int f = 0; f < 7; f++) p_to_f_impl(o, out[f]->data(), ph[f].data());
    for (int k = 1; k <= o->K; k++)
        for (int j = 1; j <= o->ny; j++)
            for (int i = 1; i <= o->nx; i++) {
                size_t q = o->id(i, j, k), p = o->id2(i, j);
                double U = o->uxb[p], V = o->uyb[p], W = o->wzb[p], T = o->thb[p];
                a[q] = V * o->wx[q] - U * o->wy[q] + a[q];
                b[q] = U * o->wz[q] + o->ux[q] * W + b[q];
                c[q] = -V * o->wz[q] - o->uy[q] * W + c[q];
                d[q] = 2.0 * U * o->ux[q] + d[q];
                uth[q] = U * o->th[q] + o->ux[q] * T + uth[q];
                vth[q] = V * o->th[q] + o->uy[q] * T + vth[q];
                wth[q] = o->uz[q] * T + wth[q];
            }
    std::vector<C> dadx(N3), dbdx(N3), dddx(N3), duthdx(N3), dady(N3), dcdy(N3), dvthdy(N3), txx(N3), tyy(N3);
    std::vector<C> xx[3] = {std::vector<C>(N3), std::vector<C>(N3), std::vector<C>(N3)};
    std::vector<C> yy[3] = {std::vector<C>(N3), std::vector<C>(N3), std::vector<C>(N3)};
    derparx_impl(o, dadx.data(), a.data());
    derparx_impl(o, dbdx.data(), b.data());
    derparx_impl(o, dddx.data(), d.data());
    derparx_impl(o, duthdx.data(), uth.data());
    dery_impl(o, dady.data(), a.data(), 0);
    dery_impl(o, dcdy.data(), c.data(), 0);
    dery_impl(o, dvthdy.data(), vth.data(), 0);
    derparxx_impl(o, xx[0].data(), o->wx.data());
    derparxx_impl(o, xx[1].data(), o->wy.data());
    derparxx_impl(o, xx[2].data(), o->wz.data());
    derparxx_impl(o, txx.data(), o->th.data());
    dery_impl(o, yy[0].data(), o->wx.data(), 2);
    dery_impl(o, yy[1].data(), o->wy.data(), 2);
    dery_impl(o, yy[2].data(), o->wz.data(), 2);
    dery_impl(o, tyy.data(), o->th.data(), 2);
    const double Re = o->Re, fy = o->fac_y, varg = o->cfg.go_number * o->cfg.go_number / std::sqrt(Re);
    const double RePr = Re * o->cfg.Pr;
    for (int k = 1; k <= o->K; k++) {
        C vkb = o->v_kb[k - 1];
        double k2 = o->v_k2b2[k - 1];
        for (int j = 2; j <= o->ny; j++)
            for (int i = 1; i <= o->nx; i++) {
                size_t q = o->id(i, j, k);
                dvx[q] = -dady[q] + vkb * b[q] - vkb * d[q] * varg + (xx[0][q] + yy[0][q] * fy + k2 * o->wx[q]) / Re;
                dvy[q] = -(vkb * c[q]) + dadx[q] + (xx[1][q] + yy[1][q] * fy + k2 * o->wy[q]) / Re;
                dvz[q] = -dbdx[q] + dcdy[q] + varg * dddx[q] + (xx[2][q] + yy[2][q] * fy + k2 * o->wz[q]) / Re;
                dvt[q] = -duthdx[q] - dvthdy[q] - vkb * wth[q] + (txx[q] + tyy[q] + k2 * o->th[q]) / RePr;
            }
    }
}

// les_par.f:6-211 (terms whose results the reference never uses -- the
// x/y/z derivatives of nu_t and the nu_t spectrum -- are not formed).
void les_terms_impl(ora_ctx* o, C* Fx, C* Fy, C* Fz) {
    size_t n2 = (size_t)o->nx * o->ny, NP = n2 * o->P, N3 = o->N3();
    std::vector<C> dud(N3), dvd(N3), dwd(N3);
    std::vector<double> dudx(NP), dvdx(NP), dwdx(NP), dudy(NP), dvdy(NP), dwdy(NP), dudz(NP), dvdz(NP), dwdz(NP);
    derparx_impl(o, dud.data(), o->ux.data());
    derparx_impl(o, dvd.data(), o->uy.data());
    derparx_impl(o, dwd.data(), o->uz.data());
    f_to_p_impl(o, dudx.data(), dud.data());
    f_to_p_impl(o, dvdx.data(), dvd.data());
    f_to_p_impl(o, dwdx.data(), dwd.data());
    dery_impl(o, dud.data(), o->ux.data(), 0);
    dery_impl(o, dvd.data(), o->uy.data(), 1);
    dery_impl(o, dwd.data(), o->uz.data(), 0);
    f_to_p_impl(o, dudy.data(), dud.data());
    f_to_p_impl(o, dvdy.data(), dvd.data());
    f_to_p_impl(o, dwdy.data(), dwd.data());
    for (int k = 1; k <= o->K; k++)
        for (size_t q = 0; q < n2; q++) {
            size_t p = q + n2 * (k - 1);
            dud[p] = o->v_kb[k - 1] * o->ux[p];
            dvd[p] = o->v_kb[k - 1] * o->uy[p];
            dwd[p] = o->v_kb[k - 1] * o->uz[p];
        }
    f_to_p_impl(o, dudz.data(), dud.data());
    f_to_p_impl(o, dvdz.data(), dvd.data());
    f_to_p_impl(o, dwdz.data(), dwd.data());
    std::vector<double> nu(NP);
    double dz = o->dz;
    double delta_les = std::pow(o->dx * o->dy * dz, 1.0 / 3.0);
    for (int z = 1; z <= o->P; z++)
        for (int j = 1; j <= o->ny; j++) {
            double y = (o->stf == 1.0) ? (double)(j - 1) * o->dy : o->dy * (powi(o->stf, j - 1) - 1.0) / (o->stf - 1.0);
            for (int i = 1; i <= o->nx; i++) {
                size_t q = o->id2(i, j) + n2 * (z - 1);
                // les_par.f:194; les_damping bit 2 takes |wz_wall| (the reference's
                // square root is NaN where the wall vorticity is negative)
                double wz0 = o->wz[o->id(i, 1, 1)].re;
                if (o->cfg.les_damping & 2) wz0 = std::fabs(wz0);
                double yplus = std::sqrt(o->Re * wz0 / std::sqrt(o->fac_y)) * y;
                double damp;
                if (o->cfg.les_damping & 1) {
                    double e = 1.0 - std::exp(-yplus / o->cfg.A_plus);
                    damp = e * e;
                } else {
                    // min(y+/A, 100): fmin's IEEE minNum gives 100 for a NaN y+
                    // (Fortran leaves MIN with a NaN argument unspecified)
                    double ratio = std::fmin(yplus / o->cfg.A_plus, 100.0);
                    ratio = powi(ratio, 3);
                    damp = 1.0 - std::exp(-ratio);
                }
                double cte = o->cfg.C_s * o->cfg.C_s * delta_les * delta_les * damp;
                double Sxx = dudx[q], Syy = dvdy[q], Szz = dwdz[q];
                double Sxy = 0.5 * (dudy[q] + dvdx[q]), Sxz = 0.5 * (dudz[q] + dwdx[q]), Syz = 0.5 * (dvdz[q] + dwdy[q]);
                nu[q] = cte * std::sqrt(2.0 * (Sxx * Sxx + Syy * Syy + Szz * Szz + 2.0 * (Sxy * Sxy + Sxz * Sxz + Syz * Syz)));
            }
        }
    std::vector<C> d2x(N3), d2y(N3), lap(N3);
    std::vector<double> lp(NP);
    const std::vector<C>* us[3] = {&o->ux, &o->uy, &o->uz};
    C* outs[3] = {Fx, Fy, Fz};
    std::vector<std::vector<double>> laps(3, std::vector<double>(NP));
    for (int f = 0; f < 3; f++) {
        derparxx_impl(o, d2x.data(), us[f]->data());
        dery_impl(o, d2y.data(), us[f]->data(), 2);
        for (int k = 1; k <= o->K; k++)
            for (size_t q = 0; q < n2; q++) {
                size_t p = q + n2 * (k - 1);
                lap[p] = d2x[p] + d2y[p] + o->v_k2b2[k - 1] * (*us[f])[p];
            }
        f_to_p_impl(o, laps[f].data(), lap.data());
    }
    for (int f = 0; f < 3; f++) {
        for (size_t q = 0; q < NP; q++) lp[q] = nu[q] * laps[f][q];
        p_to_f_impl(o, outs[f], lp.data());
    }
}
void cvirt_impl(ora_ctx* o, C* Fx, C* Fy, C* Fz) {  // immersed_par.f:262-313
    size_t n2 = (size_t)o->nx * o->ny, NP = n2 * o->P;
    std::vector<double> up(NP), fp(NP);
    const std::vector<C>* us[3] = {&o->ux, &o->uy, &o->uz};
    C* outs[3] = {Fx, Fy, Fz};
    for (int f = 0; f < 3; f++) {
        f_to_p_impl(o, up.data(), us[f]->data());
        for (size_t q = 0; q < NP; q++) fp[q] = o->cfg.irf * o->delta_no[q] * up[q];
        p_to_f_impl(o, outs[f], fp.data());
        for (int k = 1; k <= o->K; k++)
            for (size_t q = 0; q < n2; q++) outs[f][q + n2 * (k - 1)] = o->gibbs[k - 1] * outs[f][q + n2 * (k - 1)];
    }
}
void drv_impl(ora_ctx* o, C* dvx, C* dvy, C* dvz) {  // main_par.f:1264-1336 / 1487-1574
    if (o->cfg.my_form == 1) { drv_gv_impl(o, dvx, dvy, dvz); return; }
    if (o->cfg.my_form == 2) { drv_gvth_impl(o, dvx, dvy, dvz, (dvx == o->dv1x.data() ? o->dv1t : o->dv2t).data()); return; }
    size_t N3 = o->N3();
    std::vector<C> a(N3), b(N3), c(N3), dadx(N3), dbdx(N3), dady(N3), dcdy(N3);
    std::vector<C> xx[3] = {std::vector<C>(N3), std::vector<C>(N3), std::vector<C>(N3)};
    std::vector<C> yy[3] = {std::vector<C>(N3), std::vector<C>(N3), std::vector<C>(N3)};
    nlterms_impl(o, a.data(), b.data(), c.data());
    derparx_impl(o, dadx.data(), a.data());
    derparx_impl(o, dbdx.data(), b.data());
    dery_impl(o, dady.data(), a.data(), 0);
    dery_impl(o, dcdy.data(), c.data(), 0);
    derparxx_impl(o, xx[0].data(), o->wx.data());
    derparxx_impl(o, xx[1].data(), o->wy.data());
    derparxx_impl(o, xx[2].data(), o->wz.data());
    dery_impl(o, yy[0].data(), o->wx.data(), 2);
    dery_impl(o, yy[1].data(), o->wy.data(), 2);
    dery_impl(o, yy[2].data(), o->wz.data(), 2);
    bool les = o->cfg.my_form == 4, ibm = o->cfg.ibm != 0;
    bool force = les || ibm;
    std::vector<C> dfydx, dfzdx, dfxdy, dfzdy;
    if (force) {
        std::fill(o->fx.begin(), o->fx.end(), mk(0, 0));
        std::fill(o->fy.begin(), o->fy.end(), mk(0, 0));
        std::fill(o->fz.begin(), o->fz.end(), mk(0, 0));
        if (les) les_terms_impl(o, o->fx.data(), o->fy.data(), o->fz.data());
        if (ibm) {
            std::vector<C> gx(N3), gy(N3), gz(N3);
            cvirt_impl(o, gx.data(), gy.data(), gz.data());
            for (size_t q = 0; q < N3; q++) { o->fx[q] = o->fx[q] + gx[q]; o->fy[q] = o->fy[q] + gy[q]; o->fz[q] = o->fz[q] + gz[q]; }
        }
        dfydx.resize(N3); dfzdx.resize(N3); dfxdy.resize(N3); dfzdy.resize(N3);
        derparx_impl(o, dfydx.data(), o->fy.data());
        derparx_impl(o, dfzdx.data(), o->fz.data());
        dery_impl(o, dfxdy.data(), o->fx.data(), 0);
        dery_impl(o, dfzdy.data(), o->fz.data(), 0);
    }
    double Re = o->Re, fy = o->fac_y;
    for (int k = 1; k <= o->K; k++) {
        C vkb = o->v_kb[k - 1];
        double k2 = o->v_k2b2[k - 1];
        for (int j = 2; j <= o->ny; j++)
            for (int i = 1; i <= o->nx; i++) {
                size_t q = o->id(i, j, k);
                C vx = -dady[q] + vkb * b[q] + (xx[0][q] + yy[0][q] * fy + k2 * o->wx[q]) / Re;
                C vy = -(vkb * c[q]) + dadx[q] + (xx[1][q] + yy[1][q] * fy + k2 * o->wy[q]) / Re;
                C vz = -dbdx[q] + dcdy[q] + (xx[2][q] + yy[2][q] * fy + k2 * o->wz[q]) / Re;
                if (force) {
                    vx = vx + vkb * o->fy[q] / fy - dfzdy[q];
                    vy = vy + dfzdx[q] - vkb * o->fx[q];
                    vz = vz + dfxdy[q] - dfydx[q] / fy;
                }
                dvx[q] = vx; dvy[q] = vy; dvz[q] = vz;
            }
    }
}
void loop_impl(ora_ctx* o, double erro, bool filter) {  // main_par.f:1762-1785
    if (filter) filter_trid_impl(o);
    bzone_impl(o);
    size_t N3 = o->N3();
    std::vector<C> dwzdx(N3), duydy(N3), lapv((size_t)o->nx * o->K);
    outuy_impl(o, dwzdx.data());
    poi_uy_impl(o, dwzdx.data(), erro);
    poi_ux_impl(o, duydy.data());
    poi_uz_impl(o, duydy.data());
    wx_wall_impl(o, lapv.data());
    wz_wall_impl(o, lapv.data());
    bzonew_impl(o);
}

// ---------------------------------------------------------------------------
// Set-up (init_fi main_par.f:551-772, create_ctes 1828-1892, derivs_k,
// var_ts 1688-1736, gibbs_function immersed_par.f:205, delta 98-181).
void setup_constants(ora_ctx* o) {
    const tb_config& c = o->cfg;
    int nx = o->nx, ny = o->ny, msh = o->msh;
    // create_ctes
    o->v_dy0.assign(msh, 0); o->v_stf.assign(msh, 0); o->v_dx2.assign(msh, 0);
    for (int l = 1; l <= msh; l++) {
        if (o->stf != 1.0) o->v_dy0[l - 1] = o->dy * ((powi(o->stf, 1 << (l - 1)) - 1.0) / (o->stf - 1.0));
        else o->v_dy0[l - 1] = o->dy * powi(2.0, l - 1);
    }
    for (int l = 1; l <= msh; l++) {
        o->v_stf[l - 1] = powi(o->stf, 1 << (l - 1));
        o->v_dx2[l - 1] = powi(o->dx * (double)(1 << (l - 1)), 2);
    }
    o->v_qdy.assign(ny, 0.0);
    for (int j = 1; j <= ny - 1; j++) {
        if (o->stf != 1.0) o->v_qdy[j - 1] = 1.0 / (o->v_dy0[0] * powi(o->v_stf[0], j - 1));
        else o->v_qdy[j - 1] = 1.0 / o->v_dy0[0];
    }
    o->v_qdy2.assign((size_t)ny * msh, 0.0);
    for (int l = 1; l <= msh; l++)
        for (int j = 1; j <= (ny - 1) / (1 << (l - 1)); j++) {
            double aux = (o->stf != 1.0) ? o->v_dy0[l - 1] * powi(o->v_stf[l - 1], j - 1) : o->v_dy0[l - 1];
            o->QDY2(j, l) = 1.0 / powi(aux, 2);
        }
    o->v_ptsx.assign(msh, 0); o->v_ptsy.assign(msh, 0);
    o->v_ptsx[0] = nx; o->v_ptsy[0] = ny;
    for (int l = 2; l <= msh; l++) {
        o->v_ptsx[l - 1] = (o->v_ptsx[l - 2] + 1) / 2;
        o->v_ptsy[l - 1] = (o->v_ptsy[l - 2] + 1) / 2;
    }
    o->v_k2b2.assign(o->K, 0.0); o->v_kb.assign(o->K, mk(0, 0));
    for (int k = 1; k <= o->K; k++) {
        o->v_k2b2[k - 1] = -(double)(k - 1) * (double)(k - 1) * o->beta * o->beta;
        C mim = mk(-0.0, -1.0);  // -im
        o->v_kb[k - 1] = (mim * (double)(k - 1)) * o->beta;
    }
    // coefx / coeffx (derivs_par.f:1145-1210)
    o->a1x.assign(nx, 0); o->b1x.assign(nx, 0); o->c1x.assign(nx, 0);
    o->a2x.assign(nx, 0); o->b2x.assign(nx, 0); o->c2x.assign(nx, 0);
    o->a1x[0] = 0; o->b1x[0] = 1; o->c1x[0] = 0;
    o->a1x[1] = 1; o->b1x[1] = 6; o->c1x[1] = 2;
    for (int i = 2; i < nx - 2; i++) { o->a1x[i] = 1; o->b1x[i] = 3; o->c1x[i] = 1; }
    o->a1x[nx - 2] = 2; o->b1x[nx - 2] = 6; o->c1x[nx - 2] = 1;
    o->a1x[nx - 1] = 4; o->b1x[nx - 1] = 1; o->c1x[nx - 1] = 0;
    o->a2x[0] = 0; o->b2x[0] = 13; o->c2x[0] = 137;
    o->a2x[1] = 1; o->b2x[1] = 12; o->c2x[1] = 3;
    for (int i = 2; i < nx - 2; i++) { o->a2x[i] = 2; o->b2x[i] = 11; o->c2x[i] = 2; }
    o->a2x[nx - 2] = 3; o->b2x[nx - 2] = 12; o->c2x[nx - 2] = 1;
    o->a2x[nx - 1] = 137; o->b2x[nx - 1] = 13; o->c2x[nx - 1] = 0;
    // lhs_tridf (filter_par.f:181-220)
    o->afil.assign(nx, 0); o->bfil.assign(nx, 1); o->cfil.assign(nx, 0);
    for (int i = 3; i < nx - 3; i++) { o->afil[i] = c.alphaf; o->cfil[i] = c.alphaf; }
    // var_ts (main_par.f:1688-1736)
    int i1 = c.i1, i2 = c.i2;
    o->fcx.assign(i2, 0.0); o->fcllx.assign(i2, 0.0);
    {
        double imed = (double)(i1 + i2) / 2.0;
        double div = 1.0 / ((double)(imed - i1) * o->dx);
        double A = -(19683.0 / 4096.0 * powi(div, 8)), B = 177147.0 / 4096.0 * powi(div, 7);
        double Cc = -(19683.0 / 128.0 * powi(div, 6)), D = 137781.0 / 512.0 * powi(div, 5);
        double E = -(59049.0 / 256.0 * powi(div, 4)), F = 19683.0 / 256.0 * powi(div, 3);
        double fcmax = 0.0;
        for (int i = i1; i <= (i1 + i2) / 2; i++) {
            double x = (double)(i - i1) * o->dx;
            double v = (((((A * x + B) * x + Cc) * x + D) * x + E) * x + F) * powi(x, 4);
            fcmax = std::max(fcmax, std::fabs(v));
        }
        for (int i = i1; i <= (i1 + i2) / 2; i++) {
            double x = (double)(i - i1) * o->dx;
            double v = (((((A * x + B) * x + Cc) * x + D) * x + E) * x + F) * powi(x, 4) / fcmax;
            if (std::fabs(v) < 1e-15) v = 0.0;
            o->fcx[i - 1] = v;
            o->fcx[i2 + i1 - i - 1] = -o->fcx[i - 1];
            double w = (((((72.0 * A * x + 56.0 * B) * x + 42.0 * Cc) * x + 30.0 * D) * x + 20.0 * E) * x + 12.0 * F) * x * x / fcmax;
            if (std::fabs(w) < 1e-15) w = 0.0;
            o->fcllx[i - 1] = w;
            o->fcllx[i2 + i1 - i - 1] = -o->fcllx[i - 1];
        }
    }
    // buffer ramps (main_par.f:737-756)
    o->bdfc.assign(nx, 0.0);
    for (int i = 1; i <= c.i0; i++) {
        double ep = (double)(i - 1) / (double)(c.i0 - 1);
        o->bdfc[i - 1] = ((6.0 * ep - 15.0) * ep + 10.0) * powi(ep, 3);
    }
    for (int i = c.i0; i <= c.i3; i++) o->bdfc[i - 1] = 1.0;
    for (int i = c.i3; i <= c.i4; i++) {
        double ep = (double)(i - c.i3) / (double)(c.i4 - c.i3);
        o->bdfc[i - 1] = powi(1.0 - powi(ep, 50), 4) * std::exp(-powi(ep, 4) / 10.0);
    }
    for (int i = c.i4; i <= nx; i++) o->bdfc[i - 1] = 0.0;
    // bdfc(2,:): init_gv's ramp over i = 1 .. 2 (i1 + i2) (main_par.f:991-996)
    o->bdfc2 = o->bdfc;
    if (c.my_form == 1) {
        int igv = std::min(2 * (c.i1 + c.i2), nx);
        for (int i = 1; i <= igv; i++) {
            double ep = (double)(i - 1) / (double)(igv - 1);
            o->bdfc2[i - 1] = ((6.0 * ep - 15.0) * ep + 10.0) * powi(ep, 3);
        }
    }
    // var_gv (main_par.f:1739-1759)
    o->fcx2.assign(nx, 0.0); o->fcllx2.assign(nx, 0.0);
    for (int i = c.i1; i <= c.i2 && i <= nx; i++) {
        double x = PI * (double)(i - c.i1) / (double)(c.i2 - c.i1);
        o->fcx2[i - 1] = powi(std::sin(x), 3);
        o->fcllx2[i - 1] = 6.0 * powi(std::cos(x), 2) * std::sin(x) - 3.0 * powi(std::sin(x), 3);
    }
    // gibbs_function (immersed_par.f:205-259): final form exp(-theta^2)
    o->gibbs.assign(o->K, 1.0);
    for (int k = 1; k <= o->K; k++) {
        if (o->K == 1) { o->gibbs[k - 1] = 1.0; continue; }
        double theta = PI * (double)(k - 1) / (double)(o->K - 1);
        o->gibbs[k - 1] = std::exp(-(theta * theta));
    }
}
void setup_lhs_y(ora_ctx* o) {  // coefy / coefy_fv / coeffy (derivs_par.f:1040-1142)
    int J = o->ny;
    auto set = [&](std::vector<double>& a, std::vector<double>& b, std::vector<double>& c, const double* first3,
                   const double* sp, const double* cp, const double* pp, const double* lp) {
        a.assign(J, 0); b.assign(J, 0); c.assign(J, 0);
        a[0] = first3[0]; b[0] = first3[1]; c[0] = first3[2];
        a[1] = sp[0]; b[1] = sp[1]; c[1] = sp[2];
        for (int j = 2; j < J - 2; j++) { a[j] = cp[0]; b[j] = cp[1]; c[j] = cp[2]; }
        a[J - 2] = pp[2]; b[J - 2] = pp[1]; c[J - 2] = pp[0];
        a[J - 1] = lp[1]; b[J - 1] = lp[0]; c[J - 1] = 0.0;
    };
    double f1[3] = {0.0, o->fp_fd_e[0], 0.0};
    double ffv[3] = {0.0, 1.0, 0.0};
    double f2[3] = {0.0, o->fp_sd[0], o->fp_sd[1]};
    set(o->a1y, o->b1y, o->c1y, f1, o->sp_fd, o->cp_fd, o->pp_fd, o->lp_fd);
    set(o->a1fv, o->b1fv, o->c1fv, ffv, o->sp_fd, o->cp_fd, o->pp_fd, o->lp_fd);
    set(o->a2y, o->b2y, o->c2y, f2, o->sp_sd, o->cp_sd, o->pp_sd, o->lp_sd);
}
void setup_delta(ora_ctx* o) {  // delta (immersed_par.f:98-181)
    size_t n2 = (size_t)o->nx * o->ny;
    o->delta_no.assign(n2 * o->P, 0.0);
    if (!o->cfg.ibm) return;
    double sigx = 1.0, sigy = 1.0, dz = o->dz;
    double xc = o->cfg.ibm_xc, zc = o->cfg.ibm_zc, h = o->cfg.ibm_h, R = o->cfg.ibm_R;
    for (int k = 1; k <= o->P; k++) {
        double z = (double)(k - 1) * dz;
        for (int j = 1; j <= o->ny; j++) {
            double y = (o->stf == 1.0) ? (double)(j - 1) * o->dy : o->dy * (powi(o->stf, j - 1) - 1.0) / (o->stf - 1.0);
            for (int i = 1; i <= o->nx; i++) {
                double x = o->cfg.x0 + (double)(i - 1) * o->dx;
                size_t q = o->id2(i, j) + n2 * (k - 1);
                if (y <= h) {
                    double dist = std::sqrt(powi(x - xc, 2) + powi(z - zc, 2));
                    double xs = xc - (R * (xc - x)) / dist;
                    double zs = zc - (R * (zc - z)) / dist;
                    double v = std::exp(-powi((x - xs) / sigx / dz, 2) - powi((z - zs) / sigy / dz, 2)) / (sigx * sigy);
                    if (dist < R) v = 1.0;
                    if (v < 1e-14) v = 0.0;
                    o->delta_no[q] = v;
                }
            }
        }
    }
    std::vector<C> df(o->N3());
    p_to_f_impl(o, df.data(), o->delta_no.data());
    for (int k = 1; k <= o->K; k++)
        for (size_t q = 0; q < n2; q++) df[q + n2 * (k - 1)] = o->gibbs[k - 1] * df[q + n2 * (k - 1)];
    f_to_p_impl(o, o->delta_no.data(), df.data());
}

}  // namespace

// ===========================================================================
extern "C" {

ora_ctx* ora_create(const tb_config* cfg) {
    if (!cfg || cfg->nx < 16 || cfg->ny < 16 || cfg->kfour < 1 || cfg->kphys < 2 || 2 * cfg->kfour > cfg->kphys + 1)
        return nullptr;
    ora_ctx* o = new ora_ctx();
    o->cfg = *cfg;
    o->nx = cfg->nx; o->ny = cfg->ny; o->K = cfg->kfour; o->P = cfg->kphys; o->msh = cfg->msh;
    o->dx = cfg->dx; o->dxx = o->dx * o->dx; o->dy = cfg->dy; o->dyy = o->dy * o->dy; o->stf = cfg->stf;
    o->Re = cfg->Re; o->fac_y = cfg->fac_y; o->alpha = cfg->alpha; o->omega = cfg->omega; o->beta = cfg->beta;
    o->dt = (2.0 * PI) / o->omega / (double)cfg->stpp;
    o->dt2 = 0.5 * o->dt; o->dt6 = o->dt / 6.0;
    o->dz = (2.0 * PI) / ((double)o->P * o->beta);
    size_t N3 = o->N3();
    for (auto* v : {&o->ux, &o->uy, &o->uz, &o->wx, &o->wy, &o->wz, &o->wx1, &o->wy1, &o->wz1, &o->dv1x, &o->dv1y, &o->dv1z,
                    &o->dv2x, &o->dv2y, &o->dv2z, &o->fx, &o->fy, &o->fz})
        v->assign(N3, mk(0, 0));
    o->d2uydx2.assign((size_t)o->nx * o->K, mk(0, 0));
    o->uxb.assign((size_t)o->nx * o->ny, 0.0); o->uyb = o->uxb; o->wzb = o->uxb; o->thb = o->uxb;
    for (auto* v : {&o->th, &o->th1, &o->dv1t, &o->dv2t}) v->assign(N3, mk(0, 0));
    o->duexmdx.assign(o->nx, 0.0);
    o->sp_poi.assign(7 * o->msh, 0); o->cp_poi.assign(8 * o->msh, 0); o->pp_poi.assign(4 * o->msh, 0); o->lp_poi.assign(5 * o->msh, 0);
    setup_constants(o);
    setup_delta(o);
    return o;
}
void ora_destroy(ora_ctx* o) { delete o; }

int ora_set_coefs(ora_ctx* o, const double* b) {
    const double* p = b;
    auto take = [&](double* dst, int n) { std::memcpy(dst, p, sizeof(double) * n); p += n; };
    take(o->fp_fd_e, 6); take(o->sp_fd, 9); take(o->cp_fd, 8); take(o->pp_fd, 9); take(o->lp_fd, 7);
    take(o->fp_sd, 8); take(o->sp_sd, 10); take(o->cp_sd, 8); take(o->pp_sd, 10); take(o->lp_sd, 8);
    take(o->sp_poi.data(), 7 * o->msh); take(o->cp_poi.data(), 8 * o->msh);
    take(o->pp_poi.data(), 4 * o->msh); take(o->lp_poi.data(), 5 * o->msh);
    take(o->w_at_w, 9); take(o->dwydy, 8);
    setup_lhs_y(o);
    o->have_coefs = true;
    return 0;
}
int ora_set_baseflow(ora_ctx* o, const double* uxb, const double* uyb, const double* wzb) {
    size_t n2 = (size_t)o->nx * o->ny;
    o->uxb.assign(uxb, uxb + n2); o->uyb.assign(uyb, uyb + n2); o->wzb.assign(wzb, wzb + n2);
    // derparxue (derivs_par.f:32-45) on ue = uxb(:, jmax) -> duexmdx
    std::vector<double> ue(o->nx), r(o->nx), gam(o->nx), u(o->nx);
    for (int i = 1; i <= o->nx; i++) ue[i - 1] = o->uxb[o->id2(i, o->ny)];
    rhsx_line<double>(ue.data(), r.data(), o->nx, o->dx);
    thomas_r(o->a1x.data(), o->b1x.data(), o->c1x.data(), r.data(), o->nx, 1, gam, u);
    o->duexmdx = r;
    o->have_base = true;
    return 0;
}
int ora_init_fields(ora_ctx* o) {  // main_par.f:601-641
    for (auto* v : {&o->ux, &o->uy, &o->uz, &o->wx, &o->wy, &o->wz, &o->wx1, &o->wy1, &o->wz1, &o->dv1x, &o->dv1y, &o->dv1z,
                    &o->dv2x, &o->dv2y, &o->dv2z, &o->fx, &o->fy, &o->fz})
        std::fill(v->begin(), v->end(), mk(0, 0));
    std::fill(o->d2uydx2.begin(), o->d2uydx2.end(), mk(0, 0));
    for (auto* v : {&o->th, &o->th1, &o->dv1t, &o->dv2t}) std::fill(v->begin(), v->end(), mk(0, 0));
    if (o->cfg.my_form == 1 || o->cfg.my_form == 2) return 0;   // init_gv / init_gvth: every mode a disturbance, all zero
    for (int j = 1; j <= o->ny; j++)
        for (int i = 1; i <= o->nx; i++) {
            o->ux[o->id(i, j, 1)] = mk(o->uxb[o->id2(i, j)], 0.0);
            o->uy[o->id(i, j, 1)] = mk(o->uyb[o->id2(i, j)], 0.0);
            o->wz[o->id(i, j, 1)] = mk(o->wzb[o->id2(i, j)], 0.0);
        }
    return 0;
}
static void cp_in(std::vector<C>& d, const double* s) { std::memcpy(d.data(), s, d.size() * sizeof(C)); }
static void cp_out(double* d, const std::vector<C>& s) { std::memcpy(d, s.data(), s.size() * sizeof(C)); }
int ora_put_state(ora_ctx* o, const double* ux, const double* uy, const double* uz, const double* wx, const double* wy,
                  const double* wz) {
    cp_in(o->ux, ux); cp_in(o->uy, uy); cp_in(o->uz, uz); cp_in(o->wx, wx); cp_in(o->wy, wy); cp_in(o->wz, wz);
    return 0;
}
int ora_get_state(ora_ctx* o, double* ux, double* uy, double* uz, double* wx, double* wy, double* wz) {
    cp_out(ux, o->ux); cp_out(uy, o->uy); cp_out(uz, o->uz); cp_out(wx, o->wx); cp_out(wy, o->wy); cp_out(wz, o->wz);
    return 0;
}
int ora_put_wall(ora_ctx* o, const double* d) { cp_in(o->d2uydx2, d); return 0; }
int ora_set_baseflow_th(ora_ctx* o, const double* thb) { std::memcpy(o->thb.data(), thb, o->thb.size() * sizeof(double)); return 0; }
int ora_put_th(ora_ctx* o, const double* th) { cp_in(o->th, th); return 0; }
int ora_get_th(ora_ctx* o, double* th) { cp_out(th, o->th); return 0; }
int ora_get_wall(ora_ctx* o, double* d) { cp_out(d, o->d2uydx2); return 0; }

#define AS_C(p) reinterpret_cast<C*>(p)
#define AS_CC(p) reinterpret_cast<const C*>(p)
int ora_derparx(ora_ctx* o, double* d, const double* f) { derparx_impl(o, AS_C(d), AS_CC(f)); return 0; }
int ora_derparxx(ora_ctx* o, double* d, const double* f) { derparxx_impl(o, AS_C(d), AS_CC(f)); return 0; }
int ora_dery(ora_ctx* o, double* d, const double* f) { dery_impl(o, AS_C(d), AS_CC(f), 0); return 0; }
int ora_deryfv(ora_ctx* o, double* d, const double* f) { dery_impl(o, AS_C(d), AS_CC(f), 1); return 0; }
int ora_deryy(ora_ctx* o, double* d, const double* f) { dery_impl(o, AS_C(d), AS_CC(f), 2); return 0; }
int ora_f_to_p(ora_ctx* o, double* phys, const double* four) { f_to_p_impl(o, phys, AS_CC(four)); return 0; }
int ora_p_to_f(ora_ctx* o, double* four, const double* phys) {
    std::vector<double> tmp(phys, phys + (size_t)o->nx * o->ny * o->P);
    p_to_f_impl(o, AS_C(four), tmp.data());
    return 0;
}
int ora_nlterms(ora_ctx* o, double* a, double* b, double* c) { nlterms_impl(o, AS_C(a), AS_C(b), AS_C(c)); return 0; }
int ora_drv(ora_ctx* o, double* x, double* y, double* z) { drv_impl(o, AS_C(x), AS_C(y), AS_C(z)); return 0; }
int ora_filter_trid(ora_ctx* o) { filter_trid_impl(o); return 0; }
int ora_bzone(ora_ctx* o) { bzone_impl(o); return 0; }
int ora_bzonew(ora_ctx* o) { bzonew_impl(o); return 0; }
int ora_outuy(ora_ctx* o, double* d) { outuy_impl(o, AS_C(d)); return 0; }
int ora_poi_uy(ora_ctx* o, const double* d, double erro) { poi_uy_impl(o, AS_CC(d), erro); return 0; }
int ora_poi_ux(ora_ctx* o, double* d) { poi_ux_impl(o, AS_C(d)); return 0; }
int ora_poi_uz(ora_ctx* o, const double* d) { poi_uz_impl(o, AS_CC(d)); return 0; }
int ora_wx_wall(ora_ctx* o, double* l) { wx_wall_impl(o, AS_C(l)); return 0; }
int ora_wz_wall(ora_ctx* o, const double* l) { wz_wall_impl(o, AS_CC(l)); return 0; }
int ora_ts_pert(ora_ctx* o, int t, double tempt) {
    if (o->cfg.my_form == 1) gv_pert_impl(o, t);
    else ts_pert_impl(o, t, tempt);
    return 0;
}
int ora_les_terms(ora_ctx* o, double* x, double* y, double* z) { les_terms_impl(o, AS_C(x), AS_C(y), AS_C(z)); return 0; }
int ora_cvirt(ora_ctx* o, double* x, double* y, double* z) { cvirt_impl(o, AS_C(x), AS_C(y), AS_C(z)); return 0; }
int ora_loop(ora_ctx* o, double erro) { loop_impl(o, erro, erro < 1.0e-5); return 0; }

// One RK4 stage of solver case 0 / case 4 (main_par.f:165-247, 461-536).
int ora_rk_stage(ora_ctx* o, int stage, int t) {
    int i_ini = 3;
    const tb_config& c = o->cfg;
    std::vector<C>& d1x = o->dv1x; std::vector<C>& d1y = o->dv1y; std::vector<C>& d1z = o->dv1z;
    std::vector<C>& d2x = o->dv2x; std::vector<C>& d2y = o->dv2y; std::vector<C>& d2z = o->dv2z;
    if (stage == 1) drv_impl(o, d1x.data(), d1y.data(), d1z.data());
    else drv_impl(o, d2x.data(), d2y.data(), d2z.data());
    for (int k = 1; k <= o->K; k++)
        for (int j = 2; j <= o->ny - 1; j++)
            for (int i = i_ini; i <= o->nx; i++) {
                size_t q = o->id(i, j, k);
                if (stage == 1) {
                    o->wx1[q] = o->wx[q]; o->wy1[q] = o->wy[q]; o->wz1[q] = o->wz[q];
                    o->wx[q] = o->wx1[q] + d1x[q] * o->dt2;
                    o->wy[q] = o->wy1[q] + d1y[q] * o->dt2;
                    o->wz[q] = o->wz1[q] + d1z[q] * o->dt2;
                } else if (stage == 2 || stage == 3) {
                    double h = (stage == 2) ? o->dt2 : o->dt;
                    o->wx[q] = o->wx1[q] + d2x[q] * h;
                    o->wy[q] = o->wy1[q] + d2y[q] * h;
                    o->wz[q] = o->wz1[q] + d2z[q] * h;
                    d1x[q] = d1x[q] + 2.0 * d2x[q];
                    d1y[q] = d1y[q] + 2.0 * d2y[q];
                    d1z[q] = d1z[q] + 2.0 * d2z[q];
                } else {
                    o->wx[q] = o->wx1[q] + o->dt6 * (d1x[q] + d2x[q]);
                    o->wy[q] = o->wy1[q] + o->dt6 * (d1y[q] + d2y[q]);
                    o->wz[q] = o->wz1[q] + o->dt6 * (d1z[q] + d2z[q]);
                }
                if (c.my_form == 2) {   // main_par.f:366-440
                    if (stage == 1) { o->th1[q] = o->th[q]; o->th[q] = o->th1[q] + o->dv1t[q] * o->dt2; }
                    else if (stage == 2 || stage == 3) {
                        double h = (stage == 2) ? o->dt2 : o->dt;
                        o->th[q] = o->th1[q] + o->dv2t[q] * h;
                        o->dv1t[q] = o->dv1t[q] + 2.0 * o->dv2t[q];
                    } else {
                        o->th[q] = o->th1[q] + o->dt6 * (o->dv1t[q] + o->dv2t[q]);
                    }
                }
            }
    if (stage == 1 || stage == 3) {
        if (c.my_form == 1) gv_pert_impl(o, t);
        else ts_pert_impl(o, t, stage == 1 ? 0.5 : 1.0);
    }
    if (stage < 4) loop_impl(o, c.tol_stage, false);
    else loop_impl(o, c.tol_final, true);
    return 0;
}
int ora_step(ora_ctx* o, int t) {
    for (int s = 1; s <= 4; s++) ora_rk_stage(o, s, t);
    return 0;
}
int ora_poisson_stats(ora_ctx* o, int* v, double* r) {
    for (int k = 0; k < (int)o->pv.size(); k++) { v[k] = o->pv[k]; r[k] = o->pres[k]; }
    return (int)o->pv.size();
}

// Host threads for the parallel loops (independent lines and modes).
int ora_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

}  // extern "C"

// Diagnostic: smoothing-only convergence at the finest level for mode k
// (function_source, nsweeps sor sweeps, defect); returns max|defect|.
extern "C" double ora_debug_sor(ora_ctx* o, const double* dwzdx, int k, int nsweeps, int mesh) {
    Poi p(o);
    p.function_source(reinterpret_cast<const C*>(dwzdx), k);
    if (mesh > 1) {
        // restrict the fine problem down to 'mesh' without smoothing
        for (int l = 1; l < mesh; l++) { p.defect(-1.0, k, l); p.restrict_(l); p.defect(1.0, k, l + 1); }
    }
    p.sor(k, nsweeps, mesh);
    p.defect(-1.0, k, mesh);
    double e = 0.0;
    for (int j = 2; j <= o->v_ptsy[mesh - 1]; j++)
        for (int i = 2; i <= o->v_ptsx[mesh - 1] - 1; i++) e = std::max(e, cabs_(p.FT(i, j, 1)));
    return e;
}
