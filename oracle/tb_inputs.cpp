// tb_inputs.cpp -- CPU restatement of the reference's pre-processing: the
// stretched-grid compact-scheme tables (pre_processing/derivative.f90,
// coef_generation.f90) and the Falkner-Skan / Blasius base flow
// (pre_processing/fs_sch.f90, main_fs.f90).
//
// TEST INFRASTRUCTURE ONLY: it lets the CPU baseline of the benchmark (and the
// tests that cross-check the library's own generator) build a workload's
// inputs without the GPU library.  Pinned by the reference's golden
// pre_processing/coefs.bin (records 2-20, stretching 1.01, 4 levels) and
// lst_ts/fpp.dat (Blasius f''(0)).
//
// Each table of derivative.f90 is the solution of a Taylor-matching system:
// the weights alpha_l of derivative values f^(d)(e_l) (left-hand side) and
// a_m of function values f(h_m) (right-hand side) with
//     sum_l alpha_l e_l^(q-d)/(q-d)!  -  sum_m a_m h_m^q/q!  =  0
// for the listed orders q, plus rows that fix single weights.  Offsets are in
// units of the stencil's first spacing, spacings growing by the stretching
// factor from cell to cell.  derivative.f90 assembles the same systems row by
// row and solves them with an unpivoted Doolittle LU (solvers.f90:68-128), in
// real*8 for the derivative tables and real*10 for the Poisson and wall
// tables, zeroing solution entries below 1e-14 (solvers.f90:122).  Here the
// solve is Gaussian elimination with partial pivoting in long double, with the
// same zeroing rule.
#include "tb_oracle.h"
#include <cmath>
#include <cstring>
#include <vector>

namespace {

typedef long double LD;

struct Term {
    int lhs;   // 1: derivative weight on the left-hand side, 0: function weight on the right
    int d;     // derivative order of the term
    LD at;     // offset from the stencil point
};

LD ipow(LD x, int n) { LD r = 1; while (n-- > 0) r *= x; return r; }
// real*8 ** integer as libgcc's __powidf2 (binary exponentiation).
double powi(double x, int m) {
    unsigned n = m < 0 ? -m : m;
    double y = (n % 2) ? x : 1.0;
    while (n >>= 1) { x = x * x; if (n % 2) y = y * x; }
    return m < 0 ? 1.0 / y : y;
}
LD fac(int n) { LD r = 1; for (int i = 2; i <= n; i++) r *= i; return r; }

// Solve A x = b (n x n, row-major) with partial pivoting; zero |x_i| < 1e-14
// for every unknown but the last, as the reference's back substitution does.
bool gauss(std::vector<LD> A, std::vector<LD> b, int n, double* out) {
    for (int c = 0; c < n; c++) {
        int p = c;
        for (int r = c + 1; r < n; r++)
            if (fabsl(A[(size_t)r * n + c]) > fabsl(A[(size_t)p * n + c])) p = r;
        if (A[(size_t)p * n + c] == 0) return false;
        for (int k = 0; k < n && p != c; k++) std::swap(A[(size_t)c * n + k], A[(size_t)p * n + k]);
        std::swap(b[c], b[p]);
        for (int r = c + 1; r < n; r++) {
            LD f = A[(size_t)r * n + c] / A[(size_t)c * n + c];
            for (int k = c; k < n; k++) A[(size_t)r * n + k] -= f * A[(size_t)c * n + k];
            b[r] -= f * b[c];
        }
    }
    std::vector<LD> x(n);
    for (int r = n - 1; r >= 0; r--) {
        LD s = b[r];
        for (int k = r + 1; k < n; k++) s -= A[(size_t)r * n + k] * x[k];
        x[r] = s / A[(size_t)r * n + r];
        if (r < n - 1 && fabsl(x[r]) < 1e-14L) x[r] = 0;
    }
    for (int i = 0; i < n; i++) out[i] = (double)x[i];
    return true;
}

// One scheme: terms (the unknowns, in the reference's column order), fixed
// weights (column, value), moment orders; 'bump' adds a constant to one
// matrix entry (moment order, column) as the reference's wall row does.
struct Scheme {
    std::vector<Term> t;
    std::vector<std::pair<int, LD>> fixed;
    int q_lo, q_hi;
    int bump_q = -1, bump_col = -1;
    LD bump = 0;
};

bool solve_scheme(const Scheme& s, double* out) {
    int n = (int)s.t.size();
    if ((int)s.fixed.size() + (s.q_hi - s.q_lo + 1) != n) return false;
    std::vector<LD> A((size_t)n * n, 0), b(n, 0);
    int r = 0;
    for (auto& f : s.fixed) { A[(size_t)r * n + f.first] = 1; b[r] = f.second; r++; }
    for (int q = s.q_lo; q <= s.q_hi; q++, r++)
        for (int c = 0; c < n; c++) {
            const Term& u = s.t[c];
            LD v = 0;
            if (q >= u.d) v = ipow(u.at, q - u.d) / fac(q - u.d);
            A[(size_t)r * n + c] = u.lhs ? v : -v;
            if (q == s.bump_q && c == s.bump_col) A[(size_t)r * n + c] += s.bump;
        }
    return gauss(A, b, n, out);
}

Term D(int d, LD at) { return Term{1, d, at}; }
Term F(LD at) { return Term{0, 0, at}; }

// Offsets of the points above the wall point: h_k = sum_{i<=k} s^(p0+i).
std::vector<LD> up(LD s, int p0, int n) {
    std::vector<LD> h(n);
    LD acc = 0;
    for (int k = 0; k < n; k++) { acc += ipow(s, p0 + k); h[k] = acc; }
    return h;
}
// Offsets below the top point: spacings s^p0, s^(p0-1), ...
std::vector<LD> down(LD s, int p0, int n) {
    std::vector<LD> h(n);
    LD acc = 0;
    for (int k = 0; k < n; k++) { acc += ipow(s, p0 - k); h[k] = -acc; }
    return h;
}

bool first_derivative(LD s, double* fp7, double* fpe6, double* sp9, double* cp8, double* pp9, double* lp7) {
    bool ok = true;
    std::vector<LD> h = up(s, 0, 4), g = up(s, 1, 4), m = down(s, 3, 4);
    // first point, compact (derivative.f90:15-104)
    ok &= solve_scheme({{D(1, 0), D(1, h[0]), F(0), F(h[0]), F(h[1]), F(h[2]), F(h[3])}, {{0, 1}}, 0, 5}, fp7);
    // first point, explicit, scaled to 12 f'(0)
    ok &= solve_scheme({{D(1, 0), F(0), F(h[0]), F(h[1]), F(h[2]), F(h[3])}, {{0, 12}}, 0, 4}, fpe6);
    // second point: alpha_{-1} = 1, a_0 = -2.5
    ok &= solve_scheme({{D(1, -1), D(1, 0), D(1, g[0]), F(-1), F(0), F(g[0]), F(g[1]), F(g[2]), F(g[3])},
                        {{0, 1}, {4, -2.5L}}, 0, 6}, sp9);
    // centre: spacings 1, s | s^2, s^3 around the point
    LD a1 = s, a2 = 1 + s, b1 = s * s, b2 = s * s + s * s * s;
    ok &= solve_scheme({{D(1, -a1), D(1, 0), D(1, b1), F(-a2), F(-a1), F(0), F(b1), F(b2)}, {{1, 1}}, 0, 6}, cp8);
    // penultimate: mirror of the second point with the top spacings
    LD t1 = ipow(s, 4);
    ok &= solve_scheme({{D(1, t1), D(1, 0), D(1, m[0]), F(t1), F(0), F(m[0]), F(m[1]), F(m[2]), F(m[3])},
                        {{0, 1}, {4, 2.5L}}, 0, 6}, pp9);
    // last point
    ok &= solve_scheme({{D(1, 0), D(1, m[0]), F(0), F(m[0]), F(m[1]), F(m[2]), F(m[3])}, {{0, 1}}, 0, 5}, lp7);
    return ok;
}

bool second_derivative(LD s, double* fp8, double* sp10, double* cp8, double* pp10, double* lp8) {
    bool ok = true;
    std::vector<LD> h = up(s, 0, 5), g = up(s, 1, 5), m = down(s, 4, 5);
    ok &= solve_scheme({{D(2, 0), D(2, h[0]), F(0), F(h[0]), F(h[1]), F(h[2]), F(h[3]), F(h[4])}, {{0, 1}}, 0, 6}, fp8);
    ok &= solve_scheme({{D(2, -1), D(2, 0), D(2, g[0]), F(-1), F(0), F(g[0]), F(g[1]), F(g[2]), F(g[3]), F(g[4])},
                        {{0, 1}, {5, 5.25L}}, 0, 7}, sp10);
    LD a1 = s, a2 = 1 + s, b1 = s * s, b2 = s * s + s * s * s;
    ok &= solve_scheme({{D(2, -a1), D(2, 0), D(2, b1), F(-a2), F(-a1), F(0), F(b1), F(b2)}, {{1, 1}}, 0, 6}, cp8);
    LD t1 = ipow(s, 5);
    ok &= solve_scheme({{D(2, t1), D(2, 0), D(2, m[0]), F(t1), F(0), F(m[0]), F(m[1]), F(m[2]), F(m[3]), F(m[4])},
                        {{0, 1}, {5, 5.25L}}, 0, 7}, pp10);
    ok &= solve_scheme({{D(2, 0), D(2, m[0]), F(0), F(m[0]), F(m[1]), F(m[2]), F(m[3]), F(m[4])}, {{0, 1}}, 0, 6}, lp8);
    return ok;
}

// Compact Poisson weights of one multigrid level with stretching t
// (poisson_coefficient_generation, derivative.f90:1850-1882).
bool poisson(LD t, double* sp7, double* cp8, double* pp4, double* lp5) {
    bool ok = true;
    ok &= solve_scheme({{D(1, -1), D(2, 0), D(2, t), F(-1), F(0), F(t), F(t + t * t)}, {{1, 0.8L}}, 0, 5}, sp7);
    LD a1 = t, a2 = 1 + t, b1 = t * t, b2 = t * t + t * t * t;
    ok &= solve_scheme({{D(2, -a1), D(2, 0), D(2, b1), F(-a2), F(-a1), F(0), F(b1), F(b2)},
                        {{1, 11.0L / 15.0L}}, 0, 6}, cp8);
    ok &= solve_scheme({{D(2, 0), F(-1), F(0), F(t)}, {{0, 1}}, 0, 2}, pp4);
    ok &= solve_scheme({{D(2, 0), Term{0, 1, 0}, F(0), F(-t), F(-(t + 1))}, {{0, 1}}, 0, 3}, lp5);
    return ok;
}

// Wall curvature of v from the wall slope and seven values, with the extra -1
// on the wall value in the slope row (vorticity_at_wall_matrix_coef), and the
// 7-point one-sided wall slope (dwydy_matrix_coef).
bool wall(LD s, double* w9, double* d8) {
    std::vector<LD> h = up(s, 0, 6);
    Scheme w{{D(2, 0), D(1, 0), F(0), F(h[0]), F(h[1]), F(h[2]), F(h[3]), F(h[4]), F(h[5])}, {{8, -1.0L / 18.0L}}, 0, 7};
    w.bump_q = 1; w.bump_col = 2; w.bump = -1;
    bool ok = solve_scheme(w, w9);
    ok &= solve_scheme({{D(1, 0), F(0), F(h[0]), F(h[1]), F(h[2]), F(h[3]), F(h[4]), F(h[5])}, {{0, 1}}, 0, 6}, d8);
    return ok;
}

// ---------------------------------------------------------------------------
// Falkner-Skan similarity solution (fs_sch.f90).
typedef void (*Rhs)(const double* f, double* d, double beta, double pr);

void derivs(const double* f, double* d, double beta, double) {  // fs_sch.f90 derivs
    d[0] = f[1];
    d[1] = f[2];
    d[2] = -f[0] * f[2] - beta * (1.0 - f[1] * f[1]);
    d[3] = f[4];
    d[4] = f[5];
    d[5] = -f[3] * f[2] - f[0] * f[5] + 2.0 * beta * f[1] * f[4];
}
void derivs_theta(const double* f, double* d, double beta, double pr) {  // fs_sch.f90:432-446
    d[0] = f[1];
    d[1] = f[2];
    d[2] = -f[0] * f[2] - (beta * (1.0 - f[1] * f[1]));
    d[3] = f[4];
    d[4] = -f[0] * f[4] * pr;
    d[5] = 0.0;
}
void rk4(double* f, double h, Rhs der, double beta, double pr) {  // fs_sch.f90 rk4 / rk4_theta
    double hh = h * 0.5, h6 = h / 6.0, d1[6], d2[6], ft[6];
    der(f, d1, beta, pr);
    for (int q = 0; q < 6; q++) ft[q] = f[q] + hh * d1[q];
    der(ft, d2, beta, pr);
    for (int q = 0; q < 6; q++) { ft[q] = f[q] + hh * d2[q]; d1[q] = d1[q] + 2.0 * d2[q]; }
    der(ft, d2, beta, pr);
    for (int q = 0; q < 6; q++) { ft[q] = f[q] + h * d2[q]; d1[q] = d1[q] + 2.0 * d2[q]; }
    der(ft, d2, beta, pr);
    for (int q = 0; q < 6; q++) f[q] = f[q] + h6 * (d1[q] + d2[q]);
}

}  // namespace

extern "C" {

int ora_generate_coefs(double stf, int msh, double* blob) {
    if (!blob || msh < 1 || msh > 6 || !(stf > 0)) return TB_ERR_ARG;
    LD s = stf;
    double fp7[7];
    double *fpe = blob, *sp = fpe + 6, *cp = sp + 9, *pp = cp + 8, *lp = pp + 9;
    double *fsd = lp + 7, *ssd = fsd + 8, *csd = ssd + 10, *psd = csd + 8, *lsd = psd + 10;
    double *spoi = lsd + 8, *cpoi = spoi + 7 * msh, *ppoi = cpoi + 8 * msh, *lpoi = ppoi + 4 * msh;
    double *w9 = lpoi + 5 * msh, *d8 = w9 + 9;
    bool ok = first_derivative(s, fp7, fpe, sp, cp, pp, lp) && second_derivative(s, fsd, ssd, csd, psd, lsd);
    for (int l = 1; l <= msh && ok; l++) {
        double t = powi(stf, 1 << (l - 1));  // stf**2**(l-1) in real*8 (coef_generation.f90:33)
        ok = poisson((LD)t, spoi + 7 * (l - 1), cpoi + 8 * (l - 1), ppoi + 4 * (l - 1), lpoi + 5 * (l - 1));
    }
    ok = ok && wall(s, w9, d8);
    return ok ? TB_OK : TB_ERR_ARG;
}

int ora_generate_fp_fd(double stf, double* out7) {
    double fpe[6], sp[9], cp[8], pp[9], lp[7];
    return first_derivative(stf, out7, fpe, sp, cp, pp, lp) ? TB_OK : TB_ERR_ARG;
}

// fpp_finder (fs_sch.f90:10-52): Newton on f''(0) with the integration end
// eta_adp pushed out by eta_variation until (1 - f')^2 + f''^2 <= gtol_fs.
int ora_fs_wall_shear(double beta, double* fpp_out) {
    if (!fpp_out) return TB_ERR_ARG;
    const double tol_fs = 1.0e-13, gtol_fs = 1.0e-23, eta_variation = 0.01, deta = 1.0e-4;  // constants.f90:24-29
    double fpp = 1.1, eta_adp = 0.5, ls_err = 1.0, f[6];
    int cont = 1;
    while (std::fabs(ls_err) > gtol_fs && cont < 10000) {
        double delta = 100.0;
        int steps = (int)(eta_adp / deta + 1.0);
        int it = 0;
        while (std::fabs(delta / fpp) > tol_fs) {
            f[0] = 0.0; f[1] = 0.0; f[2] = fpp; f[3] = 0.0; f[4] = 0.0; f[5] = 1.0;
            for (int j = 2; j <= steps; j++) rk4(f, deta, derivs, beta, 0.0);
            delta = (-f[4] * f[1] - (f[5] * f[2]) + f[4]) / (f[4] * f[4] + f[5] * f[5]);
            fpp = fpp + delta;
            if (++it > 200) return TB_ERR_NOCONV;
        }
        ls_err = (1.0 - f[1]) * (1.0 - f[1]) + f[2] * f[2];
        eta_adp = eta_adp + eta_variation;
        cont++;
    }
    *fpp_out = fpp;
    return TB_OK;
}

// baseflow_fs (fs_sch.f90:58-162) with one f''(0) for every station (the
// reference's beta_fs.dist is uniform), thp = 0; outputs (ny, nx) row-major,
// i fastest, as the Fortran arrays ux(imax, jmax).
int ora_baseflow_fs(const tb_config* cf, double beta, double* uxb, double* uyb, double* wzb) {
    if (!cf || !uxb || !uyb || !wzb) return TB_ERR_ARG;
    double fpp;
    int r = ora_fs_wall_shear(beta, &fpp);
    if (r) return r;
    const double Pr = 0.72;
    const int nx = cf->nx, ny = cf->ny;
    const double Re = cf->Re, dy0 = cf->dy, stf = cf->stf, fac_y = cf->fac_y;
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 1; i <= nx; i++) {
        double m = beta / (2.0 - beta);
        double xad = cf->x0 + (double)(i - 1) * cf->dx;
        double ue = std::pow(xad, m);
        double deta0 = (dy0 / std::sqrt(fac_y)) * std::sqrt(0.5 * Re * ue * (m + 1.0) / xad);
        double f[6] = {0.0, 0.0, fpp, 0.0, 0.0, 0.0};
        size_t c0 = (size_t)(i - 1);
        uxb[c0] = 0.0;
        uyb[c0] = 0.0;
        wzb[c0] = ue * deta0 * f[2] / (dy0 / std::sqrt(fac_y));
        wzb[c0] = wzb[c0] / std::sqrt(fac_y);
        for (int j = 2; j <= ny; j++) {
            double h = deta0 * powi(stf, j - 2);
            int pt = (int)(h / 1.0e-4);
            if (pt < 1) pt = 1;
            h = h / (double)pt;
            for (int k = 1; k <= pt; k++) rk4(f, h, derivs_theta, beta, Pr);
            double eta = (stf != 1.0) ? deta0 * (powi(stf, j - 1) - 1.0) / (stf - 1.0) : deta0 * (double)(j - 1);
            double yad = eta / std::sqrt(0.5 * Re * ue * (m + 1.0) / xad);
            size_t q = c0 + (size_t)nx * (j - 1);
            uxb[q] = ue * f[1];
            uyb[q] = -std::sqrt(0.5 * ue * (m + 1.0) / (xad * Re)) * f[0] - 0.5 * (m - 1.0) * yad * ue * f[1] / xad;
            uyb[q] = uyb[q] * std::sqrt(fac_y);
            wzb[q] = ue * std::sqrt(0.5 * (m + 1.0) * Re * ue / xad) * f[2];
            wzb[q] = wzb[q] / std::sqrt(fac_y);
        }
    }
    return TB_OK;
}

}  // extern "C"
