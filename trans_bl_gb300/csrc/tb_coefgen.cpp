// tb_coefgen.cpp -- stretched-grid compact-scheme coefficients
// (pre_processing/derivative.f90:15-2081, driver 1762-1882).
//
// Every table of the reference is the solution of a small Taylor-matching
// system: unknown weights on derivative values (left-hand side, derivative
// order d at offset e) and on function values (right-hand side, offset h)
// such that  sum_l alpha_l f^(d)(e_l) - sum_m a_m f(h_m)  vanishes for the
// polynomial orders q listed, plus normalisation rows that fix one weight.
// Offsets are in units of the first spacing of the stencil, the spacing
// growing by the stretching factor from cell to cell.  The systems are the
// reference's; here they are assembled from that description and solved by
// Gaussian elimination with partial pivoting in long double (the reference
// uses an unpivoted Doolittle LU in real*8 or real*10).
#include "tb_internal.h"
#include <cmath>
#include <cstring>
#include <vector>

namespace {

typedef long double LD;

struct Unknown {
    int side;   // +1: left-hand derivative weight, -1: right-hand weight
    int d;      // derivative order the weight multiplies
    LD e;       // signed offset
};
struct Fix { int col; LD val; };

LD fact(int n) { LD f = 1; for (int i = 2; i <= n; i++) f *= i; return f; }
LD pw(LD x, int n) { LD r = 1; for (int i = 0; i < n; i++) r *= x; return r; }

// Entry of unknown u in the order-q moment row.
LD moment(const Unknown& u, int q) {
    if (q < u.d) return 0;
    return (LD)u.side * pw(u.e, q - u.d) / fact(q - u.d);
}

bool solve(std::vector<LD>& A, std::vector<LD>& b, int n) {
    for (int c = 0; c < n; c++) {
        int p = c;
        for (int r = c + 1; r < n; r++)
            if (fabsl(A[r * n + c]) > fabsl(A[p * n + c])) p = r;
        if (A[p * n + c] == 0) return false;
        if (p != c) {
            for (int k = 0; k < n; k++) std::swap(A[c * n + k], A[p * n + k]);
            std::swap(b[c], b[p]);
        }
        for (int r = c + 1; r < n; r++) {
            LD f = A[r * n + c] / A[c * n + c];
            if (f == 0) continue;
            for (int k = c; k < n; k++) A[r * n + k] -= f * A[c * n + k];
            b[r] -= f * b[c];
        }
    }
    for (int r = n - 1; r >= 0; r--) {
        LD s = b[r];
        for (int k = r + 1; k < n; k++) s -= A[r * n + k] * b[k];
        b[r] = s / A[r * n + r];
    }
    return true;
}

// Build and solve: rows = fixes + one row per listed moment order.
// 'extra' adds (row-moment q, column, value) entries on top of the moments.
struct Extra { int q, col; LD val; };
bool scheme(const std::vector<Unknown>& U, const std::vector<Fix>& F, const std::vector<int>& Q, double* out,
            const std::vector<Extra>& X = {}) {
    int n = (int)U.size();
    if ((int)(F.size() + Q.size()) != n) return false;
    std::vector<LD> A((size_t)n * n, 0), b(n, 0);
    int r = 0;
    for (const Fix& f : F) { A[r * n + f.col] = 1; b[r] = f.val; r++; }
    for (int q : Q) {
        for (int c = 0; c < n; c++) A[r * n + c] = moment(U[c], q);
        for (const Extra& x : X) if (x.q == q) A[r * n + x.col] += x.val;
        r++;
    }
    if (!solve(A, b, n)) return false;
    for (int c = 0; c < n; c++) out[c] = (double)b[c];
    return true;
}

std::vector<int> orders(int lo, int hi) { std::vector<int> v; for (int q = lo; q <= hi; q++) v.push_back(q); return v; }

// Cumulative offsets of a geometric stencil: first spacing s^p0, growing by s.
// up[k] = sum_{i<k+1} s^(p0+i) for k = 0..n-1.
std::vector<LD> cum(LD s, int p0, int n) {
    std::vector<LD> v(n);
    LD acc = 0;
    for (int k = 0; k < n; k++) { acc += pw(s, p0 + k); v[k] = acc; }
    return v;
}
std::vector<LD> cumdown(LD s, int p0, int n) {  // s^p0 + s^(p0-1) + ... (toward the wall side)
    std::vector<LD> v(n);
    LD acc = 0;
    for (int k = 0; k < n; k++) { acc += pw(s, p0 - k); v[k] = acc; }
    return v;
}

Unknown L(int d, LD e) { return Unknown{+1, d, e}; }
Unknown R(LD h) { return Unknown{-1, 0, h}; }

}  // namespace

// First-derivative schemes (derivative.f90:15-612, 2002-2081).
static bool first_derivative(LD s, double* fp7, double* fpe6, double* sp9, double* cp8, double* pp9, double* lp7) {
    bool ok = true;
    {   // first point, compact: f'(0) + alpha f'(1) = sum a f(h), h = 0, 1, 1+s, ...
        std::vector<LD> h = cum(s, 0, 4);
        std::vector<Unknown> U = {L(1, 0), L(1, h[0]), R(0), R(h[0]), R(h[1]), R(h[2]), R(h[3])};
        ok &= scheme(U, {{0, 1}}, orders(0, 5), fp7);
    }
    {   // first point, explicit, normalised to 12 f'(0)
        std::vector<LD> h = cum(s, 0, 4);
        std::vector<Unknown> U = {L(1, 0), R(0), R(h[0]), R(h[1]), R(h[2]), R(h[3])};
        ok &= scheme(U, {{0, 12}}, orders(0, 4), fpe6);
    }
    {   // second point: alpha_{-1}=1, a(0) = -2.5
        std::vector<LD> h = cum(s, 1, 4);
        std::vector<Unknown> U = {L(1, -1), L(1, 0), L(1, h[0]), R(-1), R(0), R(h[0]), R(h[1]), R(h[2]), R(h[3])};
        ok &= scheme(U, {{0, 1}, {4, -2.5}}, orders(0, 6), sp9);
    }
    {   // centre: stencil j-2..j+2 with spacings 1, s | s^2, s^3
        LD hm1 = s, hm2 = 1 + s, hp1 = s * s, hp2 = hp1 + s * s * s;
        std::vector<Unknown> U = {L(1, -hm1), L(1, 0), L(1, hp1), R(-hm2), R(-hm1), R(0), R(hp1), R(hp2)};
        ok &= scheme(U, {{1, 1}}, orders(0, 6), cp8);
    }
    {   // penultimate: mirror of the second point with the top spacings
        LD hp1 = pw(s, 4);
        std::vector<LD> hm = cumdown(s, 3, 4);
        std::vector<Unknown> U = {L(1, hp1), L(1, 0), L(1, -hm[0]), R(hp1), R(0), R(-hm[0]), R(-hm[1]), R(-hm[2]), R(-hm[3])};
        ok &= scheme(U, {{0, 1}, {4, 2.5}}, orders(0, 6), pp9);
    }
    {   // last point
        std::vector<LD> hm = cumdown(s, 3, 4);
        std::vector<Unknown> U = {L(1, 0), L(1, -hm[0]), R(0), R(-hm[0]), R(-hm[1]), R(-hm[2]), R(-hm[3])};
        ok &= scheme(U, {{0, 1}}, orders(0, 5), lp7);
    }
    return ok;
}

// Second-derivative schemes (derivative.f90:617-1267).
static bool second_derivative(LD s, double* fp8, double* sp10, double* cp8, double* pp10, double* lp8) {
    bool ok = true;
    {
        std::vector<LD> h = cum(s, 0, 5);
        std::vector<Unknown> U = {L(2, 0), L(2, h[0]), R(0), R(h[0]), R(h[1]), R(h[2]), R(h[3]), R(h[4])};
        ok &= scheme(U, {{0, 1}}, orders(0, 6), fp8);
    }
    {   // second point: alpha_{-1} = 1, a(+1st) = 5.25
        std::vector<LD> h = cum(s, 1, 5);
        std::vector<Unknown> U = {L(2, -1), L(2, 0), L(2, h[0]), R(-1), R(0), R(h[0]), R(h[1]), R(h[2]), R(h[3]), R(h[4])};
        ok &= scheme(U, {{0, 1}, {5, 5.25}}, orders(0, 7), sp10);
    }
    {
        LD hm1 = s, hm2 = 1 + s, hp1 = s * s, hp2 = hp1 + s * s * s;
        std::vector<Unknown> U = {L(2, -hm1), L(2, 0), L(2, hp1), R(-hm2), R(-hm1), R(0), R(hp1), R(hp2)};
        ok &= scheme(U, {{1, 1}}, orders(0, 6), cp8);
    }
    {
        LD hp1 = pw(s, 5);
        std::vector<LD> hm = cumdown(s, 4, 5);
        std::vector<Unknown> U = {L(2, hp1), L(2, 0), L(2, -hm[0]), R(hp1), R(0), R(-hm[0]), R(-hm[1]), R(-hm[2]), R(-hm[3]), R(-hm[4])};
        ok &= scheme(U, {{0, 1}, {5, 5.25}}, orders(0, 7), pp10);
    }
    {
        std::vector<LD> hm = cumdown(s, 4, 5);
        std::vector<Unknown> U = {L(2, 0), L(2, -hm[0]), R(0), R(-hm[0]), R(-hm[1]), R(-hm[2]), R(-hm[3]), R(-hm[4])};
        ok &= scheme(U, {{0, 1}}, orders(0, 6), lp8);
    }
    return ok;
}

// Compact Poisson weights at one multigrid level with stretching t
// (derivative.f90:1272-1613, poisson_coefficient_generation 1850-1882).
static bool poisson(LD t, double* sp7, double* cp8, double* pp4, double* lp5) {
    bool ok = true;
    {   // second point: wall slope weight, curvature weights at j and j+1 (alpha_j = 4/5)
        LD hp1 = t, hp2 = t + t * t;
        std::vector<Unknown> U = {L(1, -1), L(2, 0), L(2, hp1), R(-1), R(0), R(hp1), R(hp2)};
        ok &= scheme(U, {{1, (LD)4 / 5}}, orders(0, 5), sp7);
    }
    {
        LD hm1 = t, hm2 = 1 + t, hp1 = t * t, hp2 = hp1 + t * t * t;
        std::vector<Unknown> U = {L(2, -hm1), L(2, 0), L(2, hp1), R(-hm2), R(-hm1), R(0), R(hp1), R(hp2)};
        ok &= scheme(U, {{1, (LD)11 / 15}}, orders(0, 6), cp8);
    }
    {   // penultimate: explicit 3-point curvature
        std::vector<Unknown> U = {L(2, 0), R(-1), R(0), R(t)};
        ok &= scheme(U, {{0, 1}}, orders(0, 2), pp4);
    }
    {   // top point: curvature + slope (Robin condition) from three values
        std::vector<Unknown> U = {L(2, 0), Unknown{-1, 1, 0}, R(0), R(-t), R(-(t + 1))};
        ok &= scheme(U, {{0, 1}}, orders(0, 3), lp5);
    }
    return ok;
}

// Wall curvature of v from the wall slope and seven values (derivative.f90:1618-1757),
// and the 7-point one-sided wall slope (1887-1998).
static bool wall(LD s, double* w9, double* d8) {
    bool ok = true;
    {
        std::vector<LD> h = cum(s, 0, 6);
        std::vector<Unknown> U = {L(2, 0), L(1, 0), R(0), R(h[0]), R(h[1]), R(h[2]), R(h[3]), R(h[4]), R(h[5])};
        // the reference's slope (q = 1) row also carries -1 on the wall value
        ok &= scheme(U, {{8, (LD)-1 / 18}}, orders(0, 7), w9, {{1, 2, -1}});
    }
    {
        std::vector<LD> h = cum(s, 0, 6);
        std::vector<Unknown> U = {L(1, 0), R(0), R(h[0]), R(h[1]), R(h[2]), R(h[3]), R(h[4]), R(h[5])};
        ok &= scheme(U, {{0, 1}}, orders(0, 6), d8);
    }
    return ok;
}

extern "C" int tb_generate_coefs(double stf, int msh, double* blob) {
    if (!blob || msh < 1 || msh > TB_MAX_MSH || !(stf > 0)) { tb_set_error("tb_generate_coefs: bad argument"); return TB_ERR_ARG; }
    LD s = stf;
    double fp7[7];
    double* p = blob;
    double *fpe = p, *sp = p + 6, *cp = sp + 9, *pp = cp + 8, *lp = pp + 9;
    double *fsd = lp + 7, *ssd = fsd + 8, *csd = ssd + 10, *psd = csd + 8, *lsd = psd + 10;
    double* spoi = lsd + 8;
    double* cpoi = spoi + 7 * msh;
    double* ppoi = cpoi + 8 * msh;
    double* lpoi = ppoi + 4 * msh;
    double* w9 = lpoi + 5 * msh;
    double* d8 = w9 + 9;
    bool ok = first_derivative(s, fp7, fpe, sp, cp, pp, lp);
    ok = ok && second_derivative(s, fsd, ssd, csd, psd, lsd);
    for (int l = 1; l <= msh && ok; l++) {
        LD t = pw(s, 1 << (l - 1));  // stf**2**(l-1) (coef_generation.f90:33)
        ok = poisson(t, spoi + 7 * (l - 1), cpoi + 8 * (l - 1), ppoi + 4 * (l - 1), lpoi + 5 * (l - 1));
    }
    ok = ok && wall(s, w9, d8);
    if (!ok) { tb_set_error("tb_generate_coefs: singular system"); return TB_ERR_ARG; }
    return TB_OK;
}

// The compact first-point first-derivative weights fp_fd_coef(7); the
// reference file pre_processing/coefs.bin stores these as its first record.
extern "C" int tb_generate_fp_fd(double stf, double* out7) {
    if (!out7) return TB_ERR_ARG;
    double fpe[6], sp[9], cp[8], pp[9], lp[7];
    if (!first_derivative(stf, out7, fpe, sp, cp, pp, lp)) { tb_set_error("singular system"); return TB_ERR_ARG; }
    return TB_OK;
}
