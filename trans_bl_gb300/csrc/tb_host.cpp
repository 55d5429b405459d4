// tb_host.cpp -- host-side set-up of the trans_bl stage: configuration,
// constant tables and the once-per-run factorizations that the reference
// recomputes inside every call (derivs_k, create_ctes, lhs5+ludecomp,
// coef_center/coef_border+band5_poi, var_ts, buffer ramps, gibbs_function).
#include "tb_internal.h"
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>

static thread_local char g_err[512] = "";

void tb_set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

extern "C" const char* tb_last_error(void) { return g_err; }

double tb_powi(double x, int m) {  // real**integer by binary exponentiation
    unsigned n = m < 0 ? -m : m;
    double y = (n % 2) ? x : 1.0;
    while (n >>= 1) { x = x * x; if (n % 2) y = y * x; }
    return m < 0 ? 1.0 / y : y;
}

static const double PI = 3.141592653589793;  // par.for:49

extern "C" int tb_config_default(tb_config* c) {
    if (!c) return TB_ERR_ARG;
    std::memset(c, 0, sizeof *c);
    // Grid of par.for scaled down; physics constants as in par.for:34-129.
    c->nx = 129; c->ny = 65; c->kfour = 4; c->kphys = 8; c->msh = 3; c->my_form = 0;
    c->i0 = 10; c->i1 = 22; c->i2 = 36; c->i3 = 100; c->i4 = 115;
    c->stpp = 368; c->max_vcycles = 11; c->ibm = 0; c->precision = TB_FORM_PLAIN_FP64;
    c->les_damping = 0; c->warm_start = 2; c->step_graph = 1;
    c->Re = 5.0 * 0.1 / 1.509479531e-5;
    c->dx = 0.02962963; c->dy = 0.15 / 182.0; c->stf = 1.0; c->x0 = 1.0;
    c->alpha = 0.45723605; c->omega = 2.6; c->beta = 34.9; c->fac_y = 1.0; c->alphaf = 0.48;
    c->tol_stage = 1e-5; c->tol_final = 1e-6;
    c->C_s = 0.032; c->A_plus = 25.0; c->irf = -0.1 * c->Re;
    c->ibm_xc = 1.7; c->ibm_zc = 0.0; c->ibm_h = 0.0; c->ibm_R = 1e-2 / 0.1;
    c->n_forced = 1; c->forced_mode[0] = 0; c->forced_amp[0] = 1e-5; c->forced_phase[0] = 0.0;
    c->Pr = 0.72;
    return TB_OK;
}

extern "C" double tb_dt(const tb_config* c) { return (2.0 * PI) / c->omega / (double)c->stpp; }

extern "C" int tb_coef_count(int msh) { return 100 + 24 * msh; }

// CUDA-event brackets around a kernel family (no-ops unless tb_profile is on).
int tb_prof_begin(tb_ctx* c, int id, cudaEvent_t* start) {
    (void)id;
    *start = nullptr;
    if (!c->prof) return TB_OK;
    cudaEvent_t e;
    if (!c->prof_pool.empty()) { e = c->prof_pool.back(); c->prof_pool.pop_back(); }
    else TB_CUDA(cudaEventCreate(&e));
    TB_CUDA(cudaEventRecord(e, c->stream));
    *start = e;
    return TB_OK;
}
int tb_prof_end(tb_ctx* c, int id, cudaEvent_t start) {
    if (!c->prof || !start) return TB_OK;
    cudaEvent_t e;
    if (!c->prof_pool.empty()) { e = c->prof_pool.back(); c->prof_pool.pop_back(); }
    else TB_CUDA(cudaEventCreate(&e));
    TB_CUDA(cudaEventRecord(e, c->stream));
    c->prof_open.push_back(tb_ctx::ProfRec{id, start, e});
    return TB_OK;
}

// ---------------------------------------------------------------------------
// Table construction (runs once per context after the coefficients are set).
namespace {

struct Coefs {
    double fp_fd_e[6], sp_fd[9], cp_fd[8], pp_fd[9], lp_fd[7];
    double fp_sd[8], sp_sd[10], cp_sd[8], pp_sd[10], lp_sd[8];
    std::vector<double> sp_poi, cp_poi, pp_poi, lp_poi;
    double w_at_w[9], dwydy[8];
};
void unpack(const std::vector<double>& blob, int msh, Coefs& c) {
    const double* p = blob.data();
    auto take = [&](double* d, int n) { std::memcpy(d, p, sizeof(double) * n); p += n; };
    take(c.fp_fd_e, 6); take(c.sp_fd, 9); take(c.cp_fd, 8); take(c.pp_fd, 9); take(c.lp_fd, 7);
    take(c.fp_sd, 8); take(c.sp_sd, 10); take(c.cp_sd, 8); take(c.pp_sd, 10); take(c.lp_sd, 8);
    c.sp_poi.resize(7 * msh); c.cp_poi.resize(8 * msh); c.pp_poi.resize(4 * msh); c.lp_poi.resize(5 * msh);
    take(c.sp_poi.data(), 7 * msh); take(c.cp_poi.data(), 8 * msh);
    take(c.pp_poi.data(), 4 * msh); take(c.lp_poi.data(), 5 * msh);
    take(c.w_at_w, 9); take(c.dwydy, 8);
}

// Thomas factors of a constant tridiagonal (same recurrence as tridparx/tridy).
void thomas_factors(const std::vector<double>& a, const std::vector<double>& b, const std::vector<double>& c,
                    std::vector<double>& g, std::vector<double>& ib) {
    int n = (int)a.size();
    g.assign(n, 0.0); ib.assign(n, 0.0);
    double bet = b[0];
    ib[0] = 1.0 / bet;
    for (int i = 1; i < n; i++) {
        g[i] = c[i - 1] / bet;
        bet = b[i] - a[i] * g[i];
        ib[i] = 1.0 / bet;
    }
}

template <class T>
int upload(T** dst, const std::vector<T>& src) {
    if (*dst) cudaFree(*dst);
    *dst = nullptr;
    if (src.empty()) return TB_OK;
    TB_CUDA(cudaMalloc((void**)dst, src.size() * sizeof(T)));
    TB_CUDA(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
    return TB_OK;
}

// Chunk tables of a Thomas sweep split over 32 lanes of S rows (TriLHS).
void chunk_tri(const std::vector<double>& a, const std::vector<double>& g, const std::vector<double>& ib, int S,
               std::vector<double>& hf, std::vector<double>& hb, std::vector<double>& pf, std::vector<double>& pb) {
    int n = (int)a.size();
    hf.assign(n, 0.0); hb.assign(n, 0.0); pf.assign(160, 0.0); pb.assign(160, 0.0);
    double Af[32], Ab[32];
    for (int t = 0; t < 32; t++) {
        int r0 = t * S, r1 = std::min(n, r0 + S);
        double h = 1.0;
        for (int i = r0; i < r1; i++) { h *= -a[i] * ib[i]; hf[i] = h; }
        Af[t] = (r1 > r0) ? hf[r1 - 1] : 1.0;
        h = 1.0;
        for (int i = r1 - 1; i >= r0; i--) { h = (r1 < n) ? h * -g[i + 1] : 0.0; hb[i] = h; }
        Ab[t] = (r1 > r0) ? hb[r0] : 1.0;
    }
    for (int d = 0, off = 1; d < 5; d++, off <<= 1) {
        double nf[32], nb[32];
        for (int t = 0; t < 32; t++) {
            pf[d * 32 + t] = Af[t];
            pb[d * 32 + t] = Ab[t];
            nf[t] = (t >= off) ? Af[t] * Af[t - off] : Af[t];
            nb[t] = (t + off < 32) ? Ab[t] * Ab[t + off] : Ab[t];
        }
        std::copy(nf, nf + 32, Af);
        std::copy(nb, nb + 32, Ab);
    }
}

int upload_tri(TriLHS& t, const std::vector<double>& a, const std::vector<double>& b, const std::vector<double>& c,
               bool chunked = false) {
    std::vector<double> g, ib;
    thomas_factors(a, b, c, g, ib);
    int r;
    if ((r = upload(&t.a, a))) return r;
    if ((r = upload(&t.g, g))) return r;
    if ((r = upload(&t.ib, ib))) return r;
    if (!chunked) return TB_OK;
    int n = (int)a.size();
    t.S = (n + 31) / 32;
    std::vector<double> hf, hb, pf, pb;
    chunk_tri(a, g, ib, t.S, hf, hb, pf, pb);
    if ((r = upload(&t.hf, hf))) return r;
    if ((r = upload(&t.hb, hb))) return r;
    if ((r = upload(&t.pf, pf))) return r;
    if ((r = upload(&t.pb, pb))) return r;
    auto f32 = [](const std::vector<double>& v) { return std::vector<float>(v.begin(), v.end()); };
    if ((r = upload(&t.af, f32(a))) || (r = upload(&t.gf, f32(g))) || (r = upload(&t.ibf, f32(ib))) ||
        (r = upload(&t.hff, f32(hf))) || (r = upload(&t.hbf, f32(hb))) || (r = upload(&t.pff, f32(pf))))
        return r;
    return upload(&t.pbf, f32(pb));
}

// lhs5 (loop_par.f:258-299) + ludecomp (penta_par.f:6-50), 1-based (n,5).
void lhs5(int n, double k2b2, std::vector<double>& a) {
    a.assign((size_t)n * 5, 0.0);
    auto A = [&](int i, int c) -> double& { return a[(size_t)(i - 1) + (size_t)n * (c - 1)]; };
    A(1, 3) = 1.0;
    A(2, 2) = 1.0 + k2b2 / 12.0; A(2, 3) = -2.0 + k2b2 / 1.2; A(2, 4) = 1.0 + k2b2 / 12.0;
    for (int i = 3; i <= n - 2; i++) {
        A(i, 1) = 3.0; A(i, 2) = 48.0 + 8.0 * k2b2; A(i, 3) = -102.0 + 44.0 * k2b2; A(i, 4) = 48.0 + 8.0 * k2b2; A(i, 5) = 3.0;
    }
    A(n - 1, 2) = 1.0 + k2b2 / 12.0; A(n - 1, 3) = -2.0 + k2b2 / 1.2; A(n - 1, 4) = 1.0 + k2b2 / 12.0;
    A(n, 3) = 1.0;
}
void ludecomp(int n, const std::vector<double>& a, std::vector<double>& lu) {
    lu.assign((size_t)n * 5, 0.0);
    auto A = [&](int i, int c) -> double { return a[(size_t)(i - 1) + (size_t)n * (c - 1)]; };
    auto L = [&](int i, int c) -> double& { return lu[(size_t)(i - 1) + (size_t)n * (c - 1)]; };
    for (int i = 1; i <= n - 2; i++) {
        int jj = std::min(i - 1, 2);
        for (int j = 3; j <= 5; j++) {
            int kk = 2; double soma = 0.0;
            for (int k = 1; k <= jj; k++) { soma = soma + L(i, kk) * L(i - k, j + k); kk--; }
            jj--;
            L(i, j) = A(i, j) - soma;
        }
        int j = 2, ii = std::min(i - 1, 1);
        for (int it = i + 1; it <= i + 2; it++) {
            double soma = 0.0;
            for (int k = 1; k <= ii; k++) soma = L(it, k) * L(i - 1, j + 2);
            L(it, j) = (A(it, j) - soma) / L(i, 3);
            ii--; j--;
        }
    }
    int i = n - 1;
    L(i, 3) = A(i, 3) - L(i, 2) * L(i - 1, 4) - L(i, 1) * L(i - 2, 5);
    L(i, 4) = A(i, 4) - L(i, 2) * L(i - 1, 5);
    L(i + 1, 2) = (A(i + 1, 2) - L(i + 1, 1) * L(i - 1, 4)) / L(i, 3);
    i = n;
    L(i, 3) = A(i, 3) - L(i, 2) * L(i - 1, 4) - L(i, 1) * L(i - 2, 5);
}

}  // namespace

// band5_poi (penta_par.f:308-364): NR banded LU, m1 = m2 = 2, no pivoting.
// Returns per row (0-based j): L1 = al(j-1,1), L2 = al(j-2,2), U1 = a(j,2),
// U2 = a(j,3) and 1/a(j,1) so that
//   y_j = r_j - L2_j y_{j-2} - L1_j y_{j-1},  x_j = (y_j - U1_j x_{j+1} - U2_j x_{j+2}) / D_j.
void tb_band5_factor(int n, std::vector<double>& a /*(n,5) band, modified*/, double* L1, double* L2, double* U1,
                     double* U2, double* ID) {
    std::vector<double> al((size_t)n * 5, 0.0);
    auto A = [&](int i, int c) -> double& { return a[(size_t)(i - 1) + (size_t)n * (c - 1)]; };
    auto AL = [&](int i, int c) -> double& { return al[(size_t)(i - 1) + (size_t)n * (c - 1)]; };
    const double TINY = (double)1.e-20f;
    int m1 = 2, mm = 5, l = m1;
    for (int i = 1; i <= m1; i++) {
        for (int j = m1 + 2 - i; j <= mm; j++) A(i, j - l) = A(i, j);
        l--;
        for (int j = mm - l; j <= mm; j++) A(i, j) = 0.0;
    }
    l = m1;
    for (int k = 1; k <= n; k++) {
        double dum = A(k, 1);
        if (l < n) l++;
        if (dum == 0.0) A(k, 1) = TINY;
        for (int i = k + 1; i <= l; i++) {
            dum = A(i, 1) / A(k, 1);
            AL(k, i - k) = dum;
            for (int j = 2; j <= mm; j++) A(i, j - 1) = A(i, j) - dum * A(k, j);
            A(i, mm) = 0.0;
        }
    }
    for (int j = 1; j <= n; j++) {
        L1[j - 1] = (j >= 2) ? AL(j - 1, 1) : 0.0;
        L2[j - 1] = (j >= 3) ? AL(j - 2, 2) : 0.0;
        U1[j - 1] = (j <= n - 1) ? A(j, 2) : 0.0;
        U2[j - 1] = (j <= n - 2) ? A(j, 3) : 0.0;
        ID[j - 1] = 1.0 / A(j, 1);
    }
}


// Poisson y-line matrix of coef_center / coef_border (poisson_par.f:229-340)
// for y-level lvl with x-spacing^2 dx2.
void tb_poisson_band_matrix_dx(const tb_ctx* c, int type, int lvl /*1-based*/, int k /*1-based*/, double dx2,
                               std::vector<double>& a) {
    const tb_config& cf = c->cfg;
    int ny = c->g.ny, msh = c->g.msh;
    const double* blob = c->coefs.data();
    const double* sp = blob + 83;             // sp_poi(7, msh)
    const double* cp = sp + 7 * msh;
    const double* pp = cp + 8 * msh;
    const double* lp = pp + 4 * msh;
    auto SP = [&](int i) { return sp[(i - 1) + 7 * (lvl - 1)]; };
    auto CP = [&](int i) { return cp[(i - 1) + 8 * (lvl - 1)]; };
    auto PP = [&](int i) { return pp[(i - 1) + 4 * (lvl - 1)]; };
    auto LP = [&](int i) { return lp[(i - 1) + 5 * (lvl - 1)]; };
    auto Q = [&](int j) { return c->h_qdy2[(size_t)(j - 1) + (size_t)ny * (lvl - 1)]; };
    int n = c->g.ptsy[lvl - 1];
    double k2b2 = c->h_k2b2[k - 1];
    double qx = (type == 0 ? -30.0 : -15.0) / (12.0 * dx2);
    double add = (qx + k2b2) / cf.fac_y;
    a.assign((size_t)n * 5, 0.0);
    auto A = [&](int j, int col) -> double& { return a[(size_t)(j - 1) + (size_t)n * (col - 1)]; };
    A(1, 3) = 1.0;
    A(2, 2) = SP(4) * Q(1);
    A(2, 3) = SP(5) * Q(1) + SP(2) * add;
    A(2, 4) = SP(6) * Q(1) + SP(3) * add;
    A(2, 5) = SP(7) * Q(1);
    for (int j = 3; j <= n - 2; j++) {
        double q = Q(j - 2);
        A(j, 1) = CP(4) * q;
        A(j, 2) = CP(5) * q + CP(1) * add;
        A(j, 3) = CP(6) * q + CP(2) * add;
        A(j, 4) = CP(7) * q + CP(3) * add;
        A(j, 5) = CP(8) * q;
    }
    double q = Q(n - 2);
    A(n - 1, 2) = PP(2) * q;
    A(n - 1, 3) = PP(3) * q + add;
    A(n - 1, 4) = PP(4) * q;
    A(n, 1) = LP(5) * q;
    A(n, 2) = LP(4) * q;
    A(n, 3) = LP(3) * q + add - LP(2) * std::sqrt(q) * std::sqrt((cf.alpha * cf.alpha - k2b2) / cf.fac_y);
    (void)msh;
}

void tb_poisson_band_matrix(const tb_ctx* c, int type, int lvl /*1-based*/, int k /*1-based*/, std::vector<double>& a) {
    tb_poisson_band_matrix_dx(c, type, lvl, k, c->h_dx2[lvl - 1], a);
}

int tb_host_build_tables(tb_ctx* c) {
    const tb_config& cf = c->cfg;
    TbGrid& g = c->g;
    int nx = g.nx, ny = g.ny, K = g.K, msh = g.msh;
    Coefs co;
    unpack(c->coefs, msh, co);
    int r;
    // create_ctes (main_par.f:1828-1892)
    std::vector<double> dy0(msh), vstf(msh);
    c->h_dx2.assign(msh, 0.0);
    for (int l = 1; l <= msh; l++) {
        dy0[l - 1] = (cf.stf != 1.0) ? cf.dy * ((tb_powi(cf.stf, 1 << (l - 1)) - 1.0) / (cf.stf - 1.0))
                                     : cf.dy * tb_powi(2.0, l - 1);
        vstf[l - 1] = tb_powi(cf.stf, 1 << (l - 1));
        c->h_dx2[l - 1] = tb_powi(cf.dx * (double)(1 << (l - 1)), 2);
    }
    c->h_qdy.assign(ny, 0.0);
    for (int j = 1; j <= ny - 1; j++)
        c->h_qdy[j - 1] = (cf.stf != 1.0) ? 1.0 / (dy0[0] * tb_powi(vstf[0], j - 1)) : 1.0 / dy0[0];
    c->h_qdy2.assign((size_t)ny * msh, 0.0);
    for (int l = 1; l <= msh; l++)
        for (int j = 1; j <= (ny - 1) / (1 << (l - 1)); j++) {
            double aux = (cf.stf != 1.0) ? dy0[l - 1] * tb_powi(vstf[l - 1], j - 1) : dy0[l - 1];
            c->h_qdy2[(size_t)(j - 1) + (size_t)ny * (l - 1)] = 1.0 / tb_powi(aux, 2);
        }
    c->h_k2b2.assign(K, 0.0);
    for (int k = 1; k <= K; k++) c->h_k2b2[k - 1] = -(double)(k - 1) * (double)(k - 1) * cf.beta * cf.beta;
    if ((r = upload(&c->k2b2, c->h_k2b2))) return r;
    if ((r = upload(&c->pqdy2, c->h_qdy2))) return r;

    // x compact LHS (coefx/coeffx derivs_par.f:1145-1210) and filter (lhs_tridf filter_par.f:181)
    {
        std::vector<double> a(nx), b(nx), cc(nx);
        a[0] = 0; b[0] = 1; cc[0] = 0; a[1] = 1; b[1] = 6; cc[1] = 2;
        for (int i = 2; i < nx - 2; i++) { a[i] = 1; b[i] = 3; cc[i] = 1; }
        a[nx - 2] = 2; b[nx - 2] = 6; cc[nx - 2] = 1; a[nx - 1] = 4; b[nx - 1] = 1; cc[nx - 1] = 0;
        if ((r = upload_tri(c->tx1, a, b, cc, true))) return r;
        a[0] = 0; b[0] = 13; cc[0] = 137; a[1] = 1; b[1] = 12; cc[1] = 3;
        for (int i = 2; i < nx - 2; i++) { a[i] = 2; b[i] = 11; cc[i] = 2; }
        a[nx - 2] = 3; b[nx - 2] = 12; cc[nx - 2] = 1; a[nx - 1] = 137; b[nx - 1] = 13; cc[nx - 1] = 0;
        if ((r = upload_tri(c->tx2, a, b, cc, true))) return r;
        std::fill(a.begin(), a.end(), 0.0); std::fill(b.begin(), b.end(), 1.0); std::fill(cc.begin(), cc.end(), 0.0);
        for (int i = 3; i < nx - 3; i++) { a[i] = cf.alphaf; cc[i] = cf.alphaf; }
        if ((r = upload_tri(c->tfil, a, b, cc, true))) return r;
    }
    // y compact LHS (coefy/coefy_fv/coeffy derivs_par.f:1040-1142) and RHS row weights
    {
        auto lhs = [&](const double* first3, const double* sp, const double* cp, const double* pp, const double* lp,
                       TriLHS& t) {
            std::vector<double> a(ny), b(ny), cc(ny);
            a[0] = first3[0]; b[0] = first3[1]; cc[0] = first3[2];
            a[1] = sp[0]; b[1] = sp[1]; cc[1] = sp[2];
            for (int j = 2; j < ny - 2; j++) { a[j] = cp[0]; b[j] = cp[1]; cc[j] = cp[2]; }
            a[ny - 2] = pp[2]; b[ny - 2] = pp[1]; cc[ny - 2] = pp[0];
            a[ny - 1] = lp[1]; b[ny - 1] = lp[0]; cc[ny - 1] = 0.0;
            return upload_tri(t, a, b, cc);
        };
        double f1[3] = {0.0, co.fp_fd_e[0], 0.0}, ffv[3] = {0.0, 1.0, 0.0}, f2[3] = {0.0, co.fp_sd[0], co.fp_sd[1]};
        if ((r = lhs(f1, co.sp_fd, co.cp_fd, co.pp_fd, co.lp_fd, c->ty1))) return r;
        if ((r = lhs(ffv, co.sp_fd, co.cp_fd, co.pp_fd, co.lp_fd, c->tyfv))) return r;
        if ((r = lhs(f2, co.sp_sd, co.cp_sd, co.pp_sd, co.lp_sd, c->ty2))) return r;
        // RHS weights (rhsy derivs_par.f:400-449, rhsyfv 504, rhsyy 552): row j uses
        // f[j + off .. j + off + cnt - 1] with weights scaled by v_qdy / v_qdy2.
        auto q1 = [&](int j1) { return c->h_qdy[j1 - 1]; };
        auto q2 = [&](int j1) { return c->h_qdy2[j1 - 1]; };
        std::vector<double> w((size_t)ny * 7, 0.0);
        std::vector<int> off(ny), cnt(ny);
        auto row = [&](int j0, int o, const double* src, int n, double s, bool rev) {
            off[j0] = o; cnt[j0] = n;
            for (int m = 0; m < n; m++) w[(size_t)j0 * 7 + m] = (rev ? src[n - 1 - m] : src[m]) * s;
        };
        // first derivative
        auto build1 = [&](bool fv, YRhs& out) {
            std::fill(w.begin(), w.end(), 0.0);
            if (fv) { off[0] = 0; cnt[0] = 0; } else row(0, 0, co.fp_fd_e + 1, 5, q1(1), false);
            row(1, -1, co.sp_fd + 3, 6, q1(1), false);
            for (int j = 2; j < ny - 2; j++) row(j, -2, co.cp_fd + 3, 5, q1(j + 1 - 2), false);
            // rhs(jmax-1) = q(jmax-5) * (pp4 f(J) + pp5 f(J-1) + ... + pp9 f(J-5)): stored ascending from f(J-5)
            row(ny - 2, -4, co.pp_fd + 3, 6, q1(ny - 5), true);
            row(ny - 1, -4, co.lp_fd + 2, 5, q1(ny - 4), true);
            int rr;
            if ((rr = upload(&out.w, w))) return rr;
            if ((rr = upload(&out.off, off))) return rr;
            return upload(&out.cnt, cnt);
        };
        if ((r = build1(false, c->ry1))) return r;
        if ((r = build1(true, c->ryfv))) return r;
        std::fill(w.begin(), w.end(), 0.0);
        row(0, 0, co.fp_sd + 2, 6, q2(1), false);
        row(1, -1, co.sp_sd + 3, 7, q2(1), false);
        for (int j = 2; j < ny - 2; j++) row(j, -2, co.cp_sd + 3, 5, q2(j + 1 - 2), false);
        row(ny - 2, -5, co.pp_sd + 3, 7, q2(ny - 6), true);
        row(ny - 1, -5, co.lp_sd + 2, 6, q2(ny - 5), true);
        if ((r = upload(&c->ry2.w, w))) return r;
        if ((r = upload(&c->ry2.off, off))) return r;
        if ((r = upload(&c->ry2.cnt, cnt))) return r;
    }
    // x-penta LU per mode (lhs5 + ludecomp; reciprocal of the diagonal in column 3)
    {
        std::vector<double> all((size_t)K * 5 * nx, 0.0), a, lu;
        for (int k = 2; k <= K; k++) {
            double k2b2 = cf.dx * cf.dx * c->h_k2b2[k - 1];
            lhs5(nx, k2b2, a);
            ludecomp(nx, a, lu);
            for (int col = 0; col < 5; col++)
                for (int i = 0; i < nx; i++) {
                    double v = lu[(size_t)i + (size_t)nx * col];
                    if (col == 2) v = 1.0 / v;
                    all[((size_t)(k - 1) * 5 + col) * nx + i] = v;
                }
        }
        if ((r = upload(&c->px.lu, all))) return r;
    }
    {
        // Poisson coefficients per level for the device kernels: sp(7) cp(8) pp(4) lp(5)
        std::vector<double> pc((size_t)24 * msh);
        for (int l = 0; l < msh; l++) {
            for (int m = 0; m < 7; m++) pc[24 * l + m] = co.sp_poi[7 * l + m];
            for (int m = 0; m < 8; m++) pc[24 * l + 7 + m] = co.cp_poi[8 * l + m];
            for (int m = 0; m < 4; m++) pc[24 * l + 15 + m] = co.pp_poi[4 * l + m];
            for (int m = 0; m < 5; m++) pc[24 * l + 19 + m] = co.lp_poi[5 * l + m];
        }
        if ((r = upload(&c->pcoef, pc))) return r;
        const double* wat = c->coefs.data() + 100 + 24 * msh - 17;
        if ((r = upload(&c->wcoef, std::vector<double>(wat, wat + 17)))) return r;
    }
    // var_ts (main_par.f:1688-1736)
    {
        int i1 = cf.i1, i2 = cf.i2;
        c->h_fcx.assign(nx, 0.0); c->h_fcllx.assign(nx, 0.0);
        double imed = (double)(i1 + i2) / 2.0;
        double div = 1.0 / ((double)(imed - i1) * cf.dx);
        double A = -(19683.0 / 4096.0 * tb_powi(div, 8)), B = 177147.0 / 4096.0 * tb_powi(div, 7);
        double Cc = -(19683.0 / 128.0 * tb_powi(div, 6)), D = 137781.0 / 512.0 * tb_powi(div, 5);
        double E = -(59049.0 / 256.0 * tb_powi(div, 4)), F = 19683.0 / 256.0 * tb_powi(div, 3);
        double fcmax = 0.0;
        for (int i = i1; i <= (i1 + i2) / 2; i++) {
            double x = (double)(i - i1) * cf.dx;
            fcmax = std::max(fcmax, std::fabs((((((A * x + B) * x + Cc) * x + D) * x + E) * x + F) * tb_powi(x, 4)));
        }
        for (int i = i1; i <= (i1 + i2) / 2; i++) {
            double x = (double)(i - i1) * cf.dx;
            double v = (((((A * x + B) * x + Cc) * x + D) * x + E) * x + F) * tb_powi(x, 4) / fcmax;
            if (std::fabs(v) < 1e-15) v = 0.0;
            c->h_fcx[i - 1] = v;
            c->h_fcx[i2 + i1 - i - 1] = -v;
            double w = (((((72.0 * A * x + 56.0 * B) * x + 42.0 * Cc) * x + 30.0 * D) * x + 20.0 * E) * x + 12.0 * F) * x * x / fcmax;
            if (std::fabs(w) < 1e-15) w = 0.0;
            c->h_fcllx[i - 1] = w;
            c->h_fcllx[i2 + i1 - i - 1] = -w;
        }
        if ((r = upload(&c->fcx, c->h_fcx))) return r;
        if ((r = upload(&c->fcllx, c->h_fcllx))) return r;
    }
    // var_gv (main_par.f:1739-1759): the steady Goertler strip sin^3 and its
    // second x-derivative factor, over i1..i2
    {
        int i1 = cf.i1, i2 = cf.i2;
        c->h_fcx2.assign(nx, 0.0); c->h_fcllx2.assign(nx, 0.0);
        for (int i = i1; i <= i2 && i <= nx; i++) {
            double x = PI * (double)(i - i1) / (double)(i2 - i1);
            double sx = std::sin(x), cx = std::cos(x);
            c->h_fcx2[i - 1] = sx * sx * sx;
            c->h_fcllx2[i - 1] = 6.0 * cx * cx * sx - 3.0 * sx * sx * sx;
        }
        if ((r = upload(&c->fcx2, c->h_fcx2))) return r;
        if ((r = upload(&c->fcllx2, c->h_fcllx2))) return r;
    }
    // buffer ramps (main_par.f:737-756)
    {
        c->h_bdfc.assign(nx, 0.0);
        for (int i = 1; i <= cf.i0; i++) {
            double ep = (double)(i - 1) / (double)(cf.i0 - 1);
            c->h_bdfc[i - 1] = ((6.0 * ep - 15.0) * ep + 10.0) * tb_powi(ep, 3);
        }
        for (int i = cf.i0; i <= cf.i3; i++) c->h_bdfc[i - 1] = 1.0;
        for (int i = cf.i3; i <= cf.i4; i++) {
            double ep = (double)(i - cf.i3) / (double)(cf.i4 - cf.i3);
            c->h_bdfc[i - 1] = tb_powi(1.0 - tb_powi(ep, 50), 4) * std::exp(-tb_powi(ep, 4) / 10.0);
        }
        for (int i = cf.i4; i <= nx; i++) c->h_bdfc[i - 1] = 0.0;
        // second row, for mode 2 (bzone's bdt = 2, loop_par.f:19-20): equal to
        // the first, except in the Goertler form (init_gv, main_par.f:991-996),
        // where it ramps up over i = 1 .. 2 (i1 + i2)
        c->h_bdfc.resize(2 * (size_t)nx);
        for (int i = 0; i < nx; i++) c->h_bdfc[nx + i] = c->h_bdfc[i];
        if (cf.my_form == 1) {
            int igv = std::min(2 * (cf.i1 + cf.i2), nx);
            for (int i = 1; i <= igv; i++) {
                double ep = (double)(i - 1) / (double)(igv - 1);
                c->h_bdfc[nx + i - 1] = ((6.0 * ep - 15.0) * ep + 10.0) * tb_powi(ep, 3);
            }
        }
        if ((r = upload(&c->bdfc, c->h_bdfc))) return r;
    }
    // gibbs_function final form exp(-theta^2) (immersed_par.f:248-249); K = 1 guarded
    {
        c->h_gibbs.assign(K, 1.0);
        for (int k = 1; k <= K && K > 1; k++) {
            double th = PI * (double)(k - 1) / (double)(K - 1);
            c->h_gibbs[k - 1] = std::exp(-(th * th));
        }
        if ((r = upload(&c->gibbs, c->h_gibbs))) return r;
    }
    return TB_OK;
}

// Base flow upload + derparxue (derivs_par.f:32-45): d(ue)/dx from uxb(:,jmax).
int tb_host_upload_baseflow(tb_ctx* c) {
    int nx = c->g.nx, ny = c->g.ny;
    double dx = c->cfg.dx;
    std::vector<double> f(nx), rr(nx);
    for (int i = 0; i < nx; i++) f[i] = c->h_uxb[(size_t)i + (size_t)nx * (ny - 1)];
    int m = nx - 1;
    rr[0] = (-(25.0 * f[0]) + 48.0 * f[1] - 36.0 * f[2] + 16.0 * f[3] - 3.0 * f[4]) / (12.0 * dx);
    rr[1] = (-(406.0 * f[0]) - 300.0 * f[1] + 760.0 * f[2] - 80.0 * f[3] + 30.0 * f[4] - 4.0 * f[5]) / (120.0 * dx);
    for (int i = 2; i < nx - 2; i++) rr[i] = (f[i + 2] - f[i - 2] + 28.0 * (f[i + 1] - f[i - 1])) / (12.0 * dx);
    rr[m - 1] = (-(406.0 * f[m]) - 300.0 * f[m - 1] + 760.0 * f[m - 2] - 80.0 * f[m - 3] + 30.0 * f[m - 4] - 4.0 * f[m - 5]) / (-(120.0 * dx));
    rr[m] = (-(74.0 * f[m]) + 16.0 * f[m - 1] + 72.0 * f[m - 2] - 16.0 * f[m - 3] + 2.0 * f[m - 4]) / (-(24.0 * dx));
    std::vector<double> a(nx), b(nx), cc(nx), g, ib;
    a[0] = 0; b[0] = 1; cc[0] = 0; a[1] = 1; b[1] = 6; cc[1] = 2;
    for (int i = 2; i < nx - 2; i++) { a[i] = 1; b[i] = 3; cc[i] = 1; }
    a[nx - 2] = 2; b[nx - 2] = 6; cc[nx - 2] = 1; a[nx - 1] = 4; b[nx - 1] = 1; cc[nx - 1] = 0;
    // same recurrence as tridparxue (reference divides by bet; identical quotient sequence)
    std::vector<double> gam(nx), u(nx);
    double bet = b[0];
    u[0] = rr[0] / bet;
    for (int i = 1; i < nx; i++) {
        gam[i] = cc[i - 1] / bet;
        bet = b[i] - a[i] * gam[i];
        u[i] = (rr[i] - a[i] * u[i - 1]) / bet;
    }
    for (int i = nx - 2; i >= 0; i--) u[i] = u[i] - gam[i + 1] * u[i + 1];
    c->h_duexmdx = u;
    int r;
    if ((r = upload(&c->uxb, c->h_uxb))) return r;
    if ((r = upload(&c->uyb, c->h_uyb))) return r;
    if ((r = upload(&c->wzb, c->h_wzb))) return r;
    return upload(&c->duexmdx, c->h_duexmdx);
}

// ---------------------------------------------------------------------------
// Falkner-Skan / Blasius base flow (pre_processing/fs_sch.f90, main_fs.f90).
namespace {

// derivs (fs_sch.f90:232-247): f, f', f'' and their sensitivities to f''(0).
inline void fs_derivs(const double* f, double* d, double beta_fs) {
    d[0] = f[1];
    d[1] = f[2];
    d[2] = -f[0] * f[2] - beta_fs * (1.0 - f[1] * f[1]);
    d[3] = f[4];
    d[4] = f[5];
    d[5] = -f[3] * f[2] - f[0] * f[5] + 2.0 * beta_fs * f[1] * f[4];
}
// derivs_theta (fs_sch.f90:432-447) with Prandtl number Pr.
inline void fs_derivs_theta(const double* f, double* d, double beta_fs, double Pr) {
    d[0] = f[1];
    d[1] = f[2];
    d[2] = -f[0] * f[2] - (beta_fs * (1.0 - f[1] * f[1]));
    d[3] = f[4];
    d[4] = -f[0] * f[4] * Pr;
    d[5] = 0.0;
}
// classical RK4 step in the reference's staging (fs_sch.f90:202-227, 404-429)
template <class D>
inline void fs_rk4(double* f, double h, D derivs) {
    double hh = h * 0.5, h6 = h / 6.0, d1[6], d2[6], ft[6];
    derivs(f, d1);
    for (int q = 0; q < 6; q++) ft[q] = f[q] + hh * d1[q];
    derivs(ft, d2);
    for (int q = 0; q < 6; q++) { ft[q] = f[q] + hh * d2[q]; d1[q] = d1[q] + 2.0 * d2[q]; }
    derivs(ft, d2);
    for (int q = 0; q < 6; q++) { ft[q] = f[q] + h * d2[q]; d1[q] = d1[q] + 2.0 * d2[q]; }
    derivs(ft, d2);
    for (int q = 0; q < 6; q++) f[q] = f[q] + h6 * (d1[q] + d2[q]);
}

}  // namespace

// fpp_finder (fs_sch.f90:11-54) started as in main_fs.f90:17-19.
extern "C" int tb_fs_wall_shear(double beta_fs, double* fpp_out) {
    if (!fpp_out) return TB_ERR_ARG;
    const double tol_fs = 1.0e-13, gtol_fs = 1.0e-23, eta_variation = 0.01, deta = 1.0e-4;
    double fpp = 1.1, eta_adp = 0.5;  // etapp_guess, eta_zero (constants.f90:24-28)
    double ls_err = 1.0;
    int cont = 1;
    auto der = [&](const double* f, double* d) { fs_derivs(f, d, beta_fs); };
    while (std::fabs(ls_err) > gtol_fs && cont < 10000) {
        double delta_fpp = 100.0;
        int steps_eta = (int)(eta_adp / deta + 1.0);
        double f[6];
        int newton = 0;
        while (std::fabs(delta_fpp / fpp) > tol_fs) {
            f[0] = 0.0; f[1] = 0.0; f[2] = fpp; f[3] = 0.0; f[4] = 0.0; f[5] = 1.0;
            for (int j = 2; j <= steps_eta; j++) fs_rk4(f, deta, der);
            delta_fpp = (-f[4] * f[1] - (f[5] * f[2]) + f[4]) / (f[4] * f[4] + f[5] * f[5]);
            fpp = fpp + delta_fpp;
            if (++newton > 200) { tb_set_error("fs shooting: Newton did not converge"); return TB_ERR_NOCONV; }
        }
        ls_err = (1.0 - f[1]) * (1.0 - f[1]) + f[2] * f[2];
        eta_adp = eta_adp + eta_variation;
        cont++;
    }
    *fpp_out = fpp;
    return TB_OK;
}

// baseflow_fs (fs_sch.f90:58-162) for a constant pressure-gradient parameter
// (the reference's beta_fs.dist is all zeros: Blasius).  Every station shares
// f''(0), so the shooting runs once instead of once per station.
extern "C" int tb_baseflow_fs(const tb_config* cf, double beta_fs, double* uxb, double* uyb, double* wzb) {
    if (!cf || !uxb || !uyb || !wzb) return TB_ERR_ARG;
    double fpp;
    int r = tb_fs_wall_shear(beta_fs, &fpp);
    if (r) return r;
    const double Pr = 0.72, thp = 0.0;
    int nx = cf->nx, ny = cf->ny;
    double Re = cf->Re, dy0 = cf->dy, stf = cf->stf, fac_y = cf->fac_y;
    auto der = [&](const double* f, double* d) { fs_derivs_theta(f, d, beta_fs, Pr); };
    for (int i = 1; i <= nx; i++) {
        double m = beta_fs / (2.0 - beta_fs);
        double xad = cf->x0 + (double)(i - 1) * cf->dx;
        double ue = std::pow(xad, m);
        double deta0 = (dy0 / std::sqrt(fac_y)) * std::sqrt(0.5 * Re * ue * (m + 1.0) / xad);
        double f[6] = {0.0, 0.0, fpp, 0.0, thp, 0.0};
        size_t c0 = (size_t)(i - 1);
        uxb[c0] = 0.0;
        uyb[c0] = 0.0;
        wzb[c0] = ue * deta0 * f[2] / (dy0 / std::sqrt(fac_y)) / std::sqrt(fac_y);
        for (int j = 2; j <= ny; j++) {
            double h = deta0 * tb_powi(stf, j - 2);
            int pt = (int)(h / 1.0e-4);
            if (pt < 1) pt = 1;  // the reference would divide by zero here
            h = h / (double)pt;
            for (int k = 1; k <= pt; k++) fs_rk4(f, h, der);
            double eta = (stf != 1.0) ? deta0 * (tb_powi(stf, j - 1) - 1.0) / (stf - 1.0) : deta0 * (double)(j - 1);
            double yad = eta / std::sqrt(0.5 * Re * ue * (m + 1.0) / xad);
            size_t q = c0 + (size_t)nx * (j - 1);
            uxb[q] = ue * f[1];
            uyb[q] = (-std::sqrt(0.5 * ue * (m + 1.0) / (xad * Re)) * f[0] - 0.5 * (m - 1.0) * yad * ue * f[1] / xad) *
                     std::sqrt(fac_y);
            wzb[q] = ue * std::sqrt(0.5 * (m + 1.0) * Re * ue / xad) * f[2] / std::sqrt(fac_y);
        }
    }
    return TB_OK;
}
