// tb_mixed.cu -- mixed-precision form of the v-Poisson solve (poi_uy).
//
// The reference solves each mode's v-Poisson problem with an FP64 FAS
// multigrid whose smoother relaxes the y-lines in lexicographic x order
// (poisson_par.f:6-963): every line waits for the one before it.  This form
// keeps the reference's discrete problem and its stopping rule and changes
// how the answer is reached:
//
//   outer loop, FP64 (defect correction on the reference's fine operator):
//     d = sc - L u        -- same kernel as the plain form (poisson_par.f:543-793)
//     stop a mode once max|d| < tol  (verifica_poi, poisson_par.f:945-963)
//     solve L e = d       -- FP32 correction-scheme multigrid, e = 0 at start
//     u += e
//
// The FP32 multigrid uses the reference's level operators (compact y-weights
// and 4th-order x-stencils of coef_center/coef_border), full-weighting
// restriction and bilinear prolongation on the reference's msh levels.  Below
// them it keeps coarsening in x only (same y-level operators, dx doubled,
// (1/4, 1/2, 1/4) restriction, linear prolongation) until a level has at most
// DIRECT_MAX unknowns, which is solved exactly: its operator is inverted per
// mode at set-up (FP64 Gauss-Jordan, stored in FP32) and applied as one
// batched matrix-vector product.  The smoother relaxes y-lines in four
// groups: the two border lines, then the centre lines by colour i mod 3.  The
// centre stencil reaches i+-2 and the border stencil reaches 4 lines inwards,
// so the lines of one group never read each other and a whole group is solved
// at once, one warp per (line, mode).
//
// Layout: FP32 levels are stored per mode with each y-line contiguous
// (element (i, j) of level l at off[l] + i*ptsy[l] + j), so a warp reads
// a line and its x-neighbours with unit stride.  At 1025 x 193 x 32 modes one
// FP32 level-0 field is 51 MB: the three FP32 arrays of the fine level fit in
// the 129 MB L2 between sweeps.
#include "tb_internal.h"
#include <cmath>
#include <cstring>
#include <algorithm>
#include <thread>

namespace {

// Relaxation sweeps before / after the coarse correction, V-cycles per FP64
// correction, and whether the hierarchy starts with x-only coarsening
// (until dx >= the largest y-spacing, so that y-coupling dominates at every
// point of the coarser levels and y-line relaxation smooths everywhere).
#ifndef TB_MG_NU_PRE
#define TB_MG_NU_PRE 1
#endif
#ifndef TB_MG_NU_POST
#define TB_MG_NU_POST 2
#endif
#ifndef TB_MG_INNER
#define TB_MG_INNER 2
#endif
#ifndef TB_MG_SEMI_FIRST
#define TB_MG_SEMI_FIRST 1
#endif
constexpr int NU_PRE = TB_MG_NU_PRE, NU_POST = TB_MG_NU_POST, INNER_VCYCLES = TB_MG_INNER;
constexpr int RELAX_THREADS = 128;   // 4 warps, one line each
#ifndef TB_RELAX_MIN_BLOCKS
#define TB_RELAX_MIN_BLOCKS 8
#endif
constexpr int RELAX_MIN_BLOCKS = TB_RELAX_MIN_BLOCKS;   // resident blocks per SM the register budget allows
constexpr int MG_MAX = 16;           // levels of the FP32 hierarchy
constexpr int DIRECT_MAX = 400;      // unknowns per mode below which coarsening stops
constexpr int DIRECT_LIMIT = 2048;   // largest directly solved level accepted

struct Mixed {
    float2 *e = nullptr, *r = nullptr, *rr = nullptr;   // per mode blocks of `elems` (line-contiguous)
    float* tab = nullptr;     // [type][level][k] blocks of tb_poi_blk_size(ny): L1 L2 U1 U2 ID h1 h2 k1 k2 Pf Pb
    float* coef = nullptr;    // sp(7) cp(8) pp(4) lp(5) per reference level
    float* qdy2 = nullptr;    // (ny, msh)
    float* ainv = nullptr;    // (K, N, N) inverse of the coarsest operator per mode
    unsigned long long* maxsq = nullptr;   // (K) max |defect|^2 as double bits
    // warm start: per RK stage the v of the last two steps' solves (h0 the
    // newer), how many of them are usable (device, per stage) and the step
    // of the last solve (host)
    cplx* hist[4][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
    int* hvalid = nullptr;
    int last_t[4] = {-9, -9, -9, -9};
    int hv_host[4] = {0, 0, 0, 0};   // host copy of hvalid for host-launched solves
    int* lkeep = nullptr;            // (K, 2) learned correction kept per mode, in the layout of pstate
    int* iter = nullptr;      // corrections tested so far in a recorded solve loop
    int NL = 0, N = 0;
    int ptsx[MG_MAX], ptsy[MG_MAX], ylvl[MG_MAX], semi[MG_MAX], S[MG_MAX];
    double dx2[MG_MAX];
    size_t off[MG_MAX], elems = 0;
};

struct MgDev {
    float2 *e, *r, *rr;
    const float* tab;
    const float* coef;
    const float* qdy2;
    const float* ainv;
    const double* k2b2;
    const int* state;
    int ny, K, NL, N;
    int ptsx[MG_MAX], ptsy[MG_MAX], ylvl[MG_MAX];
    size_t off[MG_MAX], elems, bs;
    float qx[MG_MAX];       // 1 / (12 dx_l^2 fac_y)
    float ify, alpha2;      // 1 / fac_y, alpha^2
};

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// x-stencil of the line operator without its diagonal: centre lines
// 16(f[i-1] + f[i+1]) - (f[i-2] + f[i+2]); border lines (i = 1, mirrored at
// i = nxl-2) 10 f[i-1] - 4 f[i+1] + 14 f[i+2] - 6 f[i+3] + f[i+4]
// (rhs_center / rhs_border, poisson_par.f:229-540).
__device__ __forceinline__ float2 xsum(const float2* E, int n, int i, int j, int type, int e) {
    auto at = [&](int ii) { return E[(size_t)n * ii + j]; };
    if (type == 0) {
        float2 a = at(i - 2), b = at(i - 1), c = at(i + 1), d = at(i + 2);
        return f2(16.f * (b.x + c.x) - (a.x + d.x), 16.f * (b.y + c.y) - (a.y + d.y));
    }
    float2 a = at(i - e), b = at(i + e), c = at(i + 2 * e), d = at(i + 3 * e), f = at(i + 4 * e);
    return f2(10.f * a.x - 4.f * b.x + 14.f * c.x - 6.f * d.x + f.x, 10.f * a.y - 4.f * b.y + 14.f * c.y - 6.f * d.y + f.y);
}

// Relax one group of lines at level l: lines i = first + step*t, t < nlines,
// in every active mode; e(i, :) <- line solve of L e = r with the other lines
// frozen.  One warp per (line, mode); the pentadiagonal solve is split into
// 32 row chunks (local recurrences, warp scan of precomputed 2x2 chunk
// propagators, fix-up with precomputed homogeneous responses).
template <int S>
__global__ void __launch_bounds__(RELAX_THREADS, RELAX_MIN_BLOCKS) k_relax(MgDev M, int l, int first, int step, int nlines) {
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gw = blockIdx.x * (RELAX_THREADS / 32) + wib;
    const int k = gw / nlines;
    if (k >= M.K || !M.state[2 * k]) return;   // uniform over the warp
    const int i = first + step * (gw - k * nlines);
    const int nxl = M.ptsx[l], n = M.ptsy[l];
    const int type = (i == 1 || i == nxl - 2) ? 1 : 0, dir = (i == 1) ? 1 : -1;
    extern __shared__ float2 smf[];
    float2* g = smf + (size_t)wib * 2 * n;
    float2* rs = g + n;
    float2* E = M.e + (size_t)k * M.elems + M.off[l];
    const float2* R = M.r + (size_t)k * M.elems + M.off[l] + (size_t)n * i;
    // rows j = lane + 32 q, q < S (32 S >= n): all loads of the line issue at once
    float2 rv[S];
#pragma unroll
    for (int q = 0; q < S; q++) {
        int j = lane + 32 * q;
        if (j < n) { g[j] = xsum(E, n, i, j, type, dir); rv[q] = R[j]; }
    }
    __syncwarp();
    const float* cf = M.coef + 24 * M.ylvl[l];
    const float sp2 = cf[1], sp3 = cf[2], cp1 = cf[7], cp2 = cf[8], cp3 = cf[9];
    const float qx = M.qx[l];
#pragma unroll
    for (int q = 0; q < S; q++) {
        int j = lane + 32 * q;
        if (j >= n) break;
        float2 v = f2(0.f, 0.f);
        if (j >= 1) {
            float2 t;
            if (j == 1) t = f2(sp3 * g[2].x + sp2 * g[1].x, sp3 * g[2].y + sp2 * g[1].y);
            else if (j <= n - 3)
                t = f2(cp1 * g[j - 1].x + cp2 * g[j].x + cp3 * g[j + 1].x, cp1 * g[j - 1].y + cp2 * g[j].y + cp3 * g[j + 1].y);
            else t = g[j];
            float2 s = rv[q];
            v = f2(s.x - qx * t.x, s.y - qx * t.y);
        }
        rs[j] = v;
    }
    __syncwarp();
    const float* T = M.tab + (((size_t)type * M.NL + l) * M.K + k) * M.bs;
    const int ny = M.ny;
    const float *L1 = T, *L2 = T + ny, *U1 = T + 2 * ny, *U2 = T + 3 * ny, *ID = T + 4 * ny;
    const float *h1 = T + 5 * ny, *h2 = T + 6 * ny, *k1 = T + 7 * ny, *k2 = T + 8 * ny;
    const float* Pf = T + 9 * ny;
    const float* Pb = Pf + 640;
    const int r0 = lane * S, r1 = min(n, r0 + S);
    float2 y[S];
    float2 ym1 = f2(0.f, 0.f), ym2 = f2(0.f, 0.f);
#pragma unroll
    for (int s = 0; s < S; s++) {
        int j = r0 + s;
        if (j < r1) {
            float2 v = rs[j];
            float a1 = L1[j], a2 = L2[j];
            float2 yy = f2(v.x - a2 * ym2.x - a1 * ym1.x, v.y - a2 * ym2.y - a1 * ym1.y);
            y[s] = yy; ym2 = ym1; ym1 = yy;
        }
    }
    float2 b0 = ym1, b1 = ym2;
#pragma unroll
    for (int d = 0, off = 1; d < 5; d++, off <<= 1) {
        float2 o0, o1;
        o0.x = __shfl_up_sync(0xffffffffu, b0.x, off); o0.y = __shfl_up_sync(0xffffffffu, b0.y, off);
        o1.x = __shfl_up_sync(0xffffffffu, b1.x, off); o1.y = __shfl_up_sync(0xffffffffu, b1.y, off);
        if (lane >= off) {
            const float* P = Pf + (d * 32 + lane) * 4;
            b0 = f2(b0.x + P[0] * o0.x + P[1] * o1.x, b0.y + P[0] * o0.y + P[1] * o1.y);
            b1 = f2(b1.x + P[2] * o0.x + P[3] * o1.x, b1.y + P[2] * o0.y + P[3] * o1.y);
        }
    }
    float2 Y1, Y2;
    Y1.x = __shfl_up_sync(0xffffffffu, b0.x, 1); Y1.y = __shfl_up_sync(0xffffffffu, b0.y, 1);
    Y2.x = __shfl_up_sync(0xffffffffu, b1.x, 1); Y2.y = __shfl_up_sync(0xffffffffu, b1.y, 1);
    if (lane == 0) { Y1 = f2(0.f, 0.f); Y2 = f2(0.f, 0.f); }
#pragma unroll
    for (int s = 0; s < S; s++) {
        int j = r0 + s;
        if (j < r1) y[s] = f2(y[s].x + h1[j] * Y1.x + h2[j] * Y2.x, y[s].y + h1[j] * Y1.y + h2[j] * Y2.y);
    }
    float2 xp1 = f2(0.f, 0.f), xp2 = f2(0.f, 0.f);
#pragma unroll
    for (int s = S - 1; s >= 0; s--) {
        int j = r0 + s;
        if (j < r1) {
            float u1 = U1[j], u2 = U2[j], id = ID[j];
            float2 xx = f2((y[s].x - u1 * xp1.x - u2 * xp2.x) * id, (y[s].y - u1 * xp1.y - u2 * xp2.y) * id);
            y[s] = xx; xp2 = xp1; xp1 = xx;
        }
    }
    b0 = xp1; b1 = xp2;
#pragma unroll
    for (int d = 0, off = 1; d < 5; d++, off <<= 1) {
        float2 o0, o1;
        o0.x = __shfl_down_sync(0xffffffffu, b0.x, off); o0.y = __shfl_down_sync(0xffffffffu, b0.y, off);
        o1.x = __shfl_down_sync(0xffffffffu, b1.x, off); o1.y = __shfl_down_sync(0xffffffffu, b1.y, off);
        if (lane + off < 32) {
            const float* P = Pb + (d * 32 + lane) * 4;
            b0 = f2(b0.x + P[0] * o0.x + P[1] * o1.x, b0.y + P[0] * o0.y + P[1] * o1.y);
            b1 = f2(b1.x + P[2] * o0.x + P[3] * o1.x, b1.y + P[2] * o0.y + P[3] * o1.y);
        }
    }
    float2 X1, X2;
    X1.x = __shfl_down_sync(0xffffffffu, b0.x, 1); X1.y = __shfl_down_sync(0xffffffffu, b0.y, 1);
    X2.x = __shfl_down_sync(0xffffffffu, b1.x, 1); X2.y = __shfl_down_sync(0xffffffffu, b1.y, 1);
    if (lane == 31) { X1 = f2(0.f, 0.f); X2 = f2(0.f, 0.f); }
    __syncwarp();
#pragma unroll
    for (int s = 0; s < S; s++) {
        int j = r0 + s;
        if (j < r1) rs[j] = f2(y[s].x + k1[j] * X1.x + k2[j] * X2.x, y[s].y + k1[j] * X1.y + k2[j] * X2.y);
    }
    __syncwarp();
    float2* Ei = E + (size_t)n * i;
#pragma unroll
    for (int q = 0; q < S; q++) {
        int j = lane + 32 * q;
        if (j >= 1 && j < n) Ei[j] = rs[j];
    }
}

// FP32 residual rr = r - L e at level l (interior columns, rows >= 1):
// the operator of defect (poisson_par.f:543-793) on the line-contiguous layout.
__global__ void k_resid(MgDev M, int l) {
    const int nxl = M.ptsx[l], n = M.ptsy[l];
    size_t per = (size_t)(nxl - 2) * (n - 1);
    size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= per * M.K) return;
    int k = (int)(q / per);
    if (!M.state[2 * k]) return;
    size_t rq = q % per;
    int j = 1 + (int)(rq % (n - 1)), i = 1 + (int)(rq / (n - 1));
    const int yl = M.ylvl[l];
    const float* cf = M.coef + 24 * yl;
    const float *SP = cf, *CP = cf + 7, *PP = cf + 15, *LP = cf + 19;
    const float* Q2 = M.qdy2 + (size_t)M.ny * yl;
    const float k2b2 = (float)M.k2b2[k];
    const float den = M.qx[l];
    const float2* E = M.e + (size_t)k * M.elems + M.off[l];
    auto f = [&](int ii, int jj) -> float2 { return E[(size_t)n * ii + jj]; };
    auto bx = [&](int jj) -> float2 {
        if (i == 1 || i == nxl - 2) {
            int e = (i == 1) ? 1 : -1;
            float2 a = f(i - e, jj), c0 = f(i, jj), b = f(i + e, jj), c = f(i + 2 * e, jj), d = f(i + 3 * e, jj), g = f(i + 4 * e, jj);
            return f2(10.f * a.x - 15.f * c0.x - 4.f * b.x + 14.f * c.x - 6.f * d.x + g.x,
                      10.f * a.y - 15.f * c0.y - 4.f * b.y + 14.f * c.y - 6.f * d.y + g.y);
        }
        float2 a = f(i - 2, jj), b = f(i - 1, jj), c0 = f(i, jj), c = f(i + 1, jj), d = f(i + 2, jj);
        return f2(-a.x + 16.f * b.x - 30.f * c0.x + 16.f * c.x - d.x, -a.y + 16.f * b.y - 30.f * c0.y + 16.f * c.y - d.y);
    };
    float2 b, cc, d;
    float q2, top = 0.f;
    if (j == 1) {
        float2 b1 = bx(1), b2 = bx(2);
        b = f2(SP[2] * b2.x + SP[1] * b1.x, SP[2] * b2.y + SP[1] * b1.y);
        float2 g0 = f(i, 0), g1 = f(i, 1), g2 = f(i, 2), g3 = f(i, 3);
        cc = f2(SP[3] * g0.x + SP[4] * g1.x + SP[5] * g2.x + SP[6] * g3.x, SP[3] * g0.y + SP[4] * g1.y + SP[5] * g2.y + SP[6] * g3.y);
        d = f2(k2b2 * (SP[1] * g1.x + SP[2] * g2.x), k2b2 * (SP[1] * g1.y + SP[2] * g2.y));
        q2 = Q2[0];
    } else if (j <= n - 3) {
        float2 ba = bx(j - 1), bb = bx(j), bc = bx(j + 1);
        b = f2(CP[0] * ba.x + CP[1] * bb.x + CP[2] * bc.x, CP[0] * ba.y + CP[1] * bb.y + CP[2] * bc.y);
        float2 fm2 = f(i, j - 2), fm1 = f(i, j - 1), g0 = f(i, j), fp1 = f(i, j + 1), fp2 = f(i, j + 2);
        cc = f2(CP[3] * fm2.x + CP[4] * fm1.x + CP[5] * g0.x + CP[6] * fp1.x + CP[7] * fp2.x,
                CP[3] * fm2.y + CP[4] * fm1.y + CP[5] * g0.y + CP[6] * fp1.y + CP[7] * fp2.y);
        d = f2(k2b2 * (CP[0] * fm1.x + CP[1] * g0.x + CP[2] * fp1.x), k2b2 * (CP[0] * fm1.y + CP[1] * g0.y + CP[2] * fp1.y));
        q2 = Q2[j - 2];
    } else if (j == n - 2) {
        b = bx(j);
        float2 fm1 = f(i, j - 1), g0 = f(i, j), fp1 = f(i, j + 1);
        cc = f2(PP[3] * fp1.x + PP[2] * g0.x + PP[1] * fm1.x, PP[3] * fp1.y + PP[2] * g0.y + PP[1] * fm1.y);
        d = f2(k2b2 * g0.x, k2b2 * g0.y);
        q2 = Q2[j - 1];
    } else {
        b = bx(j);
        float2 fm2 = f(i, j - 2), fm1 = f(i, j - 1), g0 = f(i, j);
        cc = f2(LP[2] * g0.x + LP[3] * fm1.x + LP[4] * fm2.x, LP[2] * g0.y + LP[3] * fm1.y + LP[4] * fm2.y);
        d = f2(k2b2 * g0.x, k2b2 * g0.y);
        q2 = Q2[j - 2];
        top = LP[1] * sqrtf((M.alpha2 - k2b2) * M.ify) * sqrtf(q2);
    }
    float2 fij = f(i, j);
    size_t o = (size_t)k * M.elems + M.off[l] + (size_t)n * i + j;
    float2 s = M.r[o];
    M.rr[o] = f2(s.x - (b.x * den + cc.x * q2 + d.x * M.ify - top * fij.x),
                 s.y - (b.y * den + cc.y * q2 + d.y * M.ify - top * fij.y));
}

// Full-weighting restriction of rr(l) into r(l+1) with the weights of
// restrict (poisson_par.f:796-874); the coarse correction e(l+1) starts at 0.
__global__ void k_restrict32(MgDev M, int l) {
    const int nxc = M.ptsx[l + 1], nyc = M.ptsy[l + 1], nyf = M.ptsy[l];
    size_t per = (size_t)nxc * nyc;
    size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= per * M.K) return;
    int k = (int)(q / per);
    if (!M.state[2 * k]) return;
    int j = (int)((q % per) % nyc), i = (int)((q % per) / nyc);
    size_t oc = (size_t)k * M.elems + M.off[l + 1] + (size_t)nyc * i + j;
    M.e[oc] = f2(0.f, 0.f);
    float2 v = f2(0.f, 0.f);
    if (i >= 1 && i <= nxc - 2 && j >= 1) {
        const float2* D = M.rr + (size_t)k * M.elems + M.off[l];
        auto df = [&](int ii, int jj) { return D[(size_t)nyf * ii + jj]; };
        int fi = 2 * i, fj = 2 * j;
        if (j <= nyc - 2) {
            float2 a = df(fi - 1, fj), b = df(fi + 1, fj), c = df(fi, fj - 1), d = df(fi, fj + 1), e = df(fi, fj);
            float2 g1 = df(fi + 1, fj + 1), g2 = df(fi + 1, fj - 1), g3 = df(fi - 1, fj + 1), g4 = df(fi - 1, fj - 1);
            v.x = 0.0625f * (2.f * (a.x + b.x + c.x + d.x) + 4.f * e.x + g1.x + g2.x + g3.x + g4.x);
            v.y = 0.0625f * (2.f * (a.y + b.y + c.y + d.y) + 4.f * e.y + g1.y + g2.y + g3.y + g4.y);
        } else {
            fj = nyf - 1;
            float2 a = df(fi - 1, fj), e = df(fi, fj), b = df(fi + 1, fj);
            v = f2(0.25f * (a.x + 2.f * e.x + b.x), 0.25f * (a.y + 2.f * e.y + b.y));
        }
    }
    M.r[oc] = v;
}

// Bilinear prolongation of e(l) added to e(l-1) (intpol, poisson_par.f:877-920).
__global__ void k_prolong32(MgDev M, int l) {
    const int nyc = M.ptsy[l], nxf = M.ptsx[l - 1], nyf = M.ptsy[l - 1];
    size_t per = (size_t)nxf * nyf;
    size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= per * M.K) return;
    int k = (int)(q / per);
    if (!M.state[2 * k]) return;
    int j = (int)((q % per) % nyf), i = (int)((q % per) / nyf);
    if (i < 1 || i > nxf - 2 || j < 1) return;
    const float2* C = M.e + (size_t)k * M.elems + M.off[l];
    auto cv = [&](int ci, int cj) { return C[(size_t)nyc * ci + cj]; };
    auto row = [&](int jj) -> float2 {
        int cj = jj / 2;
        if ((i & 1) == 0) return cv(i / 2, cj);
        float2 a = cv(i / 2, cj), b = cv(i / 2 + 1, cj);
        return f2(0.5f * (a.x + b.x), 0.5f * (a.y + b.y));
    };
    float2 t;
    if ((j & 1) == 0) t = row(j);
    else { float2 a = row(j + 1), b = row(j - 1); t = f2(0.5f * (a.x + b.x), 0.5f * (a.y + b.y)); }
    float2& fe = M.e[(size_t)k * M.elems + M.off[l - 1] + (size_t)nyf * i + j];
    fe = f2(fe.x + t.x, fe.y + t.y);
}

// x-only restriction of rr(l) into r(l+1), weights (1/4, 1/2, 1/4) in x;
// the coarse correction e(l+1) starts at 0.
__global__ void k_restrict_x(MgDev M, int l) {
    const int nxc = M.ptsx[l + 1], n = M.ptsy[l + 1];
    size_t per = (size_t)nxc * n;
    size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= per * M.K) return;
    int k = (int)(q / per);
    if (!M.state[2 * k]) return;
    int j = (int)((q % per) % n), i = (int)((q % per) / n);
    size_t oc = (size_t)k * M.elems + M.off[l + 1] + (size_t)n * i + j;
    M.e[oc] = f2(0.f, 0.f);
    float2 v = f2(0.f, 0.f);
    if (i >= 1 && i <= nxc - 2 && j >= 1) {
        const float2* D = M.rr + (size_t)k * M.elems + M.off[l] + j;
        float2 a = D[(size_t)n * (2 * i - 1)], b = D[(size_t)n * (2 * i)], c = D[(size_t)n * (2 * i + 1)];
        v = f2(0.25f * (a.x + 2.f * b.x + c.x), 0.25f * (a.y + 2.f * b.y + c.y));
    }
    M.r[oc] = v;
}

// Linear prolongation in x of e(l) added to e(l-1).
__global__ void k_prolong_x(MgDev M, int l) {
    const int nxf = M.ptsx[l - 1], n = M.ptsy[l - 1];
    size_t per = (size_t)nxf * n;
    size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= per * M.K) return;
    int k = (int)(q / per);
    if (!M.state[2 * k]) return;
    int j = (int)((q % per) % n), i = (int)((q % per) / n);
    if (i < 1 || i > nxf - 2 || j < 1) return;
    const float2* C = M.e + (size_t)k * M.elems + M.off[l] + j;
    float2 t;
    if ((i & 1) == 0) t = C[(size_t)n * (i / 2)];
    else {
        float2 a = C[(size_t)n * (i / 2)], b = C[(size_t)n * (i / 2 + 1)];
        t = f2(0.5f * (a.x + b.x), 0.5f * (a.y + b.y));
    }
    float2& fe = M.e[(size_t)k * M.elems + M.off[l - 1] + (size_t)n * i + j];
    fe = f2(fe.x + t.x, fe.y + t.y);
}

// Exact solve on the coarsest level: e = A_k^{-1} r, one warp per (mode, row).
// Unknown q is the interior point (1 + q / (n-1), 1 + q % (n-1)).
__global__ void k_direct(MgDev M) {
    const int lane = threadIdx.x & 31;
    const long gw = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int N = M.N;
    const int k = (int)(gw / N);
    if (k >= M.K || !M.state[2 * k]) return;
    const int p = (int)(gw - (long)k * N);
    const int l = M.NL - 1, n = M.ptsy[l], m = n - 1;
    const float* A = M.ainv + ((size_t)k * N + p) * N;
    const float2* R = M.r + (size_t)k * M.elems + M.off[l];
    float ax = 0.f, ay = 0.f;
    for (int q = lane; q < N; q += 32) {
        float a = A[q];
        float2 v = R[(size_t)n * (1 + q / m) + 1 + q % m];
        ax = fmaf(a, v.x, ax);
        ay = fmaf(a, v.y, ay);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ax += __shfl_xor_sync(0xffffffffu, ax, o);
        ay += __shfl_xor_sync(0xffffffffu, ay, o);
    }
    if (lane == 0) M.e[(size_t)k * M.elems + M.off[l] + (size_t)n * (1 + p / m) + 1 + p % m] = f2(ax, ay);
}

// Warm start of one stage's solve from its history h0 (previous step), h1
// (the step before), of which *valid are usable: with both, fc = 2 h0 - h1
// on the interior of the FP64 fine level (the boundary rows and columns keep
// this stage's Dirichlet data).  h1 <- h0 then makes room for this solve,
// which the caller copies into h0.
__global__ void k_extrap(cplx* fc, size_t elems64, cplx* h0, cplx* h1, const int* valid, int nx, int ny, int K,
                         int shift) {
    const int nv = *valid;
    if (nv == 0) return;
    size_t per = (size_t)nx * ny;
    size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= per * K) return;
    int k = (int)(q / per);
    int i = (int)((q % per) % nx), j = (int)((q % per) / nx);
    cplx a = h0[q];
    if (nv >= 2 && i >= 1 && i <= nx - 2 && j >= 1) {
        cplx b = h1[q];
        fc[(size_t)k * elems64 + (q % per)] = make_double2(2.0 * a.x - b.x, 2.0 * a.y - b.y);
    }
    if (shift) h1[q] = a;
}

// warm_start = 2: the previous solve's solution fc (stage p = s - 1 of this
// step, or stage 4 of the last step for s = 1) plus the increment between
// the same two solves one step earlier, fc + v_s(n-1) - v_p(n-1), from this
// stage's newest history entry h0 and stage p's older one hp1.  Stages 2 and 4
// solve at the same time as the stage before them, so the increment is the
// difference of two RK stage estimates and changes by O(dt^3) per step;
// stages 1 and 3 carry half a step of time change, O(dt^2) with half the
// constant of the linear extrapolation.  Needs one entry of this stage's
// history and two of stage p's; shifts this stage's history as k_extrap.
__global__ void k_extrap_inc(cplx* fc, size_t elems64, cplx* h0, cplx* h1, const cplx* hp1, const int* valid,
                             const int* valid_p, int nx, int ny, int K, int shift) {
    const int nv = *valid, np = *valid_p;
    if (nv == 0) return;
    const size_t per = (size_t)nx * ny;
    const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= per * K) return;
    const int k = (int)(q / per);
    const int i = (int)((q % per) % nx), j = (int)((q % per) / nx);
    const cplx a = h0[q];
    if (np >= 2 && i >= 1 && i <= nx - 2 && j >= 1) {
        cplx& f = fc[(size_t)k * elems64 + (q % per)];
        const cplx b = hp1[q];
        f = make_double2(f.x + (a.x - b.x), f.y + (a.y - b.y));
    }
    if (shift) h1[q] = a;
}

// ---- learned first correction (network and training in tb_learn.cu) -------
// Per mode maxima over both parts of |v1| and |v1 - v2| (history,
// x-contiguous) and of |D^-1 d0| (d0: the FP32 copy r of the FP64 defect of
// the guess, line-contiguous), as float bits in scl (K, 3).
__global__ void k_learn_scale(MgDev M, const cplx* h0, const cplx* h1, const int* valid, unsigned* scl, const float* invD,
                              int nx) {
    if (*valid < 2) return;
    const int k = blockIdx.y, ny = M.ny;
    const size_t per = (size_t)nx * ny;
    float a = 0.f, b = 0.f, d = 0.f;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < per; q += (size_t)gridDim.x * blockDim.x) {
        const cplx u = h0[(size_t)k * per + q], w = h1[(size_t)k * per + q];
        a = fmaxf(a, fmaxf(fabsf((float)u.x), fabsf((float)u.y)));
        b = fmaxf(b, fmaxf(fabsf((float)(u.x - w.x)), fabsf((float)(u.y - w.y))));
        const float2 r = M.r[(size_t)k * M.elems + M.off[0] + q];   // point (q / ny, q % ny)
        d = fmaxf(d, invD[(size_t)k * ny + q % ny] * fmaxf(fabsf(r.x), fabsf(r.y)));
    }
    for (int o = 16; o > 0; o >>= 1) {
        a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
        b = fmaxf(b, __shfl_xor_sync(0xffffffffu, b, o));
        d = fmaxf(d, __shfl_xor_sync(0xffffffffu, d, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&scl[3 * k], __float_as_uint(a));
        atomicMax(&scl[3 * k + 1], __float_as_uint(b));
        atomicMax(&scl[3 * k + 2], __float_as_uint(d));
    }
}

// The network's input planes X (2K, 4, nx, ny) and the history shift
// h1 <- h0 that k_extrap leaves to this kernel when the network runs.
__global__ void k_learn_prep(MgDev M, const cplx* h0, cplx* h1, const int* valid, const float* scl, const float* invD,
                             const float* mfeat, float* X, int nx) {
    const int nv = *valid;
    if (nv == 0) return;
    __shared__ float2 t0[32][33], t1[32][33];   // [j][i]: v1, v1 - v2
    const int k = blockIdx.z, ny = M.ny, i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
    const size_t per = (size_t)nx * ny;
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int i = i0 + threadIdx.x, j = j0 + r;
        float2 a = f2(0.f, 0.f), b = f2(0.f, 0.f);
        if (i < nx && j < ny) {
            const size_t o = (size_t)k * per + (size_t)j * nx + i;
            const cplx u = h0[o], w = h1[o];
            a = f2((float)u.x, (float)u.y);
            b = f2((float)(u.x - w.x), (float)(u.y - w.y));
            h1[o] = u;
        }
        t0[r][threadIdx.x] = a;
        t1[r][threadIdx.x] = b;
    }
    if (nv < 2) return;   // uniform over the block
    __syncthreads();
    // one scale for the three field planes: s = max|v1 - v2|
    const float si = scl[3 * k + 1];
    const float ii = si > 0.f ? 1.f / si : 0.f, iv = ii, id = ii;
    float* Xr = X + (size_t)(2 * k) * 4 * per;   // planes of the real part, then of the imaginary part
    float* Xi = Xr + 4 * per;
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int i = i0 + r, j = j0 + threadIdx.x;
        if (i >= nx || j >= ny) continue;
        const float2 a = t0[threadIdx.x][r], b = t1[threadIdx.x][r];
        const float2 d = M.r[(size_t)k * M.elems + M.off[0] + (size_t)ny * i + j];
        const float sj = invD[(size_t)k * ny + j] * id, mf = mfeat[(size_t)k * ny + j];
        const size_t o = (size_t)ny * i + j;
        Xr[o] = a.x * iv; Xr[per + o] = b.x * ii; Xr[2 * per + o] = d.x * sj; Xr[3 * per + o] = mf;
        Xi[o] = a.y * iv; Xi[per + o] = b.y * ii; Xi[2 * per + o] = d.y * sj; Xi[3 * per + o] = mf;
    }
}

// Candidate correction e = max|v1 - v2| * network output on the fine interior.
__global__ void k_learn_emit(MgDev M, const float* out, const float* scl, const int* valid, int nx) {
    if (*valid < 2) return;
    const int ny = M.ny;
    const size_t per = (size_t)(nx - 2) * (ny - 1), img = (size_t)nx * ny;
    const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= per * M.K) return;
    const int k = (int)(q / per);
    const size_t rq = q % per;
    const int j = 1 + (int)(rq % (ny - 1)), i = 1 + (int)(rq / (ny - 1));
    const float s = scl[3 * k + 1];
    const size_t o = (size_t)ny * i + j;
    M.e[(size_t)k * M.elems + M.off[0] + o] = f2(s * out[(size_t)(2 * k) * img + o], s * out[(size_t)(2 * k + 1) * img + o]);
}

// max |r - L e|^2 per mode (blockIdx.y) over the fine interior, float bits.
__global__ void k_learn_judge(MgDev M, unsigned* jmax, const int* valid, int nx) {
    if (*valid < 2) return;
    const int k = blockIdx.y, ny = M.ny;
    const size_t per = (size_t)(nx - 2) * (ny - 1);
    float m = 0.f;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < per; q += (size_t)gridDim.x * blockDim.x) {
        const int j = 1 + (int)(q % (ny - 1)), i = 1 + (int)(q / (ny - 1));
        const float2 v = M.rr[(size_t)k * M.elems + M.off[0] + (size_t)ny * i + j];
        m = fmaxf(m, v.x * v.x + v.y * v.y);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&jmax[k], __float_as_uint(m));
}

// Gated evaluation of the network for one stage's solve.  It runs the first
// time, once every `probe` solves, and in the solve after one where it ran
// and the solve needed fewer corrections than the stage's last solve
// without it: the network is kept on only while it saves multigrid work;
// otherwise the solve falls back to the warm-start guess without running it.
// g (per stage): [solves since it last ran, ran in the last solve,
// evaluations, solves, corrections of the last solve without it, of the
// last solve with it].  The decision goes to a conditional graph node (h)
// or, for host-launched solves, to *flag.
__global__ void k_learn_gate(int* g, int probe, cudaGraphConditionalHandle h, int use_handle, int* flag) {
    const int saved = g[1] && g[5] < g[4];
    const int run = (g[2] == 0 || saved || g[0] >= probe - 1) ? 1 : 0;
    if (run) { g[0] = 0; g[2] += 1; }
    else g[0] += 1;
    g[1] = run;
    g[3] += 1;
    if (use_handle) cudaGraphSetConditional(h, (unsigned)run);
    else *flag = run;
}

// After a gated solve: its corrections (the largest count over the modes)
// into the stage's slot for solves with or without the network.
__global__ void k_learn_after(const int* state, int K, int* g) {
    int c = 0;
    for (int k = 0; k < K; k++) {
        int v = state[2 * k + 1];
        if (v < 0) v = -v - 1;
        c = max(c, v);
    }
    if (g[1]) g[5] = c;
    else g[4] = c;
}

// Keep the candidate for a mode when it lowers the max defect by 5% or more
// (max|d0 - L e|^2 < 0.9 max|d0|^2: a zero correction, whose FP32 defect
// differs from the FP64 one by rounding only, is never kept); count the
// solves tried and the corrections kept; clear the maxima for the loop.
__global__ void k_learn_keep(unsigned long long* maxsq, unsigned* jmax, int* keep, long long* tally, const int* valid,
                             int K, int* gate_kept) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    int ok = 0;
    if (*valid >= 2) {
        const double d0 = __longlong_as_double((long long)maxsq[k]);
        const double d1 = (double)__uint_as_float(jmax[k]);
        ok = d1 < 0.9 * d0;
        tally[2 * k] += 1;
        tally[2 * k + 1] += ok;
        if (ok && gate_kept) atomicAdd(gate_kept, 1);
    }
    keep[2 * k] = ok;
    keep[2 * k + 1] = 0;
    maxsq[k] = 0ull;
    jmax[k] = 0u;
}

__global__ void k_hist_count(int* valid) { *valid = min(*valid + 1, 2); }

// u += e on the interior of the FP64 fine level (fc layout: x-contiguous).
__global__ void k_apply(MgDev M, cplx* fc, size_t elems64, int nx, int ny) {
    __shared__ float2 tile[32][33];
    const int k = blockIdx.z;
    if (!M.state[2 * k]) return;
    const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += 8) {
        int i = i0 + r, j = j0 + threadIdx.x;
        float2 v = f2(0.f, 0.f);
        if (i < nx && j < ny) v = M.e[(size_t)k * M.elems + M.off[0] + (size_t)ny * i + j];
        tile[threadIdx.x][r] = v;
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += 8) {
        int i = i0 + threadIdx.x, j = j0 + r;
        if (i >= 1 && i <= nx - 2 && j >= 1 && j < ny) {
            float2 e = tile[r][threadIdx.x];
            cplx& u = fc[(size_t)k * elems64 + (size_t)i + (size_t)nx * j];
            u = make_double2(u.x + (double)e.x, u.y + (double)e.y);
        }
    }
}

// Per-mode test of the FP64 defect (max |d| over the interior, as
// get_max_value/verifica_poi, from the max |d|^2 the defect kernel folded
// into maxsq): converged modes leave the active set with the number of
// corrections applied; a non-finite defect stops the mode with
// -1 - corrections.  maxsq is cleared for the next defect.
__device__ __forceinline__ int check_mode(unsigned long long* maxsq, int* state, double* err, int k, double tol, int it,
                                          int last) {
    if (!state[2 * k]) return 0;
    double m2 = __longlong_as_double((long long)maxsq[k]);
    maxsq[k] = 0ull;
    double e = sqrt(m2);
    if (!(e <= 1.7e308)) { err[k] = __longlong_as_double(0x7ff8000000000000LL); state[2 * k] = 0; state[2 * k + 1] = -1 - it; }
    else {
        err[k] = e;
        if (e < tol) { state[2 * k] = 0; state[2 * k + 1] = it; }
        else if (last) state[2 * k + 1] = it;   // stays active: not converged
    }
    return state[2 * k];
}
__global__ void k_check_sq(unsigned long long* maxsq, int* state, double* err, int K, double tol, int it, int last) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < K) check_mode(maxsq, state, err, k, tol, it, last);
}
// The same test inside a recorded solve (one block): the correction count
// lives in *iter, and the loop's WHILE condition becomes "some mode is still
// active and fewer than max_outer corrections were applied".
constexpr int CHECK_THREADS = 256;
__global__ void __launch_bounds__(CHECK_THREADS) k_check_loop(unsigned long long* maxsq, int* state, double* err, int K,
                                                              double tol, int* iter, int first, int max_outer,
                                                              cudaGraphConditionalHandle h) {
    const int it = first ? 0 : *iter;
    int act = 0;
    for (int k = threadIdx.x; k < K; k += blockDim.x) act |= check_mode(maxsq, state, err, k, tol, it, it == max_outer);
    act = __syncthreads_or(act);
    if (threadIdx.x == 0) {
        *iter = it + 1;
        cudaGraphSetConditional(h, (act && it < max_outer) ? 1u : 0u);
    }
}

Mixed* get(tb_ctx* c) { return static_cast<Mixed*>(c->mixed); }

MgDev make(tb_ctx* c) {
    Mixed* m = get(c);
    MgDev M;
    std::memset(&M, 0, sizeof M);
    M.e = m->e; M.r = m->r; M.rr = m->rr; M.tab = m->tab; M.coef = m->coef; M.qdy2 = m->qdy2; M.ainv = m->ainv;
    M.k2b2 = c->k2b2; M.state = c->pstate;
    M.ny = c->g.ny; M.K = c->g.K; M.NL = m->NL; M.N = m->N;
    for (int l = 0; l < m->NL; l++) {
        M.ptsx[l] = m->ptsx[l]; M.ptsy[l] = m->ptsy[l]; M.ylvl[l] = m->ylvl[l]; M.off[l] = m->off[l];
        M.qx[l] = (float)(1.0 / (12.0 * m->dx2[l] * c->cfg.fac_y));
    }
    M.elems = m->elems;
    M.bs = tb_poi_blk_size(c->g.ny);
    M.ify = (float)(1.0 / c->cfg.fac_y);
    M.alpha2 = (float)(c->cfg.alpha * c->cfg.alpha);
    return M;
}

// Rows per lane of the line solve: the smallest instantiated S with 32 S >= n.
int pick_S(int n) {
    static const int opts[] = {2, 3, 4, 5, 6, 7, 8, 10, 12, 16};
    for (int s : opts)
        if (32 * s >= n) return s;
    return 16;
}

template <class T>
int upl(T** d, const std::vector<T>& h) {
    if (*d) cudaFree(*d);
    *d = nullptr;
    TB_CUDA(cudaMalloc((void**)d, h.size() * sizeof(T)));
    TB_CUDA(cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return TB_OK;
}

// The level operator L (defect, poisson_par.f:543-793) at interior point
// (i, j) of a level with nxl x n points, applied to u (line-contiguous), FP64.
struct HostOp {
    const double *SP, *CP, *PP, *LP, *Q2;
    double den, ify, k2b2, topc;
    int nxl, n;
    double apply(const std::vector<double>& u, int i, int j) const {
        auto f = [&](int ii, int jj) { return u[(size_t)n * ii + jj]; };
        auto bx = [&](int jj) {
            if (i == 1 || i == nxl - 2) {
                int e = (i == 1) ? 1 : -1;
                return 10.0 * f(i - e, jj) - 15.0 * f(i, jj) - 4.0 * f(i + e, jj) + 14.0 * f(i + 2 * e, jj) -
                       6.0 * f(i + 3 * e, jj) + f(i + 4 * e, jj);
            }
            return -f(i - 2, jj) + 16.0 * f(i - 1, jj) - 30.0 * f(i, jj) + 16.0 * f(i + 1, jj) - f(i + 2, jj);
        };
        double b, cc, d, q2, top = 0.0;
        if (j == 1) {
            b = SP[2] * bx(2) + SP[1] * bx(1);
            cc = SP[3] * f(i, 0) + SP[4] * f(i, 1) + SP[5] * f(i, 2) + SP[6] * f(i, 3);
            d = k2b2 * (SP[1] * f(i, 1) + SP[2] * f(i, 2));
            q2 = Q2[0];
        } else if (j <= n - 3) {
            b = CP[0] * bx(j - 1) + CP[1] * bx(j) + CP[2] * bx(j + 1);
            cc = CP[3] * f(i, j - 2) + CP[4] * f(i, j - 1) + CP[5] * f(i, j) + CP[6] * f(i, j + 1) + CP[7] * f(i, j + 2);
            d = k2b2 * (CP[0] * f(i, j - 1) + CP[1] * f(i, j) + CP[2] * f(i, j + 1));
            q2 = Q2[j - 2];
        } else if (j == n - 2) {
            b = bx(j);
            cc = PP[3] * f(i, j + 1) + PP[2] * f(i, j) + PP[1] * f(i, j - 1);
            d = k2b2 * f(i, j);
            q2 = Q2[j - 1];
        } else {
            b = bx(j);
            cc = LP[2] * f(i, j) + LP[3] * f(i, j - 1) + LP[4] * f(i, j - 2);
            d = k2b2 * f(i, j);
            q2 = Q2[j - 2];
            top = LP[1] * topc * std::sqrt(q2);
        }
        return b * den + cc * q2 + d * ify - top * f(i, j);
    }
};

// Inverse of the coarsest-level operator of one mode (N x N, row-major),
// by Gauss-Jordan elimination with partial pivoting in FP64.
bool coarse_inverse(const HostOp& op, int N, float* out) {
    const int nxl = op.nxl, n = op.n, m = n - 1;
    std::vector<double> A((size_t)N * N, 0.0), X((size_t)N * N, 0.0), u((size_t)nxl * n, 0.0);
    for (int q = 0; q < N; q++) {
        int iq = 1 + q / m, jq = 1 + q % m;
        u[(size_t)n * iq + jq] = 1.0;
        for (int i = std::max(1, iq - 4); i <= std::min(nxl - 2, iq + 4); i++)
            for (int j = std::max(1, jq - 3); j <= std::min(n - 1, jq + 3); j++)
                A[(size_t)((i - 1) * m + (j - 1)) * N + q] = op.apply(u, i, j);
        u[(size_t)n * iq + jq] = 0.0;
    }
    for (int p = 0; p < N; p++) X[(size_t)p * N + p] = 1.0;
    for (int c = 0; c < N; c++) {
        int piv = c;
        for (int p = c + 1; p < N; p++)
            if (std::fabs(A[(size_t)p * N + c]) > std::fabs(A[(size_t)piv * N + c])) piv = p;
        if (A[(size_t)piv * N + c] == 0.0) return false;
        if (piv != c)
            for (int q = 0; q < N; q++) {
                std::swap(A[(size_t)piv * N + q], A[(size_t)c * N + q]);
                std::swap(X[(size_t)piv * N + q], X[(size_t)c * N + q]);
            }
        double inv = 1.0 / A[(size_t)c * N + c];
        for (int q = 0; q < N; q++) { A[(size_t)c * N + q] *= inv; X[(size_t)c * N + q] *= inv; }
        for (int p = 0; p < N; p++) {
            if (p == c) continue;
            double f = A[(size_t)p * N + c];
            if (f == 0.0) continue;
            for (int q = 0; q < N; q++) {
                A[(size_t)p * N + q] -= f * A[(size_t)c * N + q];
                X[(size_t)p * N + q] -= f * X[(size_t)c * N + q];
            }
        }
    }
    for (size_t q = 0; q < X.size(); q++) out[q] = (float)X[q];
    return true;
}

int launch_relax(tb_ctx* c, const MgDev& M, int S, int l, int first, int step, int nlines) {
    cudaEvent_t p0 = nullptr;
    int r;
    if (l == 0 && (r = tb_prof_begin(c, PROF_RELAX0, &p0))) return r;
    int nw = nlines * c->g.K;
    unsigned nb = tb_blocks((size_t)nw, RELAX_THREADS / 32);
    size_t smem = (size_t)(RELAX_THREADS / 32) * 2 * M.ptsy[l] * sizeof(float2);
    cudaStream_t st = c->stream;
    switch (S) {
        case 2: k_relax<2><<<nb, RELAX_THREADS, smem, st>>>(M, l, first, step, nlines); break;
        case 3: k_relax<3><<<nb, RELAX_THREADS, smem, st>>>(M, l, first, step, nlines); break;
        case 4: k_relax<4><<<nb, RELAX_THREADS, smem, st>>>(M, l, first, step, nlines); break;
        case 5: k_relax<5><<<nb, RELAX_THREADS, smem, st>>>(M, l, first, step, nlines); break;
        case 6: k_relax<6><<<nb, RELAX_THREADS, smem, st>>>(M, l, first, step, nlines); break;
        case 7: k_relax<7><<<nb, RELAX_THREADS, smem, st>>>(M, l, first, step, nlines); break;
        case 8: k_relax<8><<<nb, RELAX_THREADS, smem, st>>>(M, l, first, step, nlines); break;
        case 10: k_relax<10><<<nb, RELAX_THREADS, smem, st>>>(M, l, first, step, nlines); break;
        case 12: k_relax<12><<<nb, RELAX_THREADS, smem, st>>>(M, l, first, step, nlines); break;
        default: k_relax<16><<<nb, RELAX_THREADS, smem, st>>>(M, l, first, step, nlines); break;
    }
    TB_CHECK_LAUNCH(c);
    return l == 0 ? tb_prof_end(c, PROF_RELAX0, p0) : TB_OK;
}

// One relaxation sweep at level l: border lines, then centre colours 0, 1, 2.
int sweep(tb_ctx* c, const MgDev& M, int l) {
    Mixed* m = get(c);
    int nxl = m->ptsx[l], r;
    cudaEvent_t ps = nullptr;
    if ((r = tb_prof_begin(c, PROF_SOR, &ps))) return r;
    if ((r = launch_relax(c, M, m->S[l], l, 1, nxl - 3, 2))) return r;
    for (int col = 0; col < 3; col++) {
        int first = 2 + col;
        if (first > nxl - 3) break;
        int nl = (nxl - 3 - first) / 3 + 1;
        if ((r = launch_relax(c, M, m->S[l], l, first, 3, nl))) return r;
    }
    return tb_prof_end(c, PROF_SOR, ps);
}

int vcycle(tb_ctx* c, const MgDev& M) {
    Mixed* m = get(c);
    const int K = c->g.K, NL = m->NL;
    int r;
    for (int l = 0; l < NL - 1; l++) {
        for (int s = 0; s < NU_PRE; s++)
            if ((r = sweep(c, M, l))) return r;
        size_t per = (size_t)(m->ptsx[l] - 2) * (m->ptsy[l] - 1) * K;
        k_resid<<<tb_blocks(per, 256), 256, 0, c->stream>>>(M, l);
        TB_CHECK_LAUNCH(c);
        size_t pc = (size_t)m->ptsx[l + 1] * m->ptsy[l + 1] * K;
        if (m->semi[l]) k_restrict_x<<<tb_blocks(pc, 256), 256, 0, c->stream>>>(M, l);
        else k_restrict32<<<tb_blocks(pc, 256), 256, 0, c->stream>>>(M, l);
        TB_CHECK_LAUNCH(c);
    }
    k_direct<<<tb_blocks((size_t)K * m->N, 8), 256, 0, c->stream>>>(M);
    TB_CHECK_LAUNCH(c);
    for (int l = NL - 1; l >= 1; l--) {
        size_t pf = (size_t)m->ptsx[l - 1] * m->ptsy[l - 1] * K;
        if (m->semi[l - 1]) k_prolong_x<<<tb_blocks(pf, 256), 256, 0, c->stream>>>(M, l);
        else k_prolong32<<<tb_blocks(pf, 256), 256, 0, c->stream>>>(M, l);
        TB_CHECK_LAUNCH(c);
        for (int s = 0; s < NU_POST; s++)
            if ((r = sweep(c, M, l - 1))) return r;
    }
    return TB_OK;
}

}  // namespace

int tb_mixed_setup(tb_ctx* c) {
    tb_mixed_free(c);
    const int K = c->g.K, ny = c->g.ny, msh = c->g.msh;
    Mixed* m = new Mixed();
    c->mixed = m;
    // hierarchy: x-only coarsening while dx < max dy (if enabled), the
    // reference's y-levels with x and y halved together, then x-only
    // coarsening down to a level small enough for the direct solve
    double dy_max = 0.0;
    for (int j = 0; j + 1 < ny; j++) dy_max = std::max(dy_max, 1.0 / c->h_qdy[j]);
    auto push = [&](int px, int py, int yl, double dx2) {
        int l = m->NL++;
        m->ptsx[l] = px; m->ptsy[l] = py; m->ylvl[l] = yl; m->dx2[l] = dx2; m->semi[l] = 0;
    };
    m->NL = 0;
    push(c->g.nx, ny, 0, c->h_dx2[0]);
    const int full_steps = msh - 1, fdiv = 1 << full_steps;
    while (TB_MG_SEMI_FIRST && m->NL < MG_MAX - msh) {
        int l = m->NL - 1, px = m->ptsx[l];
        int pxn = (px + 1) / 2;
        if (std::sqrt(m->dx2[l]) >= dy_max || (px - 1) % 2 || (pxn - 1) % fdiv || (pxn - 1) / fdiv + 1 < 10) break;
        m->semi[l] = 1;
        push(pxn, m->ptsy[l], 0, 4.0 * m->dx2[l]);
    }
    for (int yl = 1; yl <= full_steps; yl++) {
        int l = m->NL - 1;
        push((m->ptsx[l] + 1) / 2, c->g.ptsy[yl], yl, 4.0 * m->dx2[l]);
    }
    while (m->NL < MG_MAX) {
        int l = m->NL - 1, px = m->ptsx[l], py = m->ptsy[l];
        if ((long)(px - 2) * (py - 1) <= DIRECT_MAX || (px - 1) % 2 || (px + 1) / 2 < 10) break;
        m->semi[l] = 1;
        push((px + 1) / 2, py, m->ylvl[l], 4.0 * m->dx2[l]);
    }
    const int NL = m->NL, lc = NL - 1;
    if (m->ptsx[lc] < 10) {
        tb_set_error("mixed form needs at least 10 points in x on the coarsest level (got %d)", m->ptsx[lc]);
        return TB_ERR_ARG;
    }
    m->N = (m->ptsx[lc] - 2) * (m->ptsy[lc] - 1);
    if (m->N > DIRECT_LIMIT) {
        tb_set_error("mixed form: coarsest level has %d unknowns per mode (limit %d); raise msh", m->N, DIRECT_LIMIT);
        return TB_ERR_ARG;
    }
    size_t off = 0;
    for (int l = 0; l < NL; l++) { m->off[l] = off; off += (size_t)m->ptsx[l] * m->ptsy[l]; m->S[l] = pick_S(m->ptsy[l]); }
    m->elems = off;
    size_t w = (size_t)K * m->elems;
    for (float2** p : {&m->e, &m->r, &m->rr}) {
        TB_CUDA(cudaMalloc(p, w * sizeof(float2)));
        TB_CUDA(cudaMemset(*p, 0, w * sizeof(float2)));
    }
    TB_CUDA(cudaMalloc(&m->maxsq, K * sizeof(unsigned long long)));
    TB_CUDA(cudaMemset(m->maxsq, 0, K * sizeof(unsigned long long)));
    TB_CUDA(cudaMalloc(&m->hvalid, 4 * sizeof(int)));
    TB_CUDA(cudaMemset(m->hvalid, 0, 4 * sizeof(int)));
    TB_CUDA(cudaMalloc(&m->iter, sizeof(int)));
    TB_CUDA(cudaMemset(m->iter, 0, sizeof(int)));
    TB_CUDA(cudaMalloc(&m->lkeep, 2 * K * sizeof(int)));
    TB_CUDA(cudaMemset(m->lkeep, 0, 2 * K * sizeof(int)));
    if (c->cfg.warm_start)
        for (auto& h : m->hist)
            for (cplx*& p : h) TB_CUDA(cudaMalloc(&p, tb_n3(c) * sizeof(cplx)));
    // line-solve tables per (type, level, mode): band5 factors of the level's
    // y-line matrix and chunk tables for this form's rows per lane, in FP32
    const size_t bs = tb_poi_blk_size(ny);
    std::vector<float> t32((size_t)2 * NL * K * bs, 0.f);
    std::vector<double> a, blk(bs);
    for (int type = 0; type < 2; type++)
        for (int l = 0; l < NL; l++)
            for (int k = 0; k < K; k++) {
                int n = m->ptsy[l];
                std::fill(blk.begin(), blk.end(), 0.0);
                tb_poisson_band_matrix_dx(c, type, m->ylvl[l] + 1, k + 1, m->dx2[l], a);
                tb_band5_factor(n, a, &blk[0], &blk[ny], &blk[2 * ny], &blk[3 * ny], &blk[4 * ny]);
                tb_chunk_tables(n, ny, m->S[l], &blk[0], &blk[ny], &blk[2 * ny], &blk[3 * ny], &blk[4 * ny], &blk[5 * ny]);
                float* D = &t32[(((size_t)type * NL + l) * K + k) * bs];
                for (size_t q = 0; q < bs; q++) D[q] = (float)blk[q];
            }
    int r;
    if ((r = upl(&m->tab, t32))) return r;
    const double* blob = c->coefs.data();
    std::vector<double> cf64((size_t)24 * msh);
    for (int l = 0; l < msh; l++) {   // sp_poi(7,msh) cp_poi(8,msh) pp_poi(4,msh) lp_poi(5,msh) from blob[83]
        for (int q = 0; q < 7; q++) cf64[24 * l + q] = blob[83 + 7 * l + q];
        for (int q = 0; q < 8; q++) cf64[24 * l + 7 + q] = blob[83 + 7 * msh + 8 * l + q];
        for (int q = 0; q < 4; q++) cf64[24 * l + 15 + q] = blob[83 + 15 * msh + 4 * l + q];
        for (int q = 0; q < 5; q++) cf64[24 * l + 19 + q] = blob[83 + 19 * msh + 5 * l + q];
    }
    std::vector<float> cf(cf64.begin(), cf64.end());
    if ((r = upl(&m->coef, cf))) return r;
    std::vector<float> q2(c->h_qdy2.begin(), c->h_qdy2.end());
    if ((r = upl(&m->qdy2, q2))) return r;
    // exact inverse of the coarsest operator per mode (modes in parallel)
    const int N = m->N;
    std::vector<float> ainv((size_t)K * N * N);
    std::vector<int> ok(K, 0);
    auto work = [&](int k0, int k1) {
        for (int k = k0; k < k1; k++) {
            HostOp op;
            const double* base = &cf64[24 * m->ylvl[lc]];
            op.SP = base; op.CP = base + 7; op.PP = base + 15; op.LP = base + 19;
            op.Q2 = &c->h_qdy2[(size_t)ny * m->ylvl[lc]];
            op.den = 1.0 / (12.0 * m->dx2[lc] * c->cfg.fac_y);
            op.ify = 1.0 / c->cfg.fac_y;
            op.k2b2 = c->h_k2b2[k];
            op.topc = std::sqrt((c->cfg.alpha * c->cfg.alpha - op.k2b2) / c->cfg.fac_y);
            op.nxl = m->ptsx[lc]; op.n = m->ptsy[lc];
            ok[k] = coarse_inverse(op, N, &ainv[(size_t)k * N * N]);
        }
    };
    int nt = (int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), (unsigned)K);
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++) th.emplace_back(work, K * t / nt, K * (t + 1) / nt);
    for (auto& t : th) t.join();
    for (int k = 0; k < K; k++)
        if (!ok[k]) { tb_set_error("mixed form: coarsest operator of mode %d is singular", k); return TB_ERR_ARG; }
    if ((r = upl(&m->ainv, ainv))) return r;
    return TB_OK;
}

void tb_mixed_invalidate(tb_ctx* c) {
    Mixed* m = get(c);
    if (!m) return;
    for (int& t : m->last_t) t = -9;
    for (int& v : m->hv_host) v = 0;
}

int tb_mixed_graph_pre(tb_ctx* c, int t, cudaStream_t s) {
    Mixed* m = get(c);
    if (!m) { tb_set_error("mixed form not set up"); return TB_ERR_STATE; }
    for (int q = 0; q < 4; q++)
        if (m->last_t[q] != t - 1) TB_CUDA(cudaMemsetAsync(m->hvalid + q, 0, sizeof(int), s));
    return TB_OK;
}

void tb_mixed_graph_post(tb_ctx* c, int t) {
    Mixed* m = get(c);
    if (!m || !c->cfg.warm_start) return;
    for (int q = 0; q < 4; q++) {
        m->hv_host[q] = m->last_t[q] == t - 1 ? std::min(m->hv_host[q] + 1, 2) : 1;
        m->last_t[q] = t;
    }
}

void tb_mixed_free(tb_ctx* c) {
    Mixed* m = get(c);
    if (!m) return;
    for (auto& h : m->hist)
        for (cplx* p : h)
            if (p) cudaFree(p);
    for (void* p : {(void*)m->e, (void*)m->r, (void*)m->rr, (void*)m->tab, (void*)m->coef, (void*)m->qdy2, (void*)m->ainv,
                    (void*)m->maxsq, (void*)m->hvalid, (void*)m->iter, (void*)m->lkeep})
        if (p) cudaFree(p);
    delete m;
    c->mixed = nullptr;
}

// One FP64 correction recorded as the body of the solve's WHILE node:
// INNER_VCYCLES V-cycles of the FP32 hierarchy, u += e, the new defect and
// its test (which sets the loop condition).
static int record_body(tb_ctx* c, const MgDev& M, double erro, cudaGraphConditionalHandle h) {
    Mixed* m = get(c);
    int r;
    for (int v = 0; v < INNER_VCYCLES; v++)
        if ((r = vcycle(c, M))) return r;
    dim3 tgrid(tb_blocks(c->g.nx, 32), tb_blocks(c->g.ny, 32), c->g.K), tblk(32, 8);
    k_apply<<<tgrid, tblk, 0, c->stream>>>(M, c->pfc, c->g.lvl_elems, c->g.nx, c->g.ny);
    TB_CHECK_LAUNCH(c);
    if ((r = tb_poisson_defect_f32(c, m->r, m->e, m->elems, m->maxsq))) return r;
    k_check_loop<<<1, CHECK_THREADS, 0, c->stream>>>(m->maxsq, c->pstate, c->perr, c->g.K, erro, m->iter, 0,
                                                     c->cfg.max_vcycles, h);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}

// The correction loop of a solve being recorded into a step graph: first
// defect and test, then a conditional WHILE node that repeats the body
// above until every mode has converged or max_vcycles corrections ran.
static int record_loop(tb_ctx* c, const MgDev& M, double erro) {
    Mixed* m = get(c);
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    TB_CUDA(cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &g, nullptr, nullptr, nullptr));
    if (st != cudaStreamCaptureStatusActive || !g) { tb_set_error("step graph: stream is not recording"); return TB_ERR_STATE; }
    cudaGraphConditionalHandle h;
    TB_CUDA(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
    int r;
    if ((r = tb_poisson_defect_f32(c, m->r, m->e, m->elems, m->maxsq))) return r;
    k_check_loop<<<1, CHECK_THREADS, 0, c->stream>>>(m->maxsq, c->pstate, c->perr, c->g.K, erro, m->iter, 1,
                                                     c->cfg.max_vcycles, h);
    TB_CHECK_LAUNCH(c);
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    TB_CUDA(cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &g, &deps, nullptr, &nd));
    cudaGraphNodeParams p = {};
    std::memset(&p, 0, sizeof p);
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    TB_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
    TB_CUDA(cudaStreamUpdateCaptureDependencies(c->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraph_t body = p.conditional.phGraph_out[0];
    cudaStream_t outer = c->stream;
    c->stream = c->body_stream;
    const long long l0 = c->launches;
    cudaError_t e = cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) {
        c->stream = outer;
        tb_set_error("step graph: recording the solve loop: %s", cudaGetErrorString(e));
        return TB_ERR_CUDA;
    }
    r = record_body(c, M, erro, h);
    cudaGraph_t got = nullptr;
    e = cudaStreamEndCapture(c->stream, &got);
    c->stream = outer;
    if (r) return r;
    if (e != cudaSuccess) { tb_set_error("step graph: recording the solve loop: %s", cudaGetErrorString(e)); return TB_ERR_CUDA; }
    if (c->g_stage >= 1 && c->g_stage <= 4) c->g_body[c->g_stage - 1] = c->launches - l0;
    return TB_OK;
}

// 1 / |diagonal| of the fine y-line operator per mode and row, and the share
// of k^2 beta^2 in it (rows j >= 1; the wall row is Dirichlet: 0).
int tb_mixed_line_diag(tb_ctx* c, std::vector<float>& invD, std::vector<float>& mfeat) {
    const int K = c->g.K, ny = c->g.ny;
    invD.assign((size_t)K * ny, 0.f);
    mfeat.assign((size_t)K * ny, 0.f);
    std::vector<double> a, a0;
    tb_poisson_band_matrix_dx(c, 0, 1, 1, c->h_dx2[0], a0);
    for (int k = 0; k < K; k++) {
        tb_poisson_band_matrix_dx(c, 0, 1, k + 1, c->h_dx2[0], a);
        const int n = (int)(a.size() / 5);
        if (n != ny) { tb_set_error("line operator has %d rows, expected %d", n, ny); return TB_ERR_STATE; }
        for (int j = 1; j < ny; j++) {
            const double d = a[(size_t)j + (size_t)n * 2], d0 = a0[(size_t)j + (size_t)n * 2];
            if (d != 0.0) {
                invD[(size_t)k * ny + j] = (float)(1.0 / std::fabs(d));
                mfeat[(size_t)k * ny + j] = (float)(std::fabs(d - d0) / std::fabs(d));
            }
        }
    }
    return TB_OK;
}

// The learned first correction of stage ws's solve, before the loop: the
// FP64 defect d0 of the extrapolated guess, the network's inputs (which also
// shift the stage's history), then (when applying the network) its candidate
// correction, kept per mode where max|d0 - L e| < max|d0|.  While sampling,
// the guess is kept for the training targets.
static int learned_first(tb_ctx* c, const MgDev& M, int ws, LearnSolve* L) {
    Mixed* m = get(c);
    const int K = c->g.K, nx = c->g.nx, ny = c->g.ny;
    int r;
    if ((r = tb_poisson_defect_f32(c, m->r, m->e, m->elems, m->maxsq))) return r;
    TB_CUDA(cudaMemsetAsync(L->scl, 0, 3 * K * sizeof(float), c->stream));
    const int* valid = m->hvalid + ws;
    cplx *h0 = m->hist[ws][0], *h1 = m->hist[ws][1];
    const unsigned nb = std::min<unsigned>(tb_blocks((size_t)nx * ny, 256), 64);
    k_learn_scale<<<dim3(nb, K), 256, 0, c->stream>>>(M, h0, h1, valid, reinterpret_cast<unsigned*>(L->scl), L->invD, nx);
    TB_CHECK_LAUNCH(c);
    k_learn_prep<<<dim3(tb_blocks(nx, 32), tb_blocks(ny, 32), K), dim3(32, 8), 0, c->stream>>>(M, h0, h1, valid, L->scl,
                                                                                             L->invD, L->mfeat, L->X, nx);
    TB_CHECK_LAUNCH(c);
    if (L->sample) {
        const size_t pitch = c->g.lvl_elems * sizeof(cplx);
        TB_CUDA(cudaMemcpy2DAsync(L->g0, pitch, c->pfc, pitch, (size_t)nx * ny * sizeof(cplx), K, cudaMemcpyDeviceToDevice,
                                  c->stream));
    }
    if (!L->infer) {
        TB_CUDA(cudaMemsetAsync(m->maxsq, 0, K * sizeof(unsigned long long), c->stream));
        return TB_OK;
    }
    int* gk = nullptr;
    // the network, its judge and the kept corrections; when it does not run,
    // maxsq keeps the guess's defect, which the loop's first defect recomputes
    auto network = [&]() -> int {
        int rr;
        if ((rr = tb_learn_run_net(c))) return rr;
        const size_t per = (size_t)(nx - 2) * (ny - 1);
        k_learn_emit<<<tb_blocks(per * K, 256), 256, 0, c->stream>>>(M, L->out, L->scl, valid, nx);
        TB_CHECK_LAUNCH(c);
        k_resid<<<tb_blocks(per * K, 256), 256, 0, c->stream>>>(M, 0);
        TB_CHECK_LAUNCH(c);
        const unsigned nj = std::min<unsigned>(tb_blocks(per, 256), 64);
        k_learn_judge<<<dim3(nj, K), 256, 0, c->stream>>>(M, L->jmax, valid, nx);
        TB_CHECK_LAUNCH(c);
        k_learn_keep<<<tb_blocks(K, 64), 64, 0, c->stream>>>(m->maxsq, L->jmax, m->lkeep, L->tally, valid, K, gk);
        TB_CHECK_LAUNCH(c);
        MgDev Mk = M;
        Mk.state = m->lkeep;
        dim3 tgrid(tb_blocks(nx, 32), tb_blocks(ny, 32), K), tblk(32, 8);
        k_apply<<<tgrid, tblk, 0, c->stream>>>(Mk, c->pfc, c->g.lvl_elems, nx, ny);
        TB_CHECK_LAUNCH(c);
        return TB_OK;
    };
    if (!L->gated) return network();
    if (!c->capturing) {
        k_learn_gate<<<1, 1, 0, c->stream>>>(L->gate + 8 * ws, L->probe, 0, 0, L->gate + 32);
        TB_CHECK_LAUNCH(c);
        int run = 0;
        TB_CUDA(cudaMemcpyAsync(&run, L->gate + 32, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        TB_CUDA(cudaStreamSynchronize(c->stream));
        return run ? network() : TB_OK;
    }
    // recorded step: the network's kernels become the body of a conditional
    // IF node whose condition the gate kernel sets at every replay
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    TB_CUDA(cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &g, nullptr, nullptr, nullptr));
    if (st != cudaStreamCaptureStatusActive || !g) { tb_set_error("step graph: stream is not recording"); return TB_ERR_STATE; }
    cudaGraphConditionalHandle h;
    TB_CUDA(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
    k_learn_gate<<<1, 1, 0, c->stream>>>(L->gate + 8 * ws, L->probe, h, 1, nullptr);
    TB_CHECK_LAUNCH(c);
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    TB_CUDA(cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &g, &deps, nullptr, &nd));
    cudaGraphNodeParams p = {};
    std::memset(&p, 0, sizeof p);
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    TB_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
    TB_CUDA(cudaStreamUpdateCaptureDependencies(c->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraph_t body = p.conditional.phGraph_out[0];
    cudaStream_t outer = c->stream;
    c->stream = c->body_stream;
    cudaError_t e = cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) {
        c->stream = outer;
        tb_set_error("step graph: recording the learned correction: %s", cudaGetErrorString(e));
        return TB_ERR_CUDA;
    }
    const long long l0 = c->launches;
    r = network();
    if (c->g_stage >= 1 && c->g_stage <= 4) c->g_learn[c->g_stage - 1] = c->launches - l0;
    cudaGraph_t got = nullptr;
    e = cudaStreamEndCapture(c->stream, &got);
    c->stream = outer;
    if (r) return r;
    if (e != cudaSuccess) { tb_set_error("step graph: recording the learned correction: %s", cudaGetErrorString(e)); return TB_ERR_CUDA; }
    return TB_OK;
}

int tb_mixed_fine_op(tb_ctx* c, FineOp* op) {
    Mixed* m = get(c);
    if (!m) { tb_set_error("mixed form not set up"); return TB_ERR_STATE; }
    MgDev M = make(c);
    op->coef = M.coef + 24 * M.ylvl[0];
    op->qdy2 = M.qdy2 + (size_t)M.ny * M.ylvl[0];
    op->k2b2 = M.k2b2;
    op->den = M.qx[0];
    op->ify = M.ify;
    op->alpha2 = M.alpha2;
    op->nx = m->ptsx[0];
    op->ny = M.ny;
    op->K = M.K;
    return TB_OK;
}

// -L e on the finest level of mode k alone (r = 0), through k_resid.
int tb_mixed_resid_mode(tb_ctx* c, int k, const float* e, float* out) {
    Mixed* m = get(c);
    if (!m) { tb_set_error("mixed form not set up"); return TB_ERR_STATE; }
    const int K = c->g.K, nx = c->g.nx, ny = c->g.ny;
    if (k < 0 || k >= K) { tb_set_error("mode out of range"); return TB_ERR_ARG; }
    const size_t img = (size_t)nx * ny;
    std::vector<float2> h(img);
    for (size_t q = 0; q < img; q++) h[q] = make_float2(e[q], 0.f);
    std::vector<int> st((size_t)2 * K, 0);
    st[2 * k] = 1;
    MgDev M = make(c);
    TB_CUDA(cudaStreamSynchronize(c->stream));
    TB_CUDA(cudaMemcpy(m->e + (size_t)k * m->elems, h.data(), img * sizeof(float2), cudaMemcpyHostToDevice));
    TB_CUDA(cudaMemset(m->r + (size_t)k * m->elems, 0, img * sizeof(float2)));
    TB_CUDA(cudaMemset(m->rr + (size_t)k * m->elems, 0, img * sizeof(float2)));
    TB_CUDA(cudaMemcpy(m->lkeep, st.data(), st.size() * sizeof(int), cudaMemcpyHostToDevice));
    M.state = m->lkeep;
    const size_t per = (size_t)(nx - 2) * (ny - 1);
    k_resid<<<tb_blocks(per * K, 256), 256, 0, c->stream>>>(M, 0);
    TB_CHECK_LAUNCH(c);
    TB_CUDA(cudaMemcpyAsync(h.data(), m->rr + (size_t)k * m->elems, img * sizeof(float2), cudaMemcpyDeviceToHost, c->stream));
    TB_CUDA(cudaStreamSynchronize(c->stream));
    for (size_t q = 0; q < img; q++) out[q] = h[q].x;
    TB_CUDA(cudaMemset(m->e + (size_t)k * m->elems, 0, img * sizeof(float2)));
    return TB_OK;
}

// One solve's per-mode state (hs: active flag and corrections, per mode)
// and final defect (he) into the statistics.
int tb_mixed_absorb_stats(tb_ctx* c, const int* hs, const double* he) {
    const int K = c->g.K;
    c->stats.noconv = 0;
    int nonfinite = 0;
    for (int k = 0; k < K && k < 256; k++) {
        int vc = hs[2 * k + 1];
        if (hs[2 * k]) c->stats.noconv++;
        if (vc < 0) { nonfinite = 1; vc = -vc - 1; }
        c->stats.vcycles[k] = vc;
        c->stats.residual[k] = he[k];
        c->stats.total_vcycles += vc;
    }
    c->stats.solves++;
    if (nonfinite) { tb_set_error("poi_uy (mixed form): non-finite defect"); return TB_ERR_NONFINITE; }
    return TB_OK;
}

// poi_uy (poisson_par.f:6-64), mixed form: at most max_vcycles FP64
// corrections per solve; stats.vcycles[k] counts the corrections applied to
// mode k.
int tb_poi_uy_mixed(tb_ctx* c, const cplx* dwzdx, double erro) {
    if (!c->mixed) { tb_set_error("mixed form not set up"); return TB_ERR_STATE; }
    const int K = c->g.K, nx = c->g.nx, ny = c->g.ny, max_outer = c->cfg.max_vcycles;
    MgDev M = make(c);
    Mixed* mx = get(c);
    int r;
    cudaEvent_t pall = nullptr;
    if ((r = tb_prof_begin(c, PROF_POISSON, &pall))) return r;
    if ((r = tb_poisson_begin(c, dwzdx))) return r;
    const int ws = (c->cfg.warm_start && c->ws_stage >= 1 && c->ws_stage <= 4) ? c->ws_stage - 1 : -1;
    LearnSolve* L = ws >= 0 ? tb_learn_solve(c) : nullptr;
    int hv = 0;   // usable history entries, known to the host in host-launched solves
    if (ws >= 0) {
        // a recorded step checks the continuity of its steps before each replay
        if (!c->capturing && mx->last_t[ws] != c->ws_t - 1) {
            TB_CUDA(cudaMemsetAsync(mx->hvalid + ws, 0, sizeof(int), c->stream));
            mx->hv_host[ws] = 0;
        }
        hv = mx->hv_host[ws];
        if (c->cfg.warm_start == 2) {
            const int p = (ws + 3) % 4;
            k_extrap_inc<<<tb_blocks(tb_n3(c), 256), 256, 0, c->stream>>>(
                c->pfc, c->g.lvl_elems, mx->hist[ws][0], mx->hist[ws][1], mx->hist[p][1], mx->hvalid + ws,
                mx->hvalid + p, nx, ny, K, L ? 0 : 1);
        } else {
            k_extrap<<<tb_blocks(tb_n3(c), 256), 256, 0, c->stream>>>(c->pfc, c->g.lvl_elems, mx->hist[ws][0],
                                                                      mx->hist[ws][1], mx->hvalid + ws, nx, ny, K,
                                                                      L ? 0 : 1);
        }
        TB_CHECK_LAUNCH(c);
        if (L && (r = learned_first(c, M, ws, L))) return r;
    }
    if (c->capturing) {
        if ((r = record_loop(c, M, erro))) return r;
    } else {
        std::vector<int> hs(2 * K);
        dim3 tgrid(tb_blocks(nx, 32), tb_blocks(ny, 32), K), tblk(32, 8);
        for (int it = 0; it <= max_outer; it++) {
            Mixed* m = get(c);
            if ((r = tb_poisson_defect_f32(c, m->r, m->e, m->elems, m->maxsq))) return r;
            k_check_sq<<<tb_blocks(K, 64), 64, 0, c->stream>>>(m->maxsq, c->pstate, c->perr, K, erro, it, it == max_outer);
            TB_CHECK_LAUNCH(c);
            if (it == max_outer) break;
            TB_CUDA(cudaMemcpyAsync(hs.data(), c->pstate, 2 * K * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
            TB_CUDA(cudaStreamSynchronize(c->stream));
            bool any = false;
            for (int k = 0; k < K; k++) any = any || hs[2 * k];
            if (!any) break;
            for (int v = 0; v < INNER_VCYCLES; v++)
                if ((r = vcycle(c, M))) return r;
            k_apply<<<tgrid, tblk, 0, c->stream>>>(M, c->pfc, c->g.lvl_elems, nx, ny);
            TB_CHECK_LAUNCH(c);
        }
    }
    if (L && L->infer && L->gated) {
        k_learn_after<<<1, 1, 0, c->stream>>>(c->pstate, K, L->gate + 8 * ws);
        TB_CHECK_LAUNCH(c);
    }
    if (L && L->sample && !c->capturing && hv >= 2 && (r = tb_learn_collect(c))) return r;
    if ((r = tb_poisson_end(c))) return r;
    if (ws >= 0) {   // this solve becomes the newest entry of the stage's history
        TB_CUDA(cudaMemcpyAsync(mx->hist[ws][0], c->uy, tb_n3(c) * sizeof(cplx), cudaMemcpyDeviceToDevice, c->stream));
        k_hist_count<<<1, 1, 0, c->stream>>>(mx->hvalid + ws);
        TB_CHECK_LAUNCH(c);
        if (!c->capturing) {
            mx->last_t[ws] = c->ws_t;
            mx->hv_host[ws] = std::min(hv + 1, 2);
        }
    }
    if ((r = tb_prof_end(c, PROF_POISSON, pall))) return r;
    if (c->capturing) {   // the step's statistics are read after each replay
        const int s = c->g_stage - 1;
        if (s < 0 || s > 3) { tb_set_error("step graph: solve outside a stage"); return TB_ERR_STATE; }
        TB_CUDA(cudaMemcpyAsync(c->gsnap + (size_t)2 * K * s, c->pstate, 2 * K * sizeof(int), cudaMemcpyDeviceToDevice,
                                c->stream));
        TB_CUDA(cudaMemcpyAsync(c->gerr + (size_t)K * s, c->perr, K * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        return TB_OK;
    }
    std::vector<int> hs(2 * K);
    std::vector<double> he(K);
    TB_CUDA(cudaMemcpyAsync(hs.data(), c->pstate, 2 * K * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TB_CUDA(cudaMemcpyAsync(he.data(), c->perr, K * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    TB_CUDA(cudaStreamSynchronize(c->stream));
    return tb_mixed_absorb_stats(c, hs.data(), he.data());
}
