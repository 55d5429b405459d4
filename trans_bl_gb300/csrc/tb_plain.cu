// tb_plain.cu -- multigrid v-Poisson per spanwise mode, plain FP64 form
// (poi_uy and its helpers, poisson_par.f:6-963; band solves penta_par.f:308-404).
//
// The reference relaxes y-lines in lexicographic order: in every sweep the
// border line i=2, the border line i=ptsx-1, then the centre lines 3..ptsx-2
// (1-based), each line solve using the lines i-1, i-2 already updated in the
// same sweep and i+1, i+2 from the previous one (sor, poisson_par.f:167-226).
// This file keeps that order and its iterates, and runs it as follows:
//
//  - Real and imaginary parts are independent problems (every operator
//    coefficient is real), so each (mode, part) is one CTA with its own
//    line-contiguous copy of the multigrid arrays: element (i, j) of level l
//    at off[l] + i*ptsy[l] + j, so a y-line is one contiguous run.
//  - Successive sweeps overlap as a wavefront: sweep s relaxes the centre
//    line i at step i-1+5s, the border line 2 at step 5s and the border line
//    ptsx-1 at step ptsx-8+5s (0-based line indices 1 and ptsx-2).  Every line
//    solve then reads exactly the values the sequential order gives it, and
//    no two solves of one step touch a line that the other writes (the
//    border stencils reach 4 lines inwards, which sets the lag of 5).  One
//    warp per sweep in flight.
//  - The lines the sweeps in flight touch sit in a 32-line ring in shared
//    memory (each line read from and written to global memory once per group
//    of up to five sweeps); a level small enough is held whole.
//  - Each line solve (band LU factored once at set-up) runs on one warp:
//    32 row chunks, local recurrences with zero carry, a warp scan of the
//    chunk-end 2x2 propagators and a fix-up with precomputed homogeneous
//    responses (the chunk tables of tb_chunk_tables).
// Defect, restriction, correction and interpolation are grid-parallel.
#include "tb_internal.h"
#include <algorithm>
#include <cmath>
#include <cstring>

namespace {

constexpr int LAG = 5;      // steps between successive sweeps of the wavefront
constexpr int RING = 32;    // lines in the shared-memory ring (streamed levels)
constexpr int MAX_STREAM_SWEEPS = 5;   // sweeps in flight that fit the ring: LAG*(5-1) + 9 <= 32

struct PlainDev {
    double *fc, *sc, *fct, *def;   // per block b = 2k + part: pelems doubles (fc, sc, fct), dstride (def)
    const double* tab;             // band LU and chunk tables per (type, level, mode)
    const double* coef;            // sp(7) cp(8) pp(4) lp(5) per level
    const double* qdy2;            // (ny, msh)
    const double* k2b2;
    int* state;                    // per mode: [2k] active, [2k+1] vcycles done
    double* err;
    int nx, ny, K, msh;
    int ptsx[TB_MAX_MSH], ptsy[TB_MAX_MSH];
    size_t off[TB_MAX_MSH], pelems, dstride;
    double den[TB_MAX_MSH];        // 1 / (12 dx2 fac_y)
    double fac_y, alpha, ify;
};

__host__ __device__ inline int tab_size(int n) { return 9 * n + 1280; }

// ---------------------------------------------------------------------------
// One y-line solve of sor on one warp: rhs_center / rhs_border1 / rhs_border2
// (poisson_par.f:343-540), banbk5_poi (penta_par.f:367-404) as a chunked warp
// scan, and fc = fc + rf (x - fc) for rows j >= 1 (0-based).  The five x-stencil
// lines are given as pointers into shared memory: for a centre line
// (i-2, i-1, i+1, i+2), for a border line the four inner lines in order of
// distance (and the outer line).  T holds the (type, level, mode) tables
// compactly: L1 L2 U1 U2 ID h1 h2 k1 k2 (n each), Pf (640), Pb (640).
template <int S>
__device__ __forceinline__ void line_solve(const double* __restrict__ T, int n, int border, const double* a0,
                                           const double* a1, const double* a2, const double* a3, const double* a4,
                                           double* F, const double* __restrict__ SC, const double* cf, double qx,
                                           double rf, int lane) {
    const double sp2 = cf[1], sp3 = cf[2], cp1 = cf[7], cp2 = cf[8], cp3 = cf[9];
    const int r0 = lane * S, r1 = min(n, r0 + S);
    // x-stencil sums g of rows r0-1 .. r0+S (index q = row - r0 + 1)
    double g[S + 2];
#pragma unroll
    for (int q = 0; q < S + 2; q++) {
        int j = r0 - 1 + q;
        double v = 0.0;
        if (j >= 1 && j < n) {
            if (!border) {
                // rhs_center: -(1 f(i-2)) + 16 f(i-1) + 16 f(i+1) - 1 f(i+2)
                v = -a0[j] + 16.0 * a1[j] + 16.0 * a2[j] - a3[j];
            } else {
                // rhs_border1/2: 10 f(outer) - 4 f(1) + 14 f(2) - 6 f(3) + f(4)
                v = 10.0 * a4[j] - 4.0 * a0[j] + 14.0 * a1[j] - 6.0 * a2[j] + a3[j];
            }
        }
        g[q] = v;
    }
    const double *L1 = T, *L2 = T + n, *U1 = T + 2 * n, *U2 = T + 3 * n, *ID = T + 4 * n;
    const double *h1 = T + 5 * n, *h2 = T + 6 * n, *k1 = T + 7 * n, *k2 = T + 8 * n;
    const double* Pf = T + 9 * n;
    const double* Pb = Pf + 640;
    double y[S];
    double ym1 = 0.0, ym2 = 0.0;
#pragma unroll
    for (int s = 0; s < S; s++) {
        int j = r0 + s;
        if (j < r1) {
            double r;
            if (j == 0) r = F[0];
            else {
                double t;
                if (j == 1) t = sp3 * g[s + 2] + sp2 * g[s + 1];
                else if (j <= n - 3) t = cp1 * g[s] + cp2 * g[s + 1] + cp3 * g[s + 2];
                else if (border) t = g[s + 1];
                else t = -(a3[j] + a0[j]) + 16.0 * (a2[j] + a1[j]);   // rhs_center's two top rows
                r = SC[j] - qx * t;
            }
            double yy = r - L2[j] * ym2 - L1[j] * ym1;
            y[s] = yy; ym2 = ym1; ym1 = yy;
        }
    }
    // forward scan of the chunk-end states (y_e, y_{e-1})
    double b0 = ym1, b1 = ym2;
#pragma unroll
    for (int d = 0, off = 1; d < 5; d++, off <<= 1) {
        double o0 = __shfl_up_sync(0xffffffffu, b0, off), o1 = __shfl_up_sync(0xffffffffu, b1, off);
        if (lane >= off) {
            const double* M = Pf + (d * 32 + lane) * 4;
            double n0 = b0 + M[0] * o0 + M[1] * o1;
            double n1 = b1 + M[2] * o0 + M[3] * o1;
            b0 = n0; b1 = n1;
        }
    }
    double Y1 = __shfl_up_sync(0xffffffffu, b0, 1), Y2 = __shfl_up_sync(0xffffffffu, b1, 1);
    if (lane == 0) { Y1 = 0.0; Y2 = 0.0; }
#pragma unroll
    for (int s = 0; s < S; s++) {
        int j = r0 + s;
        if (j < r1) y[s] = y[s] + h1[j] * Y1 + h2[j] * Y2;
    }
    double xp1 = 0.0, xp2 = 0.0;
#pragma unroll
    for (int s = S - 1; s >= 0; s--) {
        int j = r0 + s;
        if (j < r1) {
            double xx = (y[s] - U1[j] * xp1 - U2[j] * xp2) * ID[j];
            y[s] = xx; xp2 = xp1; xp1 = xx;
        }
    }
    b0 = xp1; b1 = xp2;
#pragma unroll
    for (int d = 0, off = 1; d < 5; d++, off <<= 1) {
        double o0 = __shfl_down_sync(0xffffffffu, b0, off), o1 = __shfl_down_sync(0xffffffffu, b1, off);
        if (lane + off < 32) {
            const double* M = Pb + (d * 32 + lane) * 4;
            double n0 = b0 + M[0] * o0 + M[1] * o1;
            double n1 = b1 + M[2] * o0 + M[3] * o1;
            b0 = n0; b1 = n1;
        }
    }
    double X1 = __shfl_down_sync(0xffffffffu, b0, 1), X2 = __shfl_down_sync(0xffffffffu, b1, 1);
    if (lane == 31) { X1 = 0.0; X2 = 0.0; }
#pragma unroll
    for (int s = 0; s < S; s++) {
        int j = r0 + s;
        if (j < r1 && j >= 1) {
            double xx = y[s] + k1[j] * X1 + k2[j] * X2;
            double fo = F[j];
            F[j] = fo + rf * (xx - fo);
        }
    }
}

// `ns` lexicographic sweeps at level l, all (mode, part) blocks with an active
// mode.  whole = 1: the level is held whole in shared memory (any ns); else
// the lines stream through a ring of RING lines (ns <= MAX_STREAM_SWEEPS).
template <int S>
__global__ void k_wsor(PlainDev P, int l, int ns, double rf, int whole) {
    const int b = blockIdx.x, k = b >> 1;
    if (!P.state[2 * k]) return;   // uniform over the block
    const int nxl = P.ptsx[l], n = P.ptsy[l], m = nxl - 2;
    extern __shared__ double smem[];
    const int tsz = tab_size(n);
    double* tabs = smem;
    double* buf = smem + 2 * tsz;
    for (int type = 0; type < 2; type++) {
        const double* Tg = P.tab + ((((size_t)type * P.msh + l) * P.K + k) * tb_poi_blk_size(P.ny));
        double* D = tabs + type * tsz;
        for (int q = threadIdx.x; q < 9 * n; q += blockDim.x) D[q] = Tg[(size_t)(q / n) * P.ny + q % n];
        for (int q = threadIdx.x; q < 1280; q += blockDim.x) D[9 * n + q] = Tg[(size_t)9 * P.ny + q];
    }
    double* Fg = P.fc + (size_t)b * P.pelems + P.off[l];
    const double* SCg = P.sc + (size_t)b * P.pelems + P.off[l];
    const double* cf = P.coef + 24 * l;
    const double qx = P.den[l];
    const int W = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    auto LN = [&](int q) -> double* { return buf + (size_t)(whole ? q : (q & (RING - 1))) * n; };
    auto centre = [&](int i) {
        line_solve<S>(tabs, n, 0, LN(i - 2), LN(i - 1), LN(i + 1), LN(i + 2), nullptr, LN(i), SCg + (size_t)i * n, cf,
                      qx, rf, lane);
    };
    auto border1 = [&]() {
        line_solve<S>(tabs + tsz, n, 1, LN(2), LN(3), LN(4), LN(5), LN(0), LN(1), SCg + (size_t)n, cf, qx, rf, lane);
    };
    auto border2 = [&]() {
        line_solve<S>(tabs + tsz, n, 1, LN(m - 1), LN(m - 2), LN(m - 3), LN(m - 4), LN(m + 1), LN(m),
                      SCg + (size_t)m * n, cf, qx, rf, lane);
    };
    if (whole) {
        for (int q = threadIdx.x; q < nxl * n; q += blockDim.x) buf[q] = Fg[q];
    }
    __syncthreads();
    if (m < 7) {
        // too few lines for the wavefront: one warp in the reference's order
        if (warp == 0) {
            for (int s = 0; s < ns; s++) {
                border1(); __syncwarp();
                border2(); __syncwarp();
                for (int i = 2; i <= m - 1; i++) { centre(i); __syncwarp(); }
            }
        }
    } else {
        const int T = m - 1 + LAG * (ns - 1);
        int loaded = -1, stored = 0;
        for (int t = 0; t < T; t++) {
            if (!whole) {
                // lines no task at step >= t touches go back to global memory,
                // lines this step's tasks reach come in
                const int hi = min(nxl - 1, t + 7);
                const int lo = max(0, t - 1 - LAG * (ns - 1));
                const int nst = lo - stored, nld = hi - loaded;
                for (int q = threadIdx.x; q < (nst + nld) * n; q += blockDim.x) {
                    int a = q / n, j = q % n;
                    if (a < nst) { int line = stored + a; Fg[(size_t)line * n + j] = LN(line)[j]; }
                    else { int line = loaded + 1 + (a - nst); LN(line)[j] = Fg[(size_t)line * n + j]; }
                }
                stored = lo; loaded = hi;
                __syncthreads();
            }
            for (int s = warp; s < ns; s += W) {
                const int u = t - LAG * s;    // step within sweep s
                if (u == 0) border1();
                if (u >= 1 && u <= m - 2) centre(u + 1);
                if (u == m - 6) border2();
            }
            __syncthreads();
        }
        if (!whole) {
            for (int q = threadIdx.x; q < (loaded + 1 - stored) * n; q += blockDim.x) {
                int line = stored + q / n, j = q % n;
                Fg[(size_t)line * n + j] = LN(line)[j];
            }
        }
    }
    if (whole) {
        __syncthreads();
        for (int q = threadIdx.x; q < nxl * n; q += blockDim.x) Fg[q] = buf[q];
    }
}

// ---------------------------------------------------------------------------
// The level-l operator of defect (poisson_par.f:543-793) at the interior point
// (i, j) of block b: L fc = den*Dxx + q2*Dyy + k2b2*ify*M - top (real part).
__device__ __forceinline__ double plain_bx(const double* F, int n, int nxl, int i, int jj) {
    auto f = [&](int ii) { return F[(size_t)ii * n + jj]; };
    if (i == 1 || i == nxl - 2) {
        int e = (i == 1) ? 1 : -1;
        return 10.0 * f(i - e) - 15.0 * f(i) - 4.0 * f(i + e) + 14.0 * f(i + 2 * e) - 6.0 * f(i + 3 * e) + f(i + 4 * e);
    }
    return -f(i - 2) + 16.0 * f(i - 1) - 30.0 * f(i) + 16.0 * f(i + 1) - f(i + 2);
}

__device__ __forceinline__ double plain_Lu(const PlainDev& P, int l, int k, const double* F, int i, int j) {
    const int nxl = P.ptsx[l], n = P.ptsy[l];
    const double* cf = P.coef + 24 * l;
    const double *SPc = cf, *CPc = cf + 7, *PPc = cf + 15, *LPc = cf + 19;
    const double k2b2 = P.k2b2[k], den = P.den[l], ify = P.ify;
    const double* Fi = F + (size_t)i * n;
    auto bx = [&](int jj) { return plain_bx(F, n, nxl, i, jj); };
    double b, cc, d, q2, top = 0.0;
    if (j == 1) {
        b = SPc[2] * bx(2) + SPc[1] * bx(1);
        cc = SPc[3] * Fi[0] + SPc[4] * Fi[1] + SPc[5] * Fi[2] + SPc[6] * Fi[3];
        d = k2b2 * (SPc[1] * Fi[1] + SPc[2] * Fi[2]);
        q2 = P.qdy2[(size_t)P.ny * l];
    } else if (j <= n - 3) {
        b = CPc[0] * bx(j - 1) + CPc[1] * bx(j) + CPc[2] * bx(j + 1);
        cc = CPc[3] * Fi[j - 2] + CPc[4] * Fi[j - 1] + CPc[5] * Fi[j] + CPc[6] * Fi[j + 1] + CPc[7] * Fi[j + 2];
        d = k2b2 * (CPc[0] * Fi[j - 1] + CPc[1] * Fi[j] + CPc[2] * Fi[j + 1]);
        q2 = P.qdy2[(j - 2) + (size_t)P.ny * l];
    } else if (j == n - 2) {
        b = bx(j);
        cc = PPc[3] * Fi[j + 1] + PPc[2] * Fi[j] + PPc[1] * Fi[j - 1];
        d = k2b2 * Fi[j];
        q2 = P.qdy2[(j - 1) + (size_t)P.ny * l];
    } else {
        b = bx(j);
        cc = LPc[2] * Fi[j] + LPc[3] * Fi[j - 1] + LPc[4] * Fi[j - 2];
        d = k2b2 * Fi[j];
        q2 = P.qdy2[(j - 2) + (size_t)P.ny * l];
        top = LPc[1] * sqrt((P.alpha * P.alpha - k2b2) / P.fac_y) * sqrt(q2);
    }
    return b * den + cc * q2 + d * ify - top * Fi[j];
}

// defect (poisson_par.f:543-793): def = sc + si * (L fc) at level l, points
// 1 <= i <= ptsx-2, 1 <= j <= ptsy-1; si > 0 also stores it into sc(l).
__global__ void k_pdefect(PlainDev P, int l, double si) {
    const int b = blockIdx.y, k = b >> 1;
    if (!P.state[2 * k]) return;
    const int nxl = P.ptsx[l], n = P.ptsy[l];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (nxl - 2) * (n - 1)) return;
    const int i = 1 + q / (n - 1), j = 1 + q % (n - 1);
    const double* F = P.fc + (size_t)b * P.pelems + P.off[l];
    double* SC = P.sc + (size_t)b * P.pelems + P.off[l];
    const size_t o = (size_t)i * n + j;
    double v = SC[o] + si * plain_Lu(P, l, k, F, i, j);
    P.def[(size_t)b * P.dstride + o] = v;
    if (si > 0) SC[o] = v;
}

// get_max_value + verifica_poi (poisson_par.f:67-108, 945-963): max |defect|
// of each mode over both parts; converged modes stop.
__global__ void k_pcheck(PlainDev P, double tol, int vcycle) {
    const int k = blockIdx.x;
    if (!P.state[2 * k]) return;
    const int nx = P.ptsx[0], n = P.ptsy[0];
    const double* Dr = P.def + (size_t)(2 * k) * P.dstride;
    const double* Di = P.def + (size_t)(2 * k + 1) * P.dstride;
    double m = 0.0;
    int nonfinite = 0;
    for (int q = threadIdx.x; q < (nx - 2) * (n - 1); q += blockDim.x) {
        size_t o = (size_t)(1 + q / (n - 1)) * n + 1 + q % (n - 1);
        double a = hypot(Dr[o], Di[o]);
        if (!(a == a) || isinf(a)) nonfinite = 1;
        m = fmax(m, a);
    }
    __shared__ double red[256];
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    if (nonfinite) bad = 1;
    red[threadIdx.x] = m;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double e = bad ? __longlong_as_double(0x7ff8000000000000LL) : red[0];
        P.err[k] = e;
        if (bad) { P.state[2 * k] = 0; P.state[2 * k + 1] = -1 - vcycle; }
        else if (e < tol) { P.state[2 * k] = 0; P.state[2 * k + 1] = vcycle - 1; }
    }
}

// restrict (poisson_par.f:796-874): level l -> l+1 (injection of fc into fc
// and fct, full weighting of the defect into sc at interior points, the top
// row from three points).
__global__ void k_prestrict(PlainDev P, int l) {
    const int b = blockIdx.y, k = b >> 1;
    if (!P.state[2 * k]) return;
    const int nxc = P.ptsx[l + 1], nyc = P.ptsy[l + 1], nxf = P.ptsx[l], nyf = P.ptsy[l];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nxc * nyc) return;
    const int i = q / nyc, j = q % nyc;
    const double* Ff = P.fc + (size_t)b * P.pelems + P.off[l];
    const double* Df = P.def + (size_t)b * P.dstride;
    double* Fc = P.fc + (size_t)b * P.pelems + P.off[l + 1];
    double* Tc = P.fct + (size_t)b * P.pelems + P.off[l + 1];
    double* Sc = P.sc + (size_t)b * P.pelems + P.off[l + 1];
    auto df = [&](int ii, int jj) { return Df[(size_t)ii * nyf + jj]; };
    int fi = (i == nxc - 1) ? nxf - 1 : 2 * i, fj = (j == nyc - 1) ? nyf - 1 : 2 * j;
    const size_t o = (size_t)i * nyc + j;
    double v = Ff[(size_t)fi * nyf + fj];
    Fc[o] = v;
    Tc[o] = v;
    if (i >= 1 && i <= nxc - 2) {
        if (j >= 1 && j <= nyc - 2) {
            Sc[o] = 6.25e-2 * (2.0 * (df(fi - 1, fj) + df(fi + 1, fj) + df(fi, fj - 1) + df(fi, fj + 1)) + 4.0 * df(fi, fj) +
                               df(fi + 1, fj + 1) + df(fi + 1, fj - 1) + df(fi - 1, fj + 1) + df(fi - 1, fj - 1));
        } else if (j == nyc - 1) {
            Sc[o] = 0.25 * (df(fi - 1, fj) + 2.0 * df(fi, fj) + df(fi + 1, fj));
        }
    }
}

// correction (poisson_par.f:923-942) at the coarse level l.
__global__ void k_pcorrection(PlainDev P, int l) {
    const int b = blockIdx.y, k = b >> 1;
    if (!P.state[2 * k]) return;
    const int nxl = P.ptsx[l], n = P.ptsy[l];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (nxl - 2) * n) return;
    const size_t o = (size_t)n + q;   // lines 1 .. nxl-2
    double* F = P.fc + (size_t)b * P.pelems + P.off[l];
    const double* T = P.fct + (size_t)b * P.pelems + P.off[l];
    F[o] = F[o] - T[o];
}

// intpol (poisson_par.f:877-920): add the bilinear interpolant of level l to
// level l-1 at lines 1 .. ptsx(l-1)-2.
__global__ void k_pintpol(PlainDev P, int l) {
    const int b = blockIdx.y, k = b >> 1;
    if (!P.state[2 * k]) return;
    const int nyc = P.ptsy[l], nxf = P.ptsx[l - 1], nyf = P.ptsy[l - 1];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (nxf - 2) * nyf) return;
    const int i = 1 + q / nyf, j = q % nyf;
    const double* C = P.fc + (size_t)b * P.pelems + P.off[l];
    auto cv = [&](int ci, int cj) { return C[(size_t)ci * nyc + cj]; };
    auto row = [&](int jj) -> double {
        int cj = jj / 2;
        if ((i & 1) == 0) return cv(i / 2, cj);
        return 0.5 * (cv(i / 2, cj) + cv(i / 2 + 1, cj));
    };
    double t = ((j & 1) == 0) ? row(j) : 0.5 * (row(j + 1) + row(j - 1));
    double* F = P.fc + (size_t)b * P.pelems + P.off[l - 1];
    F[(size_t)i * nyf + j] += t;
}

// function_source (poisson_par.f:111-164) for all modes, into the
// line-contiguous real/imaginary planes of level 0: sc and fc = uy.  32 x 32
// tiles transposed through shared memory (x-rows in, y-lines out).
__global__ void k_psource(PlainDev P, const cplx* wx, const cplx* dwzdx, const cplx* uy, const double* duexmdx,
                          const double* uyb, double beta, double dy, double stf_pow, int form) {
    __shared__ cplx ts[32][33], tu[32][33];
    const int k = blockIdx.z, J = P.ny, nx = P.nx;
    const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
    const double* c0 = P.coef;
    const double kb = (double)k * beta;
    auto S = [&](int i, int jj) {
        size_t o = (size_t)i + (size_t)nx * (jj + (size_t)J * k);
        cplx w = wx[o], d = dwzdx[o];
        return make_double2(kb * w.y - d.x, -kb * w.x - d.y);
    };
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        int i = i0 + threadIdx.x, j = j0 + r;
        if (i < nx && j < J) {
            cplx s;
            if (j == 0) s = make_double2(0, 0);
            else if (j == 1) { cplx a = S(i, 1), b = S(i, 2); s = make_double2(c0[1] * a.x + c0[2] * b.x, c0[1] * a.y + c0[2] * b.y); }
            else if (j <= J - 3) {
                cplx a = S(i, j - 1), b = S(i, j), d = S(i, j + 1);
                s = make_double2(c0[7] * a.x + c0[8] * b.x + c0[9] * d.x, c0[7] * a.y + c0[8] * b.y + c0[9] * d.y);
            } else if (j == J - 2) s = S(i, J - 2);
            else {
                s = make_double2(0, 0);
                if ((form == 0 || form == 4) && k == 0) {
                    double dya = dy * stf_pow;
                    size_t o = (size_t)i + (size_t)nx * (J - 1);
                    double lp1 = c0[19], lp2 = c0[20];
                    s = make_double2(-(lp1 * dwzdx[o].x) + lp2 * duexmdx[i] / dya - lp2 * P.alpha * uyb[o] / dya / sqrt(P.fac_y),
                                     -(lp1 * dwzdx[o].y));
                }
            }
            ts[r][threadIdx.x] = s;
            tu[r][threadIdx.x] = uy[(size_t)i + (size_t)nx * (j + (size_t)J * k)];
        }
    }
    __syncthreads();
    double *sr = P.sc + (size_t)(2 * k) * P.pelems, *si = sr + P.pelems;
    double *fr = P.fc + (size_t)(2 * k) * P.pelems, *fi = fr + P.pelems;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        int i = i0 + r, j = j0 + threadIdx.x;
        if (i < nx && j < J) {
            size_t o = (size_t)i * J + j;
            cplx s = ts[threadIdx.x][r], u = tu[threadIdx.x][r];
            sr[o] = s.x; si[o] = s.y; fr[o] = u.x; fi[o] = u.y;
        }
    }
}

// uy(i,j,k) = fc(i,j,1) for j >= 2, 2 <= i <= ptsx-1 (poisson_par.f:53-57).
__global__ void k_pwrite_uy(PlainDev P, cplx* uy) {
    __shared__ cplx tile[32][33];
    const int k = blockIdx.z, J = P.ny, nx = P.nx;
    const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
    const double *fr = P.fc + (size_t)(2 * k) * P.pelems, *fi = fr + P.pelems;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        int i = i0 + r, j = j0 + threadIdx.x;
        if (i < nx && j < J) {
            size_t o = (size_t)i * J + j;
            tile[r][threadIdx.x] = make_double2(fr[o], fi[o]);
        }
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        int i = i0 + threadIdx.x, j = j0 + r;
        if (i >= 1 && i <= nx - 2 && j >= 1 && j < J) uy[(size_t)i + (size_t)nx * (j + (size_t)J * k)] = tile[threadIdx.x][r];
    }
}

__global__ void k_pactivate(int* state, int K) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < K) { state[2 * k] = 1; state[2 * k + 1] = 0; }
}

PlainDev make_plain(tb_ctx* c) {
    PlainDev P;
    std::memset(&P, 0, sizeof P);
    P.fc = c->pl_fc; P.sc = c->pl_sc; P.fct = c->pl_fct; P.def = c->pl_def; P.tab = c->pcarry; P.coef = c->pcoef;
    P.qdy2 = c->pqdy2; P.k2b2 = c->k2b2; P.state = c->pstate; P.err = c->perr;
    P.nx = c->g.nx; P.ny = c->g.ny; P.K = c->g.K; P.msh = c->g.msh;
    for (int l = 0; l < c->g.msh; l++) {
        P.ptsx[l] = c->g.ptsx[l]; P.ptsy[l] = c->g.ptsy[l]; P.off[l] = c->g.lvl_off[l];
        P.den[l] = 1.0 / (12.0 * c->h_dx2[l] * c->cfg.fac_y);
    }
    P.ify = 1.0 / c->cfg.fac_y;
    P.pelems = c->g.lvl_elems; P.dstride = (size_t)c->g.nx * c->g.ny;
    P.fac_y = c->cfg.fac_y; P.alpha = c->cfg.alpha;
    return P;
}

template <int S>
int launch_wsor_s(tb_ctx* c, const PlainDev& P, int l, int ns, double rf, int whole, int warps, size_t smem) {
    TB_CUDA(cudaFuncSetAttribute(k_wsor<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    // at most the warps the kernel's register count allows in one block; a
    // warp then runs the tasks of two sweeps in some steps, which are independent
    cudaFuncAttributes fa;
    TB_CUDA(cudaFuncGetAttributes(&fa, k_wsor<S>));
    warps = std::max(1, std::min(warps, fa.maxThreadsPerBlock / 32));
    k_wsor<S><<<2 * c->g.K, 32 * warps, smem, c->stream>>>(P, l, ns, rf, whole);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}

// `itera` sweeps of sor at level l (poisson_par.f:167-226) for every active mode.
int plain_sor(tb_ctx* c, const PlainDev& P, int l, int itera, double rf) {
    const int nxl = c->g.ptsx[l], n = c->g.ptsy[l], m = nxl - 2;
    const int S = std::max(2, (n + 31) / 32);
    const size_t tab_bytes = (size_t)2 * tab_size(n) * sizeof(double);
    const size_t whole_bytes = tab_bytes + (size_t)nxl * n * sizeof(double);
    const bool can_whole = whole_bytes <= (size_t)200 * 1024;
    cudaEvent_t ps = nullptr;
    if (tb_prof_begin(c, PROF_SOR, &ps)) return TB_ERR_CUDA;
    int done = 0;
    while (done < itera) {
        int ns, whole, warps;
        if (m < 7 || (itera - done > MAX_STREAM_SWEEPS && can_whole)) {
            // all remaining sweeps with the level held in shared memory; warp w
            // runs the sweeps w, w + W, ... (the wavefront stays full once
            // W > (m - 2) / LAG)
            whole = 1;
            ns = itera - done;
            warps = (m < 7) ? 1 : std::min({32, ns, (m - 2) / LAG + 1});
        } else {
            whole = 0;
            ns = std::min(MAX_STREAM_SWEEPS, itera - done);
            warps = ns;
        }
        size_t smem = whole ? whole_bytes : tab_bytes + (size_t)RING * n * sizeof(double);
        int r;
        switch (S) {
            case 2: r = launch_wsor_s<2>(c, P, l, ns, rf, whole, warps, smem); break;
            case 3: r = launch_wsor_s<3>(c, P, l, ns, rf, whole, warps, smem); break;
            case 4: r = launch_wsor_s<4>(c, P, l, ns, rf, whole, warps, smem); break;
            case 5: r = launch_wsor_s<5>(c, P, l, ns, rf, whole, warps, smem); break;
            case 6: r = launch_wsor_s<6>(c, P, l, ns, rf, whole, warps, smem); break;
            case 7: r = launch_wsor_s<7>(c, P, l, ns, rf, whole, warps, smem); break;
            case 8: r = launch_wsor_s<8>(c, P, l, ns, rf, whole, warps, smem); break;
            case 9: r = launch_wsor_s<9>(c, P, l, ns, rf, whole, warps, smem); break;
            case 10: r = launch_wsor_s<10>(c, P, l, ns, rf, whole, warps, smem); break;
            case 11: r = launch_wsor_s<11>(c, P, l, ns, rf, whole, warps, smem); break;
            case 12: r = launch_wsor_s<12>(c, P, l, ns, rf, whole, warps, smem); break;
            default: r = launch_wsor_s<16>(c, P, l, ns, rf, whole, warps, smem); break;
        }
        if (r) return r;
        done += ns;
    }
    return tb_prof_end(c, PROF_SOR, ps);
}

}  // namespace

// Line-contiguous real/imaginary multigrid arrays of the plain form.
int tb_plain_setup(tb_ctx* c) {
    const int K = c->g.K;
    const size_t w = (size_t)2 * K * c->g.lvl_elems;
    for (double** p : {&c->pl_fc, &c->pl_sc, &c->pl_fct}) {
        if (*p) cudaFree(*p);
        *p = nullptr;
        TB_CUDA(cudaMalloc(p, w * sizeof(double)));
        TB_CUDA(cudaMemset(*p, 0, w * sizeof(double)));
    }
    if (c->pl_def) cudaFree(c->pl_def);
    c->pl_def = nullptr;
    const size_t d = (size_t)2 * K * c->g.nx * c->g.ny;
    TB_CUDA(cudaMalloc(&c->pl_def, d * sizeof(double)));
    TB_CUDA(cudaMemset(c->pl_def, 0, d * sizeof(double)));
    if (c->g.ny > 32 * 16) { tb_set_error("plain Poisson: ny above 512"); return TB_ERR_ARG; }
    return TB_OK;
}

// poi_uy (poisson_par.f:6-64), plain FP64 form.
int tb_poi_uy_k(tb_ctx* c, const cplx* dwzdx, double erro) {
    if (!c->pl_fc) { tb_set_error("plain Poisson arrays missing (context not in the plain form)"); return TB_ERR_STATE; }
    PlainDev P = make_plain(c);
    const int K = c->g.K, msh = c->g.msh;
    cudaEvent_t pall = nullptr;
    if (tb_prof_begin(c, PROF_POISSON, &pall)) return TB_ERR_CUDA;
    const double stf_pow = tb_powi(c->cfg.stf, c->g.ny - 3);
    {
        dim3 grid(tb_blocks(c->g.nx, 32), tb_blocks(c->g.ny, 32), K), blk(32, 8);
        k_psource<<<grid, blk, 0, c->stream>>>(P, c->wx, dwzdx, c->uy, c->duexmdx, c->uyb, c->cfg.beta, c->cfg.dy,
                                               stf_pow, c->cfg.my_form);
        TB_CHECK_LAUNCH(c);
    }
    k_pactivate<<<tb_blocks(K, 64), 64, 0, c->stream>>>(c->pstate, K);
    TB_CHECK_LAUNCH(c);
    std::vector<int> hs(2 * K);
    const int vmax = c->cfg.max_vcycles;
    auto defect = [&](int l, double si) {
        const int per = (c->g.ptsx[l] - 2) * (c->g.ptsy[l] - 1);
        cudaEvent_t ps = nullptr;
        if (tb_prof_begin(c, PROF_DEFECT, &ps)) return TB_ERR_CUDA;
        k_pdefect<<<dim3(tb_blocks(per, 128), 2 * K), 128, 0, c->stream>>>(P, l, si);
        TB_CHECK_LAUNCH(c);
        return tb_prof_end(c, PROF_DEFECT, ps);
    };
    int r;
    for (int v = 1; v <= vmax; v++) {
        for (int l = 0; l < msh - 1; l++) {
            if ((r = plain_sor(c, P, l, 3, 1.2))) return r;
            if ((r = defect(l, -1.0))) return r;
            if (l == 0) { k_pcheck<<<K, 256, 0, c->stream>>>(P, erro, v); TB_CHECK_LAUNCH(c); }
            const int per = c->g.ptsx[l + 1] * c->g.ptsy[l + 1];
            k_prestrict<<<dim3(tb_blocks(per, 128), 2 * K), 128, 0, c->stream>>>(P, l);
            TB_CHECK_LAUNCH(c);
            if ((r = defect(l + 1, 1.0))) return r;
        }
        if ((r = plain_sor(c, P, msh - 1, 60, 1.2))) return r;
        for (int l = msh - 1; l >= 1; l--) {
            const int per = (c->g.ptsx[l] - 2) * c->g.ptsy[l];
            k_pcorrection<<<dim3(tb_blocks(per, 128), 2 * K), 128, 0, c->stream>>>(P, l);
            TB_CHECK_LAUNCH(c);
            const int perf = (c->g.ptsx[l - 1] - 2) * c->g.ptsy[l - 1];
            k_pintpol<<<dim3(tb_blocks(perf, 128), 2 * K), 128, 0, c->stream>>>(P, l);
            TB_CHECK_LAUNCH(c);
            if ((r = plain_sor(c, P, l - 1, 1, 1.0))) return r;
        }
        TB_CUDA(cudaMemcpyAsync(hs.data(), c->pstate, 2 * K * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        TB_CUDA(cudaStreamSynchronize(c->stream));
        bool any = false;
        for (int k = 0; k < K; k++) any = any || hs[2 * k];
        if (!any) break;
    }
    {
        dim3 grid(tb_blocks(c->g.nx, 32), tb_blocks(c->g.ny, 32), K), blk(32, 8);
        k_pwrite_uy<<<grid, blk, 0, c->stream>>>(P, c->uy);
        TB_CHECK_LAUNCH(c);
    }
    if (tb_prof_end(c, PROF_POISSON, pall)) return TB_ERR_CUDA;
    std::vector<double> he(K);
    TB_CUDA(cudaMemcpyAsync(hs.data(), c->pstate, 2 * K * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TB_CUDA(cudaMemcpyAsync(he.data(), c->perr, K * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    TB_CUDA(cudaStreamSynchronize(c->stream));
    c->stats.noconv = 0;
    int nonfinite = 0;
    for (int k = 0; k < K && k < 256; k++) {
        int vc = hs[2 * k + 1];
        if (hs[2 * k]) { vc = vmax; c->stats.noconv++; }
        if (vc < 0) { nonfinite = 1; vc = -vc - 1; }
        c->stats.vcycles[k] = vc;
        c->stats.residual[k] = he[k];
        c->stats.total_vcycles += vc;
    }
    c->stats.solves++;
    if (nonfinite) { tb_set_error("poi_uy: non-finite defect"); return TB_ERR_NONFINITE; }
    return TB_OK;
}
