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
//    border stencils reach 4 lines inwards, which sets the lag of 5).
//  - The lines of fc and sc the sweeps in flight touch sit in 32-line rings
//    in shared memory (each line read from and written to global memory once
//    per group of up to five sweeps, the next line prefetched while a step
//    solves); a level small enough is held whole.
//  - Each line solve (band LU factored once at set-up) runs on a group of 1,
//    2 or 4 warps: row chunks with local recurrences and zero carry, a warp
//    scan of the chunk-end 2x2 propagators, the warps chained through shared
//    memory, and a fix-up with precomputed homogeneous responses.  On GB300
//    an FP64 warp instruction holds its sub-partition's FP64 pipe for ~64
//    cycles whatever the number of active lanes, so a line's latency is set
//    by the FP64 instructions per warp: one sweep in flight spreads each line
//    over four warps (all four sub-partitions), several sweeps over two.
// Defect, restriction, correction and interpolation are grid-parallel.
#include "tb_internal.h"
#include <algorithm>
#include <cmath>
#include <cstring>

namespace {

constexpr int LAG = 5;      // steps between successive sweeps of the wavefront
constexpr int RING = 32;    // lines in the shared-memory rings (streamed levels)
constexpr int MAX_STREAM_SWEEPS = 5;   // sweeps in flight that fit the ring: LAG*(5-1) + 10 <= 32
constexpr int WARP_TAB = 1544;         // per warp of a line group: Pf 640, Pb 640, R 128, Q 128, A 4, B 4
constexpr int NGROUP = 3;              // line groups of 1, 2 and 4 warps
constexpr int PREFETCH = 4;            // line elements a thread prefetches into registers per ring

__host__ __device__ inline int group_warps(int gi) { return 1 << gi; }
__host__ __device__ inline int rows_per_lane(int n, int G) { int s = (n + 32 * G - 1) / (32 * G); return s < 1 ? 1 : s; }
// one (group, type, level, mode) block of line-solve tables: L1 L2 U1 U2 ID
// h1 h2 k1 k2 (n each, compact), then WARP_TAB doubles per warp of the group
__host__ __device__ inline int tab_size(int n, int G) { return 9 * n + WARP_TAB * G; }
__host__ __device__ inline size_t tab_block(int ny) { return (size_t)tab_size(ny, 4); }

struct PlainDev {
    double *fc, *sc, *fct, *def;   // per block b = 2k + part: pelems doubles (fc, sc, fct), dstride (def)
    const double* tab;             // line-solve tables per (group, type, level, mode), blocks of tab_block(ny)
    const double* coef;            // sp(7) cp(8) pp(4) lp(5) per level
    const double* qdy2;            // (ny, msh)
    const double* k2b2;
    int* state;                    // per mode: [2k] active, [2k+1] vcycles done
    double* err;
    unsigned long long* maxsq;     // per mode: max |defect|^2 of the fine level (double bits)
    int nx, ny, K, msh;
    int ptsx[TB_MAX_MSH], ptsy[TB_MAX_MSH];
    size_t off[TB_MAX_MSH], pelems, dstride;
    double den[TB_MAX_MSH];        // 1 / (12 dx2 fac_y)
    double fac_y, alpha, ify;
};

__device__ __forceinline__ const double* tab_ptr(const PlainDev& P, int gi, int type, int l, int k) {
    return P.tab + ((((size_t)gi * 2 + type) * P.msh + l) * P.K + k) * tab_block(P.ny);
}

__device__ __forceinline__ void group_barrier(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// ---------------------------------------------------------------------------
// One y-line solve of sor on a group of G warps: rhs_center / rhs_border1 /
// rhs_border2 (poisson_par.f:343-540), banbk5_poi (penta_par.f:367-404) and
// fc = fc + rf (x - fc) for rows j >= 1 (0-based).  The rows are cut into
// 32 G chunks of S rows (warp g, lane t owns chunk 32 g + t); each chunk runs
// its local recurrences with zero carry, the chunk-end 2x2 propagators are
// scanned within each warp (Kogge-Stone), the warp totals are chained through
// shared memory, and every row is fixed up with its precomputed homogeneous
// responses.  The x-stencil lines come as pointers into shared memory: for a
// centre line (i-2, i-1, i+1, i+2), for a border line the four inner lines in
// order of distance and the outer line.  TR: row tables (stride n); TW: the
// group's warp tables.
template <int S, int G, bool BORDER>
__device__ __forceinline__ void line_solve(const double* __restrict__ TR, const double* __restrict__ TW, int n,
                                           const double* a0, const double* a1, const double* a2, const double* a3,
                                           const double* a4, double* F, const double* SC, const double* cf, double qx,
                                           double rf, int g, int lane, double* xch, int bar) {
    // rhs = sc - qx (weights . g), with qx folded into the weights
    const double sp2 = qx * cf[1], sp3 = qx * cf[2], cp1 = qx * cf[7], cp2 = qx * cf[8], cp3 = qx * cf[9];
    const int r0 = (32 * g + lane) * S, r1 = min(n, r0 + S);
    // x-stencil sums of rows r0-1 .. r0+S (index q = row - r0 + 1)
    double gs[S + 2];
#pragma unroll
    for (int q = 0; q < S + 2; q++) {
        const int j = r0 - 1 + q;
        double v = 0.0;
        if (j >= 1 && j < n) {
            if (!BORDER) v = -a0[j] + 16.0 * a1[j] + 16.0 * a2[j] - a3[j];   // -(1 f(i-2)) + 16 f(i-1) + 16 f(i+1) - 1 f(i+2)
            else v = 10.0 * a4[j] - 4.0 * a0[j] + 14.0 * a1[j] - 6.0 * a2[j] + a3[j];
        }
        gs[q] = v;
    }
    const double *L1 = TR, *L2 = TR + n, *U1 = TR + 2 * n, *U2 = TR + 3 * n, *ID = TR + 4 * n;
    const double *h1 = TR + 5 * n, *h2 = TR + 6 * n, *k1 = TR + 7 * n, *k2 = TR + 8 * n;
    const double* Tg = TW + WARP_TAB * g;
    const double *Pf = Tg, *Pb = Tg + 640, *Rm = Tg + 1280 + 4 * lane, *Qm = Tg + 1408 + 4 * lane;
    double y[S];
    double ym1 = 0.0, ym2 = 0.0;
#pragma unroll
    for (int s = 0; s < S; s++) {
        const int j = r0 + s;
        if (j < r1) {
            double r;
            if (j == 0) r = F[0];
            else if (j == 1) r = SC[j] - sp3 * gs[s + 2] - sp2 * gs[s + 1];
            else if (j <= n - 3) r = SC[j] - cp1 * gs[s] - cp2 * gs[s + 1] - cp3 * gs[s + 2];
            else if (BORDER) r = SC[j] - qx * gs[s + 1];
            else r = SC[j] - qx * (-(a3[j] + a0[j]) + 16.0 * (a2[j] + a1[j]));   // rhs_center's two top rows
            const double yy = r - L2[j] * ym2 - L1[j] * ym1;
            y[s] = yy; ym2 = ym1; ym1 = yy;
        }
    }
    // forward: scan of the chunk-end states (y_e, y_{e-1}) within the warp
    double b0 = ym1, b1 = ym2;
#pragma unroll
    for (int d = 0, off = 1; d < 5; d++, off <<= 1) {
        const double o0 = __shfl_up_sync(0xffffffffu, b0, off), o1 = __shfl_up_sync(0xffffffffu, b1, off);
        if (lane >= off) {
            const double* M = Pf + (d * 32 + lane) * 4;
            const double n0 = b0 + M[0] * o0 + M[1] * o1;
            const double n1 = b1 + M[2] * o0 + M[3] * o1;
            b0 = n0; b1 = n1;
        }
    }
    double Y1 = __shfl_up_sync(0xffffffffu, b0, 1), Y2 = __shfl_up_sync(0xffffffffu, b1, 1);
    if (lane == 0) { Y1 = 0.0; Y2 = 0.0; }
    if (G > 1) {
        // the warps' outgoing states, chained in order: z = state entering warp g
        if (lane == 31) { xch[4 * g] = b0; xch[4 * g + 1] = b1; }
        group_barrier(bar, 32 * G);
        double z0 = 0.0, z1 = 0.0;
        for (int w = 0; w < g; w++) {
            const double* A = TW + WARP_TAB * w + 1536;
            const double n0 = xch[4 * w] + A[0] * z0 + A[1] * z1;
            const double n1 = xch[4 * w + 1] + A[2] * z0 + A[3] * z1;
            z0 = n0; z1 = n1;
        }
        Y1 = Y1 + Rm[0] * z0 + Rm[1] * z1;
        Y2 = Y2 + Rm[2] * z0 + Rm[3] * z1;
    }
#pragma unroll
    for (int s = 0; s < S; s++) {
        const int j = r0 + s;
        if (j < r1) y[s] = y[s] + h1[j] * Y1 + h2[j] * Y2;
    }
    double xp1 = 0.0, xp2 = 0.0;
#pragma unroll
    for (int s = S - 1; s >= 0; s--) {
        const int j = r0 + s;
        if (j < r1) {
            const double xx = (y[s] - U1[j] * xp1 - U2[j] * xp2) * ID[j];
            y[s] = xx; xp2 = xp1; xp1 = xx;
        }
    }
    // backward: scan of the chunk-start states (x_s, x_{s+1}) from the high lanes
    b0 = xp1; b1 = xp2;
#pragma unroll
    for (int d = 0, off = 1; d < 5; d++, off <<= 1) {
        const double o0 = __shfl_down_sync(0xffffffffu, b0, off), o1 = __shfl_down_sync(0xffffffffu, b1, off);
        if (lane + off < 32) {
            const double* M = Pb + (d * 32 + lane) * 4;
            const double n0 = b0 + M[0] * o0 + M[1] * o1;
            const double n1 = b1 + M[2] * o0 + M[3] * o1;
            b0 = n0; b1 = n1;
        }
    }
    double X1 = __shfl_down_sync(0xffffffffu, b0, 1), X2 = __shfl_down_sync(0xffffffffu, b1, 1);
    if (lane == 31) { X1 = 0.0; X2 = 0.0; }
    if (G > 1) {
        if (lane == 0) { xch[4 * g + 2] = b0; xch[4 * g + 3] = b1; }
        group_barrier(bar, 32 * G);
        double z0 = 0.0, z1 = 0.0;
        for (int w = G - 1; w > g; w--) {
            const double* B = TW + WARP_TAB * w + 1540;
            const double n0 = xch[4 * w + 2] + B[0] * z0 + B[1] * z1;
            const double n1 = xch[4 * w + 3] + B[2] * z0 + B[3] * z1;
            z0 = n0; z1 = n1;
        }
        X1 = X1 + Qm[0] * z0 + Qm[1] * z1;
        X2 = X2 + Qm[2] * z0 + Qm[3] * z1;
    }
#pragma unroll
    for (int s = 0; s < S; s++) {
        const int j = r0 + s;
        if (j < r1 && j >= 1) {
            const double xx = y[s] + k1[j] * X1 + k2[j] * X2;
            const double fo = F[j];
            F[j] = fo + rf * (xx - fo);
        }
    }
}

// `ns` lexicographic sweeps at level l, all (mode, part) blocks with an active
// mode, each line solved by a group of G warps (table group gi).  whole = 1:
// the level's fc and sc are held whole in shared memory (any ns); else their
// lines stream through rings of RING lines (ns <= MAX_STREAM_SWEEPS), the
// next line prefetched into registers while the current step's lines solve.
template <int S, int G>
__global__ void k_wsor(PlainDev P, int l, int ns, double rf, int whole, int gi) {
    const int b = blockIdx.x, k = b >> 1;
    if (!P.state[2 * k]) return;   // uniform over the block
    const int nxl = P.ptsx[l], n = P.ptsy[l], m = nxl - 2;
    extern __shared__ double smem[];
    const int tsz = tab_size(n, G);
    const int lines = whole ? nxl : RING;
    double* tabc = smem;                               // centre-line tables
    double* fcb = smem + tsz;                          // fc lines
    double* scb = fcb + (size_t)lines * n;             // sc lines
    double* xch = scb + (size_t)lines * n;             // group exchange, 4 G per group
    const double* tabb = tab_ptr(P, gi, 1, l, k);      // border-line tables (global, cached)
    {
        const double* tg = tab_ptr(P, gi, 0, l, k);
        for (int q = threadIdx.x; q < tsz; q += blockDim.x) tabc[q] = tg[q];
    }
    double* Fg = P.fc + (size_t)b * P.pelems + P.off[l];
    const double* SCg = P.sc + (size_t)b * P.pelems + P.off[l];
    const double* cf = P.coef + 24 * l;
    const double qx = P.den[l];
    const int nth = blockDim.x, tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int grp = warp / G, g = warp % G, W = (blockDim.x >> 5) / G;
    double* gx = xch + 4 * G * grp;
    const int bar = 1 + grp;
    auto FL = [&](int q) -> double* { return fcb + (size_t)(whole ? q : (q & (RING - 1))) * n; };
    auto SL = [&](int q) -> double* { return scb + (size_t)(whole ? q : (q & (RING - 1))) * n; };
    auto centre = [&](int i) {
        line_solve<S, G, false>(tabc, tabc + 9 * n, n, FL(i - 2), FL(i - 1), FL(i + 1), FL(i + 2), nullptr, FL(i), SL(i),
                                cf, qx, rf, g, lane, gx, bar);
    };
    auto border1 = [&]() {
        line_solve<S, G, true>(tabb, tabb + 9 * n, n, FL(2), FL(3), FL(4), FL(5), FL(0), FL(1), SL(1), cf, qx, rf, g,
                               lane, gx, bar);
    };
    auto border2 = [&]() {
        line_solve<S, G, true>(tabb, tabb + 9 * n, n, FL(m - 1), FL(m - 2), FL(m - 3), FL(m - 4), FL(m + 1), FL(m),
                               SL(m), cf, qx, rf, g, lane, gx, bar);
    };
    const int first = whole ? nxl : min(nxl, 8);   // lines 0..7 are the first step's window
    for (int q = tid; q < first * n; q += nth) {
        const int line = q / n, j = q % n;
        FL(line)[j] = Fg[(size_t)line * n + j];
        SL(line)[j] = SCg[(size_t)line * n + j];
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
        __syncthreads();
    } else {
        const int T = m - 1 + LAG * (ns - 1);
        int stored = 0;
        double pf[PREFETCH], ps[PREFETCH];   // line t+8 of fc and sc in flight
        auto fetch = [&](int line) {
#pragma unroll
            for (int e = 0; e < PREFETCH; e++) {
                const int j = tid + e * nth;
                if (line < nxl && j < n) { pf[e] = Fg[(size_t)line * n + j]; ps[e] = SCg[(size_t)line * n + j]; }
            }
        };
        if (!whole) fetch(8);
        for (int t = 0; t < T; t++) {
            for (int s = grp; s < ns; s += W) {
                const int u = t - LAG * s;    // step within sweep s
                if (u == 0) border1();
                if (u >= 1 && u <= m - 2) centre(u + 1);
                if (u == m - 6) border2();
            }
            __syncthreads();
            if (!whole) {
                // lines no task at step >= t+1 touches go back to global memory;
                // line t+8 (step t+1's window edge) enters the rings
                const int lo = max(0, t - LAG * (ns - 1));
                for (int q = tid; q < (lo - stored) * n; q += nth) {
                    const int line = stored + q / n, j = q % n;
                    Fg[(size_t)line * n + j] = FL(line)[j];
                }
                stored = lo;
                const int line = t + 8;
                if (line < nxl) {
#pragma unroll
                    for (int e = 0; e < PREFETCH; e++) {
                        const int j = tid + e * nth;
                        if (j < n) { FL(line)[j] = pf[e]; SL(line)[j] = ps[e]; }
                    }
                    for (int j = tid + PREFETCH * nth; j < n; j += nth) {
                        FL(line)[j] = Fg[(size_t)line * n + j];
                        SL(line)[j] = SCg[(size_t)line * n + j];
                    }
                }
                fetch(t + 9);
                __syncthreads();
            }
        }
        if (!whole) {
            for (int q = tid; q < (nxl - stored) * n; q += nth) {
                const int line = stored + q / n, j = q % n;
                Fg[(size_t)line * n + j] = FL(line)[j];
            }
        }
    }
    if (whole) {
        for (int q = tid; q < nxl * n; q += nth) Fg[q] = fcb[q];
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
// 1 <= i <= ptsx-2, 1 <= j <= ptsy-1, both parts of mode blockIdx.y per
// thread; si > 0 also stores it into sc(l).  On the fine level (l = 0) the
// block's max |def|^2 goes into maxsq[k] (double bits, non-negative; a
// non-finite defect records +inf) for k_pcheck.
__global__ void k_pdefect(PlainDev P, int l, double si) {
    const int k = blockIdx.y;
    if (!P.state[2 * k]) return;   // uniform over the block
    const int nxl = P.ptsx[l], n = P.ptsy[l];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    double m = 0.0;
    bool bad = false;
    if (q < (nxl - 2) * (n - 1)) {
        const int i = 1 + q / (n - 1), j = 1 + q % (n - 1);
        const size_t o = (size_t)i * n + j;
        double v[2];
#pragma unroll
        for (int part = 0; part < 2; part++) {
            const int b = 2 * k + part;
            const double* F = P.fc + (size_t)b * P.pelems + P.off[l];
            double* SC = P.sc + (size_t)b * P.pelems + P.off[l];
            v[part] = SC[o] + si * plain_Lu(P, l, k, F, i, j);
            P.def[(size_t)b * P.dstride + o] = v[part];
            if (si > 0) SC[o] = v[part];
        }
        const double a = v[0] * v[0] + v[1] * v[1];
        if (!(a <= 1.7e308)) bad = true;
        else m = a;
    }
    if (l != 0) return;   // uniform over the block
    if (bad) m = __longlong_as_double(0x7ff0000000000000LL);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ double wm[8];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double bm = wm[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) bm = fmax(bm, wm[w]);
        atomicMax(&P.maxsq[k], (unsigned long long)__double_as_longlong(bm));
    }
}

// get_max_value + verifica_poi (poisson_par.f:67-108, 945-963): max |defect|
// of each mode from the fine-level defect's maxima; converged modes stop.
__global__ void k_pcheck(PlainDev P, double tol, int vcycle) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.K || !P.state[2 * k]) return;
    const double a = __longlong_as_double((long long)P.maxsq[k]);
    P.maxsq[k] = 0ull;
    if (!(a <= 1.7e308)) {
        P.err[k] = __longlong_as_double(0x7ff8000000000000LL);
        P.state[2 * k] = 0;
        P.state[2 * k + 1] = -1 - vcycle;
        return;
    }
    const double e = sqrt(a);
    P.err[k] = e;
    if (e < tol) { P.state[2 * k] = 0; P.state[2 * k + 1] = vcycle - 1; }
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
    P.fc = c->pl_fc; P.sc = c->pl_sc; P.fct = c->pl_fct; P.def = c->pl_def; P.tab = c->pl_tab; P.coef = c->pcoef;
    P.qdy2 = c->pqdy2; P.k2b2 = c->k2b2; P.state = c->pstate; P.err = c->perr; P.maxsq = c->pl_maxsq;
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

// Line-solve tables of one (group, type, level, mode) for G warps of 32 row
// chunks of S rows: the band LU rows (L1 L2 U1 U2 ID), the chunk-local
// homogeneous responses h1 h2 (forward, to the incoming y_{r0-1}, y_{r0-2})
// and k1 k2 (backward, to x_{r1}, x_{r1+1}), and per warp the Kogge-Stone
// step matrices Pf, Pb of its 32 chunk propagators, the prefix R (warp start
// to each chunk start, forward), the suffix Q (warp end to each chunk end,
// backward) and the warp totals A (forward) and B (backward).
void group_tables(int n, int S, int G, const double* L1, const double* L2, const double* U1, const double* U2,
                  const double* ID, double* out) {
    std::memcpy(out, L1, n * sizeof(double));
    std::memcpy(out + n, L2, n * sizeof(double));
    std::memcpy(out + 2 * n, U1, n * sizeof(double));
    std::memcpy(out + 3 * n, U2, n * sizeof(double));
    std::memcpy(out + 4 * n, ID, n * sizeof(double));
    double *h1 = out + 5 * n, *h2 = out + 6 * n, *k1 = out + 7 * n, *k2 = out + 8 * n;
    const int C = 32 * G;
    std::vector<double> Mf((size_t)C * 4), Mb((size_t)C * 4);
    for (int t = 0; t < C; t++) {
        const int r0 = t * S, r1 = std::min(n, r0 + S);
        double e0[2], e1[2];
        for (int u = 0; u < 2; u++) {
            double ym1 = (u == 0) ? 1.0 : 0.0, ym2 = (u == 0) ? 0.0 : 1.0;
            for (int j = r0; j < r1; j++) {
                double y = -L2[j] * ym2 - L1[j] * ym1;
                (u == 0 ? h1 : h2)[j] = y;
                ym2 = ym1; ym1 = y;
            }
            e0[u] = ym1; e1[u] = ym2;   // an empty chunk passes its state on unchanged
        }
        Mf[4 * t] = e0[0]; Mf[4 * t + 1] = e0[1]; Mf[4 * t + 2] = e1[0]; Mf[4 * t + 3] = e1[1];
        for (int u = 0; u < 2; u++) {
            double xp1 = (u == 0) ? 1.0 : 0.0, xp2 = (u == 0) ? 0.0 : 1.0;
            for (int j = r1 - 1; j >= r0; j--) {
                double x = (-U1[j] * xp1 - U2[j] * xp2) * ID[j];
                (u == 0 ? k1 : k2)[j] = x;
                xp2 = xp1; xp1 = x;
            }
            e0[u] = xp1; e1[u] = xp2;
        }
        Mb[4 * t] = e0[0]; Mb[4 * t + 1] = e0[1]; Mb[4 * t + 2] = e1[0]; Mb[4 * t + 3] = e1[1];
    }
    auto mul = [](const double* A, const double* B, double* Cm) {   // Cm = A B
        double c0 = A[0] * B[0] + A[1] * B[2], c1 = A[0] * B[1] + A[1] * B[3];
        double c2 = A[2] * B[0] + A[3] * B[2], c3 = A[2] * B[1] + A[3] * B[3];
        Cm[0] = c0; Cm[1] = c1; Cm[2] = c2; Cm[3] = c3;
    };
    const double I[4] = {1.0, 0.0, 0.0, 1.0};
    for (int g = 0; g < G; g++) {
        double* W = out + 9 * n + (size_t)WARP_TAB * g;
        double *Pf = W, *Pb = W + 640, *R = W + 1280, *Q = W + 1408, *A = W + 1536, *B = W + 1540;
        const double* mf = &Mf[(size_t)128 * g];
        const double* mb = &Mb[(size_t)128 * g];
        double Af[32][4], Ab[32][4];
        std::memcpy(Af, mf, sizeof Af);
        std::memcpy(Ab, mb, sizeof Ab);
        for (int d = 0, off = 1; d < 5; d++, off <<= 1) {
            for (int t = 0; t < 32; t++) {
                std::memcpy(Pf + (d * 32 + t) * 4, Af[t], 4 * sizeof(double));
                std::memcpy(Pb + (d * 32 + t) * 4, Ab[t], 4 * sizeof(double));
            }
            double nf[32][4], nb[32][4];
            for (int t = 0; t < 32; t++) {
                if (t >= off) mul(Af[t], Af[t - off], nf[t]); else std::memcpy(nf[t], Af[t], sizeof nf[t]);
                if (t + off < 32) mul(Ab[t], Ab[t + off], nb[t]); else std::memcpy(nb[t], Ab[t], sizeof nb[t]);
            }
            std::memcpy(Af, nf, sizeof Af);
            std::memcpy(Ab, nb, sizeof Ab);
        }
        // R_t = Mf_{t-1} ... Mf_0, A = Mf_31 ... Mf_0
        double acc[4];
        std::memcpy(acc, I, sizeof acc);
        for (int t = 0; t < 32; t++) {
            std::memcpy(R + 4 * t, acc, sizeof acc);
            double nx4[4];
            mul(mf + 4 * t, acc, nx4);
            std::memcpy(acc, nx4, sizeof acc);
        }
        std::memcpy(A, acc, sizeof acc);
        // Q_t = Mb_{t+1} ... Mb_31, B = Mb_0 ... Mb_31
        std::memcpy(acc, I, sizeof acc);
        for (int t = 31; t >= 0; t--) {
            std::memcpy(Q + 4 * t, acc, sizeof acc);
            double nx4[4];
            mul(mb + 4 * t, acc, nx4);
            std::memcpy(acc, nx4, sizeof acc);
        }
        std::memcpy(B, acc, sizeof acc);
    }
}

// Warps per line (as log2, the table group) for a launch of ns sweeps on
// rows of n: one sweep at a time spreads each line over four warps (one per
// SM sub-partition), several sweeps over two, unless the tuner chose; every
// warp of a group keeps at least 32 rows.
int plain_group(const tb_ctx* c, int n, int ns, int whole) {
    if (whole) return 0;
    int gi = (ns == 1) ? (c->tune_pg1 ? c->tune_pg1 - 1 : 2) : (c->tune_pg3 ? c->tune_pg3 - 1 : 1);
    while (gi > 0 && n <= 32 * group_warps(gi - 1)) gi--;
    return gi;
}

template <int S, int G>
int launch_wsor_s(tb_ctx* c, const PlainDev& P, int l, int ns, double rf, int whole, int gi, int groups) {
    const int n = c->g.ptsy[l], lines = whole ? c->g.ptsx[l] : RING;
    const size_t smem = ((size_t)tab_size(n, G) + (size_t)2 * lines * n + (size_t)4 * G * groups) * sizeof(double);
    TB_CUDA(cudaFuncSetAttribute(k_wsor<S, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // at most the groups the kernel's register count allows in one block; a
    // group then runs the tasks of several sweeps in some steps, which are independent
    cudaFuncAttributes fa;
    TB_CUDA(cudaFuncGetAttributes(&fa, k_wsor<S, G>));
    groups = std::max(1, std::min(groups, fa.maxThreadsPerBlock / (32 * G)));
    k_wsor<S, G><<<2 * c->g.K, 32 * G * groups, smem, c->stream>>>(P, l, ns, rf, whole, gi);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}

template <int G>
int launch_wsor_g(tb_ctx* c, const PlainDev& P, int l, int ns, double rf, int whole, int gi, int groups, int S) {
    switch (S) {
        case 1: return launch_wsor_s<1, G>(c, P, l, ns, rf, whole, gi, groups);
        case 2: return launch_wsor_s<2, G>(c, P, l, ns, rf, whole, gi, groups);
        case 3: return launch_wsor_s<3, G>(c, P, l, ns, rf, whole, gi, groups);
        case 4: return launch_wsor_s<4, G>(c, P, l, ns, rf, whole, gi, groups);
        case 5: return launch_wsor_s<5, G>(c, P, l, ns, rf, whole, gi, groups);
        case 6: return launch_wsor_s<6, G>(c, P, l, ns, rf, whole, gi, groups);
        case 7: return launch_wsor_s<7, G>(c, P, l, ns, rf, whole, gi, groups);
        case 8: return launch_wsor_s<8, G>(c, P, l, ns, rf, whole, gi, groups);
        default: break;
    }
    if (G == 1) {
        switch (S) {
            case 9: return launch_wsor_s<9, 1>(c, P, l, ns, rf, whole, gi, groups);
            case 10: return launch_wsor_s<10, 1>(c, P, l, ns, rf, whole, gi, groups);
            case 11: return launch_wsor_s<11, 1>(c, P, l, ns, rf, whole, gi, groups);
            case 12: return launch_wsor_s<12, 1>(c, P, l, ns, rf, whole, gi, groups);
            default: return launch_wsor_s<16, 1>(c, P, l, ns, rf, whole, gi, groups);
        }
    }
    tb_set_error("plain Poisson: %d rows per lane on %d warps per line", S, G);
    return TB_ERR_ARG;
}

// `itera` sweeps of sor at level l (poisson_par.f:167-226) for every active mode.
int plain_sor(tb_ctx* c, const PlainDev& P, int l, int itera, double rf) {
    const int nxl = c->g.ptsx[l], n = c->g.ptsy[l], m = nxl - 2;
    const size_t whole_bytes = ((size_t)tab_size(n, 1) + (size_t)2 * nxl * n + 4 * 32) * sizeof(double);
    const bool can_whole = whole_bytes <= (size_t)200 * 1024;
    cudaEvent_t ps = nullptr;
    if (tb_prof_begin(c, PROF_SOR, &ps)) return TB_ERR_CUDA;
    int done = 0;
    while (done < itera) {
        int ns, whole, groups;
        if (m < 7 || (itera - done > MAX_STREAM_SWEEPS && can_whole)) {
            // all remaining sweeps with the level held in shared memory; group w
            // runs the sweeps w, w + W, ... (the wavefront stays full once
            // W > (m - 2) / LAG)
            whole = 1;
            ns = itera - done;
            groups = (m < 7) ? 1 : std::min({32, ns, (m - 2) / LAG + 1});
        } else {
            whole = 0;
            ns = std::min(MAX_STREAM_SWEEPS, itera - done);
            groups = ns;
        }
        const int gi = (m < 7) ? 0 : plain_group(c, n, ns, whole);
        const int G = group_warps(gi), S = rows_per_lane(n, G);
        int r;
        if (G == 1) r = launch_wsor_g<1>(c, P, l, ns, rf, whole, gi, groups, S);
        else if (G == 2) r = launch_wsor_g<2>(c, P, l, ns, rf, whole, gi, groups, S);
        else r = launch_wsor_g<4>(c, P, l, ns, rf, whole, gi, groups, S);
        if (r) return r;
        done += ns;
    }
    return tb_prof_end(c, PROF_SOR, ps);
}

}  // namespace

// Times `itera` sweeps at level l with each line group in `gis`, on the plain
// form's work arrays (rebuilt from uy by every solve), and keeps the fastest.
int tb_plain_tune(tb_ctx* c, int l, int itera, const int* gis, int ngis, int* best, float* best_ms) {
    if (!c->pl_fc) { tb_set_error("plain Poisson arrays missing"); return TB_ERR_STATE; }
    PlainDev P = make_plain(c);
    cudaEvent_t a, b;
    TB_CUDA(cudaEventCreate(&a));
    TB_CUDA(cudaEventCreate(&b));
    int* keep = itera == 1 ? &c->tune_pg1 : &c->tune_pg3;
    const int old = *keep;
    *best = -1;
    *best_ms = 1e30f;
    int r = TB_OK;
    for (int q = 0; q < ngis && !r; q++) {
        *keep = gis[q] + 1;
        k_pactivate<<<tb_blocks(c->g.K, 64), 64, 0, c->stream>>>(c->pstate, c->g.K);
        r = plain_sor(c, P, l, itera, 1.0);   // warm-up
        if (r) break;
        cudaEventRecord(a, c->stream);
        for (int rep = 0; rep < 3 && !r; rep++) r = plain_sor(c, P, l, itera, 1.0);
        cudaEventRecord(b, c->stream);
        float ms = 0.f;
        if (!r && cudaEventSynchronize(b) == cudaSuccess) cudaEventElapsedTime(&ms, a, b);
        if (!r && ms / 3 < *best_ms) { *best_ms = ms / 3; *best = gis[q]; }
    }
    *keep = (*best >= 0) ? *best + 1 : old;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (!r) TB_CUDA(cudaGetLastError());
    return r;
}

// Line-contiguous real/imaginary multigrid arrays and line-solve tables of the plain form.
int tb_plain_setup(tb_ctx* c) {
    const int K = c->g.K, ny = c->g.ny, msh = c->g.msh;
    if (ny > 32 * 16) { tb_set_error("plain Poisson: ny above 512"); return TB_ERR_ARG; }
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
    if (!c->pl_maxsq) TB_CUDA(cudaMalloc(&c->pl_maxsq, K * sizeof(unsigned long long)));
    TB_CUDA(cudaMemset(c->pl_maxsq, 0, K * sizeof(unsigned long long)));
    // band LU of the y-line matrices (band5_poi, penta_par.f:308-364), factored
    // once per (type, level, mode), with the chunk tables of each line group
    const size_t bs = tab_block(ny);
    std::vector<double> all((size_t)NGROUP * 2 * msh * K * bs, 0.0), a;
    std::vector<double> L1(ny), L2(ny), U1(ny), U2(ny), ID(ny);
    for (int type = 0; type < 2; type++)
        for (int l = 0; l < msh; l++)
            for (int k = 0; k < K; k++) {
                tb_poisson_band_matrix(c, type, l + 1, k + 1, a);
                const int n = c->g.ptsy[l];
                tb_band5_factor(n, a, L1.data(), L2.data(), U1.data(), U2.data(), ID.data());
                for (int gi = 0; gi < NGROUP; gi++) {
                    const int G = group_warps(gi);
                    double* T = &all[((((size_t)gi * 2 + type) * msh + l) * K + k) * bs];
                    group_tables(n, rows_per_lane(n, G), G, L1.data(), L2.data(), U1.data(), U2.data(), ID.data(), T);
                }
            }
    if (c->pl_tab) cudaFree(c->pl_tab);
    c->pl_tab = nullptr;
    TB_CUDA(cudaMalloc(&c->pl_tab, all.size() * sizeof(double)));
    TB_CUDA(cudaMemcpy(c->pl_tab, all.data(), all.size() * sizeof(double), cudaMemcpyHostToDevice));
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
        k_pdefect<<<dim3(tb_blocks(per, 128), K), 128, 0, c->stream>>>(P, l, si);
        TB_CHECK_LAUNCH(c);
        return tb_prof_end(c, PROF_DEFECT, ps);
    };
    int r;
    for (int v = 1; v <= vmax; v++) {
        for (int l = 0; l < msh - 1; l++) {
            if ((r = plain_sor(c, P, l, 3, 1.2))) return r;
            if ((r = defect(l, -1.0))) return r;
            if (l == 0) { k_pcheck<<<tb_blocks(K, 64), 64, 0, c->stream>>>(P, erro, v); TB_CHECK_LAUNCH(c); }
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
