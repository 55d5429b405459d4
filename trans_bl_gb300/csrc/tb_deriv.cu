// tb_deriv.cu -- batched compact line operators of the stage.
//
// x-lines (derparx/derparxx, derivs_par.f:80-113 with rhsx/rhsxx 259-397 and
// tridparx 775-858; filter_trid filter_par.f:144-332) and y-lines (dery/
// deryfv/deryy derivs_par.f:116-177 with rhsy/rhsyfv/rhsyy 400-611 and tridy
// 947-975).  Every line is an independent tridiagonal solve with a constant
// LHS.  A y-line is strided by nx, so one thread per line already reads
// coalesced rows across a warp; an x-line is contiguous, so a whole warp
// shares one x-line (k_xwarp).  Launches batch several fields so that each SM
// sub-partition has full warps of FP64 work (GB300 issues one FP64 warp
// instruction per 64 cycles per sub-partition whatever the active-lane count).
#include "tb_internal.h"
#include <cstring>

namespace {

// Complex arithmetic in the working precision R (double, or float for the
// mixed form's lines of modes k >= 1).
template <class R> struct Cx;
template <> struct Cx<double> { using V = double2; };
template <> struct Cx<float> { using V = float2; };
template <class V, class R> __device__ __forceinline__ V cmul(R s, V a) { return V{s * a.x, s * a.y}; }
template <class V> __device__ __forceinline__ V cadd(V a, V b) { return V{a.x + b.x, a.y + b.y}; }
template <class V> __device__ __forceinline__ V csub(V a, V b) { return V{a.x - b.x, a.y - b.y}; }
template <class V, class R> __device__ __forceinline__ V cfma(R s, V a, V b) { return V{fma(s, a.x, b.x), fma(s, a.y, b.y)}; }

struct XArgs {
    XJob job[8];
    int njobs, nx, ny, K;
    int fp32_modes;   // lines of modes k >= 1 in FP32 (mixed form)
    double inv12dx, inv120dx, inv24dx, inv60dxx, inv360dxx, inv4dxx;
    double af, bf, cf, df;
    TriLHS t[3];
};

// The chunked Thomas tables of a TriLHS in precision R.
template <class R> struct TriT;
template <> struct TriT<double> {
    const double *a, *g, *ib, *hf, *hb, *pf, *pb;
    __device__ explicit TriT(const TriLHS& T) : a(T.a), g(T.g), ib(T.ib), hf(T.hf), hb(T.hb), pf(T.pf), pb(T.pb) {}
};
template <> struct TriT<float> {
    const float *a, *g, *ib, *hf, *hb, *pf, *pb;
    __device__ explicit TriT(const TriLHS& T) : a(T.af), g(T.gf), ib(T.ibf), hf(T.hff), hb(T.hbf), pf(T.pff), pb(T.pbf) {}
};

// A line staged in shared memory in lane chunks: row i at (i / S) * Sp + i % S
// (Sp = S rounded up to odd, so the accesses of consecutive lanes at the
// same chunk offset fall in distinct banks).
template <class V>
struct SmemLine {
    const V* F;
    int S, Sp;
    __device__ __forceinline__ V operator[](int i) const { return F[(i / S) * Sp + i % S]; }
};

// RHS of one x-line point (rows 0-based); f is a SmemLine.
template <int OP, class R, class Line>
__device__ __forceinline__ typename Cx<R>::V xrhs(const Line& f, int i, int n, const XArgs& A) {
    using V = typename Cx<R>::V;
    if (OP == XOP_D1) {
        const R i12 = (R)A.inv12dx, i120 = (R)A.inv120dx, i24 = (R)A.inv24dx;
        if (i >= 2 && i < n - 2) {
            V d2 = csub(f[i + 2], f[i - 2]), d1 = csub(f[i + 1], f[i - 1]);
            return cmul(i12, cfma((R)28, d1, d2));
        }
        if (i == 0) {
            V s = cmul((R)-25, f[0]); s = cfma((R)48, f[1], s); s = cfma((R)-36, f[2], s); s = cfma((R)16, f[3], s);
            s = cfma((R)-3, f[4], s); return cmul(i12, s);
        }
        if (i == 1) {
            V s = cmul((R)-406, f[0]); s = cfma((R)-300, f[1], s); s = cfma((R)760, f[2], s); s = cfma((R)-80, f[3], s);
            s = cfma((R)30, f[4], s); s = cfma((R)-4, f[5], s); return cmul(i120, s);
        }
        int m = n - 1;
        if (i == m - 1) {
            V s = cmul((R)-406, f[m]); s = cfma((R)-300, f[m - 1], s); s = cfma((R)760, f[m - 2], s);
            s = cfma((R)-80, f[m - 3], s); s = cfma((R)30, f[m - 4], s); s = cfma((R)-4, f[m - 5], s);
            return cmul(-i120, s);
        }
        V s = cmul((R)-74, f[m]); s = cfma((R)16, f[m - 1], s); s = cfma((R)72, f[m - 2], s); s = cfma((R)-16, f[m - 3], s);
        s = cfma((R)2, f[m - 4], s); return cmul(-i24, s);
    } else if (OP == XOP_D2) {
        const R i4 = (R)A.inv4dxx, i60 = (R)A.inv60dxx, i360 = (R)A.inv360dxx;
        if (i >= 2 && i < n - 2) {
            V s2 = cadd(f[i + 2], f[i - 2]), s1 = cadd(f[i + 1], f[i - 1]);
            V s = cmul((R)3, s2); s = cfma((R)48, s1, s); s = cfma((R)-102, f[i], s);
            return cmul(i4, s);
        }
        int m = n - 1;
        int b = (i < 2) ? 0 : m;       // anchor
        int e = (i < 2) ? 1 : -1;      // direction
        if (i == 0 || i == m) {
            V s = cmul((R)9775, f[b]); s = cfma((R)-20285, f[b + e], s); s = cfma((R)11170, f[b + 2 * e], s);
            s = cfma((R)-550, f[b + 3 * e], s); s = cfma((R)-145, f[b + 4 * e], s); s = cfma((R)35, f[b + 5 * e], s);
            return cmul(i60, s);
        }
        V s = cmul((R)4834, f[b]); s = cfma((R)-8424, f[b + e], s); s = cfma((R)1890, f[b + 2 * e], s);
        s = cfma((R)2320, f[b + 3 * e], s); s = cfma((R)-810, f[b + 4 * e], s); s = cfma((R)216, f[b + 5 * e], s);
        s = cfma((R)-26, f[b + 6 * e], s);
        return cmul(i360, s);
    } else {  // filter
        if (i >= 3 && i < n - 3) {
            V s = cmul((R)A.af, f[i]);
            s = cfma((R)A.bf, cadd(f[i + 1], f[i - 1]), s);
            s = cfma((R)A.cf, cadd(f[i + 2], f[i - 2]), s);
            s = cfma((R)A.df, cadd(f[i + 3], f[i - 3]), s);
            return s;
        }
        int m = n - 1;
        int b = (i < 3) ? 0 : m;
        int e = (i < 3) ? 1 : -1;
        int r = (i < 3) ? i : m - i;
        const R w0[3][5] = {{15, 4, -6, 4, -1}, {1, 12, 6, -4, 1}, {-1, 4, 10, 4, -1}};
        V s = cmul(w0[r][0], f[b]);
#pragma unroll
        for (int q = 1; q < 5; q++) s = cfma(w0[r][q], f[b + q * e], s);
        return cmul((R)0.0625, s);
    }
}

template <class V> __device__ __forceinline__ V to_v(cplx c);
template <> __device__ __forceinline__ double2 to_v<double2>(cplx c) { return c; }
template <> __device__ __forceinline__ float2 to_v<float2>(cplx c) { return make_float2((float)c.x, (float)c.y); }
__device__ __forceinline__ cplx to_c(double2 v) { return v; }
__device__ __forceinline__ cplx to_c(float2 v) { return make_double2((double)v.x, (double)v.y); }

// One x-line (derparx/derparxx/filter_trid) on one warp in precision R: the
// line is staged in shared memory with coalesced loads; lane t owns rows
// [tS, tS + S) and runs the Thomas sweeps over its chunk with zero carry-in,
// the carries of the forward and backward sweeps cross the lanes by a
// Kogge-Stone scan of the precomputed chunk responses (TriLHS pf/pb), and
// each row is fixed up with its precomputed response hf/hb.  HBM stays FP64.
template <int OP, class R>
__device__ __forceinline__ void xline(const XArgs& A, const TriLHS& TL, const cplx* __restrict__ f, cplx* __restrict__ o,
                                      void* wsm) {
    using V = typename Cx<R>::V;
    const TriT<R> T(TL);
    const int lane = threadIdx.x & 31;
    const int S = TL.S, Sp = S | 1, n = A.nx;
    V* F = reinterpret_cast<V*>(wsm);   // the line; the sweeps then overwrite each lane's rows in place
    for (int i = lane; i < n; i += 32) F[(i / S) * Sp + i % S] = to_v<V>(f[i]);
    __syncwarp();
    const SmemLine<V> L{F, S, Sp};
    const int H = (OP == XOP_FILTER) ? 3 : 2;
    const int r0 = lane * S, r1 = min(n, r0 + S);
    V* Ul = F + lane * Sp;
    // Before any lane overwrites its rows, each takes what it reads outside
    // them or ahead of its own sweep: the right-hand sides of its boundary
    // rows (stencils reaching up to 6 rows in), the first window of its
    // interior rows, and the H rows after its chunk.
    const int ib0 = max(r0, H), ie = min(r1, n - H);   // the chunk's interior rows [ib0, ie)
    V rs0[3], rs1[3], hi[3], w[7];
#pragma unroll
    for (int q = 0; q < 3; q++) {
        rs0[q] = V{0, 0}; rs1[q] = V{0, 0}; hi[q] = V{0, 0};
        const int e = n - H + q;
        if (q < H && q >= r0 && q < r1) rs0[q] = xrhs<OP, R>(L, q, n, A);
        if (q < H && e >= r0 && e < r1) rs1[q] = xrhs<OP, R>(L, e, n, A);
        if (q < H && r1 + q < n) hi[q] = L[r1 + q];
    }
#pragma unroll
    for (int q = 0; q < 7; q++) w[q] = V{0, 0};
    if (ib0 < ie) {
#pragma unroll
        for (int q = 0; q < 2 * H; q++) w[q] = L[ib0 - H + q];
    }
    __syncwarp();
    // forward sweep over the chunk with zero carry-in
    V u = V{0, 0};
#pragma unroll
    for (int q = 0; q < 3; q++)
        if (q < H && q >= r0 && q < r1) {
            V r = rs0[q];
            R a = T.a[q], ib = T.ib[q];
            u = V{(r.x - a * u.x) * ib, (r.y - a * u.y) * ib};
            Ul[q - r0] = u;
        }
    if (ib0 < ie) {
        int nc = (ib0 + H) / S, no = (ib0 + H) % S;   // chunk slot of row i + H
        for (int i = ib0; i < ie; i++) {
            const int d = i + H - r1;                 // >= 0: row i + H is after the chunk
            V h = hi[0];
            if (d == 1) h = hi[1];
            if (d == 2) h = hi[2];
            w[2 * H] = (d < 0) ? F[nc * Sp + no] : h;
            if (++no == S) { no = 0; nc++; }
            V r;
            if (OP == XOP_D1) {
                V d2 = csub(w[4], w[0]), d1 = csub(w[3], w[1]);
                r = cmul((R)A.inv12dx, cfma((R)28, d1, d2));
            } else if (OP == XOP_D2) {
                V q = cmul((R)3, cadd(w[4], w[0]));
                q = cfma((R)48, cadd(w[3], w[1]), q);
                q = cfma((R)-102, w[2], q);
                r = cmul((R)A.inv4dxx, q);
            } else {
                V q = cmul((R)A.af, w[3]);
                q = cfma((R)A.bf, cadd(w[4], w[2]), q);
                q = cfma((R)A.cf, cadd(w[5], w[1]), q);
                q = cfma((R)A.df, cadd(w[6], w[0]), q);
                r = q;
            }
            R a = T.a[i], ib = T.ib[i];
            u = V{(r.x - a * u.x) * ib, (r.y - a * u.y) * ib};
            Ul[i - r0] = u;
#pragma unroll
            for (int q = 0; q < 2 * H; q++) w[q] = w[q + 1];
        }
    }
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const int e = n - H + q;
        if (q < H && e >= r0 && e < r1) {
            V r = rs1[q];
            R a = T.a[e], ib = T.ib[e];
            u = V{(r.x - a * u.x) * ib, (r.y - a * u.y) * ib};
            Ul[e - r0] = u;
        }
    }
    // forward carries: true chunk-end values by a scan, carry-in = previous lane's
    V b = (r1 > r0) ? u : V{0, 0};
#pragma unroll
    for (int d = 0, off = 1; d < 5; d++, off <<= 1) {
        R ox = __shfl_up_sync(0xffffffffu, b.x, off), oy = __shfl_up_sync(0xffffffffu, b.y, off);
        if (lane >= off) { R m = T.pf[d * 32 + lane]; b.x = fma(m, ox, b.x); b.y = fma(m, oy, b.y); }
    }
    V Uin;
    Uin.x = __shfl_up_sync(0xffffffffu, b.x, 1); Uin.y = __shfl_up_sync(0xffffffffu, b.y, 1);
    if (lane == 0) Uin = V{0, 0};
    // forward fix-up fused with the backward sweep over the chunk (zero carry from the right)
    V x = V{0, 0};
    for (int q = r1 - 1; q >= r0; q--) {
        R h = T.hf[q];
        V uu = Ul[q - r0];
        uu = V{fma(h, Uin.x, uu.x), fma(h, Uin.y, uu.y)};
        if (q < r1 - 1) { R g = T.g[q + 1]; x = V{uu.x - g * x.x, uu.y - g * x.y}; }
        else x = uu;
        Ul[q - r0] = x;
    }
    // backward carries: true chunk-start values by a scan from the high lanes
    b = (r1 > r0) ? x : V{0, 0};
#pragma unroll
    for (int d = 0, off = 1; d < 5; d++, off <<= 1) {
        R ox = __shfl_down_sync(0xffffffffu, b.x, off), oy = __shfl_down_sync(0xffffffffu, b.y, off);
        if (lane + off < 32) { R m = T.pb[d * 32 + lane]; b.x = fma(m, ox, b.x); b.y = fma(m, oy, b.y); }
    }
    V Xin;
    Xin.x = __shfl_down_sync(0xffffffffu, b.x, 1); Xin.y = __shfl_down_sync(0xffffffffu, b.y, 1);
    if (lane == 31) Xin = V{0, 0};
    for (int q = r0; q < r1; q++) {
        R h = T.hb[q];
        V xx = Ul[q - r0];
        Ul[q - r0] = V{fma(h, Xin.x, xx.x), fma(h, Xin.y, xx.y)};
    }
    __syncwarp();
    for (int q = lane; q < n; q += 32) o[q] = to_c(F[(q / S) * Sp + q % S]);
}

// One warp per x-line of the batched jobs; lines of modes k >= 1 run in FP32
// when A.fp32_modes is set (the mixed form: they hold only the disturbance).
// Shared memory per warp: 32 x Sp complex FP64 (the FP32 path uses half).
template <int OP>
__global__ void __launch_bounds__(64) k_xwarp(XArgs A) {
    extern __shared__ cplx xs[];
    const int wib = threadIdx.x >> 5;
    const TriLHS& T = A.t[OP];
    const int Sp = T.S | 1, n = A.nx;
    const long gw = (long)blockIdx.x * (blockDim.x >> 5) + wib;
    const int nlines = A.ny * A.K;
    const int jb = (int)(gw / nlines);
    if (jb >= A.njobs) return;                 // uniform over the warp
    const XJob& J = A.job[jb];
    if (J.op != OP) return;
    const int line = (int)(gw - (long)jb * nlines);
    void* wsm = xs + (size_t)wib * 32 * Sp;
    const cplx* f = J.src + (size_t)line * n;
    cplx* o = J.dst + (size_t)line * n;
    if (A.fp32_modes && line >= A.ny) xline<OP, float>(A, T, f, o, wsm);   // line / ny = mode k >= 1
    else xline<OP, double>(A, T, f, o, wsm);
}

struct YArgs {
    YJob job[8];
    int njobs, nx, ny, K;
    TriLHS t[3];
    YRhs r[3];
};

template <int OP>
__global__ void __launch_bounds__(128) k_ylines(YArgs A) {
    int nlines = A.nx * A.K;
    int gid = blockIdx.x * blockDim.x + threadIdx.x;
    int jb = gid / nlines;
    int line = gid - jb * nlines;
    if (jb >= A.njobs) return;
    const YJob& J = A.job[jb];
    if (J.op != OP) return;
    int i = line % A.nx, k = line / A.nx;
    int ny = A.ny;
    size_t s = A.nx;
    size_t base = (size_t)i + (size_t)A.nx * ny * k;
    const cplx* __restrict__ f = J.src + base;
    cplx* __restrict__ o = J.dst + base;
    const TriLHS& T = A.t[OP];
    const YRhs& R = A.r[OP];
    cplx u = make_double2(0.0, 0.0);
    // one row of the forward sweep with its rhs from the tables (boundary rows)
    auto generic = [&](int j) {
        cplx r = make_double2(0.0, 0.0);
        const int c0 = R.cnt[j], of = R.off[j];
        const double* w = R.w + 7 * j;
        for (int m = 0; m < c0; m++) r = cfma(w[m], f[(size_t)(j + of + m) * s], r);
        const double a = T.a[j], ib = T.ib[j];
        u = make_double2((r.x - a * u.x) * ib, (r.y - a * u.y) * ib);
        o[(size_t)j * s] = u;
    };
    // The sweeps are sequential in j, so each row's loads are issued YPD rows
    // ahead into a register ring; the interior rows j = 2 .. ny-3 (five-point
    // rhs f[j-2 .. j+2], derivs_par.f:400-611) keep their window in registers.
    constexpr int YPD = 8;
    generic(0);
    generic(1);
    {
        cplx w0 = f[0], w1 = f[s], w2 = f[2 * s], w3 = f[3 * s];
        cplx pre[YPD];
#pragma unroll
        for (int q = 0; q < YPD; q++) pre[q] = (4 + q < ny) ? f[(size_t)(4 + q) * s] : make_double2(0.0, 0.0);
        for (int jb = 2; jb < ny - 2; jb += YPD) {
#pragma unroll
            for (int q = 0; q < YPD; q++) {
                const int j = jb + q;
                if (j < ny - 2) {
                    const cplx w4 = pre[q];   // row j + 2
                    const int nr = j + 2 + YPD;
                    if (nr < ny) pre[q] = f[(size_t)nr * s];
                    const double* w = R.w + 7 * j;
                    cplx r = cmul(w[0], w0);
                    r = cfma(w[1], w1, r);
                    r = cfma(w[2], w2, r);
                    r = cfma(w[3], w3, r);
                    r = cfma(w[4], w4, r);
                    const double a = T.a[j], ib = T.ib[j];
                    u = make_double2((r.x - a * u.x) * ib, (r.y - a * u.y) * ib);
                    o[(size_t)j * s] = u;
                    w0 = w1; w1 = w2; w2 = w3; w3 = w4;
                }
            }
        }
    }
    generic(ny - 2);
    generic(ny - 1);
    // backward sweep, rows ny-2 .. 0, the forward values read YPD rows ahead
    {
        cplx pre[YPD];
#pragma unroll
        for (int q = 0; q < YPD; q++) pre[q] = (ny - 2 - q >= 0) ? o[(size_t)(ny - 2 - q) * s] : make_double2(0.0, 0.0);
        for (int jb = ny - 2; jb >= 0; jb -= YPD) {
#pragma unroll
            for (int q = 0; q < YPD; q++) {
                const int j = jb - q;
                if (j >= 0) {
                    const cplx v = pre[q];
                    const int nr = j - YPD;
                    if (nr >= 0) pre[q] = o[(size_t)nr * s];
                    const double g = T.g[j + 1];
                    u = make_double2(v.x - g * u.x, v.y - g * u.y);
                    o[(size_t)j * s] = u;
                }
            }
        }
    }
}

}  // namespace

int tb_launch_xlines(tb_ctx* c, const XJob* jobs, int njobs) {
    if (njobs <= 0) return TB_OK;
    if (njobs > 8) {
        int r = tb_launch_xlines(c, jobs, 8);
        if (r) return r;
        return tb_launch_xlines(c, jobs + 8, njobs - 8);
    }
    XArgs A;
    std::memset(&A, 0, sizeof A);
    for (int q = 0; q < njobs; q++) {
        if (jobs[q].src == jobs[q].dst) { tb_set_error("x-line job %d: in-place operation", q); return TB_ERR_ARG; }
        A.job[q] = jobs[q];
    }
    A.njobs = njobs; A.nx = c->g.nx; A.ny = c->g.ny; A.K = c->g.K;
    A.fp32_modes = (c->cfg.precision == TB_FORM_MIXED && c->fp32_lines) ? 1 : 0;
    double dx = c->cfg.dx, dxx = dx * dx;
    A.inv12dx = 1.0 / (12.0 * dx); A.inv120dx = 1.0 / (120.0 * dx); A.inv24dx = 1.0 / (24.0 * dx);
    A.inv60dxx = 1.0 / (60.0 * dxx); A.inv360dxx = 1.0 / (360.0 * dxx); A.inv4dxx = 1.0 / (4.0 * dxx);
    double al = c->cfg.alphaf;
    A.af = (11.0 + 10.0 * al) / 16.0; A.bf = (15.0 + 34.0 * al) / 64.0;
    A.cf = (-3.0 + 6.0 * al) / 32.0; A.df = (1.0 - 2.0 * al) / 64.0;
    A.t[0] = c->tx1; A.t[1] = c->tx2; A.t[2] = c->tfil;
    size_t lines = (size_t)njobs * c->g.ny * c->g.K;   // one warp each
    bool has[3] = {false, false, false};
    for (int q = 0; q < njobs; q++) has[jobs[q].op] = true;
    const int WPB = c->tune_xw == 1 ? 1 : 2;   // warps per block (tb_autotune), at most 2 (launch bounds)
    int Sp = c->tx1.S | 1;
    size_t smem = (size_t)WPB * 32 * Sp * sizeof(cplx);
    unsigned nb = tb_blocks(lines, WPB);
    cudaEvent_t ps = nullptr;
    if (tb_prof_begin(c, PROF_XLINES, &ps)) return TB_ERR_CUDA;
    if (has[0]) {
        TB_CUDA(cudaFuncSetAttribute(k_xwarp<XOP_D1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_xwarp<XOP_D1><<<nb, 32 * WPB, smem, c->stream>>>(A); TB_CHECK_LAUNCH(c);
    }
    if (has[1]) {
        TB_CUDA(cudaFuncSetAttribute(k_xwarp<XOP_D2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_xwarp<XOP_D2><<<nb, 32 * WPB, smem, c->stream>>>(A); TB_CHECK_LAUNCH(c);
    }
    if (has[2]) {
        TB_CUDA(cudaFuncSetAttribute(k_xwarp<XOP_FILTER>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_xwarp<XOP_FILTER><<<nb, 32 * WPB, smem, c->stream>>>(A); TB_CHECK_LAUNCH(c);
    }
    return tb_prof_end(c, PROF_XLINES, ps);
}

int tb_launch_ylines(tb_ctx* c, const YJob* jobs, int njobs) {
    if (njobs <= 0) return TB_OK;
    if (njobs > 8) {
        int r = tb_launch_ylines(c, jobs, 8);
        if (r) return r;
        return tb_launch_ylines(c, jobs + 8, njobs - 8);
    }
    YArgs A;
    std::memset(&A, 0, sizeof A);
    for (int q = 0; q < njobs; q++) {
        if (jobs[q].src == jobs[q].dst) { tb_set_error("y-line job %d: in-place operation", q); return TB_ERR_ARG; }
        A.job[q] = jobs[q];
    }
    A.njobs = njobs; A.nx = c->g.nx; A.ny = c->g.ny; A.K = c->g.K;
    A.t[0] = c->ty1; A.t[1] = c->tyfv; A.t[2] = c->ty2;
    A.r[0] = c->ry1; A.r[1] = c->ryfv; A.r[2] = c->ry2;
    size_t total = (size_t)njobs * c->g.nx * c->g.K;
    bool has[3] = {false, false, false};
    for (int q = 0; q < njobs; q++) has[jobs[q].op] = true;
    const int yt = (c->tune_yt == 32 || c->tune_yt == 64) ? c->tune_yt : 128;   // threads per block (tb_autotune)
    unsigned nb = tb_blocks(total, yt);
    cudaEvent_t ps = nullptr;
    if (tb_prof_begin(c, PROF_YLINES, &ps)) return TB_ERR_CUDA;
    if (has[0]) { k_ylines<YOP_D1><<<nb, yt, 0, c->stream>>>(A); TB_CHECK_LAUNCH(c); }
    if (has[1]) { k_ylines<YOP_D1FV><<<nb, yt, 0, c->stream>>>(A); TB_CHECK_LAUNCH(c); }
    if (has[2]) { k_ylines<YOP_D2><<<nb, yt, 0, c->stream>>>(A); TB_CHECK_LAUNCH(c); }
    return tb_prof_end(c, PROF_YLINES, ps);
}
