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

__device__ __forceinline__ cplx cmul(double s, cplx a) { return make_double2(s * a.x, s * a.y); }
__device__ __forceinline__ cplx cadd(cplx a, cplx b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ cplx csub(cplx a, cplx b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ cplx cfma(double s, cplx a, cplx b) { return make_double2(fma(s, a.x, b.x), fma(s, a.y, b.y)); }

struct XArgs {
    XJob job[8];
    int njobs, nx, ny, K;
    double inv12dx, inv120dx, inv24dx, inv60dxx, inv360dxx, inv4dxx;
    double af, bf, cf, df;
    TriLHS t[3];
};

// A line staged in shared memory in lane chunks: row i at (i / S) * Sp + i % S
// (Sp = S rounded up to odd, so the 16-byte accesses of 8 consecutive lanes
// at the same chunk offset fall in distinct banks).
struct SmemLine {
    const cplx* F;
    int S, Sp;
    __device__ __forceinline__ cplx operator[](int i) const { return F[(i / S) * Sp + i % S]; }
};

// RHS of one x-line point (rows 0-based); f is a pointer or a SmemLine.
template <int OP, class Line>
__device__ __forceinline__ cplx xrhs(const Line& f, int i, int n, const XArgs& A) {
    if (OP == XOP_D1) {
        if (i >= 2 && i < n - 2) {
            cplx d2 = csub(f[i + 2], f[i - 2]), d1 = csub(f[i + 1], f[i - 1]);
            return cmul(A.inv12dx, cfma(28.0, d1, d2));
        }
        if (i == 0) {
            cplx s = cmul(-25.0, f[0]); s = cfma(48.0, f[1], s); s = cfma(-36.0, f[2], s); s = cfma(16.0, f[3], s);
            s = cfma(-3.0, f[4], s); return cmul(A.inv12dx, s);
        }
        if (i == 1) {
            cplx s = cmul(-406.0, f[0]); s = cfma(-300.0, f[1], s); s = cfma(760.0, f[2], s); s = cfma(-80.0, f[3], s);
            s = cfma(30.0, f[4], s); s = cfma(-4.0, f[5], s); return cmul(A.inv120dx, s);
        }
        int m = n - 1;
        if (i == m - 1) {
            cplx s = cmul(-406.0, f[m]); s = cfma(-300.0, f[m - 1], s); s = cfma(760.0, f[m - 2], s);
            s = cfma(-80.0, f[m - 3], s); s = cfma(30.0, f[m - 4], s); s = cfma(-4.0, f[m - 5], s);
            return cmul(-A.inv120dx, s);
        }
        cplx s = cmul(-74.0, f[m]); s = cfma(16.0, f[m - 1], s); s = cfma(72.0, f[m - 2], s); s = cfma(-16.0, f[m - 3], s);
        s = cfma(2.0, f[m - 4], s); return cmul(-A.inv24dx, s);
    } else if (OP == XOP_D2) {
        if (i >= 2 && i < n - 2) {
            cplx s2 = cadd(f[i + 2], f[i - 2]), s1 = cadd(f[i + 1], f[i - 1]);
            cplx s = cmul(3.0, s2); s = cfma(48.0, s1, s); s = cfma(-102.0, f[i], s);
            return cmul(A.inv4dxx, s);
        }
        int m = n - 1;
        int b = (i < 2) ? 0 : m;       // anchor
        int e = (i < 2) ? 1 : -1;      // direction
        if (i == 0 || i == m) {
            cplx s = cmul(9775.0, f[b]); s = cfma(-20285.0, f[b + e], s); s = cfma(11170.0, f[b + 2 * e], s);
            s = cfma(-550.0, f[b + 3 * e], s); s = cfma(-145.0, f[b + 4 * e], s); s = cfma(35.0, f[b + 5 * e], s);
            return cmul(A.inv60dxx, s);
        }
        cplx s = cmul(4834.0, f[b]); s = cfma(-8424.0, f[b + e], s); s = cfma(1890.0, f[b + 2 * e], s);
        s = cfma(2320.0, f[b + 3 * e], s); s = cfma(-810.0, f[b + 4 * e], s); s = cfma(216.0, f[b + 5 * e], s);
        s = cfma(-26.0, f[b + 6 * e], s);
        return cmul(A.inv360dxx, s);
    } else {  // filter
        if (i >= 3 && i < n - 3) {
            cplx s = cmul(A.af, f[i]);
            s = cfma(A.bf, cadd(f[i + 1], f[i - 1]), s);
            s = cfma(A.cf, cadd(f[i + 2], f[i - 2]), s);
            s = cfma(A.df, cadd(f[i + 3], f[i - 3]), s);
            return s;
        }
        int m = n - 1;
        int b = (i < 3) ? 0 : m;
        int e = (i < 3) ? 1 : -1;
        int r = (i < 3) ? i : m - i;
        const double w0[3][5] = {{15, 4, -6, 4, -1}, {1, 12, 6, -4, 1}, {-1, 4, 10, 4, -1}};
        cplx s = cmul(w0[r][0], f[b]);
#pragma unroll
        for (int q = 1; q < 5; q++) s = cfma(w0[r][q], f[b + q * e], s);
        return cmul(0.0625, s);
    }
}

// One warp per x-line (derparx/derparxx/filter_trid): the line is staged in
// shared memory with coalesced loads; lane t owns rows [tS, tS + S) and runs
// the Thomas sweeps over its chunk with zero carry-in, the carries of the
// forward and backward sweeps cross the lanes by a Kogge-Stone scan of the
// precomputed chunk responses (TriLHS pf/pb), and each row is fixed up with
// its precomputed response hf/hb.  Shared memory per warp: 2 x 32 x Sp complex.
template <int OP>
__global__ void __launch_bounds__(64) k_xwarp(XArgs A) {
    extern __shared__ cplx xs[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const TriLHS& T = A.t[OP];
    const int S = T.S, Sp = S | 1, n = A.nx;
    const long gw = (long)blockIdx.x * (blockDim.x >> 5) + wib;
    const int nlines = A.ny * A.K;
    const int jb = (int)(gw / nlines);
    if (jb >= A.njobs) return;                 // uniform over the warp
    const XJob& J = A.job[jb];
    if (J.op != OP) return;
    const int line = (int)(gw - (long)jb * nlines);
    cplx* F = xs + (size_t)wib * 64 * Sp;
    cplx* U = F + 32 * Sp;
    const cplx* __restrict__ f = J.src + (size_t)line * n;
    cplx* __restrict__ o = J.dst + (size_t)line * n;
    for (int i = lane; i < n; i += 32) F[(i / S) * Sp + i % S] = f[i];
    __syncwarp();
    const SmemLine L{F, S, Sp};
    const int H = (OP == XOP_FILTER) ? 3 : 2;
    const int r0 = lane * S, r1 = min(n, r0 + S);
    cplx* Ul = U + lane * Sp;
    // forward sweep over the chunk with zero carry-in
    cplx u = make_double2(0.0, 0.0);
    int i = r0;
    for (; i < r1 && i < H; i++) {
        cplx r = xrhs<OP>(L, i, n, A);
        double a = T.a[i], ib = T.ib[i];
        u = make_double2((r.x - a * u.x) * ib, (r.y - a * u.y) * ib);
        Ul[i - r0] = u;
    }
    if (i < r1 && i < n - H) {
        cplx w[7];
#pragma unroll
        for (int q = 0; q < 2 * H; q++) w[q] = L[i - H + q];
        int nc = (i + H) / S, no = (i + H) % S;   // chunk slot of row i + H
        for (; i < r1 && i < n - H; i++) {
            w[2 * H] = F[nc * Sp + no];
            if (++no == S) { no = 0; nc++; }
            cplx r;
            if (OP == XOP_D1) {
                cplx d2 = csub(w[4], w[0]), d1 = csub(w[3], w[1]);
                r = cmul(A.inv12dx, cfma(28.0, d1, d2));
            } else if (OP == XOP_D2) {
                cplx q = cmul(3.0, cadd(w[4], w[0]));
                q = cfma(48.0, cadd(w[3], w[1]), q);
                q = cfma(-102.0, w[2], q);
                r = cmul(A.inv4dxx, q);
            } else {
                cplx q = cmul(A.af, w[3]);
                q = cfma(A.bf, cadd(w[4], w[2]), q);
                q = cfma(A.cf, cadd(w[5], w[1]), q);
                q = cfma(A.df, cadd(w[6], w[0]), q);
                r = q;
            }
            double a = T.a[i], ib = T.ib[i];
            u = make_double2((r.x - a * u.x) * ib, (r.y - a * u.y) * ib);
            Ul[i - r0] = u;
#pragma unroll
            for (int q = 0; q < 2 * H; q++) w[q] = w[q + 1];
        }
    }
    for (; i < r1; i++) {
        cplx r = xrhs<OP>(L, i, n, A);
        double a = T.a[i], ib = T.ib[i];
        u = make_double2((r.x - a * u.x) * ib, (r.y - a * u.y) * ib);
        Ul[i - r0] = u;
    }
    // forward carries: true chunk-end values by a scan, carry-in = previous lane's
    cplx b = (r1 > r0) ? u : make_double2(0.0, 0.0);
#pragma unroll
    for (int d = 0, off = 1; d < 5; d++, off <<= 1) {
        double ox = __shfl_up_sync(0xffffffffu, b.x, off), oy = __shfl_up_sync(0xffffffffu, b.y, off);
        if (lane >= off) { double m = T.pf[d * 32 + lane]; b.x = fma(m, ox, b.x); b.y = fma(m, oy, b.y); }
    }
    cplx Uin;
    Uin.x = __shfl_up_sync(0xffffffffu, b.x, 1); Uin.y = __shfl_up_sync(0xffffffffu, b.y, 1);
    if (lane == 0) Uin = make_double2(0.0, 0.0);
    // forward fix-up fused with the backward sweep over the chunk (zero carry from the right)
    cplx x = make_double2(0.0, 0.0);
    for (int q = r1 - 1; q >= r0; q--) {
        double h = T.hf[q];
        cplx uu = Ul[q - r0];
        uu = make_double2(fma(h, Uin.x, uu.x), fma(h, Uin.y, uu.y));
        if (q < r1 - 1) { double g = T.g[q + 1]; x = make_double2(uu.x - g * x.x, uu.y - g * x.y); }
        else x = uu;
        Ul[q - r0] = x;
    }
    // backward carries: true chunk-start values by a scan from the high lanes
    b = (r1 > r0) ? x : make_double2(0.0, 0.0);
#pragma unroll
    for (int d = 0, off = 1; d < 5; d++, off <<= 1) {
        double ox = __shfl_down_sync(0xffffffffu, b.x, off), oy = __shfl_down_sync(0xffffffffu, b.y, off);
        if (lane + off < 32) { double m = T.pb[d * 32 + lane]; b.x = fma(m, ox, b.x); b.y = fma(m, oy, b.y); }
    }
    cplx Xin;
    Xin.x = __shfl_down_sync(0xffffffffu, b.x, 1); Xin.y = __shfl_down_sync(0xffffffffu, b.y, 1);
    if (lane == 31) Xin = make_double2(0.0, 0.0);
    for (int q = r0; q < r1; q++) {
        double h = T.hb[q];
        cplx xx = Ul[q - r0];
        Ul[q - r0] = make_double2(fma(h, Xin.x, xx.x), fma(h, Xin.y, xx.y));
    }
    __syncwarp();
    for (int q = lane; q < n; q += 32) o[q] = U[(q / S) * Sp + q % S];
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
    for (int j = 0; j < ny; j++) {
        cplx r = make_double2(0.0, 0.0);
        int c0 = R.cnt[j], of = R.off[j];
        const double* w = R.w + 7 * j;
        if (c0 == 5) {
            const cplx* p = f + (size_t)(j + of) * s;
            r = cmul(w[0], p[0]);
            r = cfma(w[1], p[s], r);
            r = cfma(w[2], p[2 * s], r);
            r = cfma(w[3], p[3 * s], r);
            r = cfma(w[4], p[4 * s], r);
        } else {
            for (int m = 0; m < c0; m++) r = cfma(w[m], f[(size_t)(j + of + m) * s], r);
        }
        double a = T.a[j], ib = T.ib[j];
        u = make_double2((r.x - a * u.x) * ib, (r.y - a * u.y) * ib);
        o[(size_t)j * s] = u;
    }
    for (int j = ny - 2; j >= 0; j--) {
        double g = T.g[j + 1];
        cplx v = o[(size_t)j * s];
        u = make_double2(v.x - g * u.x, v.y - g * u.y);
        o[(size_t)j * s] = u;
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
    const int WPB = 2;
    int Sp = c->tx1.S | 1;
    size_t smem = (size_t)WPB * 64 * Sp * sizeof(cplx);
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
    unsigned nb = tb_blocks(total, 128);
    cudaEvent_t ps = nullptr;
    if (tb_prof_begin(c, PROF_YLINES, &ps)) return TB_ERR_CUDA;
    if (has[0]) { k_ylines<YOP_D1><<<nb, 128, 0, c->stream>>>(A); TB_CHECK_LAUNCH(c); }
    if (has[1]) { k_ylines<YOP_D1FV><<<nb, 128, 0, c->stream>>>(A); TB_CHECK_LAUNCH(c); }
    if (has[2]) { k_ylines<YOP_D2><<<nb, 128, 0, c->stream>>>(A); TB_CHECK_LAUNCH(c); }
    return tb_prof_end(c, PROF_YLINES, ps);
}
