// tb_spectral.cu -- spanwise Fourier <-> physical transforms and the
// physical-space products of the stage.
//
// Convention of the reference (nlterms_par.f:303-428, Numerical-Recipes
// realft packing): a field with modes c_k, k = 0..K-1, has physical values
//     p_n = Re c_0 + (Im c_0 / 2) (-1)^n + sum_{k>=1} Re( c_k e^{-2 pi i k n / P} ),
// and the forward transform returns c_0 = (1/P) sum p_n, c_k = (2/P) sum p_n
// e^{+2 pi i k n / P}, zeroes components below 1e-14 and forces Im c_0 = 0.
// Both directions are computed here as a length-P/2 complex FFT plus the
// real-to-complex split, one thread per (i, j) grid line, with exact
// twiddles from a constant table instead of the reference's rotation
// recurrence.
#include "tb_internal.h"
#include "tb_tc.cuh"
#include <cuda_bf16.h>
#include <cstring>
#include <algorithm>
#include <cmath>

#define TW_N 512
__constant__ double c_twr[TW_N], c_twi[TW_N];  // e^{-2 pi i t / TW_N}
__constant__ float c_twrf[TW_N], c_twif[TW_N]; // the same, rounded to FP32

namespace {

__device__ __forceinline__ double twr(int t) { return c_twr[t & (TW_N - 1)]; }
__device__ __forceinline__ double twi(int t) { return c_twi[t & (TW_N - 1)]; }
template <class R> __device__ __forceinline__ R tw_r(int t);
template <class R> __device__ __forceinline__ R tw_i(int t);
template <> __device__ __forceinline__ double tw_r<double>(int t) { return c_twr[t & (TW_N - 1)]; }
template <> __device__ __forceinline__ double tw_i<double>(int t) { return c_twi[t & (TW_N - 1)]; }
template <> __device__ __forceinline__ float tw_r<float>(int t) { return c_twrf[t & (TW_N - 1)]; }
template <> __device__ __forceinline__ float tw_i<float>(int t) { return c_twif[t & (TW_N - 1)]; }

template <int N>
__device__ __forceinline__ int brev(int i) {
    int r = 0;
#pragma unroll
    for (int b = 1; b < N; b <<= 1) { r = (r << 1) | (i & 1); i >>= 1; }
    return r;
}

// In-place radix-2 complex FFT of length N. SIGN = -1: sum X_k e^{-2 pi i km/N};
// SIGN = +1: sum X_k e^{+2 pi i km/N}.
template <int N, int SIGN, class R = double>
__device__ __forceinline__ void cfft(R* re, R* im) {
#pragma unroll
    for (int i = 0; i < N; i++) {
        int j = brev<N>(i);
        if (j > i) {
            R t = re[i]; re[i] = re[j]; re[j] = t;
            t = im[i]; im[i] = im[j]; im[j] = t;
        }
    }
#pragma unroll
    for (int len = 2; len <= N; len <<= 1) {
        const int h = len / 2;
#pragma unroll
        for (int s = 0; s < N; s += len) {
#pragma unroll
            for (int q = 0; q < h; q++) {
                int a = s + q, b = a + h;
                R tr, ti;
                if (q == 0) {
                    tr = re[b]; ti = im[b];
                } else if (4 * q == len) {  // twiddle -SIGN*i ... e^{SIGN*i*pi/2} = SIGN*i
                    tr = (SIGN < 0) ? im[b] : -im[b];
                    ti = (SIGN < 0) ? -re[b] : re[b];
                } else {
                    R wr = tw_r<R>(q * (TW_N / len));
                    R wi = (SIGN < 0) ? tw_i<R>(q * (TW_N / len)) : -tw_i<R>(q * (TW_N / len));
                    tr = wr * re[b] - wi * im[b];
                    ti = wr * im[b] + wi * re[b];
                }
                re[b] = re[a] - tr; im[b] = im[a] - ti;
                re[a] = re[a] + tr; im[a] = im[a] + ti;
            }
        }
    }
}

// Fourier (K modes at stride cs) -> physical p[0..P-1].
template <int P>
__device__ __forceinline__ void to_phys(const cplx* __restrict__ cf, size_t cs, int K, double* p) {
    constexpr int N = P / 2;
    double re[N], im[N];
    cplx c0 = cf[0];
    double C0 = c0.x, CN = 0.5 * c0.y;
    re[0] = C0 + CN; im[0] = C0 - CN;
#pragma unroll
    for (int k = 1; k < N; k++) {
        cplx A = (k < K) ? cf[(size_t)k * cs] : make_double2(0.0, 0.0);
        cplx Bc = (N - k < K) ? cf[(size_t)(N - k) * cs] : make_double2(0.0, 0.0);
        double Br = Bc.x, Bi = -Bc.y;  // conj
        double sr = 0.5 * (A.x + Br), si = 0.5 * (A.y + Bi);
        double dr = 0.5 * (A.x - Br), di = 0.5 * (A.y - Bi);
        double wr = twr(k * (TW_N / P)), wi = twi(k * (TW_N / P));  // e^{-2 pi i k / P}
        re[k] = sr - (wr * di + wi * dr);
        im[k] = si + (wr * dr - wi * di);
    }
    cfft<N, -1>(re, im);
#pragma unroll
    for (int m = 0; m < N; m++) { p[2 * m] = re[m]; p[2 * m + 1] = im[m]; }
}

__device__ __forceinline__ double zap(double v) { return fabs(v) < 1e-14 ? 0.0 : v; }

// physical p[0..P-1] -> Fourier (K modes at stride cs).
template <int P>
__device__ __forceinline__ void to_four(const double* p, int K, cplx* __restrict__ cf, size_t cs) {
    constexpr int N = P / 2;
    double re[N], im[N];
#pragma unroll
    for (int m = 0; m < N; m++) { re[m] = p[2 * m]; im[m] = p[2 * m + 1]; }
    cfft<N, +1>(re, im);
    const double invP = 1.0 / (double)P, two_P = 2.0 / (double)P;
    cf[0] = make_double2(zap((re[0] + im[0]) * invP), 0.0);
#pragma unroll
    for (int k = 1; k < N; k++) {
        if (k >= K) continue;
        double Fr = re[k], Fi = im[k], Gr = re[N - k], Gi = -im[N - k];  // conj(F_{N-k})
        double Er = 0.5 * (Fr + Gr), Ei = 0.5 * (Fi + Gi);
        double gr = Fr - Gr, gi = Fi - Gi;
        double Or = 0.5 * gi, Oi = -0.5 * gr;  // g / (2i)
        double vr = twr(k * (TW_N / P)), vi = -twi(k * (TW_N / P));  // e^{+2 pi i k / P}
        double Hr = Er + (vr * Or - vi * Oi), Hi = Ei + (vr * Oi + vi * Or);
        cf[(size_t)k * cs] = make_double2(zap(two_P * Hr), zap(two_P * Hi));
    }
}

// ---------------------------------------------------------------------------
template <int P>
__global__ void __launch_bounds__(128) k_f_to_p(double* phys, const cplx* four, int n2, int K) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n2) return;
    double p[P];
    to_phys<P>(four + q, n2, K, p);
#pragma unroll
    for (int z = 0; z < P; z++) phys[(size_t)q + (size_t)n2 * z] = p[z];
}
template <int P>
__global__ void __launch_bounds__(128) k_p_to_f(cplx* four, const double* phys, int n2, int K) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n2) return;
    double p[P];
#pragma unroll
    for (int z = 0; z < P; z++) p[z] = phys[(size_t)q + (size_t)n2 * z];
    to_four<P>(p, K, four + q, n2);
}

// nlterms_fi (nlterms_par.f:41-86): a = uy wx - ux wy, b = ux wz - uz wx, c = uz wy - uy wz.
struct NlArgs {
    const cplx *ux, *uy, *uz, *wx, *wy, *wz;
    cplx *a, *b, *c;
    int n2, K;
};
template <int P>
__global__ void __launch_bounds__(128) k_nlterms(NlArgs A) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= A.n2) return;
    size_t cs = A.n2;
    double ph[6][P];
    to_phys<P>(A.ux + q, cs, A.K, ph[0]);
    to_phys<P>(A.uy + q, cs, A.K, ph[1]);
    to_phys<P>(A.uz + q, cs, A.K, ph[2]);
    to_phys<P>(A.wx + q, cs, A.K, ph[3]);
    to_phys<P>(A.wy + q, cs, A.K, ph[4]);
    to_phys<P>(A.wz + q, cs, A.K, ph[5]);
#pragma unroll
    for (int z = 0; z < P; z++) {
        double ux = ph[0][z], uy = ph[1][z], uz = ph[2][z], wx = ph[3][z], wy = ph[4][z], wz = ph[5][z];
        ph[0][z] = uy * wx - ux * wy;
        ph[1][z] = ux * wz - uz * wx;
        ph[2][z] = uz * wy - uy * wz;
    }
    to_four<P>(ph[0], A.K, A.a + q, cs);
    to_four<P>(ph[1], A.K, A.b + q, cs);
    to_four<P>(ph[2], A.K, A.c + q, cs);
}

// ---------------------------------------------------------------------------
// Mixed form of nlterms_fi.  With every field split into its spanwise mean
// M = Re c_0 (which carries the base flow) and its z-varying part d(z), a
// product such as uy wx transforms to
//   mode 0:   M_uy M_wx                 + T(d_uy d_wx)_0
//   mode k:   M_uy wx_k + M_wx uy_k     + T(d_uy d_wx)_k      (k >= 1)
// because T(M d)_k = M c_k(d) exactly (T the forward transform of the
// reference; d holds modes 1..K-1 and the packed Nyquist term).  The linear
// part, which dominates for a disturbance on a base flow, stays in FP64;
// only the quadratic disturbance term goes through FP32 transforms.
// Components below 1e-14 are zeroed and Im c_0 = 0, as nlterms_par.f does.

// z-varying part of a field (mean removed) -> physical p[0..P-1], FP32.
template <int P>
__device__ __forceinline__ void to_phys_dist(const cplx* __restrict__ cf, size_t cs, int K, float* p) {
    constexpr int N = P / 2;
    float re[N], im[N];
    float CN = (float)(0.5 * cf[0].y);
    re[0] = CN; im[0] = -CN;
#pragma unroll
    for (int k = 1; k < N; k++) {
        cplx A = (k < K) ? cf[(size_t)k * cs] : make_double2(0.0, 0.0);
        cplx Bc = (N - k < K) ? cf[(size_t)(N - k) * cs] : make_double2(0.0, 0.0);
        float Ar = (float)A.x, Ai = (float)A.y, Br = (float)Bc.x, Bi = -(float)Bc.y;
        float sr = 0.5f * (Ar + Br), si = 0.5f * (Ai + Bi);
        float dr = 0.5f * (Ar - Br), di = 0.5f * (Ai - Bi);
        float wr = tw_r<float>(k * (TW_N / P)), wi = tw_i<float>(k * (TW_N / P));
        re[k] = sr - (wr * di + wi * dr);
        im[k] = si + (wr * dr - wi * di);
    }
    cfft<N, -1, float>(re, im);
#pragma unroll
    for (int m = 0; m < N; m++) { p[2 * m] = re[m]; p[2 * m + 1] = im[m]; }
}

// physical p[0..P-1] -> modes 0..N-1 in FP32 (re[k], im[k]; Im c_0 = 0).
template <int P>
__device__ __forceinline__ void to_four_f(const float* p, float* cr, float* ci) {
    constexpr int N = P / 2;
    float re[N], im[N];
#pragma unroll
    for (int m = 0; m < N; m++) { re[m] = p[2 * m]; im[m] = p[2 * m + 1]; }
    cfft<N, +1, float>(re, im);
    const float invP = 1.0f / (float)P, two_P = 2.0f / (float)P;
    cr[0] = (re[0] + im[0]) * invP; ci[0] = 0.0f;
#pragma unroll
    for (int k = 1; k < N; k++) {
        float Fr = re[k], Fi = im[k], Gr = re[N - k], Gi = -im[N - k];
        float Er = 0.5f * (Fr + Gr), Ei = 0.5f * (Fi + Gi);
        float gr = Fr - Gr, gi = Fi - Gi;
        float Or = 0.5f * gi, Oi = -0.5f * gr;
        float vr = tw_r<float>(k * (TW_N / P)), vi = -tw_i<float>(k * (TW_N / P));
        cr[k] = two_P * (Er + (vr * Or - vi * Oi));
        ci[k] = two_P * (Ei + (vr * Oi + vi * Or));
    }
}

// Pass 1: one thread per (field f, point q): the FP32 physical disturbance
// d_f(z) into ph[(f * P + z) * n2 + q].
template <int P>
__global__ void __launch_bounds__(128) k_nl_phys(NlArgs A, float* __restrict__ ph) {
    const size_t n2 = A.n2;
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= 6 * n2) return;
    const int f = (int)(t / n2);
    const size_t q = t - (size_t)f * n2;
    const cplx* F = (f == 0) ? A.ux : (f == 1) ? A.uy : (f == 2) ? A.uz : (f == 3) ? A.wx : (f == 4) ? A.wy : A.wz;
    float p[P];
    to_phys_dist<P>(F + q, n2, A.K, p);
    float* o = ph + (size_t)f * P * n2 + q;
#pragma unroll
    for (int z = 0; z < P; z++) o[(size_t)z * n2] = p[z];
}

// Pass 2: one thread per (output o, point q): the quadratic disturbance term
// through the FP32 forward transform, plus the FP64 mean terms.
// out = f[p1] f[q1] - f[p2] f[q2]: a = uy wx - ux wy, b = ux wz - uz wx, c = uz wy - uy wz.
template <int P>
__global__ void __launch_bounds__(128) k_nl_four(NlArgs A, const float* __restrict__ ph) {
    constexpr int N = P / 2;
    const size_t n2 = A.n2;
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= 3 * n2) return;
    const int o = (int)(t / n2);
    const size_t q = t - (size_t)o * n2;
    const int p1 = (o == 0) ? 1 : (o == 1) ? 0 : 2, q1 = (o == 0) ? 3 : (o == 1) ? 5 : 4;
    const int p2 = (o == 0) ? 0 : (o == 1) ? 2 : 1, q2 = (o == 0) ? 4 : (o == 1) ? 3 : 5;
    const float *a1 = ph + (size_t)p1 * P * n2 + q, *b1 = ph + (size_t)q1 * P * n2 + q;
    const float *a2 = ph + (size_t)p2 * P * n2 + q, *b2 = ph + (size_t)q2 * P * n2 + q;
    float p[P];
#pragma unroll
    for (int z = 0; z < P; z++) {
        size_t zz = (size_t)z * n2;
        p[z] = a1[zz] * b1[zz] - a2[zz] * b2[zz];
    }
    float cr[N], ci[N];
    to_four_f<P>(p, cr, ci);
    auto fld = [&](int f) -> const cplx* {
        return (f == 0) ? A.ux : (f == 1) ? A.uy : (f == 2) ? A.uz : (f == 3) ? A.wx : (f == 4) ? A.wy : A.wz;
    };
    const cplx *P1 = fld(p1) + q, *Q1 = fld(q1) + q, *P2 = fld(p2) + q, *Q2 = fld(q2) + q;
    const double m1 = P1[0].x, n1 = Q1[0].x, m2 = P2[0].x, n2v = Q2[0].x;
    cplx* out = ((o == 0) ? A.a : (o == 1) ? A.b : A.c) + q;
    out[0] = make_double2(zap(m1 * n1 - m2 * n2v + (double)cr[0]), 0.0);
#pragma unroll
    for (int k = 1; k < N; k++) {
        if (k >= A.K) continue;
        size_t kk = (size_t)k * n2;
        cplx aq1 = Q1[kk], ap1 = P1[kk], aq2 = Q2[kk], ap2 = P2[kk];
        double vr = m1 * aq1.x + n1 * ap1.x - m2 * aq2.x - n2v * ap2.x + (double)cr[k];
        double vi = m1 * aq1.y + n1 * ap1.y - m2 * aq2.y - n2v * ap2.y + (double)ci[k];
        out[kk] = make_double2(zap(vr), zap(vi));
    }
}

// ---------------------------------------------------------------------------
// The same two passes on the tensor cores: the spanwise transforms of the
// disturbance as dense DFT-matrix GEMMs (tcgen05.mma, kind::f16), every FP32
// operand split into three BF16 parts (x = x0 + x1 + x2 exactly, 8 bits each)
// and the products compensated to FP32 accuracy,
//   a b ~ a0 b0 + (a0 b1 + a1 b0) + (a0 b2 + a1 b1 + a2 b0),
// accumulated in FP32 in tensor memory.  A tile is 128 points (one per
// thread and tensor-memory lane); per point the P "slots" hold Re c0 (0: the
// mean stays in FP64), Im c0 (the packed Nyquist term) and Re, Im of modes
// 1 .. P/2-1.  Pass 1: phys[pt][z] = sum_s slot[pt][s] Tinv[z][s]; pass 2:
// slot[pt][s] = sum_z prod[pt][z] Tfwd[s][z], the transforms to_phys_dist and
// to_four_f above written as matrices (tb_dft_matrices).
//
// Shared memory, K-major without swizzle: element (row r, k) of an operand
// with R rows sits at (k / 8) * (R * 16) + r * 16 + (k % 8) * 2 bytes, so a
// core matrix (8 rows x 8 k) is 128 contiguous bytes, core matrices
// adjacent in rows are 128 bytes apart and those adjacent in k R * 16 apart.
constexpr int TC_PARTS = 3;   // BF16 parts per FP32 operand

template <int P>
struct TcLayout {
    static constexpr int AB = 128 * P * 2, BB = P * P * 2;                 // bytes of one operand part
    static constexpr int A0 = 0, B0 = TC_PARTS * AB;                       // part p at A0 + p AB, B0 + p BB
    static constexpr int BAR = B0 + TC_PARTS * BB;                         // mbarrier, then the TMEM address
    static constexpr int BYTES = BAR + 16;
    static constexpr uint32_t NCOL = P < 32 ? 32 : P;                      // tensor-memory columns
    static constexpr uint32_t ID = tbtc::idesc_bf16_f32(128, P);
    // resident blocks per SM: shared memory (227 KB), tensor memory (512 columns), at most 8
    static constexpr int PER_SM_SMEM = (227 * 1024) / BYTES, PER_SM_TMEM = 512 / (int)NCOL;
    static constexpr int PER_SM0 = PER_SM_SMEM < PER_SM_TMEM ? PER_SM_SMEM : PER_SM_TMEM;
    static constexpr int PER_SM = PER_SM0 < 8 ? PER_SM0 : 8;
};

// x = x0 + x1 + x2 with BF16 parts (round to nearest at each step).
__device__ __forceinline__ void split_bf16(float x, unsigned short* p) {
#pragma unroll
    for (int q = 0; q < TC_PARTS; q++) {
        const __nv_bfloat16 b = __float2bfloat16_rn(x);
        p[q] = __bfloat16_as_ushort(b);
        x -= __bfloat162float(b);
    }
}

// Row `row` of the A operand (P values) into its BF16 parts.
template <int P>
__device__ __forceinline__ void stage_row(unsigned char* sm, int row, const float* v) {
    using Lt = TcLayout<P>;
#pragma unroll
    for (int g = 0; g < P / 8; g++) {
        unsigned short h[TC_PARTS][8];
#pragma unroll
        for (int e = 0; e < 8; e++) {
            unsigned short p[TC_PARTS];
            split_bf16(v[8 * g + e], p);
#pragma unroll
            for (int q = 0; q < TC_PARTS; q++) h[q][e] = p[q];
        }
#pragma unroll
        for (int q = 0; q < TC_PARTS; q++) {
            uint4 H;
            H.x = h[q][0] | ((uint32_t)h[q][1] << 16); H.y = h[q][2] | ((uint32_t)h[q][3] << 16);
            H.z = h[q][4] | ((uint32_t)h[q][5] << 16); H.w = h[q][6] | ((uint32_t)h[q][7] << 16);
            *reinterpret_cast<uint4*>(sm + Lt::A0 + q * Lt::AB + g * 2048 + row * 16) = H;
        }
    }
}

// One thread issues the tile's MMAs (the six part products of order <= 2
// per 16-wide k-step) and commits them.
template <int P>
__device__ __forceinline__ void tile_mma(unsigned char* sm, uint32_t tmem, uint64_t* bar) {
    using Lt = TcLayout<P>;
    const uint32_t base = tbtc::smem_u32(sm);
#pragma unroll
    for (int ks = 0; ks < P / 16; ks++) {
        const uint32_t ao = ks * 2 * 2048, bo = ks * 2 * P * 16;
        uint64_t a[TC_PARTS], b[TC_PARTS];
#pragma unroll
        for (int q = 0; q < TC_PARTS; q++) {
            a[q] = tbtc::sdesc(base + Lt::A0 + q * Lt::AB + ao, 2048, 128);
            b[q] = tbtc::sdesc(base + Lt::B0 + q * Lt::BB + bo, P * 16, 128);
        }
        tbtc::mma_bf16(tmem, a[0], b[0], Lt::ID, ks > 0);
        tbtc::mma_bf16(tmem, a[0], b[1], Lt::ID, 1);
        tbtc::mma_bf16(tmem, a[1], b[0], Lt::ID, 1);
        tbtc::mma_bf16(tmem, a[0], b[2], Lt::ID, 1);
        tbtc::mma_bf16(tmem, a[1], b[1], Lt::ID, 1);
        tbtc::mma_bf16(tmem, a[2], b[0], Lt::ID, 1);
    }
    tbtc::mma_commit(bar);
}

// Set-up shared by both passes: the constant B operand (its BF16 parts) into
// shared memory, the mbarrier, and the tensor-memory columns.
template <int P>
__device__ __forceinline__ uint32_t tc_setup(unsigned char* sm, const uint16_t* mats) {
    using Lt = TcLayout<P>;
    const int t = threadIdx.x;
    for (int i = t; i < TC_PARTS * P * P / 8; i += blockDim.x)
        reinterpret_cast<uint4*>(sm + Lt::B0)[i] = reinterpret_cast<const uint4*>(mats)[i];
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + Lt::BAR);
    uint32_t* slot = reinterpret_cast<uint32_t*>(sm + Lt::BAR + 8);
    if (t == 0) tbtc::mbar_init(bar, 1);
    if ((t >> 5) == 0) {
        tbtc::tmem_alloc(slot, Lt::NCOL);
        tbtc::tmem_relinquish();
    }
    tbtc::fence_before_sync();
    __syncthreads();
    tbtc::fence_after_sync();
    return *slot;
}

// Issue, wait (bounded) and read: returns false (for the whole block) when
// the wait ran out, after which the caller stops issuing.
// TcCtl: the wait limit in polls and, for tests of the time-out path only,
// a switch that leaves the MMAs unissued so that the wait runs out.
struct TcCtl {
    uint32_t limit;
    int skip_mma;
};

template <int P>
__device__ __forceinline__ bool tc_run(unsigned char* sm, uint32_t tmem, uint32_t& phase, const TcCtl& ctl) {
    using Lt = TcLayout<P>;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + Lt::BAR);
    tbtc::fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0 && !ctl.skip_mma) {
        tbtc::fence_after_sync();
        tile_mma<P>(sm, tmem, bar);
    }
    const bool ok = tbtc::mbar_wait(bar, phase, ctl.limit);
    tbtc::fence_after_sync();
    const bool all = !__syncthreads_or(!ok);
    if (all) phase ^= 1u;   // on a time-out `phase` stays that of the tile in flight
    return all;
}

template <int P>
__device__ __forceinline__ void tc_teardown(unsigned char* sm, uint32_t tmem, bool ok, uint32_t phase, int* err,
                                            const TcCtl& ctl) {
    using Lt = TcLayout<P>;
    if (!ok) {   // let the MMAs of the abandoned tile finish (bounded) before freeing their columns
        (void)tbtc::mbar_wait(reinterpret_cast<uint64_t*>(sm + Lt::BAR), phase, ctl.limit);
        if (threadIdx.x == 0) atomicExch(err, 1);
    }
    tbtc::fence_before_sync();
    __syncthreads();
    tbtc::fence_after_sync();
    if ((threadIdx.x >> 5) == 0) tbtc::tmem_dealloc(tmem, Lt::NCOL);
}

__device__ __forceinline__ const cplx* nl_field(const NlArgs& A, int f) {
    return (f == 0) ? A.ux : (f == 1) ? A.uy : (f == 2) ? A.uz : (f == 3) ? A.wx : (f == 4) ? A.wy : A.wz;
}

// Pass 1 on the tensor cores: tile = (field f, 128 points) -> ph[(f P + z) n2 + q].
template <int P>
__global__ void __launch_bounds__(128) k_nl_phys_tc(NlArgs A, float* __restrict__ ph, const uint16_t* __restrict__ mats,
                                                    int* err, TcCtl ctl) {
    constexpr int N = P / 2;
    extern __shared__ __align__(1024) unsigned char sm[];
    const uint32_t tmem = tc_setup<P>(sm, mats);
    const int t = threadIdx.x, warp = t >> 5;
    const size_t n2 = A.n2;
    const int tpf = (int)((n2 + 127) / 128), ntiles = 6 * tpf;
    uint32_t phase = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int f = tile / tpf;
        const size_t q = (size_t)(tile % tpf) * 128 + t;
        const cplx* F = nl_field(A, f);
        float v[P];
        v[0] = 0.f;
        v[1] = q < n2 ? (float)F[q].y : 0.f;
#pragma unroll
        for (int k = 1; k < N; k++) {
            cplx c = make_double2(0.0, 0.0);
            if (k < A.K && q < n2) c = F[(size_t)k * n2 + q];
            v[2 * k] = (float)c.x;
            v[2 * k + 1] = (float)c.y;
        }
        stage_row<P>(sm, t, v);
        if (!(ok = tc_run<P>(sm, tmem, phase, ctl))) break;
#pragma unroll
        for (int c0 = 0; c0 < P; c0 += 16) {
            float w[16];
            tbtc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + c0, w);
            if (q < n2) {
#pragma unroll
                for (int i = 0; i < 16; i++) ph[((size_t)f * P + c0 + i) * n2 + q] = w[i];
            }
        }
        tbtc::fence_before_sync();
        __syncthreads();
    }
    tc_teardown<P>(sm, tmem, ok, phase, err, ctl);
}

// Pass 2 on the tensor cores: tile = (output o, 128 points); the quadratic
// disturbance term's slots plus the FP64 mean terms, as k_nl_four.
template <int P>
__global__ void __launch_bounds__(128) k_nl_four_tc(NlArgs A, const float* __restrict__ ph,
                                                    const uint16_t* __restrict__ mats, int* err, TcCtl ctl) {
    constexpr int N = P / 2;
    extern __shared__ __align__(1024) unsigned char sm[];
    const uint32_t tmem = tc_setup<P>(sm, mats);
    const int t = threadIdx.x, warp = t >> 5;
    const size_t n2 = A.n2;
    const int tpf = (int)((n2 + 127) / 128), ntiles = 3 * tpf;
    uint32_t phase = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int o = tile / tpf;
        const size_t q = (size_t)(tile % tpf) * 128 + t;
        const int p1 = (o == 0) ? 1 : (o == 1) ? 0 : 2, q1 = (o == 0) ? 3 : (o == 1) ? 5 : 4;
        const int p2 = (o == 0) ? 0 : (o == 1) ? 2 : 1, q2 = (o == 0) ? 4 : (o == 1) ? 3 : 5;
        float v[P];
#pragma unroll
        for (int z = 0; z < P; z++) v[z] = 0.f;
        if (q < n2) {
            const float *a1 = ph + (size_t)p1 * P * n2 + q, *b1 = ph + (size_t)q1 * P * n2 + q;
            const float *a2 = ph + (size_t)p2 * P * n2 + q, *b2 = ph + (size_t)q2 * P * n2 + q;
#pragma unroll
            for (int z = 0; z < P; z++) {
                const size_t zz = (size_t)z * n2;
                v[z] = a1[zz] * b1[zz] - a2[zz] * b2[zz];
            }
        }
        stage_row<P>(sm, t, v);
        if (!(ok = tc_run<P>(sm, tmem, phase, ctl))) break;
#pragma unroll
        for (int c0 = 0; c0 < P; c0 += 16) tbtc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + c0, v + c0);
        if (q < n2) {
            const cplx *P1 = nl_field(A, p1) + q, *Q1 = nl_field(A, q1) + q, *P2 = nl_field(A, p2) + q, *Q2 = nl_field(A, q2) + q;
            const double m1 = P1[0].x, n1 = Q1[0].x, m2 = P2[0].x, n2v = Q2[0].x;
            cplx* out = ((o == 0) ? A.a : (o == 1) ? A.b : A.c) + q;
            out[0] = make_double2(zap(m1 * n1 - m2 * n2v + (double)v[0]), 0.0);
#pragma unroll
            for (int k = 1; k < N; k++) {
                if (k >= A.K) continue;
                const size_t kk = (size_t)k * n2;
                const cplx aq1 = Q1[kk], ap1 = P1[kk], aq2 = Q2[kk], ap2 = P2[kk];
                const double vr = m1 * aq1.x + n1 * ap1.x - m2 * aq2.x - n2v * ap2.x + (double)v[2 * k];
                const double vi = m1 * aq1.y + n1 * ap1.y - m2 * aq2.y - n2v * ap2.y + (double)v[2 * k + 1];
                out[kk] = make_double2(zap(vr), zap(vi));
            }
        }
        tbtc::fence_before_sync();
        __syncthreads();
    }
    tc_teardown<P>(sm, tmem, ok, phase, err, ctl);
}

// Smagorinsky eddy viscosity and force nu_t lap(u) (les_par.f:6-211).
struct LesArgs {
    const cplx *dudx, *dvdx, *dwdx, *dudy, *dvdy, *dwdy;   // Fourier gradients
    const cplx *ux, *uy, *uz;                              // z-derivatives formed as -i k beta u
    const cplx *d2x[3], *d2y[3];                           // second derivatives of ux, uy, uz
    const double* k2b2;
    const cplx* wz;                                        // wall vorticity for y+
    cplx *fx, *fy, *fz;
    int nx, ny, n2, K, damping;
    double beta, Re, fac_y, dy, stf, Cs, Aplus, delta_les;
};
template <int P>
__device__ __forceinline__ void to_phys_dz(const cplx* __restrict__ u, size_t cs, int K, double beta, double* p) {
    // z-derivative in Fourier space: v_kb(k) u = -i (k-1) beta u  (main_par.f:1888)
    constexpr int N = P / 2;
    cplx tmp[N];
#pragma unroll
    for (int k = 0; k < N; k++) {
        if (k < K) {
            cplx v = u[(size_t)k * cs];
            double kb = -(double)k * beta;
            tmp[k] = make_double2(-kb * v.y, kb * v.x);
        } else {
            tmp[k] = make_double2(0.0, 0.0);
        }
    }
    to_phys<P>(tmp, 1, K < N ? K : N, p);
}
template <int P>
__global__ void __launch_bounds__(128) k_les(LesArgs A) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= A.n2) return;
    size_t cs = A.n2;
    int i = q % A.nx, j = q / A.nx;
    double y = (A.stf == 1.0) ? (double)j * A.dy : A.dy * (pow(A.stf, (double)j) - 1.0) / (A.stf - 1.0);
    double wz0 = (A.damping & 2) ? fabs(A.wz[i].x) : A.wz[i].x;
    double yplus = sqrt(A.Re * wz0 / sqrt(A.fac_y)) * y;
    double damp;
    if (A.damping & 1) {
        double e = 1.0 - exp(-yplus / A.Aplus);
        damp = e * e;
    } else {
        double ratio = fmin(yplus / A.Aplus, 100.0);
        ratio = ratio * ratio * ratio;
        damp = 1.0 - exp(-ratio);
    }
    double cte = A.Cs * A.Cs * A.delta_les * A.delta_les * damp;
    double dg[P], of[P], t1[P], t2[P];
    to_phys<P>(A.dudx + q, cs, A.K, t1);
#pragma unroll
    for (int z = 0; z < P; z++) dg[z] = t1[z] * t1[z];
    to_phys<P>(A.dvdy + q, cs, A.K, t1);
#pragma unroll
    for (int z = 0; z < P; z++) dg[z] += t1[z] * t1[z];
    to_phys_dz<P>(A.uz + q, cs, A.K, A.beta, t1);
#pragma unroll
    for (int z = 0; z < P; z++) dg[z] += t1[z] * t1[z];
    to_phys<P>(A.dudy + q, cs, A.K, t1);
    to_phys<P>(A.dvdx + q, cs, A.K, t2);
#pragma unroll
    for (int z = 0; z < P; z++) { double s = 0.5 * (t1[z] + t2[z]); of[z] = s * s; }
    to_phys_dz<P>(A.ux + q, cs, A.K, A.beta, t1);
    to_phys<P>(A.dwdx + q, cs, A.K, t2);
#pragma unroll
    for (int z = 0; z < P; z++) { double s = 0.5 * (t1[z] + t2[z]); of[z] += s * s; }
    to_phys_dz<P>(A.uy + q, cs, A.K, A.beta, t1);
    to_phys<P>(A.dwdy + q, cs, A.K, t2);
#pragma unroll
    for (int z = 0; z < P; z++) {
        double s = 0.5 * (t1[z] + t2[z]);
        of[z] += s * s;
        dg[z] = cte * sqrt(2.0 * (dg[z] + 2.0 * of[z]));  // nu_t
    }
    const cplx* us[3] = {A.ux, A.uy, A.uz};
    cplx* outs[3] = {A.fx, A.fy, A.fz};
    constexpr int N = P / 2;
    for (int f = 0; f < 3; f++) {
        cplx lap[N];
#pragma unroll
        for (int k = 0; k < N; k++) {
            if (k < A.K) {
                size_t o = (size_t)q + cs * k;
                cplx a = A.d2x[f][o], b = A.d2y[f][o], u = us[f][o];
                double kk = A.k2b2[k];
                lap[k] = make_double2(a.x + b.x + kk * u.x, a.y + b.y + kk * u.y);
            } else {
                lap[k] = make_double2(0.0, 0.0);
            }
        }
        to_phys<P>(lap, 1, A.K < N ? A.K : N, t1);
#pragma unroll
        for (int z = 0; z < P; z++) t1[z] = dg[z] * t1[z];
        to_four<P>(t1, A.K, outs[f] + q, cs);
    }
}

// Immersed-boundary feedback force (cvirt immersed_par.f:262-313):
// f = irf delta u in physical space, back to Fourier, Gibbs-filtered.
struct IbmArgs {
    const cplx *ux, *uy, *uz;
    const double* delta;
    const double* gibbs;
    cplx *fx, *fy, *fz;
    int n2, K, accumulate;
    double irf;
};
template <int P>
__global__ void __launch_bounds__(128) k_cvirt(IbmArgs A) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= A.n2) return;
    size_t cs = A.n2;
    const cplx* us[3] = {A.ux, A.uy, A.uz};
    cplx* outs[3] = {A.fx, A.fy, A.fz};
    double p[P];
    constexpr int N = P / 2;
    for (int f = 0; f < 3; f++) {
        to_phys<P>(us[f] + q, cs, A.K, p);
#pragma unroll
        for (int z = 0; z < P; z++) p[z] = A.irf * A.delta[(size_t)q + cs * z] * p[z];
        cplx tmp[N];
        to_four<P>(p, A.K, tmp, 1);
        for (int k = 0; k < A.K && k < N; k++) {
            size_t o = (size_t)q + cs * k;
            cplx v = make_double2(A.gibbs[k] * tmp[k].x, A.gibbs[k] * tmp[k].y);
            if (A.accumulate) { cplx w = outs[f][o]; v.x += w.x; v.y += w.y; }
            outs[f][o] = v;
        }
    }
}

// delta() (immersed_par.f:98-181): smoothed roughness indicator, filtered
// through p_to_f -> gibbs -> f_to_p.
template <int P>
__global__ void k_delta_filter(double* delta, const double* gibbs, int n2, int K) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n2) return;
    constexpr int N = P / 2;
    double p[P];
    cplx tmp[N];
#pragma unroll
    for (int z = 0; z < P; z++) p[z] = delta[(size_t)q + (size_t)n2 * z];
    to_four<P>(p, K, tmp, 1);
    for (int k = 0; k < N; k++) {
        if (k < K) tmp[k] = make_double2(gibbs[k] * tmp[k].x, gibbs[k] * tmp[k].y);
        else tmp[k] = make_double2(0.0, 0.0);
    }
    to_phys<P>(tmp, 1, K < N ? K : N, p);
#pragma unroll
    for (int z = 0; z < P; z++) delta[(size_t)q + (size_t)n2 * z] = p[z];
}

bool g_tw_ready[64] = {false};

int ensure_twiddles(tb_ctx* c) {
    int dev = c->device;
    if (dev >= 0 && dev < 64 && g_tw_ready[dev]) return TB_OK;
    double hr[TW_N], hi[TW_N];
    for (int t = 0; t < TW_N; t++) {
        long double ang = -2.0L * 3.141592653589793238462643383279502884L * (long double)t / (long double)TW_N;
        hr[t] = (double)cosl(ang);
        hi[t] = (double)sinl(ang);
    }
    TB_CUDA(cudaMemcpyToSymbol(c_twr, hr, sizeof hr));
    TB_CUDA(cudaMemcpyToSymbol(c_twi, hi, sizeof hi));
    float fr[TW_N], fi[TW_N];
    for (int t = 0; t < TW_N; t++) { fr[t] = (float)hr[t]; fi[t] = (float)hi[t]; }
    TB_CUDA(cudaMemcpyToSymbol(c_twrf, fr, sizeof fr));
    TB_CUDA(cudaMemcpyToSymbol(c_twif, fi, sizeof fi));
    if (dev >= 0 && dev < 64) g_tw_ready[dev] = true;
    return TB_OK;
}

#define TB_DISPATCH_P(P, STMT)                                           \
    switch (P) {                                                         \
        case 2: { constexpr int PP = 2; STMT; } break;                   \
        case 4: { constexpr int PP = 4; STMT; } break;                   \
        case 8: { constexpr int PP = 8; STMT; } break;                   \
        case 16: { constexpr int PP = 16; STMT; } break;                 \
        case 32: { constexpr int PP = 32; STMT; } break;                 \
        case 64: { constexpr int PP = 64; STMT; } break;                 \
        case 128: { constexpr int PP = 128; STMT; } break;               \
        default: tb_set_error("kphys %d not supported", P); return TB_ERR_ARG; \
    }

}  // namespace

int tb_launch_f_to_p(tb_ctx* c, double* phys, const cplx* four) {
    int r = ensure_twiddles(c);
    if (r) return r;
    int n2 = (int)tb_n2(c);
    unsigned nb = tb_blocks(n2, 128);
    TB_DISPATCH_P(c->g.P, (k_f_to_p<PP><<<nb, 128, 0, c->stream>>>(phys, four, n2, c->g.K)));
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}
int tb_launch_p_to_f(tb_ctx* c, cplx* four, const double* phys) {
    int r = ensure_twiddles(c);
    if (r) return r;
    int n2 = (int)tb_n2(c);
    unsigned nb = tb_blocks(n2, 128);
    TB_DISPATCH_P(c->g.P, (k_p_to_f<PP><<<nb, 128, 0, c->stream>>>(four, phys, n2, c->g.K)));
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}
// ---- the DFT matrices of the tensor-core passes ------------------------------
static uint16_t bf16_bits(float f) {   // round to nearest even
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}
static float bf16_value(uint16_t h) {
    uint32_t u = (uint32_t)h << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// to_phys_dist and to_four_f in double precision on slot vectors, with the
// length-N complex transforms of cfft written as plain sums.
static const double TB_PI = 3.14159265358979323846;
static void host_cdft(int N, int sign, std::vector<double>& re, std::vector<double>& im) {
    std::vector<double> r(N, 0.0), i(N, 0.0);
    for (int m = 0; m < N; m++)
        for (int k = 0; k < N; k++) {
            const double a = sign * 2.0 * TB_PI * (double)((long)k * m % N) / N;
            r[m] += re[k] * std::cos(a) - im[k] * std::sin(a);
            i[m] += re[k] * std::sin(a) + im[k] * std::cos(a);
        }
    re = r;
    im = i;
}
static void host_phys_from_slots(int P, const double* s, double* p) {
    const int N = P / 2;
    std::vector<double> re(N), im(N);
    re[0] = 0.5 * s[1];
    im[0] = -0.5 * s[1];
    for (int k = 1; k < N; k++) {
        const double Ar = s[2 * k], Ai = s[2 * k + 1], Br = s[2 * (N - k)], Bi = -s[2 * (N - k) + 1];
        const double sr = 0.5 * (Ar + Br), si = 0.5 * (Ai + Bi), dr = 0.5 * (Ar - Br), di = 0.5 * (Ai - Bi);
        const double wr = std::cos(2.0 * TB_PI * k / P), wi = -std::sin(2.0 * TB_PI * k / P);
        re[k] = sr - (wr * di + wi * dr);
        im[k] = si + (wr * dr - wi * di);
    }
    host_cdft(N, -1, re, im);
    for (int m = 0; m < N; m++) { p[2 * m] = re[m]; p[2 * m + 1] = im[m]; }
}
static void host_slots_from_phys(int P, const double* p, double* s) {
    const int N = P / 2;
    std::vector<double> re(N), im(N);
    for (int m = 0; m < N; m++) { re[m] = p[2 * m]; im[m] = p[2 * m + 1]; }
    host_cdft(N, +1, re, im);
    s[0] = (re[0] + im[0]) / P;
    s[1] = 0.0;
    for (int k = 1; k < N; k++) {
        const double Fr = re[k], Fi = im[k], Gr = re[N - k], Gi = -im[N - k];
        const double Er = 0.5 * (Fr + Gr), Ei = 0.5 * (Fi + Gi), gr = Fr - Gr, gi = Fi - Gi;
        const double Or = 0.5 * gi, Oi = -0.5 * gr;
        const double vr = std::cos(2.0 * TB_PI * k / P), vi = std::sin(2.0 * TB_PI * k / P);
        s[2 * k] = 2.0 / P * (Er + (vr * Or - vi * Oi));
        s[2 * k + 1] = 2.0 / P * (Ei + (vr * Oi + vi * Or));
    }
}

// B operands of both passes, their TC_PARTS BF16 parts, in the K-major core
// layout of TcLayout: inverse (n = z, k = slot) then forward (n = slot, k = z).
void tb_dft_matrices(int P, std::vector<uint16_t>& out) {
    std::vector<double> Tinv((size_t)P * P), Tfwd((size_t)P * P), e(P), v(P);
    for (int s = 0; s < P; s++) {
        std::fill(e.begin(), e.end(), 0.0);
        e[s] = 1.0;
        host_phys_from_slots(P, e.data(), v.data());
        for (int z = 0; z < P; z++) Tinv[(size_t)z * P + s] = v[z];
        host_slots_from_phys(P, e.data(), v.data());   // e as a physical unit vector at z = s
        for (int q = 0; q < P; q++) Tfwd[(size_t)q * P + s] = v[q];
    }
    out.assign((size_t)2 * TC_PARTS * P * P, 0);
    auto put = [&](int first, const std::vector<double>& T) {   // T[n][k]
        for (int n = 0; n < P; n++)
            for (int k = 0; k < P; k++) {
                float x = (float)T[(size_t)n * P + k];
                const size_t o = (size_t)(k / 8) * (P * 8) + (size_t)n * 8 + (k % 8);
                for (int q = 0; q < TC_PARTS; q++) {
                    const uint16_t h = bf16_bits(x);
                    out[(size_t)(first + q) * P * P + o] = h;
                    x -= bf16_value(h);
                }
            }
    };
    put(0, Tinv);
    put(TC_PARTS, Tfwd);
}

// The two matrices in double precision, P x P row-major [n][k]: forward 0
// gives Tinv[z][slot], forward 1 gives Tfwd[slot][z].
extern "C" int tb_dft_matrix(int P, int forward, double* out) {
    if (!out || P < 4 || (P & (P - 1))) { tb_set_error("P must be a power of two >= 4"); return TB_ERR_ARG; }
    std::vector<double> e(P), v(P);
    for (int s = 0; s < P; s++) {
        std::fill(e.begin(), e.end(), 0.0);
        e[s] = 1.0;
        if (forward) {
            host_slots_from_phys(P, e.data(), v.data());
            for (int q = 0; q < P; q++) out[(size_t)q * P + s] = v[q];
        } else {
            host_phys_from_slots(P, e.data(), v.data());
            for (int z = 0; z < P; z++) out[(size_t)z * P + s] = v[z];
        }
    }
    return TB_OK;
}

static bool tc_form(const tb_ctx* c) {
    const int P = c->g.P;
    return c->cfg.precision == TB_FORM_MIXED && c->nl_tensor && (P == 16 || P == 32 || P == 64 || P == 128);
}

static bool g_tc_attr[64][4] = {{false}};

template <int P>
static int tc_attrs(int dev) {
    const int slot = P == 16 ? 0 : P == 32 ? 1 : P == 64 ? 2 : 3;
    if (dev >= 0 && dev < 64 && g_tc_attr[dev][slot]) return TB_OK;
    TB_CUDA(cudaFuncSetAttribute(k_nl_phys_tc<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcLayout<P>::BYTES));
    TB_CUDA(cudaFuncSetAttribute(k_nl_four_tc<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcLayout<P>::BYTES));
    if (dev >= 0 && dev < 64) g_tc_attr[dev][slot] = true;
    return TB_OK;
}

static int ensure_tc(tb_ctx* c) {
    if (!tc_form(c)) return TB_OK;
    int r;
    switch (c->g.P) {
        case 16: r = tc_attrs<16>(c->device); break;
        case 32: r = tc_attrs<32>(c->device); break;
        case 64: r = tc_attrs<64>(c->device); break;
        default: r = tc_attrs<128>(c->device); break;
    }
    if (r) return r;
    if (!c->dft_tc) {
        std::vector<uint16_t> m;
        tb_dft_matrices(c->g.P, m);
        TB_CUDA(cudaMalloc(&c->dft_tc, m.size() * sizeof(uint16_t)));
        TB_CUDA(cudaMemcpy(c->dft_tc, m.data(), m.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
    }
    if (!c->tc_err) {
        TB_CUDA(cudaMalloc(&c->tc_err, sizeof(int)));
        TB_CUDA(cudaMemset(c->tc_err, 0, sizeof(int)));
    }
    return TB_OK;
}

int tb_spectral_prepare(tb_ctx* c) {
    int r = ensure_twiddles(c);
    if (r) return r;
    if (c->cfg.precision == TB_FORM_MIXED && c->g.P >= 4 && !c->nl_phys)
        TB_CUDA(cudaMalloc(&c->nl_phys, (size_t)6 * c->g.P * tb_n2(c) * sizeof(float)));
    return ensure_tc(c);
}

int tb_tc_check(tb_ctx* c) {
    if (!c->tc_err) return TB_OK;
    int e = 0;
    TB_CUDA(cudaMemcpy(&e, c->tc_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        TB_CUDA(cudaMemset(c->tc_err, 0, sizeof(int)));
        tb_set_error("nlterms (tensor cores): a bounded wait for the MMAs ran out");
        return TB_ERR_TIMEOUT;
    }
    return TB_OK;
}

int tb_launch_nlterms(tb_ctx* c, cplx* a, cplx* b, cplx* cc) {
    int r = ensure_twiddles(c);
    if (r) return r;
    NlArgs A{c->ux, c->uy, c->uz, c->wx, c->wy, c->wz, a, b, cc, (int)tb_n2(c), c->g.K};
    cudaEvent_t ps = nullptr;
    if ((r = tb_prof_begin(c, PROF_NLTERMS, &ps))) return r;
    if (tc_form(c)) {
        if (!c->capturing && (r = tb_spectral_prepare(c))) return r;
        const int P = c->g.P, sms = c->sm_count > 0 ? c->sm_count : 148;
        const size_t tiles = (A.n2 + 127) / 128;
        // a time-out test shortens the wait to a few thousand polls and leaves the MMAs unissued
        const TcCtl ctl{c->tc_timeout_test ? 4096u : (1u << 22), c->tc_timeout_test};
        switch (P) {
#define TB_TC_CASE(PP)                                                                                        \
    case PP: {                                                                                                 \
        const int per = (c->tune_nl >= 1 && c->tune_nl <= TcLayout<PP>::PER_SM) ? c->tune_nl : TcLayout<PP>::PER_SM; \
        const size_t cap = (size_t)per * sms;                                                                  \
        const unsigned g1 = (unsigned)std::min<size_t>(6 * tiles, cap), g2 = (unsigned)std::min<size_t>(3 * tiles, cap); \
        k_nl_phys_tc<PP><<<g1, 128, TcLayout<PP>::BYTES, c->stream>>>(A, c->nl_phys, c->dft_tc, c->tc_err, ctl);   \
        TB_CHECK_LAUNCH(c);                                                                                    \
        k_nl_four_tc<PP><<<g2, 128, TcLayout<PP>::BYTES, c->stream>>>(A, c->nl_phys, c->dft_tc + TC_PARTS * PP * PP, \
                                                                      c->tc_err, ctl);                         \
        break;                                                                                                 \
    }
            TB_TC_CASE(16)
            TB_TC_CASE(32)
            TB_TC_CASE(64)
            TB_TC_CASE(128)
#undef TB_TC_CASE
        }
    } else if (c->cfg.precision == TB_FORM_MIXED && c->g.P >= 4) {
        size_t need = (size_t)6 * c->g.P * A.n2;
        if (!c->nl_phys) TB_CUDA(cudaMalloc(&c->nl_phys, need * sizeof(float)));
        TB_DISPATCH_P(c->g.P, (k_nl_phys<PP><<<tb_blocks(6 * (size_t)A.n2, 128), 128, 0, c->stream>>>(A, c->nl_phys)));
        TB_CHECK_LAUNCH(c);
        TB_DISPATCH_P(c->g.P, (k_nl_four<PP><<<tb_blocks(3 * (size_t)A.n2, 128), 128, 0, c->stream>>>(A, c->nl_phys)));
    } else {
        unsigned nb = tb_blocks(A.n2, 128);
        TB_DISPATCH_P(c->g.P, (k_nlterms<PP><<<nb, 128, 0, c->stream>>>(A)));
    }
    TB_CHECK_LAUNCH(c);
    return tb_prof_end(c, PROF_NLTERMS, ps);
}

int tb_launch_les(tb_ctx* c, cplx* fx, cplx* fy, cplx* fz) {
    int r = ensure_twiddles(c);
    if (r) return r;
    // Fourier-space derivatives: x (dudx, dvdx, dwdx, d2x u,v,w) and y (dudy, dvdy(fv), dwdy, d2y u,v,w)
    cplx** t = c->tmp;
    XJob xj[6] = {{c->ux, t[0], XOP_D1}, {c->uy, t[1], XOP_D1}, {c->uz, t[2], XOP_D1},
                  {c->ux, t[6], XOP_D2}, {c->uy, t[7], XOP_D2}, {c->uz, t[8], XOP_D2}};
    YJob yj[6] = {{c->ux, t[3], YOP_D1}, {c->uy, t[4], YOP_D1FV}, {c->uz, t[5], YOP_D1},
                  {c->ux, t[9], YOP_D2}, {c->uy, t[10], YOP_D2}, {c->uz, t[11], YOP_D2}};
    if ((r = tb_launch_xlines(c, xj, 6))) return r;
    if ((r = tb_launch_ylines(c, yj, 6))) return r;
    LesArgs A;
    A.dudx = t[0]; A.dvdx = t[1]; A.dwdx = t[2]; A.dudy = t[3]; A.dvdy = t[4]; A.dwdy = t[5];
    A.ux = c->ux; A.uy = c->uy; A.uz = c->uz;
    A.d2x[0] = t[6]; A.d2x[1] = t[7]; A.d2x[2] = t[8];
    A.d2y[0] = t[9]; A.d2y[1] = t[10]; A.d2y[2] = t[11];
    A.k2b2 = c->k2b2; A.wz = c->wz; A.fx = fx; A.fy = fy; A.fz = fz;
    A.nx = c->g.nx; A.ny = c->g.ny; A.n2 = (int)tb_n2(c); A.K = c->g.K; A.damping = c->cfg.les_damping;
    A.beta = c->cfg.beta; A.Re = c->cfg.Re; A.fac_y = c->cfg.fac_y; A.dy = c->cfg.dy; A.stf = c->cfg.stf;
    A.Cs = c->cfg.C_s; A.Aplus = c->cfg.A_plus;
    A.delta_les = std::pow(c->cfg.dx * c->cfg.dy * c->dz, 1.0 / 3.0);
    unsigned nb = tb_blocks(A.n2, 128);
    TB_DISPATCH_P(c->g.P, (k_les<PP><<<nb, 128, 0, c->stream>>>(A)));
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}

int tb_launch_cvirt(tb_ctx* c, cplx* fx, cplx* fy, cplx* fz, bool accumulate) {
    int r = ensure_twiddles(c);
    if (r) return r;
    IbmArgs A{c->ux, c->uy, c->uz, c->delta_no, c->gibbs, fx, fy, fz, (int)tb_n2(c), c->g.K, accumulate ? 1 : 0,
              c->cfg.irf};
    unsigned nb = tb_blocks(A.n2, 128);
    TB_DISPATCH_P(c->g.P, (k_cvirt<PP><<<nb, 128, 0, c->stream>>>(A)));
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}

// Host construction of the roughness indicator (immersed_par.f:122-151),
// then the device-side Gibbs filtering of delta().
int tb_delta_setup(tb_ctx* c) {
    int r = ensure_twiddles(c);
    if (r) return r;
    int nx = c->g.nx, ny = c->g.ny, P = c->g.P;
    size_t n2 = tb_n2(c);
    std::vector<double> d(n2 * P, 0.0);
    const tb_config& cf = c->cfg;
    if (cf.ibm) {
        double sigx = 1.0, sigy = 1.0, dz = c->dz;
        for (int k = 1; k <= P; k++) {
            double z = (double)(k - 1) * dz;
            for (int j = 1; j <= ny; j++) {
                double y = (cf.stf == 1.0) ? (double)(j - 1) * cf.dy : cf.dy * (tb_powi(cf.stf, j - 1) - 1.0) / (cf.stf - 1.0);
                if (!(y <= cf.ibm_h)) continue;
                for (int i = 1; i <= nx; i++) {
                    double x = cf.x0 + (double)(i - 1) * cf.dx;
                    double dist = std::sqrt(tb_powi(x - cf.ibm_xc, 2) + tb_powi(z - cf.ibm_zc, 2));
                    double xs = cf.ibm_xc - (cf.ibm_R * (cf.ibm_xc - x)) / dist;
                    double zs = cf.ibm_zc - (cf.ibm_R * (cf.ibm_zc - z)) / dist;
                    double v = std::exp(-tb_powi((x - xs) / sigx / dz, 2) - tb_powi((z - zs) / sigy / dz, 2)) / (sigx * sigy);
                    if (dist < cf.ibm_R) v = 1.0;
                    if (v < 1e-14) v = 0.0;
                    d[(size_t)(i - 1) + (size_t)nx * (j - 1) + n2 * (k - 1)] = v;
                }
            }
        }
    }
    if (c->delta_no) cudaFree(c->delta_no);
    TB_CUDA(cudaMalloc(&c->delta_no, d.size() * sizeof(double)));
    TB_CUDA(cudaMemcpy(c->delta_no, d.data(), d.size() * sizeof(double), cudaMemcpyHostToDevice));
    if (cf.ibm) {
        unsigned nb = tb_blocks(n2, 128);
        TB_DISPATCH_P(P, (k_delta_filter<PP><<<nb, 128, 0, c->stream>>>(c->delta_no, c->gibbs, (int)n2, c->g.K)));
        TB_CHECK_LAUNCH(c);
    }
    return TB_OK;
}
