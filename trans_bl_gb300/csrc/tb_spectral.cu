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
    double yplus = sqrt(A.Re * A.wz[i].x / sqrt(A.fac_y)) * y;
    double damp;
    if (A.damping == 1) {
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
int tb_spectral_prepare(tb_ctx* c) {
    int r = ensure_twiddles(c);
    if (r) return r;
    if (c->cfg.precision == TB_FORM_MIXED && c->g.P >= 4 && !c->nl_phys)
        TB_CUDA(cudaMalloc(&c->nl_phys, (size_t)6 * c->g.P * tb_n2(c) * sizeof(float)));
    return TB_OK;
}

int tb_launch_nlterms(tb_ctx* c, cplx* a, cplx* b, cplx* cc) {
    int r = ensure_twiddles(c);
    if (r) return r;
    NlArgs A{c->ux, c->uy, c->uz, c->wx, c->wy, c->wz, a, b, cc, (int)tb_n2(c), c->g.K};
    cudaEvent_t ps = nullptr;
    if ((r = tb_prof_begin(c, PROF_NLTERMS, &ps))) return r;
    if (c->cfg.precision == TB_FORM_MIXED && c->g.P >= 4) {
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
