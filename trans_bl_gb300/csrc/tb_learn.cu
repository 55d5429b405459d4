// Learned first correction of the mixed v-Poisson solve: a small
// convolutional network, trained by this file's kernels on pairs that the
// solver itself generates.
//
// The reference starts each poi_uy from the current v (poisson_par.f:6-30)
// and iterates V-cycles to the tolerance.  The mixed form starts each stage's
// solve from the extrapolation 2 v(t-1) - v(t-2) of that stage's previous
// solutions; what remains, v(t) - 2 v(t-1) + v(t-2), is a second time
// difference of the flow (advection of disturbances, the oscillation of the
// TS wave) that a local network can estimate from v(t-1), v(t-1) - v(t-2) and
// the FP64 defect of the extrapolation, rhs - L(2 v(t-1) - v(t-2)).  The
// network's estimate is a candidate first correction: the solver keeps it for
// a mode only if it lowers that mode's max defect (otherwise the mode starts
// from the extrapolation), then iterates to the same tolerance as always.
//
// Network: the four input planes divided by fixed input scales, four 3x3
// convolutions with zero padding, 4 -> 32 -> 32 -> 32 -> 1 channels, GELU
// after the first three, the result times a fixed output scale.  Parameters:
// per layer the weights in [cout][cin][3][3] order, then the biases; then the
// four input scales and the output scale (RMS over the training crops of each
// input plane and of the target, set when training starts, not trained).
// Per mode k and part (re, im), with s = max|v1 - v2| over the mode's both
// parts, the inputs on the (nx, ny) fine grid (rows i, columns j) are
//   c0 = v1 / s, c1 = (v1 - v2) / s, c2 = D^-1 d0 / s,
//   c3 = share of k^2 beta^2 in D
// (D: the diagonal of the fine y-line operator at row j), so that the fields
// share one unit and the map to the correction is free of the mode's scale;
// the output times s is the correction.
//
// Training: crops of CW x CW points (a CROP x CROP interior plus the
// network's 4-point reach) with the four input planes, the target
// (v(t) - guess) / s (its RMS sets the output scale) and the crop's mode and
// position.  The loss is what the solver judges: the defect left by the
// correction e (the output times the output scale, on the grid's interior),
//   mean over the crop interiors of (w_k (d0 / s - L e))^2,
// with L the finest FP32 operator of the mixed form (k_resid's) and w_k the
// smallest 1/|D| of the mode, so that rows with the largest diagonal, where
// the max defect sits, weigh most.  Adam.  Forward, backward-data and weight-gradient kernels are FP32 on the
// CUDA cores.
#include "tb_internal.h"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <random>

namespace {

constexpr int LC = 32, LIN = 4, HALO = 4, CROP = 64, CW = CROP + 2 * HALO, PLANES = LIN + 1;
constexpr int OW1 = 0, OB1 = OW1 + LC * LIN * 9, OW2 = OB1 + LC, OB2 = OW2 + LC * LC * 9, OW3 = OB2 + LC,
              OB3 = OW3 + LC * LC * 9, OW4 = OB3 + LC, OB4 = OW4 + LC * 9, OIS = OB4 + 1, OSC = OIS + LIN,
              NPARAM = OSC + 1;
constexpr int CT = 16;   // output tile edge of the convolution kernels

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float x) {
    return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// 3x3 convolution with zero padding over a batch (blockIdx.z) of H x Wd
// images, NCHW.  Forward (TRANS false): pre = W * in + bias and, when act is
// set, act = gelu(pre) (pre may then be null); the sums are multiplied by
// *oscale when it is set, and input channel c is divided by iscale[c] when
// that is set.  Backward data (TRANS true): W is the forward layer
// [CIN][COUT][3][3] (this kernel's CIN is the forward COUT) applied
// transposed and flipped, times gelu'(gpre) when gpre is set.
template <int CIN, int COUT, bool TRANS>
__global__ void __launch_bounds__(256) k_conv(const float* __restrict__ in, const float* __restrict__ W,
                                              const float* __restrict__ bias, float* __restrict__ pre,
                                              float* __restrict__ act, const float* __restrict__ gpre, int H, int Wd,
                                              const float* __restrict__ oscale = nullptr,
                                              const float* __restrict__ iscale = nullptr) {
    constexpr int CCH = CIN < 8 ? CIN : 8;
    extern __shared__ float sm[];
    float* Ws = sm;                      // [ci][t][co]
    float* tile = sm + CIN * 9 * COUT;   // [CCH][18][18]
    for (int q = threadIdx.x; q < CIN * 9 * COUT; q += 256) {
        const int co = q % COUT, t = (q / COUT) % 9, ci = q / (9 * COUT);
        Ws[q] = TRANS ? W[((size_t)ci * COUT + co) * 9 + (8 - t)] : W[((size_t)co * CIN + ci) * 9 + t];
    }
    const int b = blockIdx.z, x0 = blockIdx.x * CT, y0 = blockIdx.y * CT;
    const int tx = threadIdx.x % CT, ty = threadIdx.x / CT;
    float acc[COUT];
#pragma unroll
    for (int o = 0; o < COUT; o++) acc[o] = (!TRANS && bias) ? bias[o] : 0.f;
    for (int c0 = 0; c0 < CIN; c0 += CCH) {
        __syncthreads();
        for (int q = threadIdx.x; q < CCH * 324; q += 256) {
            const int c = q / 324, r = q % 324, yy = y0 + r / 18 - 1, xx = x0 + r % 18 - 1;
            float v = 0.f;
            if (yy >= 0 && yy < H && xx >= 0 && xx < Wd) v = in[(((size_t)b * CIN + c0 + c) * H + yy) * Wd + xx];
            tile[q] = iscale ? v / iscale[c0 + c] : v;
        }
        __syncthreads();
#pragma unroll 1
        for (int c = 0; c < CCH; c++) {
#pragma unroll
            for (int t = 0; t < 9; t++) {
                const float v = tile[c * 324 + (ty + t / 3) * 18 + tx + t % 3];
                const float* w = Ws + ((c0 + c) * 9 + t) * COUT;
                if constexpr (COUT % 4 == 0) {
#pragma unroll
                    for (int o = 0; o < COUT; o += 4) {
                        const float4 w4 = *reinterpret_cast<const float4*>(w + o);
                        acc[o] = fmaf(w4.x, v, acc[o]);
                        acc[o + 1] = fmaf(w4.y, v, acc[o + 1]);
                        acc[o + 2] = fmaf(w4.z, v, acc[o + 2]);
                        acc[o + 3] = fmaf(w4.w, v, acc[o + 3]);
                    }
                } else {
#pragma unroll
                    for (int o = 0; o < COUT; o++) acc[o] = fmaf(w[o], v, acc[o]);
                }
            }
        }
    }
    const int y = y0 + ty, x = x0 + tx;
    if (y >= H || x >= Wd) return;
    const float sc = oscale ? *oscale : 1.f;
#pragma unroll
    for (int o = 0; o < COUT; o++) {
        acc[o] *= sc;
        const size_t off = (((size_t)b * COUT + o) * H + y) * Wd + x;
        if (!TRANS) {
            if (pre) pre[off] = acc[o];
            if (act) act[off] = gelu(acc[o]);
        } else {
            pre[off] = gpre ? acc[o] * gelu_d(gpre[off]) : acc[o];
        }
    }
}

template <int CIN, int COUT, bool TRANS>
constexpr size_t conv_smem() { return (size_t)(CIN * 9 * COUT + (CIN < 8 ? CIN : 8) * 324) * sizeof(float); }

// Weight gradient of a forward layer over the 16x16 output tiles
// blockIdx.x * tpb ... of image blockIdx.y:
//   dW[co][ci][t] += sum_p dpre[co][p] in[ci][p + off(t)],  db[co] += sum_p dpre[co][p].
// Thread (g, co) owns output channel co and input channels g, g + G, ...
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_wgrad(const float* __restrict__ in, const float* __restrict__ dpre,
                                               float* __restrict__ dW, float* __restrict__ db, int H, int Wd, int tpb) {
    constexpr int G = 256 / COUT, NCI = (CIN + G - 1) / G, SP = COUT == 1 ? 1 : COUT + 1;
    extern __shared__ float sm[];
    float* tin = sm;                 // [CIN][18][18]
    float* tdp = sm + CIN * 324;     // [256][SP]
    const int co = threadIdx.x % COUT, g = threadIdx.x / COUT, b = blockIdx.y;
    const int tX = (Wd + CT - 1) / CT, tY = (H + CT - 1) / CT, ntiles = tX * tY;
    float acc[NCI][9];
    float accb = 0.f;
#pragma unroll
    for (int n = 0; n < NCI; n++)
#pragma unroll
        for (int t = 0; t < 9; t++) acc[n][t] = 0.f;
    for (int tt = 0; tt < tpb; tt++) {
        const int tile = blockIdx.x * tpb + tt;
        if (tile >= ntiles) break;   // uniform over the block
        const int x0 = (tile % tX) * CT, y0 = (tile / tX) * CT;
        __syncthreads();
        for (int q = threadIdx.x; q < CIN * 324; q += 256) {
            const int c = q / 324, r = q % 324, yy = y0 + r / 18 - 1, xx = x0 + r % 18 - 1;
            tin[q] = (yy >= 0 && yy < H && xx >= 0 && xx < Wd) ? in[(((size_t)b * CIN + c) * H + yy) * Wd + xx] : 0.f;
        }
        for (int q = threadIdx.x; q < 256 * COUT; q += 256) {
            const int o = q / 256, p = q % 256, py = y0 + p / CT, px = x0 + p % CT;
            tdp[p * SP + o] = (py < H && px < Wd) ? dpre[(((size_t)b * COUT + o) * H + py) * Wd + px] : 0.f;
        }
        __syncthreads();
#pragma unroll 1
        for (int p = 0; p < 256; p++) {
            const float a = tdp[p * SP + co];
            const int py = p / CT, px = p % CT;
            accb += a;
#pragma unroll
            for (int n = 0; n < NCI; n++) {
                const int ci = g + n * G;
                if (ci < CIN) {
                    const float* s = tin + ci * 324 + py * 18 + px;
#pragma unroll
                    for (int t = 0; t < 9; t++) acc[n][t] = fmaf(a, s[(t / 3) * 18 + t % 3], acc[n][t]);
                }
            }
        }
    }
#pragma unroll
    for (int n = 0; n < NCI; n++) {
        const int ci = g + n * G;
        if (ci < CIN)
#pragma unroll
            for (int t = 0; t < 9; t++) atomicAdd(&dW[((size_t)co * CIN + ci) * 9 + t], acc[n][t]);
    }
    if (g == 0) atomicAdd(&db[co], accb);
}

template <int CIN, int COUT>
constexpr size_t wgrad_smem() { return (size_t)(CIN * 324 + 256 * (COUT == 1 ? 1 : COUT + 1)) * sizeof(float); }

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const float gq = g[q];
    const float mq = b1 * m[q] + (1.f - b1) * gq, vq = b2 * v[q] + (1.f - b2) * gq * gq;
    m[q] = mq;
    v[q] = vq;
    w[q] -= lr * (mq / c1) / (sqrtf(vq / c2) + eps);
}

// Sum of squares of plane blockIdx.y over the interiors of n crops (for the
// input and output scales).
__global__ void k_plane_sq(const float* __restrict__ samples, long long n, double* acc) {
    const size_t per = (size_t)PLANES * CW * CW, tot = (size_t)n * CROP * CROP;
    const int pl = blockIdx.y;
    double s = 0.0;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x) {
        const size_t c = q / (CROP * CROP);
        const int r = (int)(q % (CROP * CROP)), y = HALO + r / CROP, x = HALO + r % CROP;
        const float v = samples[c * per + (size_t)pl * CW * CW + (size_t)y * CW + x];
        s += (double)v * v;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&acc[pl], s);
}

// Batch of crops idx[b] of the sample buffer: input planes divided by their
// scales into X (B, 4, CW, CW), target plane into T (B, CW, CW).
__global__ void k_batch(const float* __restrict__ samples, const int* __restrict__ idx, float* __restrict__ X,
                        float* __restrict__ T, int B, const float* __restrict__ iscale) {
    const size_t per = (size_t)PLANES * CW * CW;
    const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= (size_t)B * per) return;
    const int b = (int)(q / per), r = (int)(q % per), pl = r / (CW * CW), pix = r % (CW * CW);
    const float v = samples[(size_t)idx[b] * per + r];
    if (pl < LIN) X[((size_t)b * LIN + pl) * CW * CW + pix] = v / iscale[pl];
    else T[(size_t)b * CW * CW + pix] = v;
}

// Crops of one solve: crop c of image im = pos[3c] (2k + part) with top-left
// (i0, j0) = (pos[3c+1], pos[3c+2]) on the (nx, ny) grid; the four input
// planes from X, the target (fc - g0) / max|v1 - v2| on the interior.
__global__ void k_crops(const float* __restrict__ X, const cplx* __restrict__ fc, const cplx* __restrict__ g0,
                        const float* __restrict__ scl, const int* __restrict__ pos, float* __restrict__ dst, int ncrop,
                        int nx, int ny, size_t elems64) {
    const size_t per = (size_t)PLANES * CW * CW;
    const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= (size_t)ncrop * per) return;
    const int c = (int)(q / per), r = (int)(q % per), pl = r / (CW * CW), pix = r % (CW * CW);
    const int im = pos[3 * c], i = pos[3 * c + 1] + pix / CW, j = pos[3 * c + 2] + pix % CW;
    float v = 0.f;
    if (i >= 0 && i < nx && j >= 0 && j < ny) {
        if (pl < LIN) {
            v = X[(((size_t)im * LIN + pl) * nx + i) * ny + j];
        } else if (i >= 1 && i <= nx - 2 && j >= 1) {
            const int k = im >> 1;
            const size_t o = (size_t)k * elems64 + (size_t)i + (size_t)nx * j;
            const double d = (im & 1) ? fc[o].y - g0[o].y : fc[o].x - g0[o].x;
            const float s = scl[3 * k + 1];
            v = s > 0.f ? (float)(d / (double)s) : 0.f;
        }
    }
    dst[q] = v;
}

// Visit the terms (i', j', coefficient) of the finest FP32 operator at
// interior point (i, j) of mode k, term by term as k_resid evaluates it
// (defect, poisson_par.f:543-793): L e = b den + cc q2 + d ify - top e.
template <class V>
__device__ __forceinline__ void fine_terms(const FineOp& F, int k, int i, int j, V&& visit) {
    const float* SP = F.coef;
    const float *CP = SP + 7, *PP = SP + 15, *LP = SP + 19;
    const int n = F.ny, nxl = F.nx;
    const float k2 = (float)F.k2b2[k], den = F.den, ify = F.ify;
    auto xs = [&](int jj, float w) {   // the x-stencil of row jj, times w
        if (i == 1 || i == nxl - 2) {
            const int e = (i == 1) ? 1 : -1;
            visit(i - e, jj, 10.f * w); visit(i, jj, -15.f * w); visit(i + e, jj, -4.f * w);
            visit(i + 2 * e, jj, 14.f * w); visit(i + 3 * e, jj, -6.f * w); visit(i + 4 * e, jj, w);
        } else {
            visit(i - 2, jj, -w); visit(i - 1, jj, 16.f * w); visit(i, jj, -30.f * w);
            visit(i + 1, jj, 16.f * w); visit(i + 2, jj, -w);
        }
    };
    if (j == 1) {
        const float q2 = F.qdy2[0];
        xs(2, SP[2] * den); xs(1, SP[1] * den);
        visit(i, 0, SP[3] * q2); visit(i, 1, SP[4] * q2 + k2 * SP[1] * ify);
        visit(i, 2, SP[5] * q2 + k2 * SP[2] * ify); visit(i, 3, SP[6] * q2);
    } else if (j <= n - 3) {
        const float q2 = F.qdy2[j - 2];
        xs(j - 1, CP[0] * den); xs(j, CP[1] * den); xs(j + 1, CP[2] * den);
        visit(i, j - 2, CP[3] * q2); visit(i, j - 1, CP[4] * q2 + k2 * CP[0] * ify);
        visit(i, j, CP[5] * q2 + k2 * CP[1] * ify); visit(i, j + 1, CP[6] * q2 + k2 * CP[2] * ify);
        visit(i, j + 2, CP[7] * q2);
    } else if (j == n - 2) {
        const float q2 = F.qdy2[j - 1];
        xs(j, den);
        visit(i, j - 1, PP[1] * q2); visit(i, j, PP[2] * q2 + k2 * ify); visit(i, j + 1, PP[3] * q2);
    } else {
        const float q2 = F.qdy2[j - 2];
        const float top = LP[1] * sqrtf((F.alpha2 - k2) * ify) * sqrtf(q2);
        xs(j, den);
        visit(i, j, LP[2] * q2 + k2 * ify - top); visit(i, j - 1, LP[3] * q2); visit(i, j - 2, LP[4] * q2);
    }
}

// Defect loss of a batch (blockIdx.x = crop b, whose mode, first row and first
// column are meta[3b] / 2, meta[3b+1], meta[3b+2]): for the correction
// e = oscale * out (zero off the grid's interior),
//   rho = w_k (d0 / s - L e) on the crop interior,  d0 / s = plane 2 / invD,
//   loss += sum rho^2 / n,  dout = -(2 / n) oscale m L^T (w_k rho).
// crops is the batch's scaled input block (B, 4, CW, CW) and *p2scale the
// scale plane 2 was divided by.  Without dout (null) only the loss; with
// zero_out the correction is 0.
constexpr int LT = 256;
__global__ void __launch_bounds__(LT) k_defect_loss(FineOp F, const float* __restrict__ crops,
                                                    const int* __restrict__ meta, const float* __restrict__ out,
                                                    float* __restrict__ dout, double* loss, const float* __restrict__ invD,
                                                    const float* __restrict__ wmode, const float* __restrict__ oscale,
                                                    const float* __restrict__ p2scale, int B, int zero_out) {
    __shared__ float es[CW * CW], gs[CW * CW];
    const int b = blockIdx.x, k = meta[3 * b] >> 1, i0 = meta[3 * b + 1], j0 = meta[3 * b + 2];
    const float sc = *oscale, wk = wmode[k];
    auto inner = [&](int i, int j) { return i >= 1 && i <= F.nx - 2 && j >= 1 && j <= F.ny - 1; };
    for (int q = threadIdx.x; q < CW * CW; q += LT) {
        const int i = i0 + q / CW, j = j0 + q % CW;
        es[q] = (!zero_out && inner(i, j)) ? sc * out[(size_t)b * CW * CW + q] : 0.f;
        gs[q] = 0.f;
    }
    __syncthreads();
    const float* d2 = crops + ((size_t)b * LIN + 2) * CW * CW;   // plane 2 of the batch's input block,
    const float p2 = *p2scale;                                     // divided there by its input scale
    float sq = 0.f;
    for (int q = threadIdx.x; q < CROP * CROP; q += LT) {
        const int y = HALO + q / CROP, x = HALO + q % CROP, i = i0 + y, j = j0 + x;
        if (!inner(i, j)) continue;
        const float iv = invD[(size_t)k * F.ny + j];
        float le = 0.f;
        fine_terms(F, k, i, j, [&](int ii, int jj, float c) { le = fmaf(c, es[(ii - i0) * CW + (jj - j0)], le); });
        const float rho = wk * (p2 * d2[y * CW + x] / iv - le);
        sq = fmaf(rho, rho, sq);
        if (dout) fine_terms(F, k, i, j, [&](int ii, int jj, float c) { atomicAdd(&gs[(ii - i0) * CW + (jj - j0)], c * wk * rho); });
    }
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if (loss && (threadIdx.x & 31) == 0 && sq != 0.f) atomicAdd(loss, (double)sq / ((double)B * CROP * CROP));
    if (!dout) return;
    __syncthreads();
    const float g = -2.f * sc / (float)((size_t)B * CROP * CROP);
    for (int q = threadIdx.x; q < CW * CW; q += LT) {
        const int i = i0 + q / CW, j = j0 + q % CW;
        dout[(size_t)b * CW * CW + q] = inner(i, j) ? g * gs[q] : 0.f;
    }
}

__global__ void k_meta(const int* __restrict__ meta, const int* __restrict__ idx, int* __restrict__ bmeta, int B) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < 3 * B) bmeta[q] = meta[3 * (size_t)idx[q / 3] + q % 3];
}

struct Learn {
    LearnSolve s;
    float *w = nullptr, *gw = nullptr, *m = nullptr, *v = nullptr;
    long long adam_t = 0;
    float *P0 = nullptr, *P1 = nullptr;          // inference ping-pong (2K, LC, nx, ny)
    float* samples = nullptr;
    int* meta = nullptr;          // (cap, 3) image (2k + part), first row, first column per crop
    float* wmode = nullptr;       // (K) smallest 1/|D| of each mode
    long long cap = 0, count = 0;
    int per_solve = 0;
    std::mt19937_64 rng;
    int* d_pos = nullptr;
    int pos_cap = 0;
    double last_loss = 0.0;
};

Learn* get(tb_ctx* c) { return static_cast<Learn*>(c->learn); }

template <typename T>
int dalloc(T** p, size_t n) {
    if (*p) return TB_OK;
    TB_CUDA(cudaMalloc((void**)p, n * sizeof(T)));
    TB_CUDA(cudaMemset(*p, 0, n * sizeof(T)));
    return TB_OK;
}

int smem_attrs() {
    static bool done[64] = {false};
    int dev = 0;
    TB_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && done[dev]) return TB_OK;
    TB_CUDA(cudaFuncSetAttribute(k_wgrad<LC, LC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wgrad_smem<LC, LC>()));
    if (dev >= 0 && dev < 64) done[dev] = true;
    return TB_OK;
}

// Forward of the network over B images of H x Wd: X (B, 4) -> out (B, 1).
// Inference (`scaled`): X holds the raw input planes, and the input and output
// scales are applied; training: X holds the scaled planes (k_batch) and the
// output is unscaled.
// P* hold the pre-activations and A* the activations of layers 1-3 (each
// (B, LC, H, Wd)); inference passes null P* and alternates two A buffers.
struct Fwd { float *P1, *A1, *P2, *A2, *P3, *A3; };
int forward(cudaStream_t st, const float* w, const float* X, float* out, const Fwd& f, int B, int H, int Wd,
            bool scaled) {
    dim3 grid((Wd + CT - 1) / CT, (H + CT - 1) / CT, B);
    k_conv<LIN, LC, false><<<grid, 256, conv_smem<LIN, LC, false>(), st>>>(X, w + OW1, w + OB1, f.P1, f.A1, nullptr, H, Wd,
                                                                         nullptr, scaled ? w + OIS : nullptr);
    k_conv<LC, LC, false><<<grid, 256, conv_smem<LC, LC, false>(), st>>>(f.A1, w + OW2, w + OB2, f.P2, f.A2, nullptr, H, Wd);
    k_conv<LC, LC, false><<<grid, 256, conv_smem<LC, LC, false>(), st>>>(f.A2, w + OW3, w + OB3, f.P3, f.A3, nullptr, H, Wd);
    k_conv<LC, 1, false><<<grid, 256, conv_smem<LC, 1, false>(), st>>>(f.A3, w + OW4, w + OB4, out, nullptr, nullptr, H, Wd,
                                                                     scaled ? w + OSC : nullptr);
    TB_CUDA(cudaGetLastError());
    return TB_OK;
}

// Backward of forward() on crops (H = Wd = CW) from dout into gw (zeroed here).
// dA, dB: (B, LC, CW, CW) work buffers.
int backward(cudaStream_t st, const float* w, float* gw, const float* X, const Fwd& f, const float* dout, float* dA,
             float* dB, int B) {
    int r;
    if ((r = smem_attrs())) return r;
    const int H = CW, Wd = CW;
    dim3 grid((Wd + CT - 1) / CT, (H + CT - 1) / CT, B);
    const int ntiles = ((Wd + CT - 1) / CT) * ((H + CT - 1) / CT), tpb = 5;
    dim3 wg((ntiles + tpb - 1) / tpb, B);
    TB_CUDA(cudaMemsetAsync(gw, 0, NPARAM * sizeof(float), st));
    // layer 4: dP4 = dout
    k_wgrad<LC, 1><<<wg, 256, wgrad_smem<LC, 1>(), st>>>(f.A3, dout, gw + OW4, gw + OB4, H, Wd, tpb);
    k_conv<1, LC, true><<<grid, 256, conv_smem<1, LC, true>(), st>>>(dout, w + OW4, nullptr, dA, nullptr, f.P3, H, Wd);
    // layer 3: dP3 = dA
    k_wgrad<LC, LC><<<wg, 256, wgrad_smem<LC, LC>(), st>>>(f.A2, dA, gw + OW3, gw + OB3, H, Wd, tpb);
    k_conv<LC, LC, true><<<grid, 256, conv_smem<LC, LC, true>(), st>>>(dA, w + OW3, nullptr, dB, nullptr, f.P2, H, Wd);
    // layer 2: dP2 = dB
    k_wgrad<LC, LC><<<wg, 256, wgrad_smem<LC, LC>(), st>>>(f.A1, dB, gw + OW2, gw + OB2, H, Wd, tpb);
    k_conv<LC, LC, true><<<grid, 256, conv_smem<LC, LC, true>(), st>>>(dB, w + OW2, nullptr, dA, nullptr, f.P1, H, Wd);
    // layer 1: dP1 = dA
    k_wgrad<LIN, LC><<<wg, 256, wgrad_smem<LIN, LC>(), st>>>(X, dA, gw + OW1, gw + OB1, H, Wd, tpb);
    TB_CUDA(cudaGetLastError());
    return TB_OK;
}

// Training buffers for a batch of B crops.
struct TrainBufs {
    float *X = nullptr, *T = nullptr, *out = nullptr, *dout = nullptr, *dA = nullptr, *dB = nullptr;
    float *P1 = nullptr, *A1 = nullptr, *P2 = nullptr, *A2 = nullptr, *P3 = nullptr, *A3 = nullptr;
    double* loss = nullptr;
    double* dloss = nullptr;   // PLANES sums of squares
    int* idx = nullptr;
    int* bmeta = nullptr;      // (B, 3) meta of the batch
    int alloc(int B) {
        const size_t img = (size_t)CW * CW, hid = (size_t)B * LC * img;
        int r;
        if ((r = dalloc(&X, (size_t)B * LIN * img)) || (r = dalloc(&T, (size_t)B * img)) || (r = dalloc(&out, (size_t)B * img)) ||
            (r = dalloc(&dout, (size_t)B * img)) || (r = dalloc(&dA, hid)) || (r = dalloc(&dB, hid)) ||
            (r = dalloc(&P1, hid)) || (r = dalloc(&A1, hid)) || (r = dalloc(&P2, hid)) || (r = dalloc(&A2, hid)) ||
            (r = dalloc(&P3, hid)) || (r = dalloc(&A3, hid)) || (r = dalloc(&loss, 1)) || (r = dalloc(&dloss, PLANES)) ||
            (r = dalloc(&idx, (size_t)B)) || (r = dalloc(&bmeta, (size_t)3 * B)))
            return r;
        return TB_OK;
    }
    void release() {
        for (void* p : {(void*)X, (void*)T, (void*)out, (void*)dout, (void*)dA, (void*)dB, (void*)P1, (void*)A1, (void*)P2,
                        (void*)A2, (void*)P3, (void*)A3, (void*)loss, (void*)dloss, (void*)idx, (void*)bmeta})
            if (p) cudaFree(p);
    }
    Fwd fwd() const { return Fwd{P1, A1, P2, A2, P3, A3}; }
};

// He-normal weights (std sqrt(2 / fan_in)), zero biases and a zero last
// layer, so an untrained network proposes no correction.
void init_weights(std::vector<float>& w, unsigned long long seed) {
    std::mt19937_64 g(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    w.assign(NPARAM, 0.f);
    auto fill = [&](int off, int n, int fan_in) {
        const float s = std::sqrt(2.f / (float)fan_in);
        for (int q = 0; q < n; q++) w[off + q] = s * nd(g);
    };
    fill(OW1, LC * LIN * 9, LIN * 9);
    fill(OW2, LC * LC * 9, LC * 9);
    fill(OW3, LC * LC * 9, LC * 9);
    for (int p = 0; p < LIN; p++) w[OIS + p] = 1.f;
    w[OSC] = 1.f;
}

int ensure(tb_ctx* c) {
    if (c->learn) return TB_OK;
    if (c->cfg.precision != TB_FORM_MIXED || !c->mixed) {
        tb_set_error("the learned correction needs the mixed form");
        return TB_ERR_STATE;
    }
    Learn* L = new (std::nothrow) Learn();
    if (!L) return TB_ERR_NOMEM;
    c->learn = L;
    const int K = c->g.K, nx = c->g.nx, ny = c->g.ny;
    const size_t img = (size_t)nx * ny;
    int r;
    if ((r = dalloc(&L->w, NPARAM)) || (r = dalloc(&L->gw, NPARAM)) || (r = dalloc(&L->m, NPARAM)) ||
        (r = dalloc(&L->v, NPARAM)) || (r = dalloc(&L->s.X, (size_t)2 * K * LIN * img)) ||
        (r = dalloc(&L->s.out, (size_t)2 * K * img)) || (r = dalloc(&L->s.scl, (size_t)3 * K)) ||
        (r = dalloc(&L->s.jmax, (size_t)K)) || (r = dalloc(&L->s.invD, (size_t)K * ny)) ||
        (r = dalloc(&L->s.mfeat, (size_t)K * ny)) || (r = dalloc(&L->s.tally, (size_t)2 * K)))
        return r;
    std::vector<float> invD, mf;
    if ((r = tb_mixed_line_diag(c, invD, mf))) return r;
    TB_CUDA(cudaMemcpy(L->s.invD, invD.data(), invD.size() * sizeof(float), cudaMemcpyHostToDevice));
    TB_CUDA(cudaMemcpy(L->s.mfeat, mf.data(), mf.size() * sizeof(float), cudaMemcpyHostToDevice));
    std::vector<float> wm(K, 0.f);
    for (int k = 0; k < K; k++) {
        float m = 0.f;
        for (int j = 1; j < ny; j++) {
            const float v = invD[(size_t)k * ny + j];
            if (v > 0.f && (m == 0.f || v < m)) m = v;
        }
        wm[k] = m;
    }
    if ((r = dalloc(&L->wmode, (size_t)K))) return r;
    TB_CUDA(cudaMemcpy(L->wmode, wm.data(), K * sizeof(float), cudaMemcpyHostToDevice));
    std::vector<float> w;
    init_weights(w, 1);
    TB_CUDA(cudaMemcpy(L->w, w.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    return TB_OK;
}

}  // namespace

LearnSolve* tb_learn_solve(tb_ctx* c) {
    Learn* L = get(c);
    return (L && (L->s.infer || L->s.sample)) ? &L->s : nullptr;
}

int tb_learn_run_net(tb_ctx* c) {
    Learn* L = get(c);
    if (!L) { tb_set_error("learned correction not set up"); return TB_ERR_STATE; }
    const int B = 2 * c->g.K, H = c->g.nx, Wd = c->g.ny;
    if (!L->P0 || !L->P1) { tb_set_error("learned correction: buffers not set up (tb_learn_enable)"); return TB_ERR_STATE; }
    int r;
    // inference keeps no pre-activations; activations alternate two buffers
    Fwd f{nullptr, L->P0, nullptr, L->P1, nullptr, L->P0};
    if ((r = forward(c->stream, L->w, L->s.X, L->s.out, f, B, H, Wd, true))) return r;
    c->launches += 4;
    return TB_OK;
}

int tb_learn_collect(tb_ctx* c) {
    Learn* L = get(c);
    if (!L || !L->s.sample || L->count >= L->cap) return TB_OK;
    const int K = c->g.K, nx = c->g.nx, ny = c->g.ny;
    const int n = (int)std::min<long long>(L->per_solve, L->cap - L->count);
    std::vector<int> pos((size_t)3 * n);
    std::uniform_int_distribution<int> dim(0, 2 * K - 1), di(-HALO, nx - CW + HALO), dj(-HALO, ny - CW + HALO);
    for (int q = 0; q < n; q++) {
        pos[3 * q] = dim(L->rng);
        pos[3 * q + 1] = nx >= CW ? di(L->rng) : -HALO;
        pos[3 * q + 2] = ny >= CW ? dj(L->rng) : -HALO;
    }
    if (L->pos_cap < n) {
        if (L->d_pos) cudaFree(L->d_pos);
        L->d_pos = nullptr;
        TB_CUDA(cudaMalloc(&L->d_pos, (size_t)3 * n * sizeof(int)));
        L->pos_cap = n;
    }
    TB_CUDA(cudaMemcpyAsync(L->d_pos, pos.data(), pos.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    const size_t per = (size_t)PLANES * CW * CW;
    k_crops<<<tb_blocks((size_t)n * per, 256), 256, 0, c->stream>>>(L->s.X, c->pfc, L->s.g0, L->s.scl, L->d_pos,
                                                                     L->samples + (size_t)L->count * per, n, nx, ny,
                                                                     c->g.lvl_elems);
    TB_CHECK_LAUNCH(c);
    TB_CUDA(cudaMemcpyAsync(L->meta + (size_t)3 * L->count, L->d_pos, (size_t)3 * n * sizeof(int), cudaMemcpyDeviceToDevice,
                            c->stream));
    L->count += n;
    return TB_OK;
}

void tb_learn_free(tb_ctx* c) {
    Learn* L = get(c);
    if (!L) return;
    for (void* p : {(void*)L->w, (void*)L->gw, (void*)L->m, (void*)L->v, (void*)L->P0, (void*)L->P1, (void*)L->samples,
                    (void*)L->meta, (void*)L->wmode,
                    (void*)L->d_pos, (void*)L->s.X, (void*)L->s.out, (void*)L->s.scl, (void*)L->s.jmax, (void*)L->s.invD,
                    (void*)L->s.mfeat, (void*)L->s.g0, (void*)L->s.tally, (void*)L->s.gate})
        if (p) cudaFree(p);
    delete L;
    c->learn = nullptr;
}

extern "C" {

int tb_learn_param_count(void) { return NPARAM; }
int tb_learn_crop_size(void) { return CW; }

int tb_learn_init(tb_ctx* c, unsigned long long seed) {
    if (!c) { tb_set_error("null context"); return TB_ERR_ARG; }
    int r = ensure(c);
    if (r) return r;
    Learn* L = get(c);
    std::vector<float> w;
    init_weights(w, seed);
    TB_CUDA(cudaMemcpy(L->w, w.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    TB_CUDA(cudaMemset(L->m, 0, NPARAM * sizeof(float)));
    TB_CUDA(cudaMemset(L->v, 0, NPARAM * sizeof(float)));
    L->adam_t = 0;
    return TB_OK;
}

int tb_learn_set_weights(tb_ctx* c, const float* w) {
    if (!c || !w) { tb_set_error("null argument"); return TB_ERR_ARG; }
    int r = ensure(c);
    if (r) return r;
    Learn* L = get(c);
    TB_CUDA(cudaStreamSynchronize(c->stream));
    TB_CUDA(cudaMemcpy(L->w, w, NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    return TB_OK;
}

int tb_learn_get_weights(tb_ctx* c, float* w) {
    if (!c || !w) { tb_set_error("null argument"); return TB_ERR_ARG; }
    int r = ensure(c);
    if (r) return r;
    TB_CUDA(cudaStreamSynchronize(c->stream));
    TB_CUDA(cudaMemcpy(w, get(c)->w, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    return TB_OK;
}

int tb_learn_enable(tb_ctx* c, int on) {
    if (!c) { tb_set_error("null context"); return TB_ERR_ARG; }
    int r = ensure(c);
    if (r) return r;
    if (!c->cfg.warm_start) { tb_set_error("the learned correction needs a warm start (warm_start > 0)"); return TB_ERR_STATE; }
    Learn* L = get(c);
    if (on < 0 || on > 2) { tb_set_error("tb_learn_enable: mode must be 0, 1 or 2"); return TB_ERR_ARG; }
    if (on) {
        const size_t hid = (size_t)2 * c->g.K * LC * c->g.nx * c->g.ny;
        if ((r = dalloc(&L->P0, hid)) || (r = dalloc(&L->P1, hid))) return r;
        if ((r = dalloc(&L->s.gate, 33))) return r;
    }
    TB_CUDA(cudaStreamSynchronize(c->stream));
    L->s.infer = on != 0;
    L->s.gated = (on == 2) ? 1 : 0;
    tb_graph_reset(c);
    return TB_OK;
}

int tb_learn_sample(tb_ctx* c, long long capacity, int crops_per_solve, unsigned long long seed) {
    if (!c) { tb_set_error("null context"); return TB_ERR_ARG; }
    int r = ensure(c);
    if (r) return r;
    Learn* L = get(c);
    TB_CUDA(cudaStreamSynchronize(c->stream));
    tb_graph_reset(c);
    if (capacity <= 0) {   // stop collecting; the crops stay for training
        L->s.sample = false;
        return TB_OK;
    }
    if (!c->cfg.warm_start) { tb_set_error("sampling needs a warm start (warm_start > 0)"); return TB_ERR_STATE; }
    if (crops_per_solve < 1) { tb_set_error("crops_per_solve must be >= 1"); return TB_ERR_ARG; }
    if (L->samples) cudaFree(L->samples);
    if (L->meta) cudaFree(L->meta);
    L->samples = nullptr;
    L->meta = nullptr;
    TB_CUDA(cudaMalloc(&L->samples, (size_t)capacity * PLANES * CW * CW * sizeof(float)));
    TB_CUDA(cudaMalloc(&L->meta, (size_t)capacity * 3 * sizeof(int)));
    if ((r = dalloc(&L->s.g0, (size_t)c->g.K * c->g.lvl_elems))) return r;
    L->cap = capacity;
    L->count = 0;
    L->per_solve = crops_per_solve;
    L->rng.seed(seed);
    L->s.sample = true;
    return TB_OK;
}

int tb_learn_train(tb_ctx* c, long long n_train, int iters, int batch, float lr, unsigned long long seed, double* loss) {
    if (!c) { tb_set_error("null context"); return TB_ERR_ARG; }
    int r = ensure(c);
    if (r) return r;
    Learn* L = get(c);
    if (L->count < 1) { tb_set_error("no training crops (tb_learn_sample, then steps)"); return TB_ERR_STATE; }
    if (n_train <= 0 || n_train > L->count) n_train = L->count;
    if (iters < 1 || batch < 1 || !(lr > 0.f)) { tb_set_error("iters, batch and lr must be positive"); return TB_ERR_ARG; }
    FineOp F;
    if ((r = tb_mixed_fine_op(c, &F))) return r;
    TrainBufs tb;
    if ((r = tb.alloc(batch))) { tb.release(); return r; }
    cudaStream_t st = c->stream;
    if (L->adam_t == 0) {   // a fresh training run: input and output scales = RMS of the planes
        double* acc = tb.dloss;
        double sq[PLANES] = {0, 0, 0, 0, 0};
        cudaError_t e = cudaMemsetAsync(acc, 0, PLANES * sizeof(double), st);
        if (e == cudaSuccess) {
            k_plane_sq<<<dim3(128, PLANES), 256, 0, st>>>(L->samples, n_train, acc);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(sq, acc, sizeof sq, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        float sc[PLANES];
        for (int p = 0; p < PLANES; p++) {
            sc[p] = (float)std::sqrt(sq[p] / ((double)n_train * CROP * CROP));
            if (!(sc[p] > 0.f) || !std::isfinite(sc[p])) sc[p] = 1.f;
        }
        if (e == cudaSuccess) e = cudaMemcpy(L->w + OIS, sc, sizeof sc, cudaMemcpyHostToDevice);   // OIS .. OIS + 3, then OSC
        if (e != cudaSuccess) {
            tb_set_error("training: %s", cudaGetErrorString(e));
            tb.release();
            return TB_ERR_CUDA;
        }
    }
    std::mt19937_64 g(seed);
    std::uniform_int_distribution<long long> pick(0, n_train - 1);
    std::vector<int> idx(batch);
    double acc = 0.0;
    int nacc = 0;
    const int tail = std::max(1, iters / 10);
    if (cudaMemsetAsync(tb.loss, 0, sizeof(double), st) != cudaSuccess) {
        tb_set_error("training: %s", cudaGetErrorString(cudaGetLastError()));
        r = TB_ERR_CUDA;
    }
    for (int it = 0; it < iters && !r; it++) {
        for (int b = 0; b < batch; b++) idx[b] = (int)pick(g);
        if (cudaMemcpyAsync(tb.idx, idx.data(), batch * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess) {
            tb_set_error("training: %s", cudaGetErrorString(cudaGetLastError()));
            r = TB_ERR_CUDA;
            break;
        }
        k_batch<<<tb_blocks((size_t)batch * PLANES * CW * CW, 256), 256, 0, st>>>(L->samples, tb.idx, tb.X, tb.T, batch,
                                                                                   L->w + OIS);
        k_meta<<<tb_blocks((size_t)3 * batch, 128), 128, 0, st>>>(L->meta, tb.idx, tb.bmeta, batch);
        if ((r = forward(st, L->w, tb.X, tb.out, tb.fwd(), batch, CW, CW, false))) break;
        const bool rec = it >= iters - tail;
        nacc += rec;
        k_defect_loss<<<batch, LT, 0, st>>>(F, tb.X, tb.bmeta, tb.out, tb.dout, rec ? tb.loss : nullptr, L->s.invD,
                                            L->wmode, L->w + OSC, L->w + OIS + 2, batch, 0);
        if ((r = backward(st, L->w, L->gw, tb.X, tb.fwd(), tb.dout, tb.dA, tb.dB, batch))) break;
        L->adam_t++;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f - std::pow(b1, (float)L->adam_t), c2 = 1.f - std::pow(b2, (float)L->adam_t);
        k_adam<<<tb_blocks(NPARAM, 256), 256, 0, st>>>(L->w, L->gw, L->m, L->v, NPARAM, lr, b1, b2, 1e-8f, c1, c2);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) { tb_set_error("training: %s", cudaGetErrorString(e)); r = TB_ERR_CUDA; }
        // bound the host's lead over the device
        if (!r && (it & 63) == 63 && cudaStreamSynchronize(st) != cudaSuccess) {
            tb_set_error("training: %s", cudaGetErrorString(cudaGetLastError()));
            r = TB_ERR_CUDA;
        }
    }
    if (!r) {
        cudaError_t e = cudaMemcpyAsync(&acc, tb.loss, sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { tb_set_error("training: %s", cudaGetErrorString(e)); r = TB_ERR_CUDA; }
    }
    tb.release();
    if (r) return r;
    L->last_loss = nacc ? acc / nacc : 0.0;
    if (loss) *loss = L->last_loss;
    return TB_OK;
}

// Defect loss of the network on crops first .. first+n-1, and of a zero
// correction (the defect the extrapolated guess leaves).
int tb_learn_eval(tb_ctx* c, long long first, long long n, double* mse, double* target_ms) {
    if (!c || !mse || !target_ms || first < 0 || n < 1) { tb_set_error("bad argument"); return TB_ERR_ARG; }
    Learn* L = get(c);
    if (!L || first + n > L->count) { tb_set_error("crops %lld..%lld not collected", first, first + n); return TB_ERR_ARG; }
    const int B = 32;
    FineOp F;
    int r = tb_mixed_fine_op(c, &F);
    if (r) return r;
    TrainBufs tb;
    r = tb.alloc(B);
    cudaStream_t st = c->stream;
    double acc[2] = {0.0, 0.0};
    std::vector<int> idx(B);
    for (long long b0 = 0; b0 < n && !r; b0 += B) {
        const int nb = (int)std::min<long long>(B, n - b0);
        for (int q = 0; q < nb; q++) idx[q] = (int)(first + b0 + q);
        double part[2] = {0.0, 0.0};
        cudaError_t e = cudaMemcpyAsync(tb.idx, idx.data(), nb * sizeof(int), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(tb.dloss, 0, 2 * sizeof(double), st);
        if (e != cudaSuccess) { tb_set_error("%s", cudaGetErrorString(e)); r = TB_ERR_CUDA; break; }
        k_batch<<<tb_blocks((size_t)nb * PLANES * CW * CW, 256), 256, 0, st>>>(L->samples, tb.idx, tb.X, tb.T, nb, L->w + OIS);
        k_meta<<<tb_blocks((size_t)3 * nb, 128), 128, 0, st>>>(L->meta, tb.idx, tb.bmeta, nb);
        if ((r = forward(st, L->w, tb.X, tb.out, tb.fwd(), nb, CW, CW, false))) break;
        k_defect_loss<<<nb, LT, 0, st>>>(F, tb.X, tb.bmeta, tb.out, nullptr, tb.dloss, L->s.invD, L->wmode, L->w + OSC,
                                         L->w + OIS + 2, nb, 0);
        k_defect_loss<<<nb, LT, 0, st>>>(F, tb.X, tb.bmeta, tb.out, nullptr, tb.dloss + 1, L->s.invD, L->wmode, L->w + OSC,
                                         L->w + OIS + 2, nb, 1);
        e = cudaMemcpyAsync(part, tb.dloss, sizeof part, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { tb_set_error("%s", cudaGetErrorString(e)); r = TB_ERR_CUDA; break; }
        acc[0] += part[0] * nb;
        acc[1] += part[1] * nb;
    }
    tb.release();
    if (r) return r;
    *mse = acc[0] / (double)n;
    *target_ms = acc[1] / (double)n;
    return TB_OK;
}

int tb_learn_get_samples(tb_ctx* c, long long first, long long n, float* dst) {
    if (!c || !dst || first < 0 || n < 0) { tb_set_error("bad argument"); return TB_ERR_ARG; }
    Learn* L = get(c);
    if (!L || first + n > L->count) { tb_set_error("crops %lld..%lld not collected", first, first + n); return TB_ERR_ARG; }
    const size_t per = (size_t)PLANES * CW * CW;
    TB_CUDA(cudaStreamSynchronize(c->stream));
    TB_CUDA(cudaMemcpy(dst, L->samples + (size_t)first * per, (size_t)n * per * sizeof(float), cudaMemcpyDeviceToHost));
    return TB_OK;
}

int tb_learn_get_stats(tb_ctx* c, tb_learn_stats* st) {
    if (!c || !st) { tb_set_error("null argument"); return TB_ERR_ARG; }
    std::memset(st, 0, sizeof *st);
    Learn* L = get(c);
    if (!L) return TB_OK;
    const int K = c->g.K;
    std::vector<long long> t((size_t)2 * K);
    TB_CUDA(cudaStreamSynchronize(c->stream));
    TB_CUDA(cudaMemcpy(t.data(), L->s.tally, t.size() * sizeof(long long), cudaMemcpyDeviceToHost));
    for (int k = 0; k < K; k++) { st->tried += t[2 * k]; st->kept += t[2 * k + 1]; }
    if (L->s.gate) {
        int g[32];
        TB_CUDA(cudaMemcpy(g, L->s.gate, sizeof g, cudaMemcpyDeviceToHost));
        for (int s = 0; s < 4; s++) { st->evaluated += g[8 * s + 2]; st->solves += g[8 * s + 3]; }
    }
    st->samples = L->count;
    st->capacity = L->cap;
    st->loss = L->last_loss;
    return TB_OK;
}

// Loss and gradient of the network on n crops (n, 5, CW, CW) with their meta
// (n, 3) (image 2k + part, first row, first column), host weights, and the
// context's operator: the training kernels alone.
int tb_learn_grad(tb_ctx* c, const float* w, const float* crops, const int* meta, int n, double* loss, float* grad) {
    if (!c || !w || !crops || !meta || n < 1 || !loss || !grad) { tb_set_error("bad argument"); return TB_ERR_ARG; }
    int r = ensure(c);
    if (r) return r;
    Learn* L = get(c);
    FineOp F;
    if ((r = tb_mixed_fine_op(c, &F))) return r;
    for (int q = 0; q < n; q++)
        if (meta[3 * q] < 0 || meta[3 * q] >= 2 * c->g.K) { tb_set_error("crop %d: image out of range", q); return TB_ERR_ARG; }
    TrainBufs tb;
    float *dw = nullptr, *dg = nullptr, *ds = nullptr;
    int* dm = nullptr;
    r = tb.alloc(n);
    const size_t per = (size_t)PLANES * CW * CW;
    if (!r) r = dalloc(&dw, NPARAM);
    if (!r) r = dalloc(&dg, NPARAM);
    if (!r) r = dalloc(&ds, (size_t)n * per);
    if (!r) r = dalloc(&dm, (size_t)3 * n);
    if (!r) {
        std::vector<int> idx(n);
        for (int q = 0; q < n; q++) idx[q] = q;
        cudaError_t e = cudaMemcpy(dw, w, NPARAM * sizeof(float), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(ds, crops, (size_t)n * per * sizeof(float), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(tb.idx, idx.data(), n * sizeof(int), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(dm, meta, (size_t)3 * n * sizeof(int), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { tb_set_error("%s", cudaGetErrorString(e)); r = TB_ERR_CUDA; }
    }
    if (!r) {
        k_batch<<<tb_blocks((size_t)n * per, 256), 256>>>(ds, tb.idx, tb.X, tb.T, n, dw + OIS);
        r = forward(0, dw, tb.X, tb.out, tb.fwd(), n, CW, CW, false);
    }
    if (!r) {
        k_defect_loss<<<n, LT>>>(F, tb.X, dm, tb.out, tb.dout, tb.loss, L->s.invD, L->wmode, dw + OSC, dw + OIS + 2, n, 0);
        r = backward(0, dw, dg, tb.X, tb.fwd(), tb.dout, tb.dA, tb.dB, n);
    }
    if (!r) {
        cudaError_t e = cudaMemcpy(loss, tb.loss, sizeof(double), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(grad, dg, NPARAM * sizeof(float), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) { tb_set_error("%s", cudaGetErrorString(e)); r = TB_ERR_CUDA; }
    }
    tb.release();
    for (void* p : {(void*)dw, (void*)dg, (void*)ds, (void*)dm})
        if (p) cudaFree(p);
    return r;
}

// The operator tables of mode k as the loss uses them: den, ify, alpha2,
// k^2 beta^2, w_k, the 24 level coefficients, qdy2 (ny), 1/|D| (ny).
int tb_learn_op_tables(tb_ctx* c, int k, float* tab) {
    if (!c || !tab) { tb_set_error("null argument"); return TB_ERR_ARG; }
    int r = ensure(c);
    if (r) return r;
    if (k < 0 || k >= c->g.K) { tb_set_error("mode out of range"); return TB_ERR_ARG; }
    Learn* L = get(c);
    FineOp F;
    if ((r = tb_mixed_fine_op(c, &F))) return r;
    const int ny = c->g.ny;
    double k2 = 0.0;
    TB_CUDA(cudaStreamSynchronize(c->stream));
    TB_CUDA(cudaMemcpy(&k2, F.k2b2 + k, sizeof(double), cudaMemcpyDeviceToHost));
    tab[0] = F.den; tab[1] = F.ify; tab[2] = F.alpha2; tab[3] = (float)k2;
    TB_CUDA(cudaMemcpy(tab + 4, L->wmode + k, sizeof(float), cudaMemcpyDeviceToHost));
    TB_CUDA(cudaMemcpy(tab + 5, F.coef, 24 * sizeof(float), cudaMemcpyDeviceToHost));
    TB_CUDA(cudaMemcpy(tab + 29, F.qdy2, ny * sizeof(float), cudaMemcpyDeviceToHost));
    TB_CUDA(cudaMemcpy(tab + 29 + ny, L->s.invD + (size_t)k * ny, ny * sizeof(float), cudaMemcpyDeviceToHost));
    return TB_OK;
}

// -L e of mode k through the solver's own residual kernel (host (nx, ny)).
int tb_learn_op_apply(tb_ctx* c, int k, const float* e, float* out) {
    if (!c || !e || !out) { tb_set_error("null argument"); return TB_ERR_ARG; }
    return tb_mixed_resid_mode(c, k, e, out);
}

// The network on n images (n, 4, H, Wd) of host memory: out (n, H, Wd).
int tb_learn_forward(const float* w, const float* x, int n, int H, int Wd, float* out) {
    if (!w || !x || !out || n < 1 || H < 1 || Wd < 1) { tb_set_error("bad argument"); return TB_ERR_ARG; }
    const size_t img = (size_t)H * Wd;
    float *dw = nullptr, *dx = nullptr, *dout = nullptr, *a = nullptr, *b = nullptr;
    int r = dalloc(&dw, NPARAM);
    if (!r) r = dalloc(&dx, (size_t)n * LIN * img);
    if (!r) r = dalloc(&dout, (size_t)n * img);
    if (!r) r = dalloc(&a, (size_t)n * LC * img);
    if (!r) r = dalloc(&b, (size_t)n * LC * img);
    if (!r) {
        cudaError_t e = cudaMemcpy(dw, w, NPARAM * sizeof(float), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(dx, x, (size_t)n * LIN * img * sizeof(float), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { tb_set_error("%s", cudaGetErrorString(e)); r = TB_ERR_CUDA; }
    }
    if (!r) r = forward(0, dw, dx, dout, Fwd{nullptr, a, nullptr, b, nullptr, a}, n, H, Wd, true);
    if (!r) {
        cudaError_t e = cudaMemcpy(out, dout, (size_t)n * img * sizeof(float), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) { tb_set_error("%s", cudaGetErrorString(e)); r = TB_ERR_CUDA; }
    }
    for (void* p : {(void*)dw, (void*)dx, (void*)dout, (void*)a, (void*)b})
        if (p) cudaFree(p);
    return r;
}

}  // extern "C"
