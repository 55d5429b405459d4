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
// Network: four 3x3 convolutions with zero padding, 4 -> 32 -> 32 -> 32 -> 1
// channels, GELU after the first three.  Parameters: per layer the weights in
// [cout][cin][3][3] order, then the biases.  Per mode k and part (re, im) the
// inputs on the (nx, ny) fine grid (rows i, columns j) are
//   c0 = v1 / max|v1|, c1 = (v1 - v2) / max|v1 - v2|,
//   c2 = D^-1 d0 / max|D^-1 d0|, c3 = share of k^2 beta^2 in D
// (D: the diagonal of the fine y-line operator at row j; maxima per mode over
// both parts), and the output times max|v1 - v2| is the correction.
//
// Training: crops of CW x CW points (a CROP x CROP interior plus the
// network's 4-point reach) with the four input planes and the target
// (v(t) - guess) / max|v1 - v2|; mean squared error over the interiors;
// Adam.  Forward, backward-data and weight-gradient kernels are FP32 on the
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
              OB3 = OW3 + LC * LC * 9, OW4 = OB3 + LC, OB4 = OW4 + LC * 9, NPARAM = OB4 + 1;
constexpr int CT = 16;   // output tile edge of the convolution kernels

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float x) {
    return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// 3x3 convolution with zero padding over a batch (blockIdx.z) of H x Wd
// images, NCHW.  Forward (TRANS false): pre = W * in + bias and, when act is
// set, act = gelu(pre) (pre may then be null).  Backward data (TRANS true): W is the forward layer
// [CIN][COUT][3][3] (this kernel's CIN is the forward COUT) applied
// transposed and flipped, times gelu'(gpre) when gpre is set.
template <int CIN, int COUT, bool TRANS>
__global__ void __launch_bounds__(256) k_conv(const float* __restrict__ in, const float* __restrict__ W,
                                              const float* __restrict__ bias, float* __restrict__ pre,
                                              float* __restrict__ act, const float* __restrict__ gpre, int H, int Wd) {
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
            tile[q] = v;
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
#pragma unroll
    for (int o = 0; o < COUT; o++) {
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

// Mean squared error over the CROP x CROP interiors of a batch of CW x CW
// outputs; dout = 2 (out - target) / n there and 0 on the margins.
__global__ void k_mse(const float* __restrict__ out, const float* __restrict__ tgt, float* __restrict__ dout,
                      double* loss, int B) {
    const size_t n = (size_t)B * CW * CW;
    const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    float sq = 0.f;
    if (q < n) {
        const int pix = (int)(q % (CW * CW)), y = pix / CW, x = pix % CW;
        float g = 0.f;
        if (y >= HALO && y < HALO + CROP && x >= HALO && x < HALO + CROP) {
            const float d = out[q] - tgt[q];
            sq = d * d;
            g = 2.f * d / (float)((size_t)B * CROP * CROP);
        }
        dout[q] = g;
    }
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if (loss && (threadIdx.x & 31) == 0 && sq != 0.f) atomicAdd(loss, (double)sq / ((double)B * CROP * CROP));
}

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

// Batch of crops idx[b] of the sample buffer: input planes into X (B, 4, CW,
// CW), target plane into T (B, CW, CW).
__global__ void k_batch(const float* __restrict__ samples, const int* __restrict__ idx, float* __restrict__ X,
                        float* __restrict__ T, int B) {
    const size_t per = (size_t)PLANES * CW * CW;
    const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= (size_t)B * per) return;
    const int b = (int)(q / per), r = (int)(q % per), pl = r / (CW * CW), pix = r % (CW * CW);
    const float v = samples[(size_t)idx[b] * per + r];
    if (pl < LIN) X[((size_t)b * LIN + pl) * CW * CW + pix] = v;
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

struct Learn {
    LearnSolve s;
    float *w = nullptr, *gw = nullptr, *m = nullptr, *v = nullptr;
    long long adam_t = 0;
    float *P0 = nullptr, *P1 = nullptr;          // inference ping-pong (2K, LC, nx, ny)
    float* samples = nullptr;
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
// P* hold the pre-activations and A* the activations of layers 1-3 (each
// (B, LC, H, Wd)); inference passes null P* and alternates two A buffers.
struct Fwd { float *P1, *A1, *P2, *A2, *P3, *A3; };
int forward(cudaStream_t st, const float* w, const float* X, float* out, const Fwd& f, int B, int H, int Wd) {
    dim3 grid((Wd + CT - 1) / CT, (H + CT - 1) / CT, B);
    k_conv<LIN, LC, false><<<grid, 256, conv_smem<LIN, LC, false>(), st>>>(X, w + OW1, w + OB1, f.P1, f.A1, nullptr, H, Wd);
    k_conv<LC, LC, false><<<grid, 256, conv_smem<LC, LC, false>(), st>>>(f.A1, w + OW2, w + OB2, f.P2, f.A2, nullptr, H, Wd);
    k_conv<LC, LC, false><<<grid, 256, conv_smem<LC, LC, false>(), st>>>(f.A2, w + OW3, w + OB3, f.P3, f.A3, nullptr, H, Wd);
    k_conv<LC, 1, false><<<grid, 256, conv_smem<LC, 1, false>(), st>>>(f.A3, w + OW4, w + OB4, out, nullptr, nullptr, H, Wd);
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
    int* idx = nullptr;
    int alloc(int B) {
        const size_t img = (size_t)CW * CW, hid = (size_t)B * LC * img;
        int r;
        if ((r = dalloc(&X, (size_t)B * LIN * img)) || (r = dalloc(&T, (size_t)B * img)) || (r = dalloc(&out, (size_t)B * img)) ||
            (r = dalloc(&dout, (size_t)B * img)) || (r = dalloc(&dA, hid)) || (r = dalloc(&dB, hid)) ||
            (r = dalloc(&P1, hid)) || (r = dalloc(&A1, hid)) || (r = dalloc(&P2, hid)) || (r = dalloc(&A2, hid)) ||
            (r = dalloc(&P3, hid)) || (r = dalloc(&A3, hid)) || (r = dalloc(&loss, 1)) || (r = dalloc(&idx, (size_t)B)))
            return r;
        return TB_OK;
    }
    void release() {
        for (void* p : {(void*)X, (void*)T, (void*)out, (void*)dout, (void*)dA, (void*)dB, (void*)P1, (void*)A1, (void*)P2,
                        (void*)A2, (void*)P3, (void*)A3, (void*)loss, (void*)idx})
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
    if ((r = forward(c->stream, L->w, L->s.X, L->s.out, f, B, H, Wd))) return r;
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
    L->count += n;
    return TB_OK;
}

void tb_learn_free(tb_ctx* c) {
    Learn* L = get(c);
    if (!L) return;
    for (void* p : {(void*)L->w, (void*)L->gw, (void*)L->m, (void*)L->v, (void*)L->P0, (void*)L->P1, (void*)L->samples,
                    (void*)L->d_pos, (void*)L->s.X, (void*)L->s.out, (void*)L->s.scl, (void*)L->s.jmax, (void*)L->s.invD,
                    (void*)L->s.mfeat, (void*)L->s.g0, (void*)L->s.tally})
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
    if (!c->cfg.warm_start) { tb_set_error("the learned correction needs warm_start = 1"); return TB_ERR_STATE; }
    Learn* L = get(c);
    if (on) {
        const size_t hid = (size_t)2 * c->g.K * LC * c->g.nx * c->g.ny;
        if ((r = dalloc(&L->P0, hid)) || (r = dalloc(&L->P1, hid))) return r;
    }
    TB_CUDA(cudaStreamSynchronize(c->stream));
    L->s.infer = on != 0;
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
    if (!c->cfg.warm_start) { tb_set_error("sampling needs warm_start = 1"); return TB_ERR_STATE; }
    if (crops_per_solve < 1) { tb_set_error("crops_per_solve must be >= 1"); return TB_ERR_ARG; }
    if (L->samples) cudaFree(L->samples);
    L->samples = nullptr;
    TB_CUDA(cudaMalloc(&L->samples, (size_t)capacity * PLANES * CW * CW * sizeof(float)));
    if ((r = dalloc(&L->s.g0, (size_t)c->g.K * c->g.lvl_elems))) return r;
    L->cap = capacity;
    L->count = 0;
    L->per_solve = crops_per_solve;
    L->rng.seed(seed);
    L->s.sample = true;
    return TB_OK;
}

int tb_learn_train(tb_ctx* c, int iters, int batch, float lr, unsigned long long seed, double* loss) {
    if (!c) { tb_set_error("null context"); return TB_ERR_ARG; }
    int r = ensure(c);
    if (r) return r;
    Learn* L = get(c);
    if (L->count < 1) { tb_set_error("no training crops (tb_learn_sample, then steps)"); return TB_ERR_STATE; }
    if (iters < 1 || batch < 1 || !(lr > 0.f)) { tb_set_error("iters, batch and lr must be positive"); return TB_ERR_ARG; }
    TrainBufs tb;
    if ((r = tb.alloc(batch))) { tb.release(); return r; }
    cudaStream_t st = c->stream;
    std::mt19937_64 g(seed);
    std::uniform_int_distribution<long long> pick(0, L->count - 1);
    std::vector<int> idx(batch);
    double acc = 0.0;
    int nacc = 0;
    const int tail = std::max(1, iters / 10);
    TB_CUDA(cudaMemsetAsync(tb.loss, 0, sizeof(double), st));
    for (int it = 0; it < iters && !r; it++) {
        for (int b = 0; b < batch; b++) idx[b] = (int)pick(g);
        TB_CUDA(cudaMemcpyAsync(tb.idx, idx.data(), batch * sizeof(int), cudaMemcpyHostToDevice, st));
        k_batch<<<tb_blocks((size_t)batch * PLANES * CW * CW, 256), 256, 0, st>>>(L->samples, tb.idx, tb.X, tb.T, batch);
        if ((r = forward(st, L->w, tb.X, tb.out, tb.fwd(), batch, CW, CW))) break;
        const bool rec = it >= iters - tail;
        if (rec) {
            k_mse<<<tb_blocks((size_t)batch * CW * CW, 256), 256, 0, st>>>(tb.out, tb.T, tb.dout, tb.loss, batch);
            nacc++;
        } else {
            k_mse<<<tb_blocks((size_t)batch * CW * CW, 256), 256, 0, st>>>(tb.out, tb.T, tb.dout, nullptr, batch);
        }
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
    st->samples = L->count;
    st->capacity = L->cap;
    st->loss = L->last_loss;
    return TB_OK;
}

// Loss and gradient of the network on n crops (n, 5, CW, CW) of host memory,
// with host weights, on the current device: the training kernels alone.
int tb_learn_grad(const float* w, const float* crops, int n, double* loss, float* grad) {
    if (!w || !crops || n < 1 || !loss || !grad) { tb_set_error("bad argument"); return TB_ERR_ARG; }
    TrainBufs tb;
    float *dw = nullptr, *dg = nullptr, *ds = nullptr;
    int r = tb.alloc(n);
    const size_t per = (size_t)PLANES * CW * CW;
    if (!r) r = dalloc(&dw, NPARAM);
    if (!r) r = dalloc(&dg, NPARAM);
    if (!r) r = dalloc(&ds, (size_t)n * per);
    if (!r) {
        std::vector<int> idx(n);
        for (int q = 0; q < n; q++) idx[q] = q;
        cudaError_t e = cudaMemcpy(dw, w, NPARAM * sizeof(float), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(ds, crops, (size_t)n * per * sizeof(float), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(tb.idx, idx.data(), n * sizeof(int), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { tb_set_error("%s", cudaGetErrorString(e)); r = TB_ERR_CUDA; }
    }
    if (!r) {
        k_batch<<<tb_blocks((size_t)n * per, 256), 256>>>(ds, tb.idx, tb.X, tb.T, n);
        r = forward(0, dw, tb.X, tb.out, tb.fwd(), n, CW, CW);
    }
    if (!r) {
        k_mse<<<tb_blocks((size_t)n * CW * CW, 256), 256>>>(tb.out, tb.T, tb.dout, tb.loss, n);
        r = backward(0, dw, dg, tb.X, tb.fwd(), tb.dout, tb.dA, tb.dB, n);
    }
    if (!r) {
        cudaError_t e = cudaMemcpy(loss, tb.loss, sizeof(double), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(grad, dg, NPARAM * sizeof(float), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) { tb_set_error("%s", cudaGetErrorString(e)); r = TB_ERR_CUDA; }
    }
    tb.release();
    for (void* p : {(void*)dw, (void*)dg, (void*)ds})
        if (p) cudaFree(p);
    return r;
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
    if (!r) r = forward(0, dw, dx, dout, Fwd{nullptr, a, nullptr, b, nullptr, a}, n, H, Wd);
    if (!r) {
        cudaError_t e = cudaMemcpy(out, dout, (size_t)n * img * sizeof(float), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) { tb_set_error("%s", cudaGetErrorString(e)); r = TB_ERR_CUDA; }
    }
    for (void* p : {(void*)dw, (void*)dx, (void*)dout, (void*)a, (void*)b})
        if (p) cudaFree(p);
    return r;
}

}  // extern "C"
