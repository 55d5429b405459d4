// tb_poisson.cu -- the pieces of poi_uy (poisson_par.f:6-164) that the mixed
// form shares: the source and start state (function_source) in the complex
// x-contiguous work arrays, the fine-level FP64 defect of the correction
// equation, the write-back of fc into uy, and the set-up of the y-line band
// LU factors with their chunk tables (band5_poi, penta_par.f:308-364) used by
// both forms.  The plain FP64 form's V-cycle is in tb_plain.cu.
#include "tb_internal.h"
#include <cmath>
#include <cstring>
#include <algorithm>



namespace {

struct PoiDev {
    cplx *fc, *sc, *fct, *def;    // per-mode blocks
    const double* coef;           // sp(7) cp(8) pp(4) lp(5) per level
    const double* qdy2;           // (ny, msh)
    const double* k2b2;
    int* state;                   // per mode: [2k] active, [2k+1] vcycles done
    double* err;
    int nx, ny, K, msh;
    int ptsx[TB_MAX_MSH], ptsy[TB_MAX_MSH];
    size_t off[TB_MAX_MSH], elems, dstride;
    double dx2[TB_MAX_MSH];
    double den[TB_MAX_MSH];       // 1 / (12 dx2 fac_y)
    double fac_y, alpha, ify;
};

__device__ __forceinline__ cplx& AT(cplx* base, const PoiDev& P, int k, int l, int i, int j) {
    return base[(size_t)k * P.elems + P.off[l] + (size_t)i + (size_t)P.ptsx[l] * j];
}

// ---------------------------------------------------------------------------
// function_source (poisson_par.f:111-164) for all modes.
__global__ void k_source(PoiDev P, const cplx* wx, const cplx* dwzdx, const cplx* uy, const double* duexmdx,
                         const double* uyb, double beta, double dy, double stf_pow, int form) {
    size_t n = (size_t)P.nx * P.ny * P.K;
    size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    int i = (int)(q % P.nx), j = (int)((q / P.nx) % P.ny), k = (int)(q / ((size_t)P.nx * P.ny));
    const double* c0 = P.coef;  // level 1
    double kb = (double)k * beta;
    int J = P.ny;
    auto S = [&](int jj) {
        size_t o = (size_t)i + (size_t)P.nx * (jj + (size_t)J * k);
        cplx w = wx[o], d = dwzdx[o];
        return make_double2(kb * w.y - d.x, -kb * w.x - d.y);
    };
    cplx s;
    if (j == 0) s = make_double2(0, 0);
    else if (j == 1) { cplx a = S(1), b = S(2); s = make_double2(c0[1] * a.x + c0[2] * b.x, c0[1] * a.y + c0[2] * b.y); }
    else if (j <= J - 3) {
        cplx a = S(j - 1), b = S(j), d = S(j + 1);
        s = make_double2(c0[7] * a.x + c0[8] * b.x + c0[9] * d.x, c0[7] * a.y + c0[8] * b.y + c0[9] * d.y);
    } else if (j == J - 2) s = S(J - 2);
    else {
        s = make_double2(0, 0);
        if ((form == 0 || form == 4) && k == 0) {
            double dya = dy * stf_pow;
            size_t o = (size_t)i + (size_t)P.nx * (J - 1);
            double lp1 = c0[19], lp2 = c0[20];
            s = make_double2(-(lp1 * dwzdx[o].x) + lp2 * duexmdx[i] / dya - lp2 * P.alpha * uyb[o] / dya / sqrt(P.fac_y),
                             -(lp1 * dwzdx[o].y));
        }
    }
    AT(P.sc, P, k, 0, i, j) = s;
    AT(P.fc, P, k, 0, i, j) = uy[q];
}

// ---------------------------------------------------------------------------
// The level-l operator of defect (poisson_par.f:543-793) applied to fc at the
// interior point (i, j) of mode k: L fc = den*Dxx + q2*Dyy + k2b2*ify*M - top.
// The x-stencil sum of row jj (rhs_center / rhs_border incl. the diagonal):
__device__ __forceinline__ cplx poi_bx(const PoiDev& P, int l, int k, int i, int jj) {
    const int nxl = P.ptsx[l];
    const cplx* F = P.fc + (size_t)k * P.elems + P.off[l] + (size_t)nxl * jj;
    if (i == 1 || i == nxl - 2) {
        int e = (i == 1) ? 1 : -1;
        cplx a = F[i - e], c0 = F[i], b = F[i + e], c = F[i + 2 * e], d = F[i + 3 * e], g = F[i + 4 * e];
        return make_double2(10.0 * a.x - 15.0 * c0.x - 4.0 * b.x + 14.0 * c.x - 6.0 * d.x + g.x,
                            10.0 * a.y - 15.0 * c0.y - 4.0 * b.y + 14.0 * c.y - 6.0 * d.y + g.y);
    }
    cplx a = F[i - 2], b = F[i - 1], c0 = F[i], c = F[i + 1], d = F[i + 2];
    return make_double2(-a.x + 16.0 * b.x - 30.0 * c0.x + 16.0 * c.x - d.x, -a.y + 16.0 * b.y - 30.0 * c0.y + 16.0 * c.y - d.y);
}

// L fc at (i, j) with the x-stencil sums supplied by bx(jj).
template <class BX>
__device__ __forceinline__ cplx poi_Lu_b(const PoiDev& P, int l, int k, int i, int j, BX bx) {
    const int nxl = P.ptsx[l], n = P.ptsy[l];
    const double* cf = P.coef + 24 * l;
    const double *SPc = cf, *CPc = cf + 7, *PPc = cf + 15, *LPc = cf + 19;
    double k2b2 = P.k2b2[k];
    double den = P.den[l], ify = P.ify;
    const cplx* F = P.fc + (size_t)k * P.elems + P.off[l];
    auto f = [&](int ii, int jj) -> cplx { return F[(size_t)ii + (size_t)nxl * jj]; };
    cplx b, cc, d;
    double q2;
    double top = 0.0;
    if (j == 1) {
        cplx b1 = bx(1), b2 = bx(2);
        b = make_double2(SPc[2] * b2.x + SPc[1] * b1.x, SPc[2] * b2.y + SPc[1] * b1.y);
        cplx f0 = f(i, 0), f1 = f(i, 1), f2 = f(i, 2), f3 = f(i, 3);
        cc = make_double2(SPc[3] * f0.x + SPc[4] * f1.x + SPc[5] * f2.x + SPc[6] * f3.x,
                          SPc[3] * f0.y + SPc[4] * f1.y + SPc[5] * f2.y + SPc[6] * f3.y);
        d = make_double2(k2b2 * (SPc[1] * f1.x + SPc[2] * f2.x), k2b2 * (SPc[1] * f1.y + SPc[2] * f2.y));
        q2 = P.qdy2[0 + (size_t)P.ny * l];
    } else if (j <= n - 3) {
        cplx ba = bx(j - 1), bb = bx(j), bc = bx(j + 1);
        b = make_double2(CPc[0] * ba.x + CPc[1] * bb.x + CPc[2] * bc.x, CPc[0] * ba.y + CPc[1] * bb.y + CPc[2] * bc.y);
        cplx fm2 = f(i, j - 2), fm1 = f(i, j - 1), f0 = f(i, j), fp1 = f(i, j + 1), fp2 = f(i, j + 2);
        cc = make_double2(CPc[3] * fm2.x + CPc[4] * fm1.x + CPc[5] * f0.x + CPc[6] * fp1.x + CPc[7] * fp2.x,
                          CPc[3] * fm2.y + CPc[4] * fm1.y + CPc[5] * f0.y + CPc[6] * fp1.y + CPc[7] * fp2.y);
        d = make_double2(k2b2 * (CPc[0] * fm1.x + CPc[1] * f0.x + CPc[2] * fp1.x), k2b2 * (CPc[0] * fm1.y + CPc[1] * f0.y + CPc[2] * fp1.y));
        q2 = P.qdy2[(j - 2) + (size_t)P.ny * l];
    } else if (j == n - 2) {
        b = bx(j);
        cplx fm1 = f(i, j - 1), f0 = f(i, j), fp1 = f(i, j + 1);
        cc = make_double2(PPc[3] * fp1.x + PPc[2] * f0.x + PPc[1] * fm1.x, PPc[3] * fp1.y + PPc[2] * f0.y + PPc[1] * fm1.y);
        d = make_double2(k2b2 * f0.x, k2b2 * f0.y);
        q2 = P.qdy2[(j - 1) + (size_t)P.ny * l];
    } else {
        b = bx(j);
        cplx fm2 = f(i, j - 2), fm1 = f(i, j - 1), f0 = f(i, j);
        cc = make_double2(LPc[2] * f0.x + LPc[3] * fm1.x + LPc[4] * fm2.x, LPc[2] * f0.y + LPc[3] * fm1.y + LPc[4] * fm2.y);
        d = make_double2(k2b2 * f0.x, k2b2 * f0.y);
        q2 = P.qdy2[(j - 2) + (size_t)P.ny * l];
        double alpha2 = sqrt((P.alpha * P.alpha - k2b2) / P.fac_y);
        top = LPc[1] * alpha2 * sqrt(q2);
    }
    cplx fij = f(i, j);
    return make_double2(b.x * den + cc.x * q2 + d.x * ify - top * fij.x, b.y * den + cc.y * q2 + d.y * ify - top * fij.y);
}

// Fine-level FP64 defect d = sc - L fc for the mixed form: stored as FP32 in
// the line-contiguous right-hand side r32 of the correction equation (element
// (i, j) of mode k at k*elems32 + i*ny + j, through a 32x32 shared tile), the
// correction e32 zeroed at the same points, and max |d|^2 of each mode
// folded into maxsq[k] (bit pattern of a non-negative double; a non-finite
// defect records +inf).
__global__ void k_defect_f32(PoiDev P, float2* r32, float2* e32, size_t elems32, unsigned long long* maxsq) {
    __shared__ float2 tile[32][33];
    __shared__ cplx bxs[34][32];   // x-stencil sums of rows j0-1 .. j0+32, computed once
    __shared__ double wmax[8];
    const int k = blockIdx.z;
    if (!P.state[2 * k]) return;   // uniform over the block
    const int nx = P.nx, ny = P.ny;
    const int i0 = 1 + blockIdx.x * 32, j0 = 1 + blockIdx.y * 32;
    {
        const int i = i0 + threadIdx.x;
        for (int r = threadIdx.y; r < 34; r += 8) {
            int jj = j0 - 1 + r;
            bxs[r][threadIdx.x] = (i <= nx - 2 && jj >= 1 && jj <= ny - 1) ? poi_bx(P, 0, k, i, jj) : make_double2(0.0, 0.0);
        }
    }
    __syncthreads();
    double m = 0.0;
    bool bad = false;
    for (int r = threadIdx.y; r < 32; r += 8) {
        int i = i0 + threadIdx.x, j = j0 + r;
        float2 v32 = make_float2(0.f, 0.f);
        if (i <= nx - 2 && j <= ny - 1) {
            cplx s = P.sc[(size_t)k * P.elems + (size_t)i + (size_t)nx * j];
            cplx Lu = poi_Lu_b(P, 0, k, i, j, [&](int jj) { return bxs[jj - j0 + 1][threadIdx.x]; });
            cplx v = make_double2(s.x - Lu.x, s.y - Lu.y);
            double a = v.x * v.x + v.y * v.y;
            if (!(a <= 1.7e308)) bad = true;
            else m = fmax(m, a);
            v32 = make_float2((float)v.x, (float)v.y);
        }
        tile[r][threadIdx.x] = v32;
    }
    if (bad) m = __longlong_as_double(0x7ff0000000000000LL);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    const int w = (threadIdx.y * 32 + threadIdx.x) >> 5;
    if ((threadIdx.x & 31) == 0) wmax[w] = m;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        double b = wmax[0];
        for (int q = 1; q < 8; q++) b = fmax(b, wmax[q]);
        atomicMax(&maxsq[k], (unsigned long long)__double_as_longlong(b));
    }
    for (int r = threadIdx.y; r < 32; r += 8) {
        int i = i0 + r, j = j0 + threadIdx.x;
        if (i <= nx - 2 && j <= ny - 1) {
            size_t o = (size_t)k * elems32 + (size_t)ny * i + j;
            r32[o] = tile[threadIdx.x][r];
            e32[o] = make_float2(0.f, 0.f);
        }
    }
}

// uy(i,j,k) = fc(i,j,1) for j >= 2, 2 <= i <= ptsx-1 (poisson_par.f:53-57).
__global__ void k_write_uy(PoiDev P, cplx* uy) {
    size_t n = (size_t)P.nx * P.ny * P.K;
    size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    int i = (int)(q % P.nx), j = (int)((q / P.nx) % P.ny), k = (int)(q / ((size_t)P.nx * P.ny));
    if (j < 1 || i < 1 || i > P.nx - 2) return;
    uy[q] = AT(P.fc, P, k, 0, i, j);
}

__global__ void k_activate(int* state, int K) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < K) { state[2 * k] = 1; state[2 * k + 1] = 0; }
}

PoiDev make_dev(tb_ctx* c) {
    PoiDev P;
    std::memset(&P, 0, sizeof P);
    P.fc = c->pfc; P.sc = c->psc; P.fct = c->pfct; P.def = c->pdef; P.coef = c->pcoef;
    P.qdy2 = c->pqdy2; P.k2b2 = c->k2b2; P.state = c->pstate; P.err = c->perr;
    P.nx = c->g.nx; P.ny = c->g.ny; P.K = c->g.K; P.msh = c->g.msh;
    for (int l = 0; l < c->g.msh; l++) {
        P.ptsx[l] = c->g.ptsx[l]; P.ptsy[l] = c->g.ptsy[l]; P.off[l] = c->g.lvl_off[l]; P.dx2[l] = c->h_dx2[l];
        P.den[l] = 1.0 / (12.0 * c->h_dx2[l] * c->cfg.fac_y);
    }
    P.ify = 1.0 / c->cfg.fac_y;
    P.elems = c->g.lvl_elems; P.dstride = (size_t)c->g.nx * c->g.ny;
    P.fac_y = c->cfg.fac_y; P.alpha = c->cfg.alpha;
    return P;
}

}  // namespace

// Host: chunk tables of the line solve for one (type, level, mode), lane
// chunks of S rows (lane t owns rows [tS, min(n, tS + S))).
void tb_chunk_tables(int n, int ny, int S, const double* L1, const double* L2, const double* U1, const double* U2,
                     const double* ID, double* out) {
    double *h1 = out, *h2 = out + ny, *k1 = out + 2 * ny, *k2 = out + 3 * ny;
    double* Pf = out + 4 * ny;
    double* Pb = Pf + 640;
    double Mf[32][4], Mb[32][4];
    for (int t = 0; t < 32; t++) {
        int r0 = t * S, r1 = std::min(n, r0 + S);
        // forward: responses to incoming (Y1 = y_{r0-1}, Y2 = y_{r0-2})
        double e0[2], e1[2];   // outgoing (y_{e}, y_{e-1}) for unit incoming
        for (int u = 0; u < 2; u++) {
            double ym1 = (u == 0) ? 1.0 : 0.0, ym2 = (u == 0) ? 0.0 : 1.0;
            for (int j = r0; j < r1; j++) {
                double y = -L2[j] * ym2 - L1[j] * ym1;
                (u == 0 ? h1 : h2)[j] = y;
                ym2 = ym1; ym1 = y;
            }
            e0[u] = ym1; e1[u] = ym2;  // for an empty chunk this is the identity
        }
        Mf[t][0] = e0[0]; Mf[t][1] = e0[1]; Mf[t][2] = e1[0]; Mf[t][3] = e1[1];
        // backward: responses to incoming (X1 = x_{r1}, X2 = x_{r1+1})
        for (int u = 0; u < 2; u++) {
            double xp1 = (u == 0) ? 1.0 : 0.0, xp2 = (u == 0) ? 0.0 : 1.0;
            for (int j = r1 - 1; j >= r0; j--) {
                double x = (-U1[j] * xp1 - U2[j] * xp2) * ID[j];
                (u == 0 ? k1 : k2)[j] = x;
                xp2 = xp1; xp1 = x;
            }
            e0[u] = xp1; e1[u] = xp2;
        }
        Mb[t][0] = e0[0]; Mb[t][1] = e0[1]; Mb[t][2] = e1[0]; Mb[t][3] = e1[1];
    }
    // Kogge-Stone: A_t before each step; b_t += A_t b_{t-off}; A_t = A_t A_{t-off}
    auto mul = [](const double* A, const double* B, double* C) {
        double c0 = A[0] * B[0] + A[1] * B[2], c1 = A[0] * B[1] + A[1] * B[3];
        double c2 = A[2] * B[0] + A[3] * B[2], c3 = A[2] * B[1] + A[3] * B[3];
        C[0] = c0; C[1] = c1; C[2] = c2; C[3] = c3;
    };
    double Af[32][4], Ab[32][4];
    std::memcpy(Af, Mf, sizeof Af);
    std::memcpy(Ab, Mb, sizeof Ab);
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
}


int tb_poisson_setup(tb_ctx* c) {
    int ny = c->g.ny, K = c->g.K;
    size_t w = (size_t)K * c->g.lvl_elems;
    for (cplx** p : {&c->pfc, &c->psc, &c->pfct}) {
        if (*p) cudaFree(*p);
        TB_CUDA(cudaMalloc(p, w * sizeof(cplx)));
        TB_CUDA(cudaMemset(*p, 0, w * sizeof(cplx)));
    }
    if (c->pdef) cudaFree(c->pdef);
    TB_CUDA(cudaMalloc(&c->pdef, (size_t)K * c->g.nx * ny * sizeof(cplx)));
    TB_CUDA(cudaMemset(c->pdef, 0, (size_t)K * c->g.nx * ny * sizeof(cplx)));
    if (!c->pstate) TB_CUDA(cudaMalloc(&c->pstate, 2 * K * sizeof(int)));
    if (!c->perr) TB_CUDA(cudaMalloc(&c->perr, K * sizeof(double)));
    return TB_OK;
}

// Pieces of poi_uy shared with the mixed form: the source and the start
// state (fc = uy, every mode active) and the write-back of fc into uy.
int tb_poisson_begin(tb_ctx* c, const cplx* dwzdx) {
    PoiDev P = make_dev(c);
    double stf_pow = tb_powi(c->cfg.stf, c->g.ny - 3);
    k_source<<<tb_blocks(tb_n3(c), 256), 256, 0, c->stream>>>(P, c->wx, dwzdx, c->uy, c->duexmdx, c->uyb, c->cfg.beta,
                                                               c->cfg.dy, stf_pow, c->cfg.my_form);
    TB_CHECK_LAUNCH(c);
    k_activate<<<tb_blocks(c->g.K, 64), 64, 0, c->stream>>>(c->pstate, c->g.K);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}

int tb_poisson_end(tb_ctx* c) {
    PoiDev P = make_dev(c);
    k_write_uy<<<tb_blocks(tb_n3(c), 256), 256, 0, c->stream>>>(P, c->uy);
    TB_CHECK_LAUNCH(c);
    return TB_OK;
}

int tb_poisson_defect_f32(tb_ctx* c, float2* r32, float2* e32, size_t elems32, unsigned long long* maxsq) {
    PoiDev P = make_dev(c);
    dim3 grid(tb_blocks(c->g.nx - 2, 32), tb_blocks(c->g.ny - 1, 32), c->g.K), blk(32, 8);
    cudaEvent_t ps = nullptr;
    if (tb_prof_begin(c, PROF_DEFECT, &ps)) return TB_ERR_CUDA;
    k_defect_f32<<<grid, blk, 0, c->stream>>>(P, r32, e32, elems32, maxsq);
    TB_CHECK_LAUNCH(c);
    return tb_prof_end(c, PROF_DEFECT, ps);
}
