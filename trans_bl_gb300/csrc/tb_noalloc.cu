// tb_noalloc.cu -- compact x-filter (filter_trid) on caller device buffers
// without any device allocation.
//
// Some hosts cannot call cudaMalloc once their time loop runs: a Fortran
// driver whose memory manager hands every free byte of the GPU to its own
// pool at start-up, or a real-time section where a device allocation (which
// may synchronise the whole device) is not allowed.  tb_filter_trid_noalloc
// serves them: the filtered lines are staged in a fixed scratch array that
// lives in the library's own device image instead of a per-context
// allocation.
//
//  - Scratch: 2^21 complex*16 elements (32 MiB), a file-scope __device__
//    array; one call filters at most nx*ny*kfour = 2^21 - 4096 points with
//    nx <= 4096 (larger grids: call once per slice of Fourier modes, which the
//    filter treats independently).  Every GPU that loads this library keeps
//    the array resident until the process exits.
//  - The first call on a device (with that device current) looks up the
//    array's device address with cudaGetSymbolAddress and keeps it for the
//    device; make that first call before any stream capture.  The kept
//    address belongs to the device's primary context: after cudaDeviceReset
//    of that device it is stale, so a process that resets a device must not
//    call this entry point on it again.
//  - All calls share the one array: calls that overlap on the GPU (two
//    streams, or two host threads) race on it.  Every element the kernels read
//    is written earlier in the same call, so nothing needs clearing.
#include "tb_internal.h"
#include <atomic>

#define TB_NOALLOC_FILTER_MAX (1u << 21)      // complex*16 elements in the scratch (32 MiB)
#define TB_NOALLOC_PIVOTS 4096                 // the last elements hold the Thomas pivots (nx <= 4096)
#define TB_NOALLOC_FIELD_MAX (TB_NOALLOC_FILTER_MAX - TB_NOALLOC_PIVOTS)

static __device__ __align__(256) double2 g_filter_scratch[TB_NOALLOC_FILTER_MAX];

namespace {

// Device address of the scratch per device ordinal, set by the first call on
// that device (concurrent first calls store the same value).
std::atomic<double2*> g_scratch_addr[64];

// Forward Thomas sweep of the filter LHS built on the fly (lhs_tridf
// filter_par.f:181, quotient sequence of tridseqx derivs_par.f:1009), one
// thread per x-line; the line of the first thread also records the pivots
// gam_i (data independent) for the backward sweep.
__global__ void k_filter_fwd(const double2* __restrict__ w, double2* __restrict__ s, double2* __restrict__ piv, int nx,
                             int nlines, double alphaf, double af, double bf, double cf, double df) {
    int line = blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= nlines) return;
    const double2* f = w + (size_t)line * nx;
    double2* o = s + (size_t)line * nx;
    auto lhs_a = [&](int i) { return (i >= 3 && i <= nx - 4) ? alphaf : 0.0; };
    auto rhs = [&](int i) -> double2 {
        if (i >= 3 && i <= nx - 4) {
            double2 a = f[i], b1 = f[i + 1], b2 = f[i - 1], c1 = f[i + 2], c2 = f[i - 2], d1 = f[i + 3], d2 = f[i - 3];
            return make_double2(af * a.x + bf * (b1.x + b2.x) + cf * (c1.x + c2.x) + df * (d1.x + d2.x),
                                af * a.y + bf * (b1.y + b2.y) + cf * (c1.y + c2.y) + df * (d1.y + d2.y));
        }
        const double wt[3][5] = {{15, 4, -6, 4, -1}, {1, 12, 6, -4, 1}, {-1, 4, 10, 4, -1}};
        int b = (i < 3) ? 0 : nx - 1, e = (i < 3) ? 1 : -1, r = (i < 3) ? i : nx - 1 - i;
        double2 acc = make_double2(0.0, 0.0);
        for (int q = 0; q < 5; q++) { double2 v = f[b + q * e]; acc.x += wt[r][q] * v.x; acc.y += wt[r][q] * v.y; }
        return make_double2(acc.x / 16.0, acc.y / 16.0);
    };
    double bet = 1.0;
    double2 u = rhs(0);
    o[0] = u;
    if (line == 0) piv[0] = make_double2(0.0, 0.0);
    for (int i = 1; i < nx; i++) {
        double a = lhs_a(i);
        double gam = lhs_a(i - 1) / bet;
        bet = 1.0 - a * gam;
        double2 r = rhs(i);
        u = make_double2((r.x - a * u.x) / bet, (r.y - a * u.y) / bet);
        o[i] = u;
        if (line == 0) piv[i] = make_double2(gam, 0.0);
    }
}

// Backward sweep u_i -= gam_{i+1} u_{i+1} on the scratch lines.
__global__ void k_filter_bwd(double2* __restrict__ s, const double2* __restrict__ piv, int nx, int nlines) {
    int line = blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= nlines) return;
    double2* o = s + (size_t)line * nx;
    double2 u = o[nx - 1];
    for (int i = nx - 2; i >= 0; i--) {
        double g = piv[i + 1].x;
        double2 v = o[i];
        u = make_double2(v.x - g * u.x, v.y - g * u.y);
        o[i] = u;
    }
}

__global__ void k_filter_copy_back(double2* w, const double2* s, int nx, int ny, int K) {
    size_t n = (size_t)nx * ny * K;
    size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    int i = (int)(q % nx), j = (int)((q / nx) % ny);
    if (i < 1 || j < 1) return;   // filter_trid copies back i >= 2, j >= 2 (filter_par.f:166-174)
    w[q] = s[q];
}

int scratch_address(double2** out) {
    int dev = 0;
    TB_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) { tb_set_error("device ordinal %d out of range", dev); return TB_ERR_ARG; }
    double2* a = g_scratch_addr[dev].load(std::memory_order_acquire);
    if (!a) {
        void* p = nullptr;
        TB_CUDA(cudaGetSymbolAddress(&p, g_filter_scratch));
        a = static_cast<double2*>(p);
        g_scratch_addr[dev].store(a, std::memory_order_release);
    }
    *out = a;
    return TB_OK;
}

}  // namespace

extern "C" int tb_filter_trid_noalloc(double* wx, double* wy, double* wz, int nx, int ny, int kfour, double alphaf,
                                      void* stream) {
    if (!wx || !wy || !wz) { tb_set_error("tb_filter_trid_noalloc: null field pointer"); return TB_ERR_ARG; }
    if (nx < 8 || nx > TB_NOALLOC_PIVOTS || ny < 2 || kfour < 1) {
        tb_set_error("tb_filter_trid_noalloc: need 8 <= nx <= %d, ny >= 2, kfour >= 1", TB_NOALLOC_PIVOTS);
        return TB_ERR_ARG;
    }
    size_t n3 = (size_t)nx * ny * kfour;
    if (n3 > TB_NOALLOC_FIELD_MAX) {
        tb_set_error("tb_filter_trid_noalloc: nx*ny*kfour = %zu exceeds the %u-element scratch (32 MiB); "
                     "filter fewer Fourier modes per call", n3, (unsigned)TB_NOALLOC_FIELD_MAX);
        return TB_ERR_ARG;
    }
    double2* s = nullptr;
    int r = scratch_address(&s);
    if (r) return r;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double af = (11.0 + 10.0 * alphaf) / 16.0, bf = (15.0 + 34.0 * alphaf) / 64.0;
    double cf = (-3.0 + 6.0 * alphaf) / 32.0, df = (1.0 - 2.0 * alphaf) / 64.0;
    int nlines = ny * kfour;
    double* fields[3] = {wx, wy, wz};
    for (double* f : fields) {
        double2* w = reinterpret_cast<double2*>(f);
        double2* piv = s + TB_NOALLOC_FIELD_MAX;
        k_filter_fwd<<<tb_blocks(nlines, 128), 128, 0, st>>>(w, s, piv, nx, nlines, alphaf, af, bf, cf, df);
        TB_CUDA(cudaGetLastError());
        k_filter_bwd<<<tb_blocks(nlines, 128), 128, 0, st>>>(s, piv, nx, nlines);
        TB_CUDA(cudaGetLastError());
        k_filter_copy_back<<<tb_blocks(n3, 256), 256, 0, st>>>(w, s, nx, ny, kfour);
        TB_CUDA(cudaGetLastError());
    }
    return TB_OK;
}
