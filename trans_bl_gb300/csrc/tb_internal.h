// tb_internal.h -- shared definitions of the GB300 trans_bl stage library.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>
#include "../../include/transbl.h"

#define TB_MAX_MSH 6
#define TB_MAX_K 256

typedef double2 cplx;  // complex*16 as (re, im)

// Error plumbing ------------------------------------------------------------
void tb_set_error(const char* fmt, ...);
#define TB_CUDA(call)                                                                      \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            tb_set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return TB_ERR_CUDA;                                                            \
        }                                                                                  \
    } while (0)
#define TB_CHECK_LAUNCH(ctx)                                                               \
    do {                                                                                   \
        cudaError_t e_ = cudaGetLastError();                                               \
        if (e_ != cudaSuccess) {                                                           \
            tb_set_error("%s:%d kernel launch: %s", __FILE__, __LINE__, cudaGetErrorString(e_)); \
            return TB_ERR_CUDA;                                                            \
        }                                                                                  \
        (ctx)->launches++;                                                                 \
    } while (0)

// Device-side line operator tables ----------------------------------------
// Thomas factors of a constant tridiagonal LHS: forward u_i = (r_i - a_i u_{i-1}) * ib_i,
// backward u_i -= g_{i+1} u_{i+1}  (tridparx/tridy, derivs_par.f:775-975).
struct TriLHS {
    double* a;   // (n)
    double* g;   // (n) gam
    double* ib;  // (n) 1/bet
    // Chunked form for one warp per line (x-lines): lane t owns rows
    // [tS, min(n, tS + S)).  hf_i = d u_i / d u_{tS-1} of the forward sweep,
    // hb_i = d x_i / d x_{tS+S} of the backward sweep, and the Kogge-Stone
    // step factors pf[d][t], pb[d][t] of the chunk-end (start) responses.
    double* hf = nullptr;   // (n)
    double* hb = nullptr;   // (n)
    double* pf = nullptr;   // (5, 32)
    double* pb = nullptr;   // (5, 32)
    int S = 0;
    // FP32 copies of the chunked form (lines of the mixed form's modes k >= 1)
    float *af = nullptr, *gf = nullptr, *ibf = nullptr, *hff = nullptr, *hbf = nullptr, *pff = nullptr, *pbf = nullptr;
};
// Row weights of the stretched-y compact RHS: row j (0-based) is
// sum_m w[7*j+m] * f[j + off[j] + m], m < cnt[j].
struct YRhs {
    double* w;   // (ny*7)
    int* off;    // (ny)
    int* cnt;    // (ny)
};
// Pentadiagonal x-LU of lhs5 per Fourier mode (penta_par.f:6-50): lu(i,c) with
// reciprocal diagonal; one block of 5*nx per mode.
struct PentaX {
    double* lu;   // (K, 5, nx): [k][c][i], c = 0..4 -> lu(:,1..5), c = 2 holds 1/lu(:,3)
};

struct TbGrid {
    int nx, ny, K, P, msh;
    int ptsx[TB_MAX_MSH], ptsy[TB_MAX_MSH];
    size_t lvl_off[TB_MAX_MSH];  // element offsets of each level inside a per-mode work block
    size_t lvl_elems;             // per-mode work block (sum of ptsx*ptsy over levels)
};

struct tb_ctx {
    tb_config cfg;
    TbGrid g;
    double dt, dt2, dt6, dz;
    cudaStream_t stream = nullptr;
    long long launches = 0;
    bool have_coefs = false, have_base = false, inited = false;
    int device = 0;

    // host copies of coefficient tables
    std::vector<double> coefs;            // blob
    std::vector<double> h_qdy, h_qdy2;    // v_qdy(ny), v_qdy2(ny*msh)
    std::vector<double> h_dx2;            // v_dx2(msh)
    std::vector<double> h_k2b2;           // v_k2b2(K)
    std::vector<double> h_bdfc, h_fcx, h_fcllx, h_fcx2, h_fcllx2, h_gibbs, h_uxb, h_uyb, h_wzb, h_duexmdx;

    // device state (comm.var) and RK storage
    cplx *ux = nullptr, *uy = nullptr, *uz = nullptr, *wx = nullptr, *wy = nullptr, *wz = nullptr;
    cplx *wx1 = nullptr, *wy1 = nullptr, *wz1 = nullptr;
    cplx *dv1x = nullptr, *dv1y = nullptr, *dv1z = nullptr, *dv2x = nullptr, *dv2y = nullptr, *dv2z = nullptr;
    cplx* d2uydx2 = nullptr;     // (nx, K)
    cplx* lapv = nullptr;        // (nx, K)
    cplx* tmp[24] = {nullptr};   // work fields (nx, ny, K)
    double* uxb = nullptr; double* uyb = nullptr; double* wzb = nullptr; double* duexmdx = nullptr;
    double* bdfc = nullptr; double* fcx = nullptr; double* fcllx = nullptr; double* gibbs = nullptr;
    double* fcx2 = nullptr; double* fcllx2 = nullptr;   // Goertler strip (var_gv)
    // thermal form (my_form 2): temperature disturbance, its RK storage, the
    // base temperature, and the seven physical-space planes of nlterms_th
    cplx *th = nullptr, *th1 = nullptr, *dv1t = nullptr, *dv2t = nullptr;
    double* thb = nullptr;
    double* th_phys = nullptr;
    double* delta_no = nullptr;  // (nx, ny, P) IBM indicator
    double* k2b2 = nullptr;      // (K)
    // line-operator tables
    TriLHS tx1, tx2, tfil, ty1, tyfv, ty2;
    YRhs ry1, ryfv, ry2;
    PentaX px;
    // Poisson work (per mode blocks of lvl_elems complex): fc, sc, fct
    cplx *pfc = nullptr, *psc = nullptr, *pfct = nullptr, *pdef = nullptr;
    // plain form: line-contiguous real/imaginary planes per (mode, part) of
    // the multigrid arrays (element (i, j) of level l at lvl_off[l] + i*ptsy[l] + j)
    double *pl_fc = nullptr, *pl_sc = nullptr, *pl_fct = nullptr, *pl_def = nullptr;
    double* pl_tab = nullptr;              // plain form: y-line band LU and chunk tables per line group
    unsigned long long* pl_maxsq = nullptr;   // plain form: per mode max |defect|^2 of the fine level
    int* pstate = nullptr;       // per mode: [0] active, [1] vcycles done
    double* perr = nullptr;      // per mode max|defect|
    double* pqdy2 = nullptr;     // v_qdy2 on device (ny*msh)
    double* pcoef = nullptr;     // Poisson coefficients sp/cp/pp/lp per level (24*msh)
    double* wcoef = nullptr;     // wall coefficients w_at_w_coef(9), dwydy_coef(8)
    // statistics
    tb_poisson_stats stats;
    // host staging for the mirrors
    std::vector<cplx> hbuf;
    // mixed form
    void* mixed = nullptr;
    int ws_stage = 0, ws_t = 0;  // RK stage and step of the running loop (0: a mirror call)
    float* nl_phys = nullptr;    // mixed nlterms: FP32 physical disturbance of the 6 fields (6, P, nx*ny)
    double* phys_stage = nullptr; // (P, nx*ny) staging of the tb_f_to_p / tb_p_to_f mirrors
    // optional CUDA-event timing of kernel families (tb_profile)
    bool prof = false;
    struct ProfRec { int id; cudaEvent_t a, b; };
    std::vector<ProfRec> prof_open;
    std::vector<cudaEvent_t> prof_pool;
    double prof_ms[16] = {0};
    long long prof_n[16] = {0};
    // tb_step replayed as a CUDA graph (mixed form): the four stages with each
    // Poisson solve's correction loop as a conditional WHILE node
    bool capturing = false;                // launches are being recorded into a graph
    cudaStream_t body_stream = nullptr;    // records the WHILE bodies
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    double* d_fct = nullptr;               // (2, 4) TS forcing amplitudes of stages 1 and 3
    int* gsnap = nullptr;                  // (4, 2K) pstate after each stage's solve
    double* gerr = nullptr;                // (4, K) perr after each stage's solve
    long long g_outer = 0;                 // kernels of the graph outside the WHILE bodies
    long long g_body[4] = {0, 0, 0, 0};    // kernels of one body iteration per stage
    long long g_learn[4] = {0, 0, 0, 0};   // kernels of the learned correction's IF body per stage
    int g_learn_seen[4] = {0, 0, 0, 0};    // network evaluations per stage counted so far
    int g_stage = 0;                       // stage being recorded (1..4)
    long long graph_gen = 0;               // bumped whenever recorded graphs go stale
    void* learn = nullptr;                 // learned first correction (tb_learn.cu)
    // spanwise transforms of the mixed nonlinear terms on the tensor cores
    int nl_tensor = 1;                     // 0: the FP32 FFT passes instead
    uint16_t* dft_tc = nullptr;            // BF16 DFT matrices (inverse hi, lo; forward hi, lo)
    int* tc_err = nullptr;                 // set when a bounded MMA wait ran out
    int tc_timeout_test = 0;               // tests only: the passes skip their MMAs so the bounded wait runs out
    int sm_count = 0;
    int fp32_lines = 0;                    // mixed form: line operators of modes k >= 1 in FP32 (opt-in)
    // launch shapes chosen by tb_autotune (0: the built-in defaults)
    int tune_xw = 0;                       // warps per block of the x-line kernel (1 or 2)
    int tune_yt = 0;                       // threads per block of the y-line kernel (32, 64 or 128)
    int tune_nl = 0;                       // resident blocks per SM of the tensor-core passes
    int tune_pg3 = 0, tune_pg1 = 0;        // plain form: 1 + log2 warps per line of multi- / single-sweep launches
};

// Kernel families timed by tb_profile (index into prof_ms / prof_n).
enum ProfId { PROF_SOR = 0, PROF_POISSON = 1, PROF_NLTERMS = 2, PROF_XLINES = 3, PROF_YLINES = 4,
              PROF_STAGE = 5, PROF_PENTA = 6, PROF_DEFECT = 7, PROF_RELAX0 = 8, PROF_COUNT = 9 };
int tb_prof_begin(tb_ctx* c, int id, cudaEvent_t* start);
int tb_prof_end(tb_ctx* c, int id, cudaEvent_t start);

// ---- host helpers (tb_host.cpp) -------------------------------------------
int tb_host_build_tables(tb_ctx* c);            // after coefficients are known
int tb_host_upload_baseflow(tb_ctx* c);
double tb_powi(double x, int m);
// Poisson y-line matrix (n, 5) of coef_center (type 0) / coef_border (type 1)
// at y-level lvl (1-based) for mode k (1-based) with x-spacing^2 dx2.
void tb_poisson_band_matrix(const tb_ctx* c, int type, int lvl, int k, std::vector<double>& a);
void tb_poisson_band_matrix_dx(const tb_ctx* c, int type, int lvl, int k, double dx2, std::vector<double>& a);
// band5_poi LU of an (n, 5) band (modified in place) into per-row L1 L2 U1 U2 1/D.
void tb_band5_factor(int n, std::vector<double>& a, double* L1, double* L2, double* U1, double* U2, double* ID);

// ---- kernel launchers ------------------------------------------------------
// Batched x-line operators (derivs_par.f:80-113, filter_par.f:144-177).
enum XOp { XOP_D1 = 0, XOP_D2 = 1, XOP_FILTER = 2 };
struct XJob { const cplx* src; cplx* dst; int op; };  // src and dst must not alias
int tb_launch_xlines(tb_ctx* c, const XJob* jobs, int njobs);
enum YOp { YOP_D1 = 0, YOP_D1FV = 1, YOP_D2 = 2 };
struct YJob { const cplx* src; cplx* dst; int op; };
int tb_launch_ylines(tb_ctx* c, const YJob* jobs, int njobs);

int tb_launch_nlterms(tb_ctx* c, cplx* a, cplx* b, cplx* cc);
int tb_launch_f_to_p(tb_ctx* c, double* phys, const cplx* four);
int tb_launch_p_to_f(tb_ctx* c, cplx* four, const double* phys);
int tb_launch_les(tb_ctx* c, cplx* fx, cplx* fy, cplx* fz);
int tb_launch_cvirt(tb_ctx* c, cplx* fx, cplx* fy, cplx* fz, bool accumulate);
int tb_delta_setup(tb_ctx* c);

int tb_drv_k(tb_ctx* c, cplx* dvx, cplx* dvy, cplx* dvz);
int tb_drv_gvth(tb_ctx* c, cplx* dvx, cplx* dvy, cplx* dvz, cplx* dvt);   // thermal form (tb_thermal.cu)
int tb_combine_gv(tb_ctx* c, const cplx* dadx, const cplx* dady, const cplx* b, const cplx* xx0, const cplx* yy0,
                  const cplx* cc, const cplx* xx1, const cplx* yy1, const cplx* dbdx, const cplx* dcdy,
                  const cplx* xx2, const cplx* yy2, const cplx* d, const cplx* dddx, double varg, cplx* dvx, cplx* dvy,
                  cplx* dvz);
int tb_rk_update_th(tb_ctx* c, int stage);
int tb_bzone_th(tb_ctx* c);
int tb_drv_forced(tb_ctx* c, cplx* dvx, cplx* dvy, cplx* dvz, cplx* f[3], cplx* df[4]);
int tb_rk_update(tb_ctx* c, int stage);
int tb_loop_impl(tb_ctx* c, double erro, bool filter);
int tb_filter(tb_ctx* c);
int tb_bzone_k(tb_ctx* c);
int tb_bzonew_k(tb_ctx* c);
int tb_outuy_k(tb_ctx* c, cplx* dwzdx);
int tb_poi_ux_k(tb_ctx* c, cplx* duydy);
int tb_poi_uz_k(tb_ctx* c, const cplx* duydy);
int tb_wx_wall_k(tb_ctx* c, cplx* lapv);
int tb_wz_wall_k(tb_ctx* c, const cplx* lapv);
int tb_ts_pert_k(tb_ctx* c, int t, double tempt);
int tb_poi_uy_k(tb_ctx* c, const cplx* dwzdx, double erro);   // plain FP64 form (tb_plain.cu)
int tb_plain_setup(tb_ctx* c);
int tb_plain_tune(tb_ctx* c, int l, int itera, const int* gis, int ngis, int* best, float* best_ms);
int tb_poisson_setup(tb_ctx* c);
int tb_poisson_begin(tb_ctx* c, const cplx* dwzdx);
int tb_poisson_defect_f32(tb_ctx* c, float2* r32, float2* e32, size_t elems32, unsigned long long* maxsq);
int tb_poisson_end(tb_ctx* c);
void tb_chunk_tables(int n, int ny, int S, const double* L1, const double* L2, const double* U1, const double* U2,
                     const double* ID, double* out);
__host__ __device__ inline size_t tb_poi_blk_size(int ny) { return (size_t)9 * ny + 1280; }
int tb_poi_uy_mixed(tb_ctx* c, const cplx* dwzdx, double erro);
// Learned first correction of the mixed solve (tb_learn.cu owns the network
// and buffers, tb_mixed.cu the solver-side kernels).
struct LearnSolve {
    bool infer = false;          // apply the network's correction in every solve
    bool sample = false;         // collect training crops from every solve
    float* X = nullptr;          // (2K, 4, nx, ny) network input planes per mode and part
    float* out = nullptr;        // (2K, nx, ny) network output
    float* scl = nullptr;        // (K, 3) input scales: max|v1|, max|v1 - v2|, max|D^-1 d0|
    unsigned* jmax = nullptr;    // (K) max |r - L e|^2 of the candidate correction, float bits
    float* invD = nullptr;       // (K, ny) 1 / |diagonal| of the fine line operator
    float* mfeat = nullptr;      // (K, ny) share of k^2 beta^2 in the diagonal
    cplx* g0 = nullptr;          // guess before any correction (while sampling)
    long long* tally = nullptr;  // (K, 2) solves tried / corrections kept per mode
    // gated evaluation (tb_learn_enable mode 2): per stage [solves since it
    // last ran, ran in the last solve, evaluations, solves, corrections of
    // the last solve without / with it, 2 spare]
    int gated = 0;
    int probe = 32;              // a stage evaluates the network at least every `probe` solves
    int* gate = nullptr;         // (4, 8) and a host-read flag
};
// The fine-level FP32 operator of the mixed form (the operator of k_resid at
// level 0): device tables and scalars.
struct FineOp {
    const float* coef;     // sp(7) cp(8) pp(4) lp(5) of the finest level
    const float* qdy2;     // (ny)
    const double* k2b2;    // (K)
    float den, ify, alpha2;
    int nx, ny, K;
};
int tb_mixed_fine_op(tb_ctx* c, FineOp* op);
// FP32 residual r - L e of the finest level for one mode (tests of the
// learned correction's operator): host r, e and out in line-contiguous (nx, ny).
int tb_mixed_resid_mode(tb_ctx* c, int k, const float* e, float* out);
LearnSolve* tb_learn_solve(tb_ctx* c);     // null unless the learned form is on
int tb_learn_run_net(tb_ctx* c);           // X -> out on c->stream
int tb_learn_collect(tb_ctx* c);           // this solve's crops into the sample buffer
void tb_learn_free(tb_ctx* c);
int tb_mixed_line_diag(tb_ctx* c, std::vector<float>& invD, std::vector<float>& mfeat);

// Step graph support (tb_graph.cu, tb_mixed.cu, tb_spectral.cu)
int tb_spectral_prepare(tb_ctx* c);               // lazy tables/buffers of the step, made before a capture
int tb_tc_check(tb_ctx* c);                       // error of the tensor-core passes since the last check
void tb_dft_matrices(int P, std::vector<uint16_t>& out);
int tb_mixed_graph_pre(tb_ctx* c, int t, cudaStream_t s);   // warm-start continuity before a replay of step t
void tb_mixed_graph_post(tb_ctx* c, int t);       // after it
int tb_mixed_absorb_stats(tb_ctx* c, const int* hs, const double* he);   // one solve's pstate/perr into stats
int tb_ts_pert_fct(tb_ctx* c, int t, double tempt, double* fct);   // forcing amplitudes per forced mode
int tb_graph_record_step(tb_ctx* c);              // the four stages on c->stream, which is capturing
int tb_graph_pre(tb_ctx* c, int t, cudaStream_t s);
int tb_graph_post(tb_ctx* c, const int* hs, const double* he);   // hs (4, 2K), he (4, K) copied from gsnap/gerr
void tb_graph_reset(tb_ctx* c);                   // drop the recorded graph (tables or buffers changed)
void tb_graph_free(tb_ctx* c);
bool tb_graph_usable(const tb_ctx* c);            // tb_step may replay a graph
int tb_graph_step(tb_ctx* c, int t);
int tb_mixed_setup(tb_ctx* c);
void tb_mixed_free(tb_ctx* c);
void tb_mixed_invalidate(tb_ctx* c);   // forget the warm-start history (new state)

// grid helpers
inline unsigned tb_blocks(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }
inline size_t tb_n3(const tb_ctx* c) { return (size_t)c->g.nx * c->g.ny * c->g.K; }
inline size_t tb_n2(const tb_ctx* c) { return (size_t)c->g.nx * c->g.ny; }
