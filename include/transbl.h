/*
 * transbl.h -- C ABI of the GB300-native per-RK4-stage hot path of the
 * trans_bl incompressible boundary-layer DNS (vorticity-velocity form,
 * compact finite differences in x/y, spanwise Fourier modes in z).
 *
 * The library keeps the whole domain resident in GPU memory and runs every
 * loop nest of one RK stage as hand-written CUDA for sm_103a.  The entry
 * points mirror the Fortran subroutines of the reference one for one, with
 * the reference's argument order (output first), so that a Fortran host can
 * bind them through ISO_C_BINDING.
 *
 * Conventions
 *  - Fields are complex*16, Fortran column-major f(nx, ny, kfour): i fastest,
 *    then j, then k; interleaved (re, im) doubles.  Host pointers passed to
 *    the mirrors below are borrowed for the duration of the call.
 *  - Indices inside the config (i0..i4) are 1-based, as in the reference.
 *  - Every function returns an int status (TB_OK = 0 or a TB_ERR_* code);
 *    tb_last_error() gives a one-line message for the last failure of the
 *    calling thread.
 *  - One host thread per context; contexts are independent.
 *
 * Reference interfaces (paths inside the trans_bl project):
 *  par.for:1-132             compile-time parameters   -> tb_config
 *  main_par.f:551-772        init_fi                   -> tb_create, tb_set_coefs, tb_init_fields
 *  main_par.f:165-254        solver RK4 loop (form 0)  -> tb_rk_stage/tb_step
 *  main_par.f:1264-1336      drv_fi                    -> tb_drv
 *  main_par.f:1487-1574      drv_les                   -> tb_drv (my_form 4)
 *  main_par.f:1762-1785      loop                      -> tb_loop
 */
#ifndef TRANSBL_H
#define TRANSBL_H

#ifdef __cplusplus
extern "C" {
#endif

#define TB_OK            0
#define TB_ERR_ARG       1  /* bad argument / config                              */
#define TB_ERR_CUDA      2  /* CUDA runtime failure (message in tb_last_error)    */
#define TB_ERR_NOCONV    3  /* Poisson V-cycle cap reached above the tolerance    */
#define TB_ERR_NONFINITE 4  /* NaN/Inf met in a residual reduction                */
#define TB_ERR_TIMEOUT   5  /* a bounded device wait gave up                       */
#define TB_ERR_STATE     6  /* call order violated (e.g. no coefficients yet)      */
#define TB_ERR_NOMEM     7  /* device allocation failed                            */

/* Precision forms of the stage. */
#define TB_FORM_PLAIN_FP64 0   /* drop-in: FP64 everywhere, lexicographic line-SOR */
#define TB_FORM_MIXED      1   /* FP32 multigrid inside FP64 defect correction      */

/* Runtime replacement of the compile-time parameters of par.for. */
typedef struct tb_config {
    int    nx;          /* imax = ptsx (whole domain, one GPU)        par.for:81-82 */
    int    ny;          /* jmax                                        par.for:73   */
    int    kfour;       /* stored Fourier modes K (k = 0..K-1)         par.for:106  */
    int    kphys;       /* physical z points P, power of two, >= 4     par.for:106  */
    int    msh;         /* multigrid levels                            par.for:102  */
    int    my_form;     /* 0: drv_fi (+optional IBM), 1: drv_gv (linear about the base
                           flow, Goertler curvature; gv_pert forcing), 2: drv_gvth (the
                           nonlinear disturbance about the base flow with a transported
                           temperature th), 4: drv_les                        par.for:14 */
    int    i0, i1, i2, i3, i4;  /* buffer ramp end, TS strip, damping  par.for:21,88 */
    int    stpp;        /* time steps per forcing period               par.for:92   */
    int    max_vcycles; /* V-cycle cap (11 in the reference)  poisson_par.f:33      */
    int    ibm;         /* 1: add immersed-boundary force (cvirt)                   */
    int    precision;   /* TB_FORM_PLAIN_FP64 or TB_FORM_MIXED                      */
    int    les_damping; /* 0: reference cubic damping 1-e^{-(y+/A)^3}, 1: van Driest
                           [1-e^{-y+/A}]^2; +2: y+ from |wall vorticity| (les_par.f:194
                           takes sqrt(Re wz_wall), undefined where wz_wall < 0)      */
    int    warm_start;  /* mixed form: 1 starts each stage's v-Poisson solve from the
                           extrapolation 2 v(t-1) - v(t-2) of the same stage's solutions
                           of the two previous steps; 2 from the current v plus the
                           increment between the same two stages' solutions one step
                           earlier; 0 from the current v, as the reference (no effect
                           on the plain form)                                       */
    int    step_graph;  /* mixed form: 1 runs tb_step/tb_steps as a recorded CUDA graph,
                           each Poisson correction loop a device-side WHILE loop, so a
                           step has no host synchronisation inside; 0 launches every
                           kernel from the host.  tb_rk_stage and profiling always
                           launch from the host.                                    */
    double Re;          /* U L / nu                                    par.for:41   */
    double dx;          /* uniform x spacing                           par.for:83   */
    double dy;          /* first wall-normal spacing dy0               par.for:73   */
    double stf;         /* geometric stretching factor in y            par.for:75   */
    double x0;          /* x of i = 1                                  par.for:41   */
    double alpha;       /* streamwise wavenumber (top Poisson BC)      par.for:56   */
    double omega;       /* forcing frequency; dt = 2 pi / omega / stpp par.for:57,93*/
    double beta;        /* spanwise wavenumber                         par.for:70   */
    double fac_y;       /* y scaling (1 or Re)                         par.for:45   */
    double alphaf;      /* compact filter alpha_f (0.48)               par.for:116  */
    double tol_stage;   /* Poisson max-defect tolerance, stages 1-3 (1e-5) main_par.f:187 */
    double tol_final;   /* Poisson max-defect tolerance, stage 4 (1e-6)   main_par.f:247 */
    double C_s;         /* Smagorinsky constant                        par.for:126  */
    double A_plus;      /* damping length in wall units (25)           les_par.f:195 */
    double irf;         /* IBM feedback gain (-0.1 Re)                 par.for:123  */
    double ibm_xc, ibm_zc, ibm_h, ibm_R;  /* roughness centre, height, radius  immersed_par.f:111-120 */
    /* Wall suction/blowing forcing per Fourier mode (ts2d_pert/ts3d_pert,
       main_par.f:1613-1685): uy(i,1,k) = A_k fcx(i) sin(omega (t+tau) dt + phi_k). */
    int    n_forced;            /* number of forced modes (<= 4)                    */
    int    forced_mode[4];      /* 0-based Fourier mode index                       */
    double forced_amp[4];       /* amplitude A_k                                    */
    double forced_phase[4];     /* phase phi_k (0 in the reference)                 */
    /* my_form 1: Goertler number Go of the wall curvature, varg = Go^2 / sqrt(Re)
       at every point (init_gv, main_par.f:944-970; 0 in the reference)             */
    double go_number;
    /* my_form 2: Prandtl number of the temperature equation (0.72, par.for:38)   */
    double Pr;
} tb_config;

typedef struct tb_ctx tb_ctx;

/* Per-solve Poisson statistics (poisson_par.f:58-60 prints k, vcycles-1, err). */
typedef struct tb_poisson_stats {
    int    vcycles[256];   /* V-cycles taken per mode in the last poi_uy     */
    double residual[256];  /* last max|defect| per mode                      */
    int    total_vcycles;  /* accumulated over the context's lifetime        */
    int    solves;         /* number of poi_uy calls accumulated             */
    int    noconv;         /* modes that hit the cap in the last poi_uy      */
} tb_poisson_stats;

const char* tb_last_error(void);

/* Fill cfg with the reference defaults of par.for scaled to a tiny grid. */
int tb_config_default(tb_config* cfg);
/* Derived quantities (dt = 2 pi / omega / stpp, par.for:93). */
double tb_dt(const tb_config* cfg);

/* ---- host set-up (pre_processing/) ---------------------------------- */
/* Number of doubles in a coefficient blob for msh levels: 100 + 24 msh.
   Layout = records 1..16 of pre_processing/coefs.bin (coef_generation.f90:38-53),
   record 1 being fp_fd_coef_e(6). */
int tb_coef_count(int msh);
/* Stretched-grid compact / Poisson / wall coefficients
   (pre_processing/derivative.f90:1762-1882, at_wall.f90:1499). */
int tb_generate_coefs(double stf, int msh, double* blob);
/* Compact first-point first-derivative weights fp_fd_coef(7)
   (derivative.f90:15-108); record 1 of pre_processing/coefs.bin holds these. */
int tb_generate_fp_fd(double stf, double* out7);
/* Falkner-Skan / Blasius wall shear by Newton shooting (fs_sch.f90:11-54):
   returns f''(0) for pressure-gradient parameter beta_fs. */
int tb_fs_wall_shear(double beta_fs, double* fpp);
/* Base flow on the (nx, ny) grid (fs_sch.f90:58-162), column-major reals. */
int tb_baseflow_fs(const tb_config* cfg, double beta_fs, double* uxb, double* uyb, double* wzb);

/* ---- linear stability theory for the TS-wave check (lst_ts/ose_bl.f) ---- */
/* Spatial Orr-Sommerfeld/Squire stability of the Falkner-Skan layer: the
   reference's continuation from a starting eigenvalue to the target
   parameters (steps per parameter: 1000 in the reference), then the march
   over stations x = 1 + (i-1) dx with Re^(1/2) = re_dns sqrt(x), scaled
   frequency w0 = omega_dns Re^(1/2)/re_dns and beta scaled the same way. */
typedef struct tb_lst_config {
    double re0, w0, alfa0_re, alfa0_im;   /* starting point and eigenvalue guess (ose3d.in)  */
    int    jedge;                         /* wall-normal points of the mapped grid           */
    double bl, etamax, beta, wslope;      /* integration fraction, eta_max, beta, f''(0)     */
    double re_dns, omega_dns, beta_dns;   /* target Re^(1/2), w/Re^(1/2), beta/Re^(1/2) (datalst.dat) */
    int    imax;                          /* stations                                        */
    double dx;                            /* station spacing in x / x0                       */
    int    steps;                         /* continuation steps per parameter                */
} tb_lst_config;
/* Outputs per station i: x, Re^(1/2), scaled frequency and the eigenvalue
   alpha0 = (alpha[2i], alpha[2i+1]); the growth rate is -Im(alpha0).
   fpp, betafs: wall shear f''(0) and Falkner-Skan beta per station. */
int tb_lst_march(const tb_lst_config* cfg, const double* fpp, const double* betafs, double* x,
                 double* re0, double* w0, double* alpha);

/* ---- lifecycle --------------------------------------------------------- */
int tb_create(const tb_config* cfg, tb_ctx** out);
int tb_destroy(tb_ctx* ctx);
int tb_set_coefs(tb_ctx* ctx, const double* blob);
int tb_set_baseflow(tb_ctx* ctx, const double* uxb, const double* uyb, const double* wzb);
/* init_fi (main_par.f:551-772): zero every field, base flow into mode 0,
   buffer ramps, filter and x-penta factors, forcing shape, IBM delta. */
int tb_init_fields(tb_ctx* ctx);
int tb_put_state(tb_ctx* ctx, const double* ux, const double* uy, const double* uz,
                 const double* wx, const double* wy, const double* wz);
int tb_get_state(tb_ctx* ctx, double* ux, double* uy, double* uz,
                 double* wx, double* wy, double* wz);
/* d2uydx2(nx, K) wall forcing curvature (common /derw/). */
int tb_put_wall(tb_ctx* ctx, const double* d2uydx2);
/* my_form 2 only: the base temperature thb(nx,ny) (/blast/, read with the base
   flow in init_gvth, main_par.f:1125) and the temperature disturbance
   th(nx,ny,kfour) (complex, comm.var), host pointers. */
int tb_set_baseflow_th(tb_ctx* ctx, const double* thb);
int tb_put_th(tb_ctx* ctx, const double* th);
int tb_get_th(tb_ctx* ctx, double* th);
int tb_get_wall(tb_ctx* ctx, double* d2uydx2);
int tb_synchronize(tb_ctx* ctx);

/* ---- time stepping (main_par.f:165-254) -------------------------------- */
int tb_rk_stage(tb_ctx* ctx, int stage, int t);   /* stage 1..4 of step t        */
int tb_step(tb_ctx* ctx, int t);                  /* four stages                 */
int tb_steps(tb_ctx* ctx, int t0, int nsteps);    /* t0 .. t0+nsteps-1           */
int tb_get_poisson_stats(tb_ctx* ctx, tb_poisson_stats* st);
/* Mixed form, opt-in: the compact x-line operators (derparx, derparxx, the
   x filter) of modes k >= 1, which hold only the disturbance, run in FP32
   on FP64 data; mode 0 (the base flow and the 2D disturbance) stays FP64.
   About 9% faster on the 1025 x 193 x 32 step, at the cost of ~1e-6
   relative on the disturbance modes after two steps and 0.2-5e-6 after
   eight: above the mixed form's 1e-6 target, hence off by default.  Default 0. */
int tb_mixed_fp32_lines(tb_ctx* ctx, int on);
/* Mixed form, P >= 16: the spanwise transforms of the disturbance products
   in the nonlinear terms run as DFT-matrix GEMMs on the tensor cores
   (operands split into three BF16 parts, products compensated to FP32
   accuracy, FP32 accumulation); 0 selects the FP32 FFT passes.
   Default 1.                                                                */
int tb_nl_tensor_cores(tb_ctx* ctx, int on);
/* Tests of the error path only: with on = 1 the tensor-core passes leave
   their MMAs unissued and wait at most a few thousand polls, so the bounded
   wait runs out; the kernels free their tensor memory and return, and the
   next synchronising call reports TB_ERR_TIMEOUT.  No MMA is in flight and
   nothing faults; the context stays usable.                                */
int tb_tc_timeout_test(tb_ctx* ctx, int on);
/* The DFT matrices of those GEMMs in double precision, P x P row-major:
   forward 0: physical z from slot s (slots: Re c0 (unused), Im c0 as the
   Nyquist term, Re and Im of modes 1 .. P/2-1); forward 1: slot from z.     */
int tb_dft_matrix(int P, int forward, double* out);

/* ---- learned first correction of the mixed v-Poisson solve ------------
   A convolutional network (four 3x3 layers, 4 -> 32 -> 32 -> 32 -> 1
   channels, GELU) estimates, per mode, the error of the extrapolated guess
   from v(t-1), v(t-1) - v(t-2) and the FP64 defect of the guess.  Its
   correction is kept per mode only where it lowers the max defect by 5%; the
   multigrid then iterates to the same tolerance.  The solver generates the
   training crops itself, and the network is trained on the GPU by the
   library's own forward and backward kernels (Adam).  Needs the mixed form
   with warm_start = 1.  Crops are collected only from host-launched steps:
   while collecting, tb_step does not replay a graph.                      */
typedef struct tb_learn_stats {
    long long samples;     /* training crops collected                          */
    long long capacity;    /* crops the sample buffer holds                     */
    long long tried;       /* mode-solves that evaluated the network            */
    long long kept;        /* of those, corrections kept (the rest fell back)   */
    double    loss;        /* mean training loss over the last tenth of training */
    long long solves;      /* gated mode: solves that passed the gate           */
    long long evaluated;   /* gated mode: of those, solves that ran the network */
} tb_learn_stats;
int tb_learn_param_count(void);                 /* floats in a weight vector        */
int tb_learn_crop_size(void);                   /* edge of a training crop (72)     */
int tb_learn_init(tb_ctx* ctx, unsigned long long seed);   /* He-normal, last layer 0 */
int tb_learn_set_weights(tb_ctx* ctx, const float* w);
int tb_learn_get_weights(tb_ctx* ctx, float* w);
/* on = 1: run the network in every solve; on = 2 (gated): a stage runs it
   in its first solve and once every 32 solves, and keeps running it while a
   solve with it needs fewer multigrid corrections than the stage's last
   solve without it; in between the solve falls back to the guess without
   running the network; 0: off.                                             */
int tb_learn_enable(tb_ctx* ctx, int on);
/* Collect crops_per_solve crops from every solve into a buffer of `capacity`
   crops; capacity 0 stops collecting and keeps the crops for training.     */
int tb_learn_sample(tb_ctx* ctx, long long capacity, int crops_per_solve, unsigned long long seed);
/* Adam on crops 0 .. n_train-1 (all when n_train <= 0); the first run from
   fresh weights sets the input and output scales from those crops.          */
int tb_learn_train(tb_ctx* ctx, long long n_train, int iters, int batch, float lr, unsigned long long seed,
                   double* loss);
/* Defect loss of the network over crops first .. first+n-1 and that of a
   zero correction (the defect the extrapolated guess leaves).             */
int tb_learn_eval(tb_ctx* ctx, long long first, long long n, double* mse, double* target_ms);
int tb_learn_get_stats(tb_ctx* ctx, tb_learn_stats* st);
/* Copy collected crops first .. first+n-1, each (5, 72, 72) floats.       */
int tb_learn_get_samples(tb_ctx* ctx, long long first, long long n, float* dst);
/* The training kernels on caller data (host memory): loss and gradient over
   n crops (n, 5, 72, 72), planes 0-3 the inputs and plane 4 the target,
   with meta (n, 3) = image (2k + part), first row, first column on the
   context's grid; and the network's output on n images (n, 4, H, W).
   tb_learn_op_tables gives mode k's operator tables as the loss uses them
   (den, ify, alpha^2, k^2 beta^2, w_k, 24 coefficients, qdy2(ny), 1/|D|(ny));
   tb_learn_op_apply gives -L e of mode k through the solver's own residual
   kernel (e, out: (nx, ny), y fastest).                                   */
int tb_learn_grad(tb_ctx* ctx, const float* w, const float* crops, const int* meta, int n, double* loss, float* grad);
int tb_learn_forward(const float* w, const float* x, int n, int H, int W, float* out);
int tb_learn_op_tables(tb_ctx* ctx, int k, float* tab);
int tb_learn_op_apply(tb_ctx* ctx, int k, const float* e, float* out);

/* ---- launch shapes ----------------------------------------------------
   tb_autotune times the candidate launch shapes of the stage's batched
   kernels on this context's grid and keeps the fastest: warps per block of
   the x-line solves (1, 2), threads per block of the y-line solves (32, 64,
   128) and, for the mixed form with P >= 16, resident blocks per SM of the
   tensor-core passes (1, 2, 4, 8, capped by shared and tensor memory), and,
   for the plain form, warps per y-line solve of the Poisson sweeps (1, 2, 4).
   It touches only scratch fields and work arrays that every solve rebuilds.
   Times are per launch of the tuned batch.  */
typedef struct tb_tune_result {
    int   xline_warps, yline_threads, nl_blocks_per_sm;
    float xline_ms, yline_ms, nl_ms;
    /* plain form: warps per y-line solve of the fine level's multi-sweep
       (pre-smoothing) and single-sweep (post-smoothing) launches (1, 2, 4) */
    int   plain_line_warps_multi, plain_line_warps_single;
    float plain_multi_ms, plain_single_ms;
} tb_tune_result;
int tb_autotune(tb_ctx* ctx, tb_tune_result* out);

/* No counterpart in the reference: the current device's FP64 throughput in
   TFLOP/s (fused multiply-adds counted as two flops), measured by a short
   kernel with CUDA events -- the denominator of the FP64-pipe rooflines the
   benchmark reports for the FP64 kernels.  Allocates a small buffer. */
int tb_fp64_peak(double* tflops);

/* ---- ensembles: independent runs advanced together --------------------
   One recorded CUDA graph advances every member by one step: the members'
   stages run concurrently on the device and the host waits once per step.
   Members use the mixed form and may differ in every size and parameter;
   between ensemble steps each stays usable on its own.  An ensemble holds
   its members' device buffers: destroy it before any member.             */
typedef struct tb_ensemble tb_ensemble;
int tb_ensemble_create(tb_ctx* const* members, int n, tb_ensemble** out);
int tb_ensemble_step(tb_ensemble* ens, const int* t);   /* t[i]: step of member i */
int tb_ensemble_destroy(tb_ensemble* ens);

/* ---- per-subroutine mirrors (host pointers, copy in / out) ------------ */
int tb_derparx (tb_ctx* ctx, double* ddx,   const double* fc);  /* derivs_par.f:80  */
int tb_derparxx(tb_ctx* ctx, double* d2dx2, const double* fc);  /* derivs_par.f:98  */
int tb_dery    (tb_ctx* ctx, double* ddy,   const double* fc);  /* derivs_par.f:116 */
int tb_deryfv  (tb_ctx* ctx, double* ddy,   const double* fc);  /* derivs_par.f:148 */
int tb_deryy   (tb_ctx* ctx, double* d2dy2, const double* fc);  /* derivs_par.f:164 */
/* nlterms_fi on the context state (nlterms_par.f:41): a, b, c out. */
int tb_nlterms (tb_ctx* ctx, double* a, double* b, double* c);
/* drv_fi / drv_les on the context state: dvx, dvy, dvz out (main_par.f:1264,1487). */
int tb_drv     (tb_ctx* ctx, double* dvx, double* dvy, double* dvz);
/* loop(erro) on the context state (main_par.f:1762). */
int tb_loop    (tb_ctx* ctx, double erro);
int tb_filter_trid(tb_ctx* ctx);                                 /* filter_par.f:144 */
int tb_bzone   (tb_ctx* ctx);                                    /* loop_par.f:6     */
int tb_bzonew  (tb_ctx* ctx);                                    /* loop_par.f:691   */
int tb_outuy   (tb_ctx* ctx, double* dwzdx);                     /* loop_par.f:48    */
int tb_poi_uy  (tb_ctx* ctx, const double* dwzdx, double erro);  /* poisson_par.f:6  */
int tb_poi_ux  (tb_ctx* ctx, double* duydy);                     /* loop_par.f:428   */
int tb_poi_uz  (tb_ctx* ctx, const double* duydy);               /* loop_par.f:569   */
int tb_wx_wall (tb_ctx* ctx, double* lapv);                      /* loop_par.f:174   */
int tb_wz_wall (tb_ctx* ctx, const double* lapv);                /* loop_par.f:361   */
int tb_ts_pert (tb_ctx* ctx, int t, double tempt);               /* main_par.f:1613  */
int tb_les_terms(tb_ctx* ctx, double* fx, double* fy, double* fz); /* les_par.f:6    */
int tb_cvirt   (tb_ctx* ctx, double* fx, double* fy, double* fz);  /* immersed_par.f:262 */
/* Spanwise transforms of one field (nlterms_par.f:303,364).
   phys: real (nx, ny, kphys); four: complex (nx, ny, kfour). */
int tb_f_to_p  (tb_ctx* ctx, double* phys, const double* four);
int tb_p_to_f  (tb_ctx* ctx, double* four, const double* phys);

/* ---- on-disk formats of the reference (escreve_par.f) ------------------ */
/* data_XX.bin checkpoint, gfortran sequential unformatted: record 1 integer*4
   t, record 2 ux,uy,uz,wx,wy,wz (escreve, escreve_par.f:6-31) -- the file the
   Fortran host writes and reads back at restart (main_par.f:762-769). */
int tb_write_checkpoint(tb_ctx* ctx, const char* path, int t);
int tb_read_checkpoint(tb_ctx* ctx, const char* path, int* t);
/* pert_XX_YY snapshot of escreve2 (escreve_par.f:34-81): one record with ux,
   the base flow removed from the real part of mode 0 in form 0. */
int tb_write_pert(tb_ctx* ctx, const char* path);
/* Largest subrecord written (default 2^31 - 9 bytes, as gfortran); records
   beyond it are split with negated markers.  A small value exercises the
   layout of records over 2 GiB on small files. */
int tb_io_set_subrecord_limit(long long bytes);

/* ---- device-resident access (no host copies) ------------------------- */
/* Device pointers of the resident fields: which = 0..5 for ux,uy,uz,wx,wy,wz. */
int tb_device_field(tb_ctx* ctx, int which, void** dptr);
/* CUDA stream (cudaStream_t) every kernel of this context is launched on. */
int tb_stream(tb_ctx* ctx, void** stream);
/* Kernel launches issued by this context so far (for launch accounting). */
long long tb_launch_count(tb_ctx* ctx);
/* CUDA-event timing of kernel families on the context stream: enable = 1
   starts recording (and clears totals), 0 stops.  tb_profile_read returns the
   accumulated device milliseconds and launch count of one family:
   0 line-relaxation sweeps (SOR in the plain form, coloured sweeps in the
   mixed form), 1 whole poi_uy, 2 nlterms, 3 x-line batches, 4 y-line
   batches, 5 RK stages, 6 x-penta solves, 7 FP64 Poisson defects,
   8 single finest-level line-relaxation launches of the mixed form. */
int tb_profile(tb_ctx* ctx, int enable);
int tb_profile_read(tb_ctx* ctx, int family, double* ms, long long* launches);

/* ---- allocation-free entry point --------------------------------------- */
/* No counterpart in the reference: filter_trid (filter_par.f:144) on caller
   DEVICE buffers wx, wy, wz (complex*16 (nx, ny, kfour)), for hosts that must
   not allocate GPU memory after start-up (a memory manager that owns all free
   device memory, or a real-time section).  Needs no context and
   allocates nothing: the filtered lines are staged in a 32 MiB array built
   into the library, so one call takes nx*ny*kfour <= 2^21 - 4096 points and
   nx <= 4096 (filter larger grids one slice of Fourier modes per call) and
   returns TB_ERR_ARG beyond that.  The first call on a device sets up the
   array's address and must precede any stream capture (after cudaDeviceReset
   of that device the kept address is stale: do not call it there again);
   calls that overlap on the GPU race on the shared array.  stream is a cudaStream_t (NULL: legacy
   default stream); the call returns once the kernels are queued. */
int tb_filter_trid_noalloc(double* wx, double* wy, double* wz, int nx, int ny, int kfour,
                           double alphaf, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TRANSBL_H */
