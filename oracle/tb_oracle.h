/*
 * tb_oracle.h -- CPU restatement of the trans_bl per-RK4-stage hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the checker for the GPU library:
 * only the test suite, the smoke check and the CPU-baseline leg of the
 * benchmark load it.  Nothing in the product links against it.
 *
 * Pinning: field-level parity unpinned by reference outputs -- the reference
 * ships no field dumps (its base-flow files are empty) and cannot be compiled
 * here (no gfortran, no MPI).  What is pinned: (a) the reference's golden
 * coefficient tables pre_processing/coefs.bin, which feed every y-operator of
 * this oracle, (b) the Blasius wall shear of lst_ts/fpp.dat; the field-level
 * routines rest on (c) exactness properties of each operator (polynomial
 * exactness of the compact schemes, realft round trips against a plain DFT,
 * the discrete Poisson equation satisfied to the stop tolerance) and on
 * following the reference's loop and operation order line by line.
 *
 * Every routine follows one reference subroutine in its loop order and
 * operation order; each cites the file:line it restates.  MPI is collapsed to
 * one rank (my_rank = numproc = 0, shift = 0).
 */
#ifndef TB_ORACLE_H
#define TB_ORACLE_H
#include "../include/transbl.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_ctx ora_ctx;

ora_ctx* ora_create(const tb_config* cfg);
void     ora_destroy(ora_ctx* o);
int      ora_set_coefs(ora_ctx* o, const double* blob);
int      ora_set_baseflow(ora_ctx* o, const double* uxb, const double* uyb, const double* wzb);
int      ora_init_fields(ora_ctx* o);
int      ora_put_state(ora_ctx* o, const double* ux, const double* uy, const double* uz,
                       const double* wx, const double* wy, const double* wz);
int      ora_get_state(ora_ctx* o, double* ux, double* uy, double* uz,
                       double* wx, double* wy, double* wz);
int      ora_put_wall(ora_ctx* o, const double* d2uydx2);
int      ora_get_wall(ora_ctx* o, double* d2uydx2);
int      ora_set_baseflow_th(ora_ctx* o, const double* thb);   /* my_form 2: base temperature (nx, ny) */
int      ora_put_th(ora_ctx* o, const double* th);             /* temperature disturbance (nx, ny, kfour) */
int      ora_get_th(ora_ctx* o, double* th);

int ora_derparx (ora_ctx* o, double* ddx,   const double* fc);
int ora_derparxx(ora_ctx* o, double* d2dx2, const double* fc);
int ora_dery    (ora_ctx* o, double* ddy,   const double* fc);
int ora_deryfv  (ora_ctx* o, double* ddy,   const double* fc);
int ora_deryy   (ora_ctx* o, double* d2dy2, const double* fc);
int ora_f_to_p  (ora_ctx* o, double* phys, const double* four);
int ora_p_to_f  (ora_ctx* o, double* four, const double* phys);
int ora_nlterms (ora_ctx* o, double* a, double* b, double* c);
int ora_drv     (ora_ctx* o, double* dvx, double* dvy, double* dvz);
int ora_filter_trid(ora_ctx* o);
int ora_bzone   (ora_ctx* o);
int ora_bzonew  (ora_ctx* o);
int ora_outuy   (ora_ctx* o, double* dwzdx);
int ora_poi_uy  (ora_ctx* o, const double* dwzdx, double erro);
int ora_poi_ux  (ora_ctx* o, double* duydy);
int ora_poi_uz  (ora_ctx* o, const double* duydy);
int ora_wx_wall (ora_ctx* o, double* lapv);
int ora_wz_wall (ora_ctx* o, const double* lapv);
int ora_ts_pert (ora_ctx* o, int t, double tempt);
int ora_les_terms(ora_ctx* o, double* fx, double* fy, double* fz);
int ora_cvirt   (ora_ctx* o, double* fx, double* fy, double* fz);
int ora_loop    (ora_ctx* o, double erro);
int ora_rk_stage(ora_ctx* o, int stage, int t);
int ora_step    (ora_ctx* o, int t);
/* V-cycles and final residual of the last poi_uy, per mode. */
int ora_poisson_stats(ora_ctx* o, int* vcycles, double* residual);
/* Host threads of the parallel loops (n <= 0: keep); returns the count in use. */
int ora_set_threads(int n);

/* Workload inputs without the GPU library (tb_inputs.cpp): the coefficient
 * blob of tb_set_coefs (100 + 24 msh doubles), the compact first-point weights
 * fp_fd_coef(7), the Falkner-Skan f''(0), and the base flow as (ny, nx). */
int ora_generate_coefs(double stf, int msh, double* blob);
int ora_generate_fp_fd(double stf, double* out7);
int ora_fs_wall_shear(double beta_fs, double* fpp);
int ora_baseflow_fs(const tb_config* cfg, double beta_fs, double* uxb, double* uyb, double* wzb);

#ifdef __cplusplus
}
#endif
#endif
