/*
 * alps_oracle.h -- CPU oracle for the ALPS dispersion-tensor hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a literal FP64 restatement of the
 * reference Fortran (danielver02/ALPS) used as the checker for the GPU
 * library.  Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline
 * may load it; the product never links or calls it.
 *
 * Parity pin: the restatement is checked against the reference's own golden
 * files tests/test_kpar_fast.{scan,eigen,heat}_kpara_1.root_1 (committed as
 * fixtures under tests/golden/).  The Fortran reference itself cannot be built
 * in this image (no gfortran, MPI or LAPACK), so there is no compiled
 * reference beside it.
 */
#ifndef ALPS_ORACLE_H
#define ALPS_ORACLE_H

#include "../include/alps_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_ctx oracle_ctx;

int oracle_create(const alps_system* sys, oracle_ctx** out);
void oracle_destroy(oracle_ctx* ctx);
int oracle_set_species(oracle_ctx* ctx, int is, const alps_species* sp,
                       const double* pperp, const double* ppar,
                       const double* f0);
int oracle_prepare(oracle_ctx* ctx);
int oracle_get_fit(oracle_ctx* ctx, int is, double* out);
int oracle_set_fit(oracle_ctx* ctx, int is, const double* in);
int oracle_get_df0(oracle_ctx* ctx, int is, double* df1, double* df2);
/* Test hook: f0_rel of a relativistic species taken as given by the next
 * oracle_prepare (in place of the spline remap). */
int oracle_set_f0_rel(oracle_ctx* ctx, int is, const double* f0_rel);
int oracle_get_f0_rel(oracle_ctx* ctx, int is, double* gamma, double* pparbar, double* f0_rel, double* df1,
                      double* df2);
int oracle_set_k(oracle_ctx* ctx, double kperp, double kpar);
int oracle_get_nmax(oracle_ctx* ctx, int* nmax);
int oracle_get_bessel(oracle_ctx* ctx, int is, double* out);
int oracle_disp(oracle_ctx* ctx, alps_complex om, alps_complex* D,
                alps_complex* chi0, alps_complex* chi0_low,
                alps_complex* wave);
/* Per species and entry, the sum over Bessel orders of |contribution| (times
 * |n_s q_s|), i.e. the scale of the rounding error of chi_ij under any
 * summation order: mag[s*9 + 3*i + j]. */
int oracle_disp_mag(oracle_ctx* ctx, alps_complex om, double* mag);
int oracle_disp_batch(oracle_ctx* ctx, int n, const alps_complex* om,
                      alps_complex* D, int nthreads);
int oracle_full_integrate(oracle_ctx* ctx, int is, alps_complex om, int nn,
                          int mode, alps_complex* out, int* resonant);
int oracle_int_ee(oracle_ctx* ctx, int is, alps_complex om, alps_complex* out);
int oracle_secant(oracle_ctx* ctx, int method, alps_complex* om, int* iters,
                  alps_complex* Dfinal);
int oracle_map(oracle_ctx* ctx, const alps_map_params* mp, alps_complex* om,
               alps_complex* cal, double* val, int nthreads);
int oracle_find_minima(const double* val, int nr, int ni, int numroots,
                       int* iroots, int* nfound);

/* om_scan for one scan definition: rows[(it*nroots + in)*4 + {kperp,kpar,
 * re, im}] for it = 0..ns (row 0 is the starting point).  wroots is updated
 * in place.  Returns ALPS_E_ROOTS_DIVERGED like alps_error(9). */
typedef struct oracle_scan_def {
  int type_s;      /* 0..4 */
  double swi, swf;
  int log_scan;
  int n_out, n_res;
  int eigen, heat; /* calc_eigen on every output row (eig[it*nroots + in]) */
} oracle_scan_def;
int oracle_scan(oracle_ctx* ctx, const oracle_scan_def* sd, int nroots,
                alps_complex* wroots, double* rows, alps_eigen* eig);

/* calc_eigen (src/ALPS_fns.f90:2605-2899) at one root, including the det D
 * evaluations at om, Re(om) and Re(om*1.000001) that the reference makes
 * around it. */
int oracle_calc_eigen(oracle_ctx* ctx, alps_complex om, int eigen, int heat,
                      alps_eigen* out);

double oracle_bessj(int n, double x);
/* exp(-x) I_n(x) and the Faddeeva function of the NHDS branch
 * (src/ALPS_NHDS.f90:537-862); oracle_wofz returns its overflow flag. */
double oracle_bessi_scaled(int n, double x);
/* interpolation/interpolation.f90: thin-plate spline of log f through n
 * samples with smoothing, on the fine grid [(nperp+1)*(npar+1)], normalised
 * if asked, times mult_f. */
int oracle_interpolate(const double* pperp_c, const double* ppar_c, const double* f_c, int n, int nperp, int npar,
                       double smoothing, double pperp_min, double pperp_max, double ppar_min, double ppar_max,
                       int do_normalize, double mult_f, double* f_out);
int oracle_wofz(double x, double y, double* u, double* v);
/* Threads used inside one disp() call (orders in parallel, summed in the
 * reference's order).  Default 1. */
void oracle_set_threads(int n);
int oracle_generate_f0(const alps_dist_params* dp, int nperp, int npar,
                       double* pperp, double* ppar, double* f0,
                       double* ideal);

#ifdef __cplusplus
}
#endif
#endif
