/*
 * alps_gb300.h -- C-ABI of the GB300-native dispersion-tensor library.
 *
 * This is the drop-in boundary beneath ALPS's disp()/root-search call surface.
 * ALPS keeps all state in module globals (src/ALPS_var.f90:19-427) and calls
 * module procedures; each entry point below replaces one of those procedures
 * (cited per function).  Every call takes plain pointers and sizes; device
 * state lives inside an opaque context, one context per plasma.
 *
 * Array conventions:
 *   - complex values are {re, im} pairs of doubles (alps_complex), layout
 *     compatible with Fortran `double complex` and C99 `double _Complex`;
 *   - momentum grids are passed per species as (nperp+1)*(npar+1) arrays in
 *     the order of the ALPS f0 table files (iperp outer, ipar inner,
 *     src/ALPS_io.f90:679-684), i.e. index iperp*(npar+1)+ipar;
 *   - tensors are 3x3 row-major: chi[s*9 + 3*i + j] = chi(s, i+1, j+1);
 *     chi_low[s*27 + 9*(n+1) + 3*i + j] = chi_low(s, i+1, j+1, n), n=-1..1.
 *   - species indices are 0-based.
 *
 * Errors: every int-returning function returns ALPS_OK or a status code.
 * Codes 1..11 mirror the reference's fatal alps_error ids
 * (src/ALPS_io.f90:937-1012); the reference aborts the MPI job on those, this
 * library returns them instead.  Device code never traps.
 */
#ifndef ALPS_GB300_H
#define ALPS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ALPS_MAX_FITS 4

/* ---- status codes ---------------------------------------------------- */
enum {
  ALPS_OK = 0,
  ALPS_E_NAMELIST = 1,        /* alps_error(1): required namelist not found   */
  ALPS_E_FIT_POINTS = 2,      /* alps_error(2): more fit parameters than data */
  ALPS_E_SCAN_OPTION = 3,     /* alps_error(3): bad scan_option               */
  ALPS_E_NSCAN = 4,           /* alps_error(4): n_scan != 2 for double scan   */
  ALPS_E_SCAN_SAME_TYPE = 5,  /* alps_error(5)                                */
  ALPS_E_SCAN_TYPE0 = 6,      /* alps_error(6)                                */
  ALPS_E_FIT_FAILED = 7,      /* alps_error(7): fit for continuation failed   */
  ALPS_E_SUBLUMINAL = 8,      /* alps_error(8)                                */
  ALPS_E_ROOTS_DIVERGED = 9,  /* alps_error(9): all roots diverged            */
  ALPS_E_POLY_KIND = 10,      /* alps_error(10): unknown polynomial basis     */
  ALPS_E_NPROC = 11,          /* alps_error(0): bad MPI rank count            */
  ALPS_E_INVALID = 20,        /* bad argument / call order                    */
  ALPS_E_CUDA = 21,           /* CUDA runtime error                           */
  ALPS_E_OOM = 22,            /* device allocation failed                     */
  ALPS_E_TIMEOUT = 23,        /* a bounded device wait ran out                */
  ALPS_E_UNSUPPORTED = 24,    /* feature not implemented in this library      */
  ALPS_E_GRID = 25,           /* grid is not a uniform tensor-product grid    */
  ALPS_E_SINGULAR = 26,       /* fit matrix singular (reference: `stop`)      */
  ALPS_E_IO = 27,             /* file input/output failed                     */
  ALPS_E_NO_DEVICE = 28       /* no CUDA device / extension unusable          */
};

typedef struct alps_complex {
  double re, im;
} alps_complex;

/* &system namelist (src/ALPS_io.f90:66-71, defaults src/ALPS_var.f90). */
typedef struct alps_system {
  int nspec;
  int nperp, npar;
  double kperp, kpar;
  double vA;
  double Bessel_zero;
  int kperp_norm;             /* logical                                      */
  int positions_principal;    /* M_I                                          */
  int n_resonance_interval;   /* M_P                                          */
  double Tlim;
  int secant_method;          /* 0 secant, 1 rtsec, 2 secant_osc              */
  int numiter;
  double D_threshold, D_prec, D_gap, D_tol;
  int maxsteps_fit;
  double lambda_initial_fit, lambdafac_fit, epsilon_fit;
  /* MPI rank count whose nmax adjustment (src/ALPS_fns.f90:4048-4071) is to
   * be reproduced; 0 means no adjustment. */
  int nproc;
  /* (Gamma, pparbar) grid of relativistic species (src/ALPS_var.f90:128-132) */
  int ngamma, npparbar;
} alps_system;

/* &spec_i, &ffit_i_j, &poly_spec_i, &bM_spec_i (src/ALPS_io.f90:302-419,
 * 563-596). */
typedef struct alps_species {
  double ns, qs, ms;
  int ac_method;              /* 0 analytic, 1 fitted functions, 2 Chebyshev */
  int n_fits;
  int relat, log_fit, use_bM;
  int fit_type[ALPS_MAX_FITS];
  double fit_init[ALPS_MAX_FITS][5];
  double perp_correction[ALPS_MAX_FITS];
  int poly_kind, poly_order;
  double poly_log_max;
  int bM_nmaxs;
  double bM_Bessel_zeros, bM_betas, bM_alphas, bM_pdrifts;
} alps_species;

/* Default &system values (src/ALPS_var.f90:83-314). */
void alps_system_defaults(alps_system* sys);
void alps_species_defaults(alps_species* sp);

typedef struct alps_ctx alps_ctx;

/* Library build tag and the device the context would use. */
const char* alps_version(void);
const char* alps_error_string(int status);

/* Creates a context on the current CUDA device.
 * Replaces init_param (src/ALPS_io.f90:46-277) + pass_instructions
 * (src/ALPS_com.f90:28-204): the parameters are copied into the context. */
int alps_create(const alps_system* sys, alps_ctx** out);
void alps_destroy(alps_ctx* ctx);

/* Loads one species' grid and f0 table (host arrays, (nperp+1)*(npar+1)).
 * Replaces read_f0 (src/ALPS_io.f90:643-692) + pass_distribution
 * (src/ALPS_com.f90:208-284).  The grid must be a uniform tensor-product grid
 * (pperp depends on iperp only, ppar on ipar only), as the reference assumes
 * (src/ALPS_fns.f90:835-836, 4244); ALPS_E_GRID otherwise. */
int alps_set_species(alps_ctx* ctx, int is, const alps_species* sp,
                     const double* pperp, const double* ppar, const double* f0);

/* Per-run preprocessing on the device: central-difference derivatives,
 * Levenberg-Marquardt fits for the analytic continuation, ee term.
 * Replaces derivative_f0 (src/ALPS_fns.f90:34-248) and determine_param_fit
 * (src/ALPS_analyt.f90:365-728). */
int alps_prepare(alps_ctx* ctx);

/* Reads back the fitted continuation parameters of species is:
 * out[(iperp*5 + ip)*n_fits + ifit], iperp=0..nperp (param_fit of
 * src/ALPS_var.f90:276). */
int alps_get_fit(alps_ctx* ctx, int is, double* out);

/* Replaces the fitted parameters of species is (same layout as
 * alps_get_fit), e.g. to share one fit between two evaluators.  No reference
 * counterpart: there the fit lives in the param_fit global. */
int alps_set_fit(alps_ctx* ctx, int is, const double* in);

/* The (Gamma, pparbar) grid of a relativistic species after alps_prepare:
 * gamma[ngamma+1], pparbar[npparbar+1], and f0_rel (-1 outside the
 * subluminal cone), df0_rel/dGamma, df0_rel/dpparbar on
 * [(igamma)*(npparbar+1) + ipparbar].  The tables the reference writes to
 * distribution/<arrayName>_f0_rel.<is>.array and _df0_rel.<is>.array
 * (derivative_f0_rel, src/ALPS_fns_rel.f90:211-289).  Any pointer may be
 * NULL.  ALPS_E_INVALID for a non-relativistic species. */
int alps_get_f0_rel(alps_ctx* ctx, int is, double* gamma, double* pparbar, double* f0_rel, double* df_dgamma,
                    double* df_dpparbar);

/* alps_prepare for n contexts at once (the per-run setup of many plasmas,
 * e.g. of an uneven batch or a request server's pool).  The
 * Levenberg-Marquardt continuation fits of every (context, species) run in
 * one launch, one warp each: the reference's warm start over the p_perp
 * rows orders a fit (src/ALPS_analyt.f90:518), but the fits of different
 * plasmas and species are independent.  Derivatives and ee terms of all
 * contexts run on a few streams; one synchronisation in all.  Contexts
 * with relativistic species or Chebyshev continuations are prepared one by
 * one.  The results are those of alps_prepare on each context.  status[i]
 * (may be NULL) receives each context's status; returns the first error. */
int alps_prepare_many(alps_ctx* const* ctx, int n, int* status);

/* Per-wavevector setup on the device: nmax from the Bessel cutoff, Bessel
 * table, and the omega-independent p_perp contraction.
 * Replaces determine_nmax + determine_bessel_array
 * (src/ALPS_fns.f90:3971-4075, 4214-4255); split_processes
 * (src/ALPS_fns.f90:4079-4207) has no counterpart: one device does all n.
 * The tables depend on kperp alone: a call that keeps the context's kperp
 * bit for bit (a k_par scan step) keeps them and moves k_par only, as
 * om_scan does for scan type 4 (src/ALPS_fns.f90:2465-2471);
 * alps_stats.k_reused counts such calls. */
int alps_set_k(alps_ctx* ctx, double kperp, double kpar);
int alps_get_nmax(alps_ctx* ctx, int* nmax /* [nspec] */);

/* alps_set_k for n contexts at once, context i at (kperp[i], kpar[i]):
 * determine_nmax for every species of every context in one launch, then
 * the Bessel tables and contractions of all contexts on a few streams with
 * one synchronisation.  Contexts whose kperp stays keep their tables.  The
 * results are those of alps_set_k on each context.  status[i] (may be
 * NULL) as in alps_prepare_many. */
int alps_set_k_many(alps_ctx* const* ctx, int n, const double* kperp,
                    const double* kpar, int* status);

/* Evaluation mode of the omega pass.
 * ALPS_PREC_FP64 (plain): every p_par pole sum is the trapezoid node sum of
 *   the reference, in FP64 (the parity path).
 * ALPS_PREC_MIXED (fast): for non-resonant orders whose pole lies well
 *   outside the p_par grid the node sum is replaced by its Laurent series
 *   about the grid centre, truncated where the remainder is below FP64
 *   rounding (rho^K <= 2^-53 (1-rho)); one-Maxwellian Landau rows are
 *   factorised where their deviation bound is below 1e-5; the node sums,
 *   series terms and principal-value sums run in double-float arithmetic
 *   (float pairs, about 46-48 bits).  Resonance decisions, windows and
 *   sample points are the reference's in both modes; results agree with the
 *   plain mode to about 1e-10 in det D on the benchmark map. */
enum { ALPS_PREC_FP64 = 0, ALPS_PREC_MIXED = 1 };
int alps_set_precision(alps_ctx* ctx, int precision);

/* det D(omega,k) for one omega, with the side results of the reference's
 * disp(): chi0 (S x 3 x 3), chi0_low (S x 3 x 3 x {-1,0,1}) and wave (3x3).
 * Any of chi0/chi0_low/wave may be NULL.
 * Replaces disp (src/ALPS_fns.f90:252-636). */
int alps_disp(alps_ctx* ctx, alps_complex om, alps_complex* D,
              alps_complex* chi0, alps_complex* chi0_low, alps_complex* wave);

/* det D for n frequencies from host memory (copies in the call). */
int alps_disp_batch(alps_ctx* ctx, int n, const alps_complex* om,
                    alps_complex* D);

/* det D for n frequencies already in device memory; stream is a
 * cudaStream_t (NULL = the context's stream).  Asynchronous. */
int alps_disp_batch_device(alps_ctx* ctx, int n, const alps_complex* d_om,
                           alps_complex* d_D, void* stream);

/* det D for n frequencies in device memory, allocating nothing.
 * No counterpart in the reference; it exists for callers that cannot let a
 * library allocate device memory while they run (an application whose own
 * caching allocator must own the whole device heap, a real-time loop that
 * cannot absorb the device-wide synchronisation of cudaMalloc/cudaFree, a
 * plugin host that forbids allocations by plugins).  Same kernels and results
 * as alps_disp_batch_device; the scratch they need comes from one static
 * 16 MiB device array per device (held until the process exits).  The first
 * call on a device looks up that array's address (cudaGetSymbolAddress) with
 * the device current; make it before any stream capture.  All calls share
 * the array: calls that overlap on the GPU race and must be serialised by the
 * caller.  Batches whose scratch would exceed 16 MiB return ALPS_E_INVALID
 * without launching; *scratch_bytes (may be NULL) receives the bytes the
 * batch needs.  stream: cudaStream_t, NULL = the context's stream. */
int alps_disp_batch_noalloc(alps_ctx* ctx, int n, const alps_complex* d_om,
                            alps_complex* d_D, void* stream,
                            size_t* scratch_bytes);

/* Device error status of the last asynchronous batch of this context
 * (alps_disp_batch_device or alps_disp_batch_noalloc).  Waits for stream
 * (cudaStream_t, NULL = the context's stream), then reads the batch's device
 * error word: ALPS_OK, ALPS_E_SUBLUMINAL (a relativistic resonance window
 * covered the whole subluminal cone: alps_error(8), src/ALPS_io.f90:982-988,
 * raised in integrate_resU_rel, src/ALPS_fns_rel.f90:656) or
 * ALPS_E_INVALID (resonant-order slots overflowed).  The reference aborts
 * the MPI job on alps_error; the synchronous entry points return these codes
 * directly, the asynchronous ones through this call.  It allocates nothing.
 * For alps_disp_batch_noalloc the word sits in the shared static scratch:
 * read the status before the next no-allocation call on the device. */
int alps_batch_status(alps_ctx* ctx, void* stream);

/* Root polishing of nroots guesses in place (om[], host memory).
 * method: 0 secant (src/ALPS_fns.f90:1815-1917), 1 rtsec (:2105-2195),
 * 2 secant_osc (:1919-2101).  iters[r] (may be NULL) receives the number of
 * iterations; Dfinal[r] (may be NULL) the det at the returned root.
 * All roots advance together: each iteration evaluates every active root's
 * det in one batched launch. */
int alps_secant(alps_ctx* ctx, int method, int nroots, alps_complex* om,
                int* iters, alps_complex* Dfinal);

/* alps_secant with a relative-step stop and a converged mask.  With
 * om_rtol > 0 a root also stops once its secant update is at most
 * om_rtol |om| (the update applied): a polish criterion independent of the
 * scale of det D, whose size keeps the reference's absolute D_threshold out
 * of reach for many roots.  om_rtol = 0 gives exactly alps_secant.
 * converged[r] (may be NULL) is 1 when a stopping rule ended root r, 0 when
 * numiter ran out (the reference then returns the best-|D| iterate,
 * src/ALPS_fns.f90:2093-2099).  No reference counterpart for om_rtol. */
int alps_secant_ex(alps_ctx* ctx, int method, int nroots, alps_complex* om,
                   double om_rtol, int* iters, alps_complex* Dfinal,
                   int* converged);

/* Root polishing of n roots, root r on its own context ctx[r] (its own
 * plasma and k: species, grids and nmax may differ from root to root; a
 * context may appear more than once), entirely on the device.
 * Replaces refine_guess's per-root secant loop (src/ALPS_fns.f90:3793-3856
 * over secant_osc :1919-2101, secant :1815-1917 or rtsec :2105-2195): the
 * root-finder state machines live in device memory, every round is one
 * fused det D launch over all roots' pending frequencies followed by a
 * device step of every machine, and the rounds repeat inside one CUDA graph
 * (a conditional WHILE node ends it when no root is active), so no round
 * waits on the host.  Each root's determinants use the launch shape of a
 * lone batch of two frequencies on its context, so a root's iterates and
 * result are bit for bit the same alone and in any batch.  om_rtol,
 * converged, iters and Dfinal as in alps_secant_ex.  Contexts with
 * relativistic or closed-form species return ALPS_E_UNSUPPORTED (use
 * alps_secant_ex).  Synchronous. */
int alps_solve_many(alps_ctx* const* ctx, int n, int method, alps_complex* om,
                    double om_rtol, int* iters, alps_complex* Dfinal,
                    int* converged);

/* Eigenfunctions and heating rates of roots (calc_eigen,
 * src/ALPS_fns.f90:2605-2899).  Fields are relative to E_x; velocities and
 * densities per species; Ps the heating rate per species over the wave
 * energy ewave (W_EM); Ps_split per species: [0] transit-time damping (the
 * n = 0 yy and yz terms), [1] Landau damping (n = 0 zy and zz), [2] n = +1
 * and [3] n = -1 cyclotron terms with E_z removed.  As in the reference,
 * electric/magnetic/vmean/ds come from det D at the complex root, Ps from
 * det D at Re(om), and ewave and Ps_split from det D at Re(om)*1.000001
 * (the last evaluation of the reference's sequence). */
#define ALPS_EIGEN_MAX_SPECIES 8
typedef struct alps_eigen {
  alps_complex electric[3];
  alps_complex magnetic[3];
  alps_complex vmean[ALPS_EIGEN_MAX_SPECIES][3];
  alps_complex ds[ALPS_EIGEN_MAX_SPECIES];
  double Ps[ALPS_EIGEN_MAX_SPECIES];
  double Ps_split[ALPS_EIGEN_MAX_SPECIES][4];
  double ewave;
} alps_eigen;

/* calc_eigen for n roots at once: all det D evaluations (n, or 3n with
 * heat) go to the device in one batch.  eigen / heat select the outputs
 * like the scan flags eigen_s / heat_s; with heat = 0 Ps, Ps_split and
 * ewave are zero, with eigen = 0 vmean and ds are zero.  The parallel flow
 * U_s = current_int/(n_s q_s) of each species is the p_par moment of its f0
 * table (derivative_f0, src/ALPS_fns.f90:157-190). */
int alps_calc_eigen(alps_ctx* ctx, int n, const alps_complex* om, int eigen,
                    int heat, alps_eigen* out);

/* Complex-frequency map (map_search, src/ALPS_fns.f90:3595-3788, without the
 * file output): om[ir*ni+ii], cal = det D with NaN/Inf sentinels, val =
 * log10|D| with sentinels.  Any output pointer may be NULL. */
typedef struct alps_map_params {
  double omi, omf, gami, gamf;
  int nr, ni;
  int loggridw, loggridg;
} alps_map_params;
int alps_map(alps_ctx* ctx, const alps_map_params* mp, alps_complex* om,
             alps_complex* cal, double* val);

/* Strict 4-neighbour minima of val[ir*ni+ii] in the reference's scan order
 * (find_minima, src/ALPS_fns.f90:3860-3966).  iroots holds (ir,ii) pairs,
 * 0-based; returns the count in *nfound.  Host-only. */
int alps_find_minima(const double* val, int nr, int ni, int numroots,
                     int* iroots, int* nfound);

/* Contents of an ALPS input file (the namelists read by init_param,
 * src/ALPS_io.f90:46-552): &system, &guess_i or &maps_1, &spec_i,
 * &ffit_i_j, &poly_spec_i, &bM_spec_i, &scan_input_i. */
#define ALPS_MAX_ROOTS 100
#define ALPS_MAX_SCANS 8
#define ALPS_MAX_INPUT_SPECIES 8
typedef struct alps_scan_def {
  int type_s;                 /* scan_type 0..4                               */
  double swi, swf;
  int log_scan;               /* swlog                                        */
  int n_out, n_res;           /* ns, nres                                     */
  int heating, eigen;
  double diff, diff2;         /* step sizes of scan_read (:426-552)           */
} alps_scan_def;
typedef struct alps_input {
  alps_system sys;
  alps_species species[ALPS_MAX_INPUT_SPECIES];
  char runname[256], arrayName[256];
  int nroots, use_map, determine_minima, scan_option, n_scan;
  int ngamma, npparbar, writeOut;
  alps_complex guess[ALPS_MAX_ROOTS];
  alps_map_params map;
  alps_scan_def scan[ALPS_MAX_SCANS];
} alps_input;

/* ------------------------------------------------------------------------
 * Request server: continuous batching of root solves, k scans and maps on
 * many plasmas.  No reference counterpart (the reference runs one plasma
 * per MPI job); each request does what the named reference driver does for
 * its plasma.
 *
 * A background thread drives the active requests.  The pending root-finder
 * evaluations of every ready plasma go into one fused launch (a round; two
 * rounds stay in flight); lattices, and plasmas with relativistic or
 * closed-form species, launch their own batch on their context's stream.
 * As a batch lands the determinants go back into the requests' root
 * finders and their next evaluations join the next round, so no request
 * waits for a slower one.  The k steps of scans run on worker threads.
 * Requests that arrive while others run are admitted as soon as their
 * estimated device footprint (the context's tables and the largest batch
 * they will launch) fits the budget.  The k steps of all scans that are ready
 * for one go to the device together (alps_set_k_many).  A fused launch evaluates each plasma
 * with the launch shape of a lone batch of its size, so every result is
 * bit for bit what the request gives alone, whatever else is in flight.
 * A map's lattice goes to the device in chunks of 2048 frequencies, with
 * the other requests' rounds launched between chunks: a lattice of at most
 * 2048 points equals alps_map bit for bit; a larger one is evaluated in
 * chunk-sized batches (the same values up to the last bits of the sums,
 * whose order follows the batch size).
 * ------------------------------------------------------------------------ */
typedef struct alps_server alps_server;

#define ALPS_REQ_POLISH 0  /* refine_guess: polish n roots (secant method of the context) */
#define ALPS_REQ_MAP 1     /* map_search lattice: det D with the reference's sentinels   */
#define ALPS_REQ_SCAN 2    /* om_scan: k steps with root following                       */

typedef struct alps_request {
  int kind;                 /* ALPS_REQ_*                                                 */
  alps_ctx* ctx;            /* prepared plasma with k set; one request at a time per ctx */
  int n;                    /* POLISH, SCAN: number of roots                               */
  alps_complex* om;         /* POLISH, SCAN: guesses in, roots out (host memory)           */
  int* iters;               /* POLISH: iterations per root (may be NULL)                   */
  alps_map_params map;      /* MAP                                                        */
  alps_complex* map_cal;    /* MAP out: nr*ni det D with sentinels (may be NULL)           */
  double* map_val;          /* MAP out: nr*ni log10 |det D| with sentinels (may be NULL)   */
  alps_scan_def scan;       /* SCAN: type, steps and diff/diff2 as alps_read_input sets    */
  double* scan_rows;        /* SCAN out: [(n_out+1) * n * 4] kperp, kpar, Re, Im           */
  int status;               /* out: ALPS_OK or an error code                               */
  double latency_ms;        /* out: submit to completion                                   */
  int rounds;               /* out: batches the request launched                           */
  double om_rtol;           /* POLISH, SCAN: relative-step stop of alps_secant_ex, 0 = the
                               reference's stopping rule only                              */
  int* converged;           /* POLISH out: 1 where the root met a stopping rule before
                               numiter (may be NULL)                                       */
} alps_request;

/* hbm_budget: bytes of device memory requests may hold at once (0: 90 % of
 * the free memory at creation); max_active: requests in flight (0: 256). */
int alps_server_create(size_t hbm_budget, int max_active, alps_server** out);
/* Waits for every submitted request, then stops the thread. */
void alps_server_destroy(alps_server* srv);
/* Queues a request (the struct and its buffers must stay valid until it is
 * done) and returns its id. */
int alps_server_submit(alps_server* srv, alps_request* req, int64_t* id);
/* *done = 1 once the request has finished (its status and outputs are set). */
int alps_server_poll(alps_server* srv, int64_t id, int* done);
/* Blocks until the request has finished; returns its status. */
int alps_server_wait(alps_server* srv, int64_t id);
/* Batches launched, peak requests in flight and peak estimated footprint so
 * far. */
int alps_server_stats(alps_server* srv, int64_t* rounds, int* peak_active, size_t* peak_bytes);
/* Where the server's time goes, summed since creation: fused rounds
 * launched and the plasma batches (jobs) in them, with the device span of
 * each round from its frequency upload to its result download; batches run
 * on a context's own stream (maps, plasmas the fused kernels do not take);
 * scan k-step batches (one alps_set_k_many over the scans ready together)
 * with the steps in them and their wall time; and the host time of the
 * server loop outside its idle waits, of which admission, landing rounds
 * (root-machine steps), the pass over the groups (own-stream launches and
 * landings, releases) and launching rounds (job tables, uploads). */
typedef struct alps_server_profile {
  int64_t rounds, round_jobs, group_batches, scan_step_batches, scan_steps;
  double round_gpu_ms, step_ms, loop_busy_ms, admit_ms, land_ms, groups_ms, round_launch_ms;
} alps_server_profile;
int alps_server_get_profile(alps_server* srv, alps_server_profile* out);

/* Parses an ALPS input file (init_param + scan_read, src/ALPS_io.f90:46-552):
 * defaults of src/ALPS_var.f90, Fortran literals (1.d-2, .true., T, 'str'),
 * `!` comments.  Missing required namelists return ALPS_E_NAMELIST. */
int alps_read_input(const char* path, alps_input* in);

/* Reads one f0 table file (read_f0, src/ALPS_io.f90:643-692): (nperp+1)*(npar+1)
 * lines "pperp ppar f0", iperp outer. */
int alps_read_f0(const char* path, int nperp, int npar, double* pperp,
                 double* ppar, double* f0);

/* Runs a whole ALPS input file (the main program src/ALPS.f90:19-147): map
 * search or guesses, refine_guess, and the k scans (scan_option 1), reading
 * f0 tables from <workdir>/distribution/<arrayName>.<is>.array and writing
 * <workdir>/solution/<runname>.roots, .map, .scan_<id><ik>.root_<in> and,
 * for scans with eigen / heating, .eigen_*, .heat_* and .heat_mech_* in the
 * reference's formats (src/ALPS_fns.f90:2346-2584, 3745, 3849). */
int alps_run_input(const char* input_path, const char* workdir);

/* f0 table generator (distribution/generate_distribution.f90:176-300):
 * kind 0 distribution_analyt (the reference's example function of species
 * 1 and 2, no normalisation, maxPperp/maxPpar as given), 1 bi-Maxwellian,
 * 2 bi-kappa, 3 Juettner, 4 bi-Moyal.  Writes
 * (nperp+1)*(npar+1) values into pperp/ppar/f0 and, if ideal!=NULL, the
 * "ideal" fit parameters {fit_1..fit_5, perpcorr}.  Host-only. */
typedef struct alps_dist_params {
  int kind;
  double ms, tau, alph, p_drift, kappa;
  double beta, vA, maxP;
  int autoscale;
  double maxPperp, maxPpar;
  double kappa1;              /* kappa of species 1 (autoscale of bi-kappa) */
  int species;                /* 1-based species index (kind 0)              */
} alps_dist_params;
int alps_generate_f0(const alps_dist_params* dp, int nperp, int npar,
                     double* pperp, double* ppar, double* f0, double* ideal);

/* The interpolation tool (interpolation/interpolation.f90): thin-plate
 * spline of log f through n scattered samples (coordinates already scaled by
 * mult_pperp / mult_ppar), the smoothing added on the diagonal of the spline
 * system, evaluated on the fine grid pperp_min + (pperp_max - pperp_min) i /
 * nperp by ppar_min + (ppar_max - ppar_min) j / npar.  With do_normalize the
 * result is divided by 2 pi sum_ij f pperp dpperp dppar (normalize,
 * interpolation.f90:520-552); the output is mult_f times it.  Outputs
 * [(nperp+1)*(npar+1)], i outer, as the reference writes its .array file
 * (any pointer may be NULL).  Solved and evaluated on the device.
 * ALPS_E_INVALID for f <= 0, n < 1 or nperp, npar < 2; ALPS_E_SINGULAR if
 * the system is. */
typedef struct alps_interp_params {
  int nperp, npar;
  double smoothing;
  double pperp_min, pperp_max, ppar_min, ppar_max;
  int do_normalize;
  double mult_f;
} alps_interp_params;
int alps_interpolate(const double* pperp_c, const double* ppar_c, const double* f_c, int n,
                     const alps_interp_params* p, double* pperp_out, double* ppar_out, double* f_out);
/* The whole program: reads the &system namelist of input_path (filename,
 * mode, threshold, smoothing, nperp, npar, p*_min_set / p*_max_set,
 * out_to_file, do_normalize, mult_pperp, mult_ppar, mult_f, with the
 * reference's defaults; empty values keep them), reads the coarse table
 * (relative paths from the input file's folder), and writes
 * <workdir>/<input name without .in>.array (out_to_file) or the same lines
 * to stdout. */
int alps_run_interpolation(const char* input_path, const char* workdir);

/* FP64-accurate dense product C = A B of row-major device arrays (A M x K,
 * B K x N, C M x N, K <= 256) on the BF16 tensor cores: the engine of the
 * mixed path's p_perp contraction.  Each row of A and column of B is split
 * into seven 8-bit slices of its own power-of-two scale (the Ozaki splitting);
 * the 28 leading slice products run as tcgen05.mma with FP32 accumulators in
 * tensor memory, exact integers up to the levels that carry FP64's precision.
 * checked = 1: B's rows are first scaled to unit size (A's columns by the
 * inverse), and every entry whose error bound exceeds 2^-44 sum_k |A B| (the
 * size of FP64 GEMM's own worst-case rounding bound) is recomputed in FP64;
 * *nfixed (may be NULL) receives their number.  checked = 0: the bare
 * product, error at most 10 K 2^-56 times the product of the row's and
 * column's power-of-two scales.  Synchronous; allocates its workspace.
 * No reference counterpart (a building block, exported for its tests). */
int alps_tc_product(const double* d_A, const double* d_B, double* d_C, int M,
                    int N, int K, int checked, int* nfixed);

/* Autotuner of the batch kernels' launch shapes.  Times the candidate
 * shapes of a batch of n frequencies on this context (its k and precision
 * path): j slices per frequency of the pole sums (1, 2, 4, 8, 16, 32) x
 * pole-sum blocks per SM (2, 4, 8) x resonant-item warps per SM (6, 12, 24),
 * each the best of two launches after a warm-up.  The fastest (if 3 % faster
 * than the default rule) is kept for every batch of the same bucket: N_perp,
 * N_par, nmax + 1 and n each rounded up to a power of two, species count
 * and precision path.  d_om: n device frequencies to tune on, or NULL for a
 * lattice over Re in [0.05, 2.5], Im in [-0.4, 0.05].  A shape changes the
 * summation order of the pole sums only (results move by rounding); lone,
 * fused and no-allocation batches of a bucket use the same shape.  No
 * reference counterpart: ALPS has one fixed loop order. */
typedef struct alps_tune_result {
  int js, blocks_per_sm, warps_per_sm; /* the shape the bucket now uses          */
  int tuned;                           /* 1: a candidate beat the default rule   */
  int candidates;                      /* shapes timed                           */
  double ms_default, ms_best;          /* per batch: default rule, chosen shape  */
} alps_tune_result;
int alps_autotune(alps_ctx* ctx, int n, const alps_complex* d_om, alps_tune_result* out);
/* Forgets every tuned shape (all buckets return to the default rule). */
int alps_tune_clear(void);

/* Device work counters of the last disp batch (for measurement). */
typedef struct alps_stats {
  int64_t n_eval;             /* frequencies evaluated                        */
  int64_t n_pole_terms;       /* (omega, n, j) terms of the non-resonant sums */
  int64_t n_resonant;         /* resonant (omega, species, n) work items      */
  int64_t n_landau;           /* of which with a Landau term                  */
  int kernels_launched;       /* kernels launched by the last disp batch      */
  int64_t graph_replays;      /* server batches replayed from a CUDA graph    */
  int64_t graph_captures;     /* server batches captured into a CUDA graph    */
  /* the p_perp contraction of the last alps_set_k: species whose product
   * ran on the tensor cores (mixed path), and of their entries those whose
   * error bound sent them to the FP64 recompute */
  int tc_contractions;
  int64_t tc_fixed_entries;
  int64_t tc_entries;
  int64_t n_eval_total;       /* frequencies evaluated since the context was created */
  int64_t k_reused;           /* k steps that kept k_perp and with it the k tables */
} alps_stats;
int alps_get_stats(alps_ctx* ctx, alps_stats* st);

/* Measurement support: when on, every disp batch records CUDA events around
 * its four kernels (classify, pole sums, resonant items, finalize) on the
 * stream it runs on; alps_get_profile returns the summed device milliseconds
 * per kernel and the number of batches since profiling was switched on. */
int alps_set_profiling(alps_ctx* ctx, int on);
int alps_get_profile(alps_ctx* ctx, double* ms /* [4] */, int64_t* batches);

#ifdef __cplusplus
}
#endif
#endif /* ALPS_GB300_H */
