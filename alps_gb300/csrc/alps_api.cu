// alps_api.cu -- the extern "C" entry points declared in include/alps_gb300.h.
//
// Host-side orchestration only: argument checks, device buffers, and the
// root finders' control flow.  Every det D evaluation runs on the device
// through launch_disp_batch (disp_kernels.cu); there is no host fallback.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "alps_internal.cuh"
#include "root_finders.h"
#include "tc_gemm.cuh"

namespace {
thread_local char g_last_err[512] = "";
typedef std::complex<double> cplx;
inline cplx C(const double2& v) { return cplx(v.x, v.y); }
inline double2 D2(const cplx& v) { return make_double2(v.real(), v.imag()); }
}  // namespace

void alps_set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
  snprintf(g_last_err, sizeof(g_last_err), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}

extern "C" {

const char* alps_version(void) { return "alps_gb300 0.1 (sm_103a)"; }

const char* alps_error_string(int st) {
  switch (st) {
    case ALPS_OK: return "ok";
    case ALPS_E_NAMELIST: return "required input namelist not found";
    case ALPS_E_FIT_POINTS: return "more fit parameters than data points";
    case ALPS_E_SCAN_OPTION: return "scan_option not set to allowable value";
    case ALPS_E_NSCAN: return "n_scan .ne. 2 for scan_option=2";
    case ALPS_E_SCAN_SAME_TYPE: return "scan(1)%type_s==scan(2)%type_s for double k scan";
    case ALPS_E_SCAN_TYPE0: return "scan(*)%type_s=0 not allowed for double k scan";
    case ALPS_E_FIT_FAILED: return "fit for analytical continuation failed";
    case ALPS_E_SUBLUMINAL: return "resonance integration covers entire subluminal cone";
    case ALPS_E_ROOTS_DIVERGED: return "all roots diverged";
    case ALPS_E_POLY_KIND: return "unspecified orthogonal representation";
    case ALPS_E_NPROC: return "number of processors must be even and greater than 2";
    case ALPS_E_INVALID: return "invalid argument or call order";
    case ALPS_E_CUDA: return g_last_err[0] ? g_last_err : "CUDA error";
    case ALPS_E_OOM: return "device memory allocation failed";
    case ALPS_E_TIMEOUT: return "device wait timed out";
    case ALPS_E_UNSUPPORTED: return "feature not supported by this library";
    case ALPS_E_GRID: return "grid is not a uniform tensor-product grid";
    case ALPS_E_SINGULAR: return "fit matrix is numerically singular";
    case ALPS_E_IO: return "file input/output failed";
    case ALPS_E_NO_DEVICE: return "no usable CUDA device";
  }
  return "unknown status";
}

void alps_system_defaults(alps_system* s) {
  memset(s, 0, sizeof(*s));
  s->nspec = 1;
  s->Bessel_zero = 1.0e-45;
  s->kperp_norm = 1;
  s->positions_principal = 5;
  s->n_resonance_interval = 100;
  s->Tlim = 0.01;
  s->secant_method = 2;
  s->numiter = 50;
  s->D_threshold = 1.0e-5;
  s->D_prec = 1.0e-5;
  s->D_gap = 1.0e-5;
  s->D_tol = 1.0e-7;
  s->maxsteps_fit = 500;
  s->lambda_initial_fit = 1.0;
  s->lambdafac_fit = 10.0;
  s->epsilon_fit = 1.0e-8;
  s->ngamma = 100;
  s->npparbar = 200;
}

void alps_species_defaults(alps_species* sp) {
  memset(sp, 0, sizeof(*sp));
  sp->ns = sp->qs = sp->ms = 1.0;
  sp->ac_method = 1;
  sp->n_fits = 1;
  sp->log_fit = 1;
  sp->bM_nmaxs = 500;
  sp->bM_Bessel_zeros = 1.0e-50;
  sp->bM_betas = 1.0;
  sp->bM_alphas = 1.0;
}

int alps_create(const alps_system* sys, alps_ctx** out) {
  if (!sys || !out) return ALPS_E_INVALID;
  *out = nullptr;
  if (sys->nspec < 1 || sys->nspec > ALPS_MAX_SPECIES) return ALPS_E_INVALID;
  if (sys->positions_principal < 0 || sys->n_resonance_interval < 1) return ALPS_E_INVALID;
  if (sys->nperp < 4 || sys->npar < 2 * sys->positions_principal + 8) return ALPS_E_INVALID;
  if (sys->secant_method < 0 || sys->secant_method > 2) return ALPS_E_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return ALPS_E_NO_DEVICE;
  alps_ctx* c = new alps_ctx();
  c->sys = *sys;
  c->spec.resize(sys->nspec);
  c->kperp = sys->kperp;
  c->kpar = sys->kpar;
  cudaGetDevice(&c->device);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return ALPS_E_CUDA;
  }
  *out = c;
  return ALPS_OK;
}

void alps_destroy(alps_ctx* c) {
  if (!c) return;
  cudaStreamSynchronize(c->stream);
  for (auto& S : c->spec) {
    cudaFree(S.d_pperp);
    cudaFree(S.d_ppar);
    cudaFree(S.d_f0);
    cudaFree(S.d_g1);
    cudaFree(S.d_g2);
    cudaFree(S.d_fit);
    cudaFree(S.d_bessel);
    cudaFree(S.d_V);
    cudaFree(S.d_A);
    cudaFree(S.d_tcws);
    cudaFree(S.d_nmax);
    cudaFree(S.d_words);
    cudaFree(S.d_fit_scratch);
    cudaFree(S.d_Rw);
    cudaFree(S.d_G);
    cudaFree(S.d_X);
    cudaFree(S.d_mom);
    cudaFree(S.d_momf);
    cudaFree(S.d_Vh);  // d_Vl points into it
    cudaFree(S.d_Vscale);
    cudaFree(S.d_Bt);
    cudaFree(S.d_Bd);
    cudaFree(S.d_pph);
    cudaFree(S.d_ppl);
    cudaFree(S.d_fit_aux);
    cudaFree(S.d_lmom);
    cudaFree(S.d_grel);
    cudaFree(S.d_prel);
    cudaFree(S.d_f0rel);
    cudaFree(S.d_dfr1);
    cudaFree(S.d_dfr2);
    cudaFree(S.d_jrel);
    cudaFree(S.d_cone);
    cudaFree(S.d_bmI);
  }
  cudaFree(c->d_om);
  cudaFree(c->d_D);
  cudaFree(c->d_part);
  cudaFree(c->d_low);
  cudaFree(c->d_count);
  cudaFree(c->d_slot_nn);
  cudaFree(c->d_items);
  cudaFree(c->d_ext);
  cudaFree(c->d_rel);
  cudaFree(c->d_bm);
  cudaFree(c->d_flags);
  if (c->h_pinned) cudaFreeHost(c->h_pinned);
  if (c->h_flag) cudaFreeHost(c->h_flag);
  if (c->ev_done) cudaEventDestroy(c->ev_done);
  if (c->d_args) cudaFree(c->d_args);
  if (c->d_job) cudaFree(c->d_job);
  if (c->h_args) cudaFreeHost(c->h_args);
  for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second.second);
  for (auto& ev : c->ev_pending)
    for (auto e : ev) cudaEventDestroy(e);
  for (auto e : c->ev_pool) cudaEventDestroy(e);
  cudaStreamDestroy(c->stream);
  delete c;
}

// rows of the fit parameter table: the pperp rows, or for a relativistic
// species the Gamma rows when there are more of them
static int fit_rows(const alps_ctx* c, int is) {
  int r = c->sys.nperp;
  if (c->spec[is].sp.relat) r = std::max(r, c->sys.ngamma);
  return r + 1;
}

// doubles in the continuation table: rows x 5 x n_fits fit parameters, or
// (nperp+1) x (poly_order+1) Chebyshev coefficients for ACmethod 2
static size_t fit_size(const alps_ctx* c, int is) {
  const alps_species& sp = c->spec[is].sp;
  if (sp.ac_method == 2 && !sp.use_bM) return (size_t)(c->sys.nperp + 1) * (sp.poly_order + 1);
  return (size_t)fit_rows(c, is) * 5 * sp.n_fits;
}

// A bi-Maxwellian or cold species evaluated in closed form (use_bM = T): no
// f0 table, no derivatives or fits (read_f0 and determine_param_fit skip
// it, src/ALPS_io.f90:672-675, src/ALPS_analyt.f90:447-451).
static int set_species_bm(alps_ctx* c, int is, const alps_species* sp) {
  if (sp->relat) return ALPS_E_UNSUPPORTED;
  if (sp->qs == 0.0 || !(sp->ms > 0.0) || !(sp->ns > 0.0) || sp->bM_betas < 0.0) return ALPS_E_INVALID;
  if (sp->bM_betas > 0.0 && (!(sp->bM_alphas > 0.0) || sp->bM_nmaxs < 0)) return ALPS_E_INVALID;
  // the cold closed form is written for kperp_norm = T (calc_chi_cold stops otherwise)
  if (sp->bM_betas == 0.0 && !c->sys.kperp_norm) return ALPS_E_INVALID;
  SpeciesHost& S = c->spec[is];
  S.sp = *sp;
  S.sp.n_fits = 1;
  S.sp.relat = 0;
  S.pperp.clear();
  S.ppar.clear();
  S.f0.clear();
  int rows = fit_rows(c, is);
  if (S.d_fit) cudaFree(S.d_fit);
  S.d_fit = nullptr;
  S.aux_ready = false;
  ALPS_CUDA_TRY(cudaMalloc(&S.d_fit, (size_t)rows * 5 * sizeof(double)));
  ALPS_CUDA_TRY(cudaMemsetAsync(S.d_fit, 0, (size_t)rows * 5 * sizeof(double), c->stream));
  ALPS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  // derivative_f0's current moment of a bi-Maxwellian (src/ALPS_fns.f90:162-166)
  S.current_int = sp->ns * sp->qs * sp->bM_pdrifts / sp->ms;
  S.int_ee = 0.0;
  S.loaded = true;
  c->prepared = false;
  c->kset = false;
  return ALPS_OK;
}

int alps_set_species(alps_ctx* c, int is, const alps_species* sp, const double* pperp, const double* ppar,
                     const double* f0) {
  if (!c || !sp || is < 0 || is >= c->sys.nspec) return ALPS_E_INVALID;
  if (sp->use_bM) return set_species_bm(c, is, sp);
  if (!pperp || !ppar || !f0) return ALPS_E_INVALID;
  if (sp->ac_method != 0 && sp->ac_method != 1 && sp->ac_method != 2) return ALPS_E_INVALID;
  if (sp->ac_method == 2) {  // Chebyshev continuation: kind 1 only (alps_error(10) otherwise)
    if (sp->poly_kind != 1) return ALPS_E_POLY_KIND;
    if (sp->poly_order < 1 || sp->poly_order > 255 || sp->relat) return ALPS_E_INVALID;
  }
  // relativistic species: continuation on the (Gamma, pparbar) rows, fit
  // types 4 and 5 (the types whose pperp argument is Gamma)
  if (sp->relat && sp->ac_method != 1) return ALPS_E_UNSUPPORTED;
  if (sp->relat && (c->sys.ngamma < 4 || c->sys.npparbar < 6)) return ALPS_E_INVALID;
  if (sp->ac_method == 1) {
    if (sp->n_fits < 1 || sp->n_fits > ALPS_MAX_FITS) return ALPS_E_INVALID;
    for (int f = 0; f < sp->n_fits; ++f) {
      int t = sp->fit_type[f];
      bool ok = sp->relat ? (t == 4 || t == 5) : (t == 1 || t == 2 || t == 3 || t == 6);
      if (!ok) return ALPS_E_UNSUPPORTED;
    }
  }
  if (sp->qs == 0.0 || sp->ms <= 0.0) return ALPS_E_INVALID;
  int N = c->sys.nperp, M = c->sys.npar, L = M + 1;
  // tensor-product, uniform, increasing grid (the reference's assumption)
  std::vector<double> pv(N + 1), qv(M + 1);
  for (int i = 0; i <= N; ++i) pv[i] = pperp[i * L];
  for (int j = 0; j <= M; ++j) qv[j] = ppar[j];
  for (int i = 0; i <= N; ++i)
    for (int j = 0; j <= M; ++j)
      if (pperp[i * L + j] != pv[i] || ppar[i * L + j] != qv[j]) return ALPS_E_GRID;
  double dp = pv[1] - pv[0], dq = qv[1] - qv[0];
  if (!(dp > 0.0) || !(dq > 0.0)) return ALPS_E_GRID;
  for (int i = 1; i <= N; ++i)
    if (std::fabs((pv[i] - pv[i - 1]) - dp) > 1e-9 * dp) return ALPS_E_GRID;
  for (int j = 1; j <= M; ++j)
    if (std::fabs((qv[j] - qv[j - 1]) - dq) > 1e-9 * dq) return ALPS_E_GRID;
  SpeciesHost& S = c->spec[is];
  S.sp = *sp;
  if (sp->ac_method != 1) S.sp.n_fits = 1;
  S.sp.relat = sp->relat ? 1 : 0;
  S.pperp = pv;
  S.ppar = qv;
  S.f0.assign(f0, f0 + (size_t)(N + 1) * L);
  size_t nn = (size_t)(N + 1) * L;
  if (!S.d_pperp) ALPS_CUDA_TRY(cudaMalloc(&S.d_pperp, (N + 1) * sizeof(double)));
  if (!S.d_ppar) ALPS_CUDA_TRY(cudaMalloc(&S.d_ppar, (M + 1) * sizeof(double)));
  if (!S.d_f0) ALPS_CUDA_TRY(cudaMalloc(&S.d_f0, nn * sizeof(double)));
  int nf = S.sp.n_fits;
  if (S.d_fit) cudaFree(S.d_fit);
  S.d_fit = nullptr;
  S.aux_ready = false;
  std::vector<double> fit(fit_size(c, is), 0.0);
  ALPS_CUDA_TRY(cudaMalloc(&S.d_fit, fit.size() * sizeof(double)));
  if (sp->ac_method == 1)
    for (int ip = 0; ip < 5; ++ip)
      for (int f = 0; f < nf; ++f) fit[(0 * 5 + ip) * nf + f] = sp->fit_init[f][ip];
  ALPS_CUDA_TRY(cudaMemcpyAsync(S.d_pperp, pv.data(), (N + 1) * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  ALPS_CUDA_TRY(cudaMemcpyAsync(S.d_ppar, qv.data(), (M + 1) * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  ALPS_CUDA_TRY(cudaMemcpyAsync(S.d_f0, S.f0.data(), nn * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  ALPS_CUDA_TRY(cudaMemcpyAsync(S.d_fit, fit.data(), fit.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  ALPS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  // parallel current moment of derivative_f0 (src/ALPS_fns.f90:157-190),
  // summed in the reference's node order
  {
    double dpperp = pv[2] - pv[1], dppar = std::fabs(qv[2] - qv[1]), ci = 0.0;
    for (int i = 0; i <= N; ++i)
      for (int j = 0; j <= M; ++j)
        ci = ci + (sp->ns * sp->qs / sp->ms) * pv[i] * qv[j] * S.f0[(size_t)i * L + j] * 2.0 * ALPS_PI * dpperp *
                      dppar;
    S.current_int = ci;
  }
  S.loaded = true;
  c->prepared = false;
  c->kset = false;
  return ALPS_OK;
}

int alps_prepare(alps_ctx* c) {
  if (!c) return ALPS_E_INVALID;
  for (int is = 0; is < c->sys.nspec; ++is)
    if (!c->spec[is].loaded) return ALPS_E_INVALID;
  // the batched setup: every species' fit in one launch, one warp each
  // (the reference's warm start orders the rows of a fit, not the species)
  if (ctx_batch_preparable(c)) return alps_prepare_many(&c, 1, nullptr);
  c->gen++;
  for (int is = 0; is < c->sys.nspec; ++is) {
    int st = launch_prepare_species(c, is);
    if (st) return st;
  }
  c->prepared = true;
  c->kset = false;
  return ALPS_OK;
}

int alps_get_fit(alps_ctx* c, int is, double* out) {
  if (!c || !out || is < 0 || is >= c->sys.nspec || !c->spec[is].loaded) return ALPS_E_INVALID;
  const SpeciesHost& S = c->spec[is];
  size_t n = fit_size(c, is);
  ALPS_CUDA_TRY(cudaMemcpyAsync(out, S.d_fit, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  ALPS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return ALPS_OK;
}

int alps_set_fit(alps_ctx* c, int is, const double* in) {
  if (!c || !in || is < 0 || is >= c->sys.nspec || !c->spec[is].loaded) return ALPS_E_INVALID;
  SpeciesHost& S = c->spec[is];
  size_t n = fit_size(c, is);
  ALPS_CUDA_TRY(cudaMemcpyAsync(S.d_fit, in, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  S.aux_ready = false;
  int st = launch_fit_aux(c, is);
  if (st) return st;
  if (c->kset && (st = launch_landau_moments(c, is))) return st;
  ALPS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  c->gen++;
  return ALPS_OK;
}

int alps_get_f0_rel(alps_ctx* c, int is, double* gamma, double* pparbar, double* f0_rel, double* df_dgamma,
                    double* df_dpparbar) {
  if (!c || is < 0 || is >= c->sys.nspec || !c->prepared || !c->spec[is].sp.relat) return ALPS_E_INVALID;
  const SpeciesHost& S = c->spec[is];
  size_t ng = c->sys.ngamma, np = c->sys.npparbar, nf = (ng + 1) * (np + 1);
  if (gamma) memcpy(gamma, S.grel.data(), (ng + 1) * sizeof(double));
  if (pparbar) memcpy(pparbar, S.prel.data(), (np + 1) * sizeof(double));
  if (f0_rel) ALPS_CUDA_TRY(cudaMemcpyAsync(f0_rel, S.d_f0rel, nf * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (df_dgamma)
    ALPS_CUDA_TRY(cudaMemcpyAsync(df_dgamma, S.d_dfr1, nf * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (df_dpparbar)
    ALPS_CUDA_TRY(cudaMemcpyAsync(df_dpparbar, S.d_dfr2, nf * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  ALPS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return ALPS_OK;
}

// The k tables of a context once nmax is known (the rest of alps_set_k);
// with sync = false the caller synchronises the context's stream and then
// calls set_k_commit.
static int set_k_tables(alps_ctx* c, double kperp, double kpar, std::vector<int> nm, bool sync);
static void set_k_commit(alps_ctx* c, double kperp, double kpar) {
  c->kperp = kperp;
  c->kpar = kpar;
  c->kset = true;
  c->gen++;
}

// The k tables (nmax, Bessel tables, contractions, moments) depend on k_perp
// alone: k_par enters per frequency, through the launch arguments and the
// resonant-order capacity.  A step that keeps k_perp bit for bit, as every
// step of a k_par scan does, keeps them and moves k_par only, the way
// om_scan skips determine_nmax and determine_bessel_array for scan type 4
// (src/ALPS_fns.f90:2465-2471).
static bool tables_hold(const alps_ctx* c, double kperp) { return c->kset && c->kperp == kperp; }

// resonant orders per omega: p_res moves by |q/k_par| per order, so at most
// width*|k_par/q| + 1 orders fall in the resonance window
static void set_rcap(alps_ctx* c, double kpar) {
  for (int is = 0; is < c->sys.nspec; ++is) {
    SpeciesHost& S = c->spec[is];
    if (S.sp.use_bM) {
      S.rcap = 1;
      continue;
    }
    const int M = c->sys.npar;
    const double dq = S.ppar[2] - S.ppar[1];
    const double width = (S.ppar[M] - S.ppar[1]) + 2.0 * c->sys.positions_principal * dq + 2.0 * dq;
    const double cnt = std::floor(width * std::fabs(kpar / S.sp.qs)) + 3.0;
    S.rcap = (int)std::min<double>(2.0 * S.nmax + 1.0, cnt);
  }
}

static int set_k_impl(alps_ctx* c, double kperp, double kpar, bool rebuild) {
  if (!c || !c->prepared) return ALPS_E_INVALID;
  if (!(kperp > 0.0) || kpar == 0.0 || !std::isfinite(kperp) || !std::isfinite(kpar)) return ALPS_E_INVALID;
  if (!rebuild && tables_hold(c, kperp)) {
    set_rcap(c, kpar);
    set_k_commit(c, kperp, kpar);
    c->stats.k_reused++;
    return ALPS_OK;
  }
  c->kset = false;  // the tables are rebuilt from here on
  int S_ = c->sys.nspec;
  std::vector<int> nm(S_);
  for (int is = 0; is < S_; ++is) {
    int st = launch_set_k_species(c, is, kperp, &nm[is]);
    if (st) return st;
  }
  return set_k_tables(c, kperp, kpar, nm, true);
}

int alps_set_k(alps_ctx* c, double kperp, double kpar) { return set_k_impl(c, kperp, kpar, false); }

static int set_k_tables(alps_ctx* c, double kperp, double kpar, std::vector<int> nm, bool sync) {
  const int S_ = c->sys.nspec;
  // nmax adjustment of a run on nproc MPI ranks (src/ALPS_fns.f90:4048-4071)
  if (c->sys.nproc > 0) {
    int max_procs = S_;
    for (int is = 0; is < S_; ++is) max_procs += nm[is];
    int is = 0;
    while (max_procs < c->sys.nproc - 1) {
      if (!c->spec[is].sp.use_bM) nm[is] += 1;
      is = (is + 1) % S_;
      max_procs++;
    }
  }
  for (int is = 0; is < S_; ++is) {
    SpeciesHost& S = c->spec[is];
    S.nmax = nm[is];
    if (S.sp.use_bM) {  // closed form: only the I_n table of k_perp
      int st = launch_nhds_bessel(c, is, kperp);
      if (st) return st;
      continue;
    }
    int st = launch_build_bessel_and_reduced(c, is, kperp);
    if (st) return st;
    if (S.sp.relat && (st = launch_rel_bessel(c, is, kperp))) return st;
    if ((st = launch_fit_aux(c, is))) return st;
    if ((st = launch_landau_moments(c, is))) return st;
  }
  set_rcap(c, kpar);
  if (!sync) return ALPS_OK;
  ALPS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  set_k_commit(c, kperp, kpar);
  return ALPS_OK;
}

int alps_prepare_many(alps_ctx* const* ctx, int n, int* status) {
  if (n < 0 || (n > 0 && !ctx)) return ALPS_E_INVALID;
  std::vector<alps_ctx*> batch;
  int first = ALPS_OK;
  for (int i = 0; i < n; ++i) {
    alps_ctx* c = ctx[i];
    if (status) status[i] = ALPS_OK;
    if (!c) return ALPS_E_INVALID;
    for (const auto& S : c->spec)
      if (!S.loaded) return ALPS_E_INVALID;
    c->gen++;
    if (ctx_batch_preparable(c)) {
      batch.push_back(c);
    } else {  // relativistic species, Chebyshev continuations: per context
      int st = alps_prepare(c);
      if (status) status[i] = st;
      if (st && !first) first = st;
    }
  }
  std::vector<int> bst(batch.size(), ALPS_OK);
  int rc = prepare_contexts(batch.data(), (int)batch.size(), bst.data());
  if (rc) return rc;
  for (size_t k = 0, i = 0; i < (size_t)n; ++i) {
    alps_ctx* c = ctx[i];
    if (k >= batch.size() || batch[k] != c) continue;
    const int st = bst[k++];
    if (status) status[i] = st;
    if (st && !first) first = st;
    c->prepared = (st == ALPS_OK);
    c->kset = false;
  }
  return first;
}

int alps_set_k_many(alps_ctx* const* ctx, int n, const double* kperp, const double* kpar, int* status) {
  if (n < 0 || (n > 0 && (!ctx || !kperp || !kpar))) return ALPS_E_INVALID;
  for (int i = 0; i < n; ++i) {
    if (!ctx[i] || !ctx[i]->prepared) return ALPS_E_INVALID;
    if (!(kperp[i] > 0.0) || kpar[i] == 0.0 || !std::isfinite(kperp[i]) || !std::isfinite(kpar[i]))
      return ALPS_E_INVALID;
    if (status) status[i] = ALPS_OK;
  }
  // contexts whose k_perp stays keep their tables (k_par steps)
  std::vector<alps_ctx*> rb;
  std::vector<double> rb_kperp;
  std::vector<int> rb_of;
  for (int i = 0; i < n; ++i) {
    alps_ctx* c = ctx[i];
    if (tables_hold(c, kperp[i])) {
      set_rcap(c, kpar[i]);
      set_k_commit(c, kperp[i], kpar[i]);
      c->stats.k_reused++;
      continue;
    }
    c->kset = false;
    rb.push_back(c);
    rb_kperp.push_back(kperp[i]);
    rb_of.push_back(i);
  }
  if (rb.empty()) return ALPS_OK;
  std::vector<std::vector<int>> nm;
  int rc = nmax_contexts(rb.data(), (int)rb.size(), rb_kperp.data(), nm);
  if (rc) return rc;
  // every context's tables on a few streams, then one synchronisation
  const int NS = 8;
  cudaStream_t st[NS];
  int plo = 0, phi = 0;  // k steps gate root following: highest priority, as the server's rounds
  ALPS_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&plo, &phi));
  for (int q = 0; q < NS; ++q) ALPS_CUDA_TRY(cudaStreamCreateWithPriority(&st[q], cudaStreamNonBlocking, phi));
  int first = ALPS_OK;
  const int nb = (int)rb.size();
  std::vector<char> ok(nb, 0);
  for (int j = 0; j < nb; ++j) {
    const int i = rb_of[j];
    alps_ctx* c = ctx[i];
    cudaStream_t own = c->stream;
    c->stream = st[j % NS];
    c->defer_sync = true;
    const int s = set_k_tables(c, kperp[i], kpar[i], nm[j], false);
    c->defer_sync = false;
    c->stream = own;
    if (status) status[i] = s;
    if (s && !first) first = s;
    ok[j] = (s == ALPS_OK);
  }
  for (int q = 0; q < NS; ++q) {
    if (cudaStreamSynchronize(st[q]) != cudaSuccess && !first) first = ALPS_E_CUDA;
    cudaStreamDestroy(st[q]);
  }
  for (int j = 0; j < nb; ++j)
    if (ok[j] && first != ALPS_E_CUDA) set_k_commit(rb[j], kperp[rb_of[j]], kpar[rb_of[j]]);
  return first;
}

int alps_get_nmax(alps_ctx* c, int* nmax) {
  if (!c || !nmax || !c->kset) return ALPS_E_INVALID;
  for (int is = 0; is < c->sys.nspec; ++is) nmax[is] = c->spec[is].nmax;
  return ALPS_OK;
}

int alps_set_precision(alps_ctx* c, int precision) {
  if (!c) return ALPS_E_INVALID;
  if (precision != ALPS_PREC_FP64 && precision != ALPS_PREC_MIXED) return ALPS_E_INVALID;
  const bool changed = c->precision != precision;
  c->precision = precision;
  c->gen++;
  // the p_perp contraction is part of the precision path (FP64 on the plain
  // path, the tensor cores on the mixed one): rebuild the k tables
  if (changed && c->kset) return set_k_impl(c, c->kperp, c->kpar, true);
  return ALPS_OK;
}

int ctx_ensure_batch(alps_ctx* c, int n, bool ext) {
  if ((size_t)n > c->batch_cap) {
    cudaFree(c->d_om);
    cudaFree(c->d_D);
    c->d_om = c->d_D = nullptr;
    c->batch_cap = 0;
    ALPS_CUDA_TRY(cudaMalloc(&c->d_om, (size_t)n * sizeof(double2)));
    ALPS_CUDA_TRY(cudaMalloc(&c->d_D, (size_t)n * sizeof(double2)));
    c->batch_cap = n;
    c->gen++;
  }
  size_t need_pin = (size_t)2 * n;
  if (need_pin > c->pinned_cap) {
    if (c->h_pinned) cudaFreeHost(c->h_pinned);
    c->h_pinned = nullptr;
    c->pinned_cap = 0;
    ALPS_CUDA_TRY(cudaMallocHost(&c->h_pinned, need_pin * sizeof(double2)));
    c->pinned_cap = need_pin;
    c->gen++;
  }
  if (!c->h_flag) ALPS_CUDA_TRY(cudaMallocHost(&c->h_flag, sizeof(int)));
  if (!c->ev_done) ALPS_CUDA_TRY(cudaEventCreateWithFlags(&c->ev_done, cudaEventDisableTiming));
  if (ext) {
    size_t ne = (size_t)n * (c->sys.nspec * 36 + 9);
    if (ne > c->ext_cap) {
      cudaFree(c->d_ext);
      c->d_ext = nullptr;
      c->ext_cap = 0;
      ALPS_CUDA_TRY(cudaMalloc(&c->d_ext, ne * sizeof(double2)));
      c->ext_cap = ne;
    }
  }
  return ALPS_OK;
}

int ctx_check_flags(alps_ctx* c) {
  int f = 0;
  ALPS_CUDA_TRY(cudaMemcpy(&f, c->d_flags, sizeof(int), cudaMemcpyDeviceToHost));
  if (f & 2) return ALPS_E_SUBLUMINAL;  // resonance window wider than the subluminal cone
  return f ? ALPS_E_INVALID : ALPS_OK;
}

// Evaluates n frequencies from host memory through pinned staging.
static int disp_host(alps_ctx* c, int n, const alps_complex* om, alps_complex* D, alps_complex* ext_out) {
  int st = ctx_ensure_batch(c, n, ext_out != nullptr);
  if (st) return st;
  double2* pin = c->h_pinned;
  memcpy(pin, om, (size_t)n * sizeof(double2));
  ALPS_CUDA_TRY(cudaMemcpyAsync(c->d_om, pin, (size_t)n * sizeof(double2), cudaMemcpyHostToDevice, c->stream));
  st = launch_disp_batch(c, n, c->d_om, c->d_D, ext_out ? c->d_ext : nullptr, c->stream);
  if (st) return st;
  ALPS_CUDA_TRY(cudaMemcpyAsync(pin + n, c->d_D, (size_t)n * sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
  if (ext_out)
    ALPS_CUDA_TRY(cudaMemcpyAsync(ext_out, c->d_ext, (size_t)n * (c->sys.nspec * 36 + 9) * sizeof(double2),
                                  cudaMemcpyDeviceToHost, c->stream));
  ALPS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if ((st = ctx_check_flags(c))) return st;
  memcpy(D, pin + n, (size_t)n * sizeof(double2));
  return ALPS_OK;
}

int alps_disp(alps_ctx* c, alps_complex om, alps_complex* D, alps_complex* chi0, alps_complex* chi0_low,
              alps_complex* wave) {
  if (!c || !D || !c->kset) return ALPS_E_INVALID;
  int S_ = c->sys.nspec;
  std::vector<alps_complex> ext((size_t)S_ * 36 + 9);
  int st = disp_host(c, 1, &om, D, ext.data());
  if (st) return st;
  if (chi0) memcpy(chi0, ext.data(), (size_t)S_ * 9 * sizeof(alps_complex));
  if (chi0_low) memcpy(chi0_low, ext.data() + S_ * 9, (size_t)S_ * 27 * sizeof(alps_complex));
  if (wave) memcpy(wave, ext.data() + S_ * 36, 9 * sizeof(alps_complex));
  return ALPS_OK;
}

int alps_disp_batch(alps_ctx* c, int n, const alps_complex* om, alps_complex* D) {
  if (!c || n < 0 || (n > 0 && (!om || !D)) || !c->kset) return ALPS_E_INVALID;
  if (n == 0) return ALPS_OK;
  return disp_host(c, n, om, D, nullptr);
}

int alps_disp_batch_device(alps_ctx* c, int n, const alps_complex* d_om, alps_complex* d_D, void* stream) {
  if (!c || n < 0 || !c->kset) return ALPS_E_INVALID;
  if (n == 0) return ALPS_OK;
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  int rc = launch_disp_batch(c, n, reinterpret_cast<const double2*>(d_om), reinterpret_cast<double2*>(d_D), nullptr,
                             st);
  if (rc == ALPS_OK) c->async_flags = c->d_flags;
  return rc;
}

// The device error word of the last asynchronous batch, read after the
// batch's stream has drained.  Reads 4 bytes with cudaMemcpy into a stack
// variable: no allocation, so it serves the no-allocation entry point too.
int alps_batch_status(alps_ctx* c, void* stream) {
  if (!c) return ALPS_E_INVALID;
  if (!c->async_flags) return ALPS_OK;
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  ALPS_CUDA_TRY(cudaStreamSynchronize(st));
  int f = 0;
  ALPS_CUDA_TRY(cudaMemcpy(&f, c->async_flags, sizeof(int), cudaMemcpyDeviceToHost));
  if (f & 2) return ALPS_E_SUBLUMINAL;
  return f ? ALPS_E_INVALID : ALPS_OK;
}

// calc_eigen (src/ALPS_fns.f90:2605-2899) for n roots; the det D evaluations
// at om, Re(om) and Re(om*1.000001) of every root go out as one batch.
int alps_calc_eigen(alps_ctx* c, int n, const alps_complex* om, int eigen, int heat, alps_eigen* out) {
  if (!c || n < 0 || (n > 0 && (!om || !out)) || !c->kset) return ALPS_E_INVALID;
  const int S_ = c->sys.nspec;
  if (S_ > ALPS_EIGEN_MAX_SPECIES) return ALPS_E_INVALID;
  if (n == 0) return ALPS_OK;
  const int per = heat ? 3 : 1;
  std::vector<alps_complex> oms((size_t)n * per), D((size_t)n * per);
  for (int r = 0; r < n; ++r) {
    oms[r] = om[r];
    if (heat) {
      oms[n + r] = alps_complex{om[r].re, 0.0};
      oms[2 * n + r] = alps_complex{(cplx(om[r].re, om[r].im) * 1.000001).real(), 0.0};
    }
  }
  const size_t ne = (size_t)S_ * 36 + 9;
  std::vector<alps_complex> ext(oms.size() * ne);
  int st = disp_host(c, (int)oms.size(), oms.data(), D.data(), ext.data());
  if (st) return st;
  const double vA = c->sys.vA, kperp = c->kperp, kpar = c->kpar;
  const cplx I(0.0, 1.0), h(-0.0, -0.5);
  auto X = [](const alps_complex& z) { return cplx(z.re, z.im); };
  for (int r = 0; r < n; ++r) {
    alps_eigen& o = out[r];
    std::memset(&o, 0, sizeof(o));
    const alps_complex* e0 = ext.data() + (size_t)r * ne;
    auto chi = [&](const alps_complex* e, int s, int i, int j) { return X(e[s * 9 + 3 * i + j]); };
    auto low = [&](const alps_complex* e, int s, int i, int j, int nn) {
      return X(e[S_ * 9 + s * 27 + (nn + 1) * 9 + 3 * i + j]);
    };
    auto W = [&](int i, int j) { return X(e0[S_ * 36 + 3 * i + j]); };
    const cplx w(om[r].re, om[r].im);
    // fields relative to E_x from the wave tensor at the root
    cplx E[3], B[3];
    E[0] = cplx(1.0, 0.0);
    E[2] = -E[0] * (W(1, 0) * W(2, 1) - W(2, 0) * W(1, 1));
    E[2] = E[2] / (W(1, 2) * W(2, 1) - W(2, 2) * W(1, 1));
    if (std::abs(W(2, 1)) != 0.0) {
      E[1] = -E[2] * W(2, 2) - E[0] * W(2, 0);
      E[1] = E[1] / W(2, 1);
    } else {  // cold plasma without drifts
      E[1] = W(1, 0) * W(0, 2) - W(0, 0) * W(1, 2);
      E[1] = E[1] / (W(1, 2) * W(0, 1) - W(1, 1) * W(0, 2));
    }
    B[0] = -1.0 * kpar * E[1] / (w * vA);
    B[1] = -1.0 * (kperp * E[2] - kpar * E[0]) / (w * vA);
    B[2] = kperp * E[1] / (w * vA);
    for (int i = 0; i < 3; ++i) {
      o.electric[i] = alps_complex{E[i].real(), E[i].imag()};
      o.magnetic[i] = alps_complex{B[i].real(), B[i].imag()};
    }
    if (eigen) {
      for (int s = 0; s < S_; ++s) {
        const SpeciesHost& Sp = c->spec[s];
        const double qn = Sp.sp.qs * Sp.sp.ns;
        const double pf = Sp.current_int / (Sp.sp.ns * Sp.sp.qs);
        auto vm = [&](int j) {
          cplx sum(0.0, 0.0);
          for (int k = 0; k < 3; ++k) sum = sum + E[k] * chi(e0, s, j, k);
          return -((vA * vA) / qn) * I * w * sum;
        };
        cplx U[3] = {vm(0), vm(1), vm(2)};
        if (pf != 0.0) {
          U[2] = U[2] - pf * kperp * U[0] / (w - kpar * pf);
          U[2] = U[2] / (1.0 + (kpar * pf) / (w - kpar * pf));
        }
        cplx d = (1.0 / vA) * (U[0] * kperp + U[2] * kpar) / (w - kpar * pf);
        for (int j = 0; j < 3; ++j) o.vmean[s][j] = alps_complex{U[j].real(), U[j].imag()};
        o.ds[s] = alps_complex{d.real(), d.imag()};
      }
    }
    if (!heat) continue;
    const alps_complex* e1 = ext.data() + (size_t)(n + r) * ne;      // Re(om)
    const alps_complex* e2 = ext.data() + (size_t)(2 * n + r) * ne;  // Re(om*1.000001)
    // anti-Hermitian part per species at Re(om), Hermitian part of the sum
    double Ps[ALPS_EIGEN_MAX_SPECIES];
    for (int s = 0; s < S_; ++s) {
      cplx sum(0.0, 0.0);
      for (int ii = 0; ii < 3; ++ii) {
        cplx term(0.0, 0.0);
        for (int k = 0; k < 3; ++k)
          term = term + std::conj(E[k]) * (-0.5 * I * (chi(e1, s, k, ii) - std::conj(chi(e1, s, ii, k))));
        sum = sum + term * E[ii];
      }
      Ps[s] = sum.real();
    }
    auto herm = [&](const alps_complex* e, int i, int j) {
      cplx a(0.0, 0.0), b(0.0, 0.0);
      for (int s = 0; s < S_; ++s) a = a + chi(e, s, i, j);
      for (int s = 0; s < S_; ++s) b = b + std::conj(chi(e, s, j, i));
      return 0.5 * (a + b);
    };
    cplx s1(0.0, 0.0), s2(0.0, 0.0);
    for (int ii = 0; ii < 3; ++ii) {
      cplx term(0.0, 0.0);
      for (int k = 0; k < 3; ++k) {
        cplx dchih = (1.000001 * herm(e2, k, ii) - herm(e1, k, ii)) / 0.000001;
        term = term + std::conj(E[k]) * dchih;
      }
      s1 = s1 + term * E[ii];
    }
    for (int ii = 0; ii < 3; ++ii) s2 = s2 + B[ii] * std::conj(B[ii]);
    const double ewave = (s1 + s2).real();
    o.ewave = ewave;
    // split by mechanism from chi0_low at Re(om*1.000001)
    for (int s = 0; s < S_; ++s) {
      cplx c22 = low(e2, s, 1, 1, 0), c23 = low(e2, s, 1, 2, 0), c32 = low(e2, s, 2, 1, 0), c33 = low(e2, s, 2, 2, 0);
      double p1 = (h * std::conj(E[1]) * E[1] * (c22 - std::conj(c22))).real();
      p1 = (p1 - 0.5 * I * (E[2] * std::conj(E[1]) * c23 - std::conj(E[2]) * E[1] * std::conj(c23))).real();
      double p2 = (h * (E[1] * std::conj(E[2]) * c32 - std::conj(E[1]) * E[2] * std::conj(c32))).real();
      p2 = (p2 - 0.5 * I * std::conj(E[2]) * E[2] * (c33 - std::conj(c33))).real();
      const cplx Exy[3] = {E[0], E[1], cplx(0.0, 0.0)};
      double pc[2];
      for (int q = 0; q < 2; ++q) {
        int nn = q == 0 ? 1 : -1;
        cplx sum(0.0, 0.0);
        for (int ii = 0; ii < 3; ++ii) {
          cplx term(0.0, 0.0);
          for (int k = 0; k < 3; ++k)
            term = term + std::conj(Exy[k]) * (h * (low(e2, s, k, ii, nn) - std::conj(low(e2, s, ii, k, nn))));
          sum = sum + term * Exy[ii];
        }
        pc[q] = sum.real();
      }
      o.Ps[s] = Ps[s] / ewave;
      o.Ps_split[s][0] = p1 / ewave;
      o.Ps_split[s][1] = p2 / ewave;
      o.Ps_split[s][2] = pc[0] / ewave;
      o.Ps_split[s][3] = pc[1] / ewave;
    }
  }
  return ALPS_OK;
}

int alps_set_profiling(alps_ctx* c, int on) {
  if (!c) return ALPS_E_INVALID;
  int st = collect_profile(c);
  if (st) return st;
  c->profiling = on != 0;
  for (int q = 0; q < 4; ++q) c->prof_ms[q] = 0.0;
  c->prof_batches = 0;
  return ALPS_OK;
}

int alps_get_profile(alps_ctx* c, double* ms, int64_t* batches) {
  if (!c || !ms) return ALPS_E_INVALID;
  int st = collect_profile(c);
  if (st) return st;
  for (int q = 0; q < 4; ++q) ms[q] = c->prof_ms[q];
  if (batches) *batches = c->prof_batches;
  return ALPS_OK;
}

int alps_get_stats(alps_ctx* c, alps_stats* st) {
  if (!c || !st) return ALPS_E_INVALID;
  *st = c->stats;
  st->tc_contractions = 0;
  st->tc_fixed_entries = 0;
  st->tc_entries = 0;
  for (const auto& S : c->spec)
    if (S.tc_used) {
      st->tc_contractions++;
      st->tc_fixed_entries += S.tc_fixed;
      st->tc_entries += (int64_t)3 * (S.nmax + 1) * 2 * (c->sys.npar - 1);
    }
  return ALPS_OK;
}

int alps_tc_product(const double* d_A, const double* d_B, double* d_C, int M, int N, int K, int checked,
                    int* nfixed) {
  if (!d_A || !d_B || !d_C || M < 1 || N < 1 || K < 1 || K > 256) return ALPS_E_INVALID;
  const size_t need = checked ? tc_checked_workspace_bytes(M, N, K) : tc_workspace_bytes(M, N, K);
  void* ws = nullptr;
  ALPS_CUDA_TRY(cudaMalloc(&ws, need));
  int fixed = 0, rc;
  if (checked)
    rc = tc_product_checked(d_A, d_B, d_C, M, N, K, ws, &fixed, 0);
  else
    rc = tc_product(d_A, K, 1, d_B, N, 1, d_C, N, 1, M, N, K, 1.0, 0.0, nullptr, ws, nullptr, 0);
  if (!rc && cudaStreamSynchronize(0) != cudaSuccess) rc = ALPS_E_CUDA;
  if (!rc && !checked) rc = tc_check(ws, M, N, K);
  cudaFree(ws);
  if (nfixed) *nfixed = fixed;
  return rc;
}


int alps_secant_ex(alps_ctx* c, int method, int nroots, alps_complex* om, double om_rtol, int* iters,
                   alps_complex* Dfinal, int* converged) {
  if (!c || !c->kset || nroots < 0 || (nroots > 0 && !om)) return ALPS_E_INVALID;
  if (method < 0 || method > 2 || !(om_rtol >= 0.0)) return ALPS_E_INVALID;
  std::vector<RootMachine> rm(nroots);
  std::vector<std::vector<cplx>> want(nroots);
  for (int r = 0; r < nroots; ++r) want[r] = rm[r].start(&c->sys, method, cplx(om[r].re, om[r].im), om_rtol);
  std::vector<alps_complex> bom, bD;
  std::vector<cplx> got;
  for (int round = 0; round < 100000; ++round) {
    bom.clear();
    for (int r = 0; r < nroots; ++r)
      for (auto& w : want[r]) bom.push_back(alps_complex{w.real(), w.imag()});
    if (bom.empty()) break;
    bD.resize(bom.size());
    int st = disp_host(c, (int)bom.size(), bom.data(), bD.data(), nullptr);
    if (st) return st;
    size_t k = 0;
    for (int r = 0; r < nroots; ++r) {
      if (want[r].empty()) continue;
      got.clear();
      for (size_t q = 0; q < want[r].size(); ++q, ++k) got.push_back(cplx(bD[k].re, bD[k].im));
      want[r] = rm[r].step(got);
    }
  }
  for (int r = 0; r < nroots; ++r) {
    const cplx o = rm[r].root(), df = rm[r].dfinal();
    om[r] = alps_complex{o.real(), o.imag()};
    if (iters) iters[r] = rm[r].iters();
    if (Dfinal) Dfinal[r] = alps_complex{df.real(), df.imag()};
    if (converged) converged[r] = rm[r].converged() ? 1 : 0;
  }
  return ALPS_OK;
}

int alps_secant(alps_ctx* c, int method, int nroots, alps_complex* om, int* iters, alps_complex* Dfinal) {
  return alps_secant_ex(c, method, nroots, om, 0.0, iters, Dfinal, nullptr);
}

// map_search values (src/ALPS_fns.f90:3595-3788)
// the (nr x ni) frequency lattice of map_search (src/ALPS_fns.f90:3684-3716)
void map_lattice(const alps_map_params* mp, std::vector<alps_complex>& oms) {
  int nr = mp->nr, ni = mp->ni;
  oms.resize((size_t)nr * ni);
  double dr = mp->omf - mp->omi, di = mp->gamf - mp->gami;
  if (nr > 1) dr = (mp->omf - mp->omi) / (1.0 * (nr - 1));
  if (ni > 1) di = (mp->gamf - mp->gami) / (1.0 * (ni - 1));
  for (int ir = 1; ir <= nr; ++ir) {
    double wr = mp->loggridw ? (nr > 1 ? mp->omi * std::pow(mp->omf / mp->omi, (1.0 * (ir - 1)) / (1.0 * (nr - 1)))
                                       : mp->omi)
                             : mp->omi + dr * (1.0 * (ir - 1));
    for (int ii = 1; ii <= ni; ++ii) {
      double wi = mp->loggridg
                      ? (ni > 1 ? mp->gami * std::pow(mp->gamf / mp->gami, (1.0 * (ii - 1)) / (1.0 * (ni - 1)))
                                : mp->gami)
                      : mp->gami + di * (1.0 * (ii - 1));
      oms[(size_t)(ir - 1) * ni + (ii - 1)] = alps_complex{wr, wi};
    }
  }
}

// map_search's sentinels on det D (:3720-3743): cal and log10 of its modulus
void map_finish(int n, const alps_complex* D, alps_complex* cal, double* val) {
  for (int k = 0; k < n; ++k) {
    cplx cc(D[k].re, D[k].im);
    double v = std::log10(std::abs(cc));
    double tmp = cc.real();
    if (cc.imag() == 0.0 && tmp != tmp) {
      cc = 999999.0;
      v = 999999.0;
    }
    if (std::fabs(tmp) > 1.0e100) {
      cc = 899999.0;
      v = 899999.0;
    }
    if (cal) cal[k] = alps_complex{cc.real(), cc.imag()};
    if (val) val[k] = v;
  }
}

int alps_map(alps_ctx* c, const alps_map_params* mp, alps_complex* om_out, alps_complex* cal, double* val) {
  if (!c || !mp || !c->kset || mp->nr < 1 || mp->ni < 1) return ALPS_E_INVALID;
  int n = mp->nr * mp->ni;
  std::vector<alps_complex> oms, D(n);
  map_lattice(mp, oms);
  int st = disp_host(c, n, oms.data(), D.data(), nullptr);
  if (st) return st;
  if (om_out) std::copy(oms.begin(), oms.end(), om_out);
  map_finish(n, D.data(), cal, val);
  return ALPS_OK;
}

}  // extern "C"
