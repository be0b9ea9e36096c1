// alps_internal.cuh -- shared declarations of the GB300 dispersion library.
//
// Layout of the device state of one context (all FP64):
//   per species s (grid N = nperp, M = npar):
//     pperp[N+1], ppar[M+1]           tensor-product grid vectors
//     f0[(N+1)(M+1)]                  f0 table, iperp-major
//     g1, g2 [(N+1)(M+1)]             df0/dpperp and pperp*df0/dppar -
//                                     ppar*df0/dpperp (interior nodes valid)
//     fit[(N+1)*5*nf]                 continuation fit parameters
//     bessel[(nmax+3)(N+1)]           J_n(k_perp pperp_i / q), n = -1..nmax+1
//     V[(nmax+1)(M-1)*12]             reduced vectors of the p_perp
//                                     contraction (k_fold_reduced)
//     mom[(nmax+1)*ALPS_KFAR*12]      Laurent moments of V about the grid
//                                     centre (k_moments)
//   per omega batch: partial sums, resonant-item slots, results.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <map>
#include <vector>

#include "../../include/alps_gb300.h"

#define ALPS_MAX_SPECIES 8
// Laurent terms kept per order for poles far from the p_par grid
#define ALPS_KFAR 128
#define ALPS_PI 3.141592653589793115997963468544185161590576171875

// ---------------------------------------------------------------------------
// complex helpers on double2
// ---------------------------------------------------------------------------
__host__ __device__ inline double2 cmk(double r, double i) { return make_double2(r, i); }
__host__ __device__ inline double2 cadd(double2 a, double2 b) { return cmk(a.x + b.x, a.y + b.y); }
__host__ __device__ inline double2 csub(double2 a, double2 b) { return cmk(a.x - b.x, a.y - b.y); }
__host__ __device__ inline double2 cmul(double2 a, double2 b) {
  return cmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ inline double2 cscale(double2 a, double s) { return cmk(a.x * s, a.y * s); }
__host__ __device__ inline double2 cneg(double2 a) { return cmk(-a.x, -a.y); }
// Smith's division (the Fortran rule for complex division).
__host__ __device__ inline double2 cdiv(double2 a, double2 b) {
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, den = b.x + b.y * r;
    return cmk((a.x + a.y * r) / den, (a.y - a.x * r) / den);
  } else {
    double r = b.x / b.y, den = b.x * r + b.y;
    return cmk((a.x * r + a.y) / den, (a.y * r - a.x) / den);
  }
}
__host__ __device__ inline double cabs_(double2 a) { return hypot(a.x, a.y); }

// ---------------------------------------------------------------------------
// per-species constants visible to kernels (one copy per species)
// ---------------------------------------------------------------------------
struct __align__(16) SpecDev {
  int N, M, nmax, nf;
  int ac_method, log_fit;
  int fit_type[ALPS_MAX_FITS];
  double perp_corr[ALPS_MAX_FITS];
  double qs, ms, ns;
  double dpperp;      // pp(2,2,1) - pp(1,2,1)
  double dppar;       // pp(2,2,2) - pp(2,1,2)  (signed; positive grids)
  double dppar_abs;   // abs of the above
  double idppar, hidpa;  // 1/dppar, 0.5/|dppar|
  double qk;          // qs / kpar at the current k
  int species_index;  // 1-based index (distribution_analyt selects on it)
  double int_ee;      // ee term (omega and k independent)
  const double* pperp;
  const double* ppar;
  const double* f0;
  const double* g1;
  const double* g2;
  const double* fit;
  const double* bessel;
  const double* V;
  const double* mom;  // Laurent moments [(nmax+1)][ALPS_KFAR][12]
  const float* momf;  // the same moments rounded to FP32 (for the series tails)
  const float* momh;  // the moments as float pairs scaled like Vh/Vl (momh + moml)
  const float* moml;
  // V as pairs of floats (hi + lo, ~48 bits) scaled by 2^-e per order, Vscale
  // = 2^e, and ppar as float pairs: the fast path's node sums run on the
  // FP32 pipes in double-float arithmetic
  const float* Vh;
  const float* Vl;
  const double* Vscale;
  const float* pph;
  const float* ppl;
  int df_sums;
  // base tables of the fast path's pole sums: the three Bessel families
  // F1 = J^2, F2 = pperp^2 J'^2, F3 = pperp J J' against g1 and g2 (reduced
  // vectors q = 0, 1, 2, 3, 6, 7), scaled by 1/Vscale[n]:
  //   Bt   [(nmax+1)][M-1][12]       node values, 6 hi then 6 lo floats
  //   mBt  [(nmax+1)][ALPS_KFAR][12] their Laurent moments, the same layout
  //   bfac [(nmax+1)][6][2]          order factors C0 v_e(n) Vscale[n] / Escale[e]
  //                                  as float pairs, entries xx yy zz xy xz yz
  //   Escale[6]                      powers of two
  //   Pre  [(nmax+1)][M][6]          FP64 prefix sums over j of the weighted
  //                                  vectors F1, F3, ppar F1 (g1, g2 each)
  //   Cfull[(nmax+1)][6]             their full-range trapezoid sums
  // FP32 resonance bounds
  const float *Bt, *mBt, *bfac;
  const double *Escale, *Pre, *Cfull;
  float qlo, qhi;        // below / above these Re p_res is not resonant
  float qlo_in, qhi_in;  // between these it is
  float kaph, kapl;   // k_par / m_s as a float pair
  float hidh, hidl;   // hidpa as a float pair
  float dpph, dppl;   // dppar (signed) as a float pair
  float idph, idpl;   // 1/dppar as a float pair
  float tpmh, tpml;   // 2 pi M_P as a float pair
  double kappa;       // k_par / m_s
  double pvc;         // 2 pi dpperp/4 (-q/(2 k_par)): the principal-value scale over smdelta
  double pcen, prad;  // centre and half-width of ppar[1..M-1]
  float pcen32, prad32;  // the same rounded to FP32
  int kfar;           // max Laurent terms used (<= ALPS_KFAR)
  int rcap;           // resonant-item slots per (omega, species)
  // [(N+1)][nf][4] = {p1 exp(-pc pperp^2), p2, p3, exp(-p2 dppar^2)} when
  // every fit term is a Maxwellian (ACmethod 1, type 1); else null
  const double* fit_aux;
  // factorised Landau sums (one Maxwellian term): moments
  // lmom[((n*3 + F)*2 + w)*5 + m], reference row Gaussian exp(-p2r (p-p3r)^2),
  // bounds of the row deviation delta_i(p) = la p^2 + lb p + lc, smallest a0
  const double* lmom;
  double p2r, p3r, la, lb, lc, min_a0;
  double lgc;  // exp(-p2r dppar^2)
  // the fast path's copy of the moments: per (n, F) ten float pairs scaled
  // by 2^-e (hi 0..9, lo 10..19, e at 20, 24 floats); the bound's
  // coefficients in FP32, lgc as a float pair, -2 p2r dppar, and the
  // exponents of min_a0 and lgc (the underflow test of the row Gaussians)
  const float* lmomf;
  float la32, lb32, lc32, lgch, lgcl;
  double lcx;
  int lze, lge;
  // relativistic species (src/ALPS_fns_rel.f90): (Gamma, pparbar) grid
  int relat, ng, np;
  const double* grel;   // [ng+1]
  const double* prel;   // [np+1]
  const double* f0rel;  // [(ng+1)*(np+1)], -1 outside the subluminal cone
  const double* dfr1;   // d f0_rel / d Gamma
  const double* dfr2;   // d f0_rel / d pparbar
  const double* jrel;   // [(n)*(ng+1)*(np+1)], n = 0..nmax+1: J_n at each node
  const int2* cone;     // [ng+1] first and last pparbar index inside the cone
  double int_ee_rel;
  // Chebyshev continuation (ACmethod 2): order, log10 cut, p_par end points
  int poly_order;
  double poly_log_max, ppar_lo, ppar_hi;
  // bi-Maxwellian / cold species through the NHDS closed form (use_bM)
  int bm;
  int bm_nrun;          // Bessel orders -bm_nrun..bm_nrun
  double bm_beta, bm_alpha, bm_pdrift;
  const double* bmI;    // exp(-z) I_n(z), n = 0..bm_nrun+1, z from k_perp
};

struct __align__(16) SysDev {
  int nspec;
  int kperp_norm;
  int M_I, M_P;
  double Tlim, vA;
  double kperp, kpar;
  double ikpar;  // 1 / kpar
};

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct SpeciesHost {
  alps_species sp;
  bool loaded = false;
  std::vector<double> pperp, ppar, f0;   // host copies (grid vectors, table)
  double *d_pperp = nullptr, *d_ppar = nullptr, *d_f0 = nullptr;
  double *d_g1 = nullptr, *d_g2 = nullptr, *d_fit = nullptr;
  double* d_bessel = nullptr;
  size_t bessel_cap = 0;
  double* d_V = nullptr;
  size_t V_cap = 0;
  double* d_A = nullptr;                  // contraction output scratch
  size_t A_cap = 0;
  void* d_tcws = nullptr;                 // tensor-core contraction workspace (mixed path)
  size_t tcws_cap = 0;
  int tc_used = 0;                        // the current reduced vectors came from the tensor cores
  int tc_fixed = 0;                       // of their entries, recomputed in FP64
  int* d_nmax = nullptr;                  // determine_nmax's result word
  double* d_words = nullptr;              // ee term and fit status words of prepare
  double* d_fit_scratch = nullptr;        // Levenberg-Marquardt scratch
  size_t fit_scratch_cap = 0;
  double* d_Rw = nullptr;                 // weighted Bessel rows scratch
  size_t Rw_cap = 0;
  double* d_G = nullptr;                  // contraction RHS [2][N-1][M-1]
  double* d_X = nullptr;                  // x_j^k, x_j = (ppar_j - pcen)/prad
  double* d_mom = nullptr;                // Laurent moments
  float* d_momf = nullptr;                // the same in FP32; the pairs below share its allocation
  float *d_momh = nullptr, *d_moml = nullptr;  // the moments as float pairs (scale Vscale per order)
  float* d_Bt = nullptr;                  // base tables of the fast pole sums: Bt, mBt, bfac
  size_t Bt_cap = 0;
  double* d_Bd = nullptr;                 // and their FP64 part: Escale[8], Cfull, Pre
  size_t Bd_cap = 0;
  float qlo = 0.0f, qhi = 0.0f;           // FP32 bounds of the resonance interval (margin outward)
  float qlo_in = 1.0f, qhi_in = -1.0f;    // the same with the margin inward
  float *d_Vh = nullptr, *d_Vl = nullptr;  // V as float pairs (one allocation, lo after hi)
  size_t Vf_cap = 0;
  double* d_Vscale = nullptr;             // per-order scale of the pairs
  size_t Vs_cap = 0;
  float *d_pph = nullptr, *d_ppl = nullptr;  // ppar as float pairs
  size_t momf_cap = 0;
  double* d_fit_aux = nullptr;            // Maxwellian continuation factors
  bool aux_ready = false;                 // d_fit_aux and the Landau row bounds are those of the current fit
  double* d_lmom = nullptr;               // factorised Landau moments
  size_t lmom_cap = 0;
  double p2r = 0, p3r = 0, la = 0, lb = 0, lc = 0, min_a0 = 0;
  bool lfact = false;
  // relativistic species
  std::vector<double> grel, prel;         // host copies of the grid vectors
  double *d_grel = nullptr, *d_prel = nullptr, *d_f0rel = nullptr, *d_dfr1 = nullptr, *d_dfr2 = nullptr;
  double* d_jrel = nullptr;
  int2* d_cone = nullptr;
  // NHDS species: exp(-z) I_n(z) table of the current k_perp
  double* d_bmI = nullptr;
  int bm_nrun = 0;
  size_t jrel_cap = 0;
  double int_ee_rel = 0.0;
  size_t mom_cap = 0;
  int nmax = 0;
  double int_ee = 0.0;
  double current_int = 0.0;  // n q P_par / m moment of the f0 table
  int rcap = 1;
};

struct alps_ctx {
  alps_system sys;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<SpeciesHost> spec;
  bool prepared = false, kset = false;
  double kperp = 0, kpar = 0;
  int precision = ALPS_PREC_FP64;
  // batch buffers
  size_t batch_cap = 0;
  double2* d_om = nullptr;      // [n]
  double2* d_D = nullptr;       // [n]
  double2* d_part = nullptr;    // [n][S][nchunk][6]
  size_t part_cap = 0;
  double2* d_low = nullptr;     // [n][S][nchunk][3][6]
  size_t low_cap = 0;
  int* d_count = nullptr;       // [n][S]
  size_t count_cap = 0;
  int* d_slot_nn = nullptr;     // [n][S][rcap]
  double2* d_items = nullptr;   // [n][S][rcap][6]
  size_t items_cap = 0;
  double2* d_ext = nullptr;     // [n][S*9 + S*27 + 9] extended outputs
  double2* d_rel = nullptr;     // [n][S][2*nmax+1][6] relativistic orders
  size_t rel_cap = 0;
  double2* d_bm = nullptr;      // [n][S][24] NHDS chi (6) and chi_low (3 x 6)
  size_t bm_cap = 0;
  size_t ext_cap = 0;
  int* d_flags = nullptr;       // error flags
  bool defer_sync = false;      // set_k of a batch (alps_set_k_many): no per-context synchronisation
  // error word of the last asynchronous batch (alps_disp_batch_device: d_flags;
  // alps_disp_batch_noalloc: a word of the static scratch), read by
  // alps_batch_status
  const int* async_flags = nullptr;
  alps_stats stats = {};
  // profiling: pending event sets (5 events per batch) and totals
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::vector<cudaEvent_t>> ev_pending;
  double prof_ms[4] = {0, 0, 0, 0};
  int64_t prof_batches = 0;
  // host pinned staging
  double2* h_pinned = nullptr;
  size_t pinned_cap = 0;
  int* h_flag = nullptr;                // pinned copy of the device error flags
  cudaEvent_t ev_done = nullptr;        // completion of an asynchronous batch
  // CUDA graphs of whole batches (upload, kernels, download) by batch size,
  // valid while gen (bumped by every change of the plasma, k, precision or
  // any batch buffer address) is unchanged
  uint64_t gen = 1;
  std::map<int, std::pair<uint64_t, cudaGraphExec_t>> graphs;
  std::map<int, uint64_t> graph_seen;  // gen of the last uncaptured batch of each size
  // device copy of the kernel arguments for fused batches, valid while
  // args_gen == gen
  void* d_args = nullptr;
  void* d_job = nullptr;  // the job table of a lone batch
  void* h_args = nullptr;
  uint64_t args_gen = 0;
  int args_maxn = 0, args_rcap = 0;
};

// ---------------------------------------------------------------------------
// kernels / launchers (setup_kernels.cu, disp_kernels.cu)
// ---------------------------------------------------------------------------
int launch_prepare_species(alps_ctx* c, int is);
// host helpers shared by the entry points and the request server (defined
// inside the extern "C" block of alps_api.cu and server.cu)
extern "C" {
int ctx_ensure_batch(alps_ctx* c, int n, bool ext);  // d_om, d_D, pinned staging for n frequencies
int ctx_check_flags(alps_ctx* c);                    // device error flags of the last batch
size_t ctx_device_bytes(const alps_ctx* c);          // device memory a context holds (estimate)
void map_lattice(const alps_map_params* mp, std::vector<alps_complex>& oms);
void map_finish(int n, const alps_complex* D, alps_complex* cal, double* val);
}
int launch_glls(alps_ctx* c, int is);
// batched setup of many contexts (setup_kernels.cu)
bool ctx_batch_preparable(const alps_ctx* c);
int prepare_contexts(alps_ctx* const* ctx, int n, int* status);
int nmax_contexts(alps_ctx* const* ctx, int n, const double* kperp, std::vector<std::vector<int>>& nm);
int launch_set_k_species(alps_ctx* c, int is, double kperp, int* nmax_out);
int launch_build_bessel_and_reduced(alps_ctx* c, int is, double kperp);
int launch_fit_aux(alps_ctx* c, int is);
int launch_landau_moments(alps_ctx* c, int is);
int launch_rel_prepare(alps_ctx* c, int is);
int launch_rel_bessel(alps_ctx* c, int is, double kperp);
// NHDS species: the I_n table of k_perp (per k) and chi per omega,
// out[(w*nspec + s)*24 + {0..5 chi, 6 + 6*(n+1) + e chi_low}]
int launch_nhds_bessel(alps_ctx* c, int is, double kperp);
int launch_nhds(const SysDev& sys, const SpecDev* sp, int n, const double2* d_om, double2* d_out, cudaStream_t st);
// relativistic orders: REL_RB blocks of REL_THREADS threads per (omega,
// species, signed order), each with its own partial slot
// a launch shape of the batch kernels chosen by the autotuner (0: the
// default rule's value)
struct TuneShape {
  int js = 0;             // j slices per omega of the pole sums (power of 2, <= 32)
  int blocks_per_sm = 0;  // pole-sum blocks per SM the order chunks aim at
  int warps_per_sm = 0;   // resident warps per SM the resonant slots spread over
};
// moves whenever the autotuner's table changes (captured graphs compare it)
uint64_t tune_epoch();

#define REL_RB 4
#define REL_THREADS 256
// per-order relativistic partials out[(((w*nspec + s)*relcap + n)*2 + sign)*REL_RB + rb][6]
int launch_rel_orders(const SysDev& sys, const SpecDev* sp, int relcap, int n, const double2* d_om, double2* d_out,
                      int* d_flags, cudaStream_t st);
int launch_disp_batch(alps_ctx* c, int n, const double2* d_om, double2* d_D, double2* d_ext,
                      cudaStream_t st);
// Fused batches: nj contexts, context j with n[j] frequencies at
// d_om[o_j ...] (o_j = n[0] + ... + n[j-1]), det D to d_D at the same
// offsets and the error flags of context j to d_flags[j].  Every context is
// evaluated with the launch shape, and so the sums, of a lone batch of its
// size.  Contexts with relativistic or closed-form species are not fusable.
struct MultiScratch;
int launch_disp_multi(alps_ctx* const* ctx, const int* n, int nj, const double2* d_om, double2* d_D, int* d_flags,
                      MultiScratch** scratch, cudaStream_t st);
void multi_scratch_free(MultiScratch* m);
// The same split in two: prepare_disp_multi builds and uploads the job table
// and sizes the scratch (host work, synchronous allocations);
// run_disp_multi launches the kernels of a prepared batch (device work only,
// so it can be captured, also into a conditional graph body).  The prepared
// batch stays valid while the contexts, their k and precision and the
// scratch are unchanged.
struct MultiLaunch {
  const void* jobs;  // device job table
  int nj;
  long blocks[4];    // grids of classify, pole sums, resonant, finalize
  size_t smem;       // dynamic shared memory of k_resonant_multi
  int* flags;        // error words, one per job
};
int prepare_disp_multi(alps_ctx* const* ctx, const int* n, int nj, const double2* d_om, double2* d_D, int* d_flags,
                       MultiScratch** scratch, cudaStream_t st, MultiLaunch* out);
int run_disp_multi(const MultiLaunch& ml, cudaStream_t st);
void disp_job_layout(size_t* stride, size_t* n_offset);
bool ctx_fusable(const alps_ctx* c);
void fill_spec_dev(const alps_ctx* c, int is, SpecDev* out);
int collect_profile(alps_ctx* c);
void fill_sys_dev(const alps_ctx* c, SysDev* out);

#define ALPS_CUDA_TRY(x)                                  \
  do {                                                    \
    cudaError_t _e = (x);                                 \
    if (_e != cudaSuccess) {                              \
      alps_set_last_cuda_error(_e, #x, __FILE__, __LINE__); \
      return (_e == cudaErrorMemoryAllocation) ? ALPS_E_OOM : ALPS_E_CUDA; \
    }                                                     \
  } while (0)

void alps_set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line);
