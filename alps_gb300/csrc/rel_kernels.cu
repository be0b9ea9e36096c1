// rel_kernels.cu -- relativistic species (src/ALPS_fns_rel.f90).
//
// Setup per run (launch_rel_prepare): the (Gamma, pparbar) grid spanning the
// f0 table, a thin-plate-spline interpolation of log f0 onto it (dense
// saddle-point system, LU with partial pivoting as dgesv does), the subluminal-cone
// mask (f0_rel = -1 outside), normalisation, and the one-sided derivatives at
// the cone edge (derivative_f0_rel, :36-289; polyharmonic_spline, :293-426),
// then the ee term (int_ee_rel, :1097-1215).
// Per k (launch_rel_bessel): J_n at every (Gamma, pparbar) node; the
// reference calls BESSJ there once per point and mode (int_T_rel, :1297-1298),
// with omega-independent arguments, so a table holds the same values.
// Per omega batch (launch_rel_orders): one block per (omega, species, n):
// the resonance test over the whole (pperp, ppar) grid (determine_resonances,
// src/ALPS_fns.f90:680-702), then either the regular-grid trapezoid sum with
// the Lorentz factor in resU (src/ALPS_fns.f90:799-864, 1560-1596) or the
// Gamma-row integrals with their principal-value windows and the Landau term
// (integrate_res_rel :460-913, landau_integrate_rel :1005-1092).
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include <cusolverDn.h>

#include "alps_internal.cuh"
#include "device_math.cuh"

namespace {

__device__ __host__ inline double cube(double x) { return x * x * x; }

// ---------------------------------------------------------------------------
// thin-plate spline
// ---------------------------------------------------------------------------
__device__ inline double tps_phi(double r) {
  if (r >= 1.0) return r * r * log(r);
  if (r == 0.0) return 0.0;
  return r * log(pow(r, r));
}

// column-major (n+3)^2 system of polyharmonic_spline, the smoothing added
// on the diagonal of the kernel block
__global__ void k_tps_matrix(const double* __restrict__ gc, const double* __restrict__ pc, int n, double smoothing,
                             double* A) {
  long m = n + 3;
  long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m * m) return;
  int i = (int)(t % m), j = (int)(t / m);
  double v = 0.0;
  if (i < n && j < n) {
    double dg = gc[i] - gc[j], dp = pc[i] - pc[j];
    v = tps_phi(sqrt(dg * dg + dp * dp));
    if (i == j) v = v + smoothing;
  } else if (i < n && j >= n) {
    v = (j == n) ? 1.0 : (j == n + 1 ? gc[i] : pc[i]);
  } else if (j < n && i >= n) {
    v = (i == n) ? 1.0 : (i == n + 1 ? gc[j] : pc[j]);
  }
  A[t] = v;
}

// Dense LU with partial pivoting, column by column (the dgetrf/dgetrs pair of
// dgesv).  Column-major m x m.  Step k: k_lu_pivot (one block) picks the
// first row of largest |A(i,k)|, swaps the whole rows and scales column k;
// k_lu_update applies the rank-1 update to columns k+1..m-1.
__global__ void k_lu_pivot(double* A, int m, int k, int* piv, int* status) {
  __shared__ double sv[1024];
  __shared__ int si[1024];
  __shared__ int sp;
  if (*status) return;
  double mx = -1.0;
  int p = m;
  for (int i = k + threadIdx.x; i < m; i += blockDim.x) {
    double v = fabs(A[(size_t)i + (size_t)m * k]);
    if (v > mx) {
      mx = v;
      p = i;
    }
  }
  sv[threadIdx.x] = mx;
  si[threadIdx.x] = p;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      double v2 = sv[threadIdx.x + s];
      int i2 = si[threadIdx.x + s];
      if (v2 > sv[threadIdx.x] || (v2 == sv[threadIdx.x] && i2 < si[threadIdx.x])) {
        sv[threadIdx.x] = v2;
        si[threadIdx.x] = i2;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    int q = si[0];
    if (q >= m) q = k;  // column of NaNs: keep the diagonal
    sp = q;
    piv[k] = q;
    if (A[(size_t)q + (size_t)m * k] == 0.0) *status = 1;
  }
  __syncthreads();
  const int q = sp;
  if (q != k)
    for (int j = threadIdx.x; j < m; j += blockDim.x) {
      double t = A[(size_t)k + (size_t)m * j];
      A[(size_t)k + (size_t)m * j] = A[(size_t)q + (size_t)m * j];
      A[(size_t)q + (size_t)m * j] = t;
    }
  __syncthreads();
  const double dk = A[(size_t)k + (size_t)m * k];
  if (dk != 0.0)
    for (int i = k + 1 + threadIdx.x; i < m; i += blockDim.x)
      A[(size_t)i + (size_t)m * k] = __ddiv_rn(A[(size_t)i + (size_t)m * k], dk);
}

__global__ void k_lu_update(double* A, int m, int k, const int* status) {
  if (*status) return;
  const int j = k + 1 + blockIdx.x;
  if (j >= m) return;
  const double f = A[(size_t)k + (size_t)m * j];
  if (f == 0.0) return;
  double* colj = A + (size_t)m * j;
  const double* colk = A + (size_t)m * k;
  for (int i = k + 1 + threadIdx.x; i < m; i += blockDim.x) colj[i] = __dsub_rn(colj[i], __dmul_rn(colk[i], f));
}

// row interchanges, then the unit-lower and upper triangular solves
__global__ void k_lu_solve(const double* A, int m, const int* piv, double* w, const int* status) {
  if (*status) return;
  if (threadIdx.x == 0)
    for (int k = 0; k < m; ++k) {
      double t = w[k];
      w[k] = w[piv[k]];
      w[piv[k]] = t;
    }
  __syncthreads();
  for (int j = 0; j < m; ++j) {
    const double wj = w[j];
    for (int i = j + 1 + threadIdx.x; i < m; i += blockDim.x)
      w[i] = __dsub_rn(w[i], __dmul_rn(A[(size_t)i + (size_t)m * j], wj));
    __syncthreads();
  }
  for (int j = m - 1; j >= 0; --j) {
    if (threadIdx.x == 0) w[j] = __ddiv_rn(w[j], A[(size_t)j + (size_t)m * j]);
    __syncthreads();
    const double wj = w[j];
    for (int i = threadIdx.x; i < j; i += blockDim.x)
      w[i] = __dsub_rn(w[i], __dmul_rn(A[(size_t)i + (size_t)m * j], wj));
    __syncthreads();
  }
}

// f0_rel = exp(spline) on the fine grid, -1 outside the subluminal cone
__global__ void k_tps_eval(const double* __restrict__ w, const double* __restrict__ gc, const double* __restrict__ pc,
                           int n, const double* __restrict__ grel, const double* __restrict__ prel, int ng, int np,
                           double* f0rel) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (ng + 1) * (np + 1)) return;
  int ig = t / (np + 1), ip = t % (np + 1);
  double g = grel[ig], pb = prel[ip], f = 0.0;
  for (int k = 0; k < n; ++k) {
    double dg = g - gc[k], dp = pb - pc[k];
    double r = sqrt(dg * dg + dp * dp);
    if (r >= 1.0) f = f + w[k] * r * r * log(r);
    else if (r != 0.0) f = f + w[k] * r * log(pow(r, r));
  }
  f = f + w[n] + w[n + 1] * g + w[n + 2] * pb;
  f = exp(f);
  // outside the subluminal cone, decided as the reference rounds it (no FMA)
  if (__dsub_rn(__dmul_rn(g, g), 1.0) < __dmul_rn(pb, pb)) f = -1.0;
  f0rel[t] = f;
}

// integral of f0_rel over the cone (one block, fixed reduction order)
__global__ void k_rel_norm(double* f0rel, const double* __restrict__ grel, int ng, int np, double scale) {
  __shared__ double red[256];
  double acc = 0.0;
  int tot = (ng + 1) * (np + 1);
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    double f = f0rel[t];
    if (f > -1.0) acc += grel[t / (np + 1)] * f * scale;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  double integ = red[0];
  __syncthreads();
  for (int t = threadIdx.x; t < tot; t += blockDim.x)
    if (f0rel[t] != -1.0) f0rel[t] = f0rel[t] / integ;
}

__global__ void k_rel_deriv(const double* __restrict__ f, const double* __restrict__ grel,
                            const double* __restrict__ prel, int ng, int np, double* d1, double* d2) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (ng + 1) * (np + 1)) return;
  int ig = t / (np + 1), ip = t % (np + 1);
  d1[t] = 0.0;
  d2[t] = 0.0;
  if (ig < 1 || ig > ng - 1 || ip < 1 || ip > np - 1) return;
  int L = np + 1;
  auto F = [&](int a, int b) { return f[a * L + b]; };
  if ((F(ig - 1, ip) > 0.0) && (F(ig + 1, ip) > 0.0)) d1[t] = (F(ig + 1, ip) - F(ig - 1, ip)) / (grel[ig + 1] - grel[ig - 1]);
  if ((F(ig, ip + 1) > 0.0) && (F(ig, ip - 1) > 0.0)) d2[t] = (F(ig, ip + 1) - F(ig, ip - 1)) / (prel[ip + 1] - prel[ip - 1]);
  if (F(ig, ip) >= 0.0) {
    if ((F(ig, ip + 1) <= 0.0) && (F(ig, ip - 1) > 0.0)) d2[t] = (F(ig, ip) - F(ig, ip - 1)) / (prel[ip] - prel[ip - 1]);
    if ((F(ig, ip + 1) > 0.0) && (F(ig, ip - 1) <= 0.0)) d2[t] = (F(ig, ip + 1) - F(ig, ip)) / (prel[ip + 1] - prel[ip]);
  }
}

__device__ inline void cone_limits(const double* fr, int np, int& lower, int& upper) {
  bool fl = false, fu = false;
  lower = 1;
  upper = np - 1;
  for (int ip = 1; ip <= np - 1; ++ip) {
    if (!fl && fr[ip - 1] <= -1.0 && fr[ip] > -1.0) { lower = ip; fl = true; }
    if (!fu && fr[ip] > -1.0 && fr[ip + 1] <= -1.0) { upper = ip; fu = true; }
  }
}

// int_ee_rel: one block
__global__ void k_rel_ee(const double* __restrict__ f0rel, const double* __restrict__ dfr2,
                         const double* __restrict__ prel, int ng, int np, double scale, double* out) {
  __shared__ double red[256];
  double acc = 0.0;
  int L = np + 1;
  for (int ig = 1 + threadIdx.x; ig <= ng - 1; ig += blockDim.x) {
    int lo, up;
    cone_limits(f0rel + (size_t)ig * L, np, lo, up);
    auto t = [&](int ip) { return prel[ip] * dfr2[(size_t)ig * L + ip]; };
    double wi = (ig == ng - 1) ? 1.0 : 2.0;   // Gamma weight; pparbar weights 1 at ends, 2 inside
    double row = t(lo) + t(up);
    for (int ip = lo + 1; ip <= up - 1; ++ip) row += 2.0 * t(ip);
    acc += wi * row;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0] * scale;
}

// J_n(z(ig, ip)), z = (k_perp m/(vA q)) sqrt(Gamma^2 - 1 - pparbar^2)
__global__ void k_rel_jtab(const double* __restrict__ grel, const double* __restrict__ prel, int ng, int np, int nrows,
                           double zfac, double* jrel) {
  long tot = (long)(ng + 1) * (np + 1);
  long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= tot * nrows) return;
  int n = (int)(t / tot);
  long pt = t % tot;
  int ig = (int)(pt / (np + 1)), ip = (int)(pt % (np + 1));
  double g = grel[ig], pb = prel[ip];
  double pperpbar = sqrt(g * g - 1.0 - pb * pb);
  double z = zfac * pperpbar;
  jrel[t] = (z == z) ? alps_bessj(n, z) : z;
}

// first and last pparbar index inside the cone of each Gamma row
// (integrate_resU_rel, src/ALPS_fns_rel.f90:603-617)
__global__ void k_rel_cone(const double* __restrict__ f0rel, int ng, int np, int2* cone) {
  int ig = blockIdx.x * blockDim.x + threadIdx.x;
  if (ig > ng) return;
  int lo, up;
  cone_limits(f0rel + (size_t)ig * (np + 1), np, lo, up);
  cone[ig] = make_int2(lo, up);
}

// right-hand side of the spline system: log f at the samples, three zeros
__global__ void k_tps_rhs(const double* __restrict__ f, int n, double* w) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) w[k] = log(f[k]);
  else if (k < n + 3) w[k] = 0.0;
}

// spline (log f) on the tensor grid pperp[i] x ppar[j], [i*(npar+1) + j]
// (the evaluation loop of polyharmonic_spline, interpolation.f90:610-630)
__global__ void k_tps_eval_grid(const double* __restrict__ w, const double* __restrict__ gc,
                                const double* __restrict__ pc, int n, const double* __restrict__ pperp,
                                const double* __restrict__ ppar, int nperp, int npar, double* g) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (nperp + 1) * (npar + 1)) return;
  const int i = t / (npar + 1), j = t % (npar + 1);
  const double x = pperp[i], y = ppar[j];
  double f = 0.0;
  for (int k = 0; k < n; ++k) {
    double dg = x - gc[k], dp = y - pc[k];
    double r = sqrt(dg * dg + dp * dp);
    if (r >= 1.0) f = f + w[k] * r * r * log(r);
    else if (r != 0.0) f = f + w[k] * r * log(pow(r, r));
  }
  g[t] = f + w[n] + w[n + 1] * x + w[n + 2] * y;
}

// f = mult exp(g - shift), shift = log(2 pi dpperp dppar sum_ij exp(g) pperp_i)
// when normalising (normalize, interpolation.f90:520-552); one block, fixed
// reduction order
__global__ void k_interp_finish(const double* __restrict__ g, const double* __restrict__ pperp, int nperp, int npar,
                                double dpp, double dpl, int normalize, double mult, double* f) {
  __shared__ double red[256];
  const int tot = (nperp + 1) * (npar + 1);
  double shift = 0.0;
  if (normalize) {
    double acc = 0.0;
    for (int t = threadIdx.x; t < tot; t += blockDim.x) acc += exp(g[t]) * pperp[t / (npar + 1)];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
      __syncthreads();
    }
    shift = log(red[0] * dpp * dpl * 2.0 * ALPS_PI);
  }
  for (int t = threadIdx.x; t < tot; t += blockDim.x) f[t] = mult * exp(g[t] - shift);
}

}  // namespace

// ---------------------------------------------------------------------------
// Large spline systems: cuSOLVER's blocked LU with partial pivoting (getrf,
// getrs: the dgesv pair), loaded on first use.  The column-by-column LU above
// restates dgesv's arithmetic for the sizes the oracle can check; from
// TPS_BLOCKED_M unknowns on (a 128 x 256 input grid has 33 156) its one pass
// per column would take minutes, and the blocked factorisation runs at the
// FP64 GEMM rate instead.
// ---------------------------------------------------------------------------
#define TPS_BLOCKED_M 4096

struct CusolverApi {
  bool tried = false, ok = false;
  cusolverStatus_t (*create)(cusolverDnHandle_t*) = nullptr;
  cusolverStatus_t (*destroy)(cusolverDnHandle_t) = nullptr;
  cusolverStatus_t (*set_stream)(cusolverDnHandle_t, cudaStream_t) = nullptr;
  cusolverStatus_t (*getrf_ws)(cusolverDnHandle_t, int, int, double*, int, int*) = nullptr;
  cusolverStatus_t (*getrf)(cusolverDnHandle_t, int, int, double*, int, double*, int*, int*) = nullptr;
  cusolverStatus_t (*getrs)(cusolverDnHandle_t, cublasOperation_t, int, int, const double*, int, const int*,
                            double*, int, int*) = nullptr;
};
std::mutex g_cusolver_mu;
CusolverApi g_cusolver;

const CusolverApi* cusolver_api() {
  std::lock_guard<std::mutex> lk(g_cusolver_mu);
  if (g_cusolver.tried) return g_cusolver.ok ? &g_cusolver : nullptr;
  g_cusolver.tried = true;
  const char* names[] = {"libcusolver.so.12", "libcusolver.so", "/usr/local/cuda/lib64/libcusolver.so.12",
                         "/usr/local/cuda/lib64/libcusolver.so"};
  void* h = nullptr;
  for (const char* nm : names)
    if ((h = dlopen(nm, RTLD_NOW | RTLD_LOCAL))) break;
  if (!h) return nullptr;
  CusolverApi& a = g_cusolver;
  a.create = reinterpret_cast<decltype(a.create)>(dlsym(h, "cusolverDnCreate"));
  a.destroy = reinterpret_cast<decltype(a.destroy)>(dlsym(h, "cusolverDnDestroy"));
  a.set_stream = reinterpret_cast<decltype(a.set_stream)>(dlsym(h, "cusolverDnSetStream"));
  a.getrf_ws = reinterpret_cast<decltype(a.getrf_ws)>(dlsym(h, "cusolverDnDgetrf_bufferSize"));
  a.getrf = reinterpret_cast<decltype(a.getrf)>(dlsym(h, "cusolverDnDgetrf"));
  a.getrs = reinterpret_cast<decltype(a.getrs)>(dlsym(h, "cusolverDnDgetrs"));
  a.ok = a.create && a.destroy && a.set_stream && a.getrf_ws && a.getrf && a.getrs;
  return a.ok ? &a : nullptr;
}

// LU with partial pivoting and the solve of A w = w (column-major m x m, d_A
// overwritten) through cuSOLVER; ALPS_E_SINGULAR for an exactly singular
// pivot, ALPS_E_UNSUPPORTED when the library cannot be loaded
int tps_lu_blocked(double* d_A, int m, double* d_w, cudaStream_t st) {
  const CusolverApi* api = cusolver_api();
  if (!api) return ALPS_E_UNSUPPORTED;
  cusolverDnHandle_t h = nullptr;
  if (api->create(&h) != CUSOLVER_STATUS_SUCCESS) return ALPS_E_CUDA;
  int status = ALPS_OK, lwork = 0, info = 0;
  double* d_work = nullptr;
  int *d_piv = nullptr, *d_info = nullptr;
  if (api->set_stream(h, st) != CUSOLVER_STATUS_SUCCESS || api->getrf_ws(h, m, m, d_A, m, &lwork) !=
                                                               CUSOLVER_STATUS_SUCCESS)
    status = ALPS_E_CUDA;
  if (!status && (cudaMalloc(&d_work, (size_t)std::max(lwork, 1) * sizeof(double)) != cudaSuccess ||
                  cudaMalloc(&d_piv, (size_t)m * sizeof(int)) != cudaSuccess ||
                  cudaMalloc(&d_info, sizeof(int)) != cudaSuccess))
    status = ALPS_E_OOM;
  if (!status && api->getrf(h, m, m, d_A, m, d_work, d_piv, d_info) != CUSOLVER_STATUS_SUCCESS) status = ALPS_E_CUDA;
  if (!status) {
    if (cudaMemcpyAsync(&info, d_info, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      status = ALPS_E_CUDA;
    else if (info != 0)
      status = ALPS_E_SINGULAR;
  }
  if (!status && api->getrs(h, CUBLAS_OP_N, m, 1, d_A, m, d_piv, d_w, m, d_info) != CUSOLVER_STATUS_SUCCESS)
    status = ALPS_E_CUDA;
  if (!status && cudaStreamSynchronize(st) != cudaSuccess) status = ALPS_E_CUDA;
  cudaFree(d_work);
  cudaFree(d_piv);
  cudaFree(d_info);
  api->destroy(h);
  return status;
}

// Weights of the thin-plate spline through n samples (gc, pc) with the
// right-hand side already in d_w (n + 3 entries): the dense system of
// polyharmonic_spline solved by LU with partial pivoting (dgesv).
int tps_solve_device(const double* d_gc, const double* d_pc, int n, double smoothing, double* d_w, cudaStream_t st) {
  const int m = n + 3;
  double* d_A = nullptr;
  int *d_piv = nullptr, *d_info = nullptr;
  int status = ALPS_OK;
  if (cudaMalloc(&d_A, (size_t)m * m * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&d_piv, m * sizeof(int)) != cudaSuccess || cudaMalloc(&d_info, sizeof(int)) != cudaSuccess) {
    status = ALPS_E_OOM;
  }
  if (!status && cudaMemsetAsync(d_info, 0, sizeof(int), st) != cudaSuccess) status = ALPS_E_CUDA;
  if (!status) {
    long mm = (long)m * m;
    k_tps_matrix<<<(unsigned)((mm + 255) / 256), 256, 0, st>>>(d_gc, d_pc, n, smoothing, d_A);
    if (cudaGetLastError() != cudaSuccess) status = ALPS_E_CUDA;
  }
  if (!status && m >= TPS_BLOCKED_M) {
    status = tps_lu_blocked(d_A, m, d_w, st);
    cudaFree(d_A);
    cudaFree(d_piv);
    cudaFree(d_info);
    return status;
  }
  for (int k = 0; k < m && !status; ++k) {
    k_lu_pivot<<<1, 1024, 0, st>>>(d_A, m, k, d_piv, d_info);
    if (k + 1 < m) k_lu_update<<<m - k - 1, 256, 0, st>>>(d_A, m, k, d_info);
    if (cudaGetLastError() != cudaSuccess) status = ALPS_E_CUDA;
  }
  if (!status) {
    k_lu_solve<<<1, 1024, 0, st>>>(d_A, m, d_piv, d_w, d_info);
    int info = 0;
    cudaMemcpyAsync(&info, d_info, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) status = ALPS_E_CUDA;
    else if (info != 0) status = ALPS_E_SINGULAR;
  }
  cudaFree(d_A);
  cudaFree(d_piv);
  cudaFree(d_info);
  return status;
}

// ===========================================================================
int launch_rel_prepare(alps_ctx* c, int is) {
  SpeciesHost& S = c->spec[is];
  const double vA = c->sys.vA, ms = S.sp.ms;
  const int N = c->sys.nperp, M = c->sys.npar, ng = c->sys.ngamma, np = c->sys.npparbar;
  cudaStream_t st = c->stream;
  // grid spanning the table (derivative_f0_rel :120-171), on the host
  double pmin = 999999.0, pmax = -999999.0, gmin = 999999.0, gmax = -1.0;
  int n = (N + 1) * (M + 1);
  std::vector<double> gc(n), pc(n), grid(n);
  for (int i = 0; i <= N; ++i)
    for (int j = 0; j <= M; ++j) {
      double p1 = S.pperp[i], p2 = S.ppar[j];
      double g = std::sqrt((p1 * p1 + p2 * p2) * (vA * vA) / (ms * ms) + 1.0);
      gmax = std::max(gmax, g);
      gmin = std::min(gmin, g);
      pmin = std::min(pmin, p2);
      pmax = std::max(pmax, p2);
      int k = i * (M + 1) + j;
      gc[k] = std::sqrt(1.0 + (p1 * p1 + p2 * p2) * vA * vA / (ms * ms));
      pc[k] = p2 * vA / ms;
      grid[k] = std::log(S.f0[k]);
    }
  pmin = pmin * vA / ms;
  pmax = pmax * vA / ms;
  double pn = S.pperp[N];
  double gmax_use = std::sqrt(1.0 + pn * pn * (vA * vA) / (ms * ms));
  S.grel.resize(ng + 1);
  S.prel.resize(np + 1);
  for (int ig = 0; ig <= ng; ++ig) S.grel[ig] = gmin + ((gmax_use - gmin) * ig) / (1.0 * ng);
  for (int ip = 0; ip <= np; ++ip) S.prel[ip] = pmin + ((pmax - pmin) * ip) / (1.0 * np);
  size_t nf = (size_t)(ng + 1) * (np + 1);
  if (!S.d_grel) ALPS_CUDA_TRY(cudaMalloc(&S.d_grel, (ng + 1) * sizeof(double)));
  if (!S.d_prel) ALPS_CUDA_TRY(cudaMalloc(&S.d_prel, (np + 1) * sizeof(double)));
  if (!S.d_f0rel) ALPS_CUDA_TRY(cudaMalloc(&S.d_f0rel, nf * sizeof(double)));
  if (!S.d_dfr1) ALPS_CUDA_TRY(cudaMalloc(&S.d_dfr1, nf * sizeof(double)));
  if (!S.d_dfr2) ALPS_CUDA_TRY(cudaMalloc(&S.d_dfr2, nf * sizeof(double)));
  if (!S.d_cone) ALPS_CUDA_TRY(cudaMalloc(&S.d_cone, (ng + 1) * sizeof(int2)));
  ALPS_CUDA_TRY(cudaMemcpyAsync(S.d_grel, S.grel.data(), (ng + 1) * sizeof(double), cudaMemcpyHostToDevice, st));
  ALPS_CUDA_TRY(cudaMemcpyAsync(S.d_prel, S.prel.data(), (np + 1) * sizeof(double), cudaMemcpyHostToDevice, st));
  // dense thin-plate-spline system (the reference sets its smoothing to 0
  // for the relativistic remap, src/ALPS_fns_rel.f90:149-151)
  int m = n + 3;
  double *d_gc = nullptr, *d_pc = nullptr, *d_w = nullptr;
  ALPS_CUDA_TRY(cudaMalloc(&d_gc, n * sizeof(double)));
  ALPS_CUDA_TRY(cudaMalloc(&d_pc, n * sizeof(double)));
  ALPS_CUDA_TRY(cudaMalloc(&d_w, m * sizeof(double)));
  std::vector<double> w(m, 0.0);
  for (int k = 0; k < n; ++k) w[k] = grid[k];
  ALPS_CUDA_TRY(cudaMemcpyAsync(d_gc, gc.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
  ALPS_CUDA_TRY(cudaMemcpyAsync(d_pc, pc.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
  ALPS_CUDA_TRY(cudaMemcpyAsync(d_w, w.data(), m * sizeof(double), cudaMemcpyHostToDevice, st));
  int status = tps_solve_device(d_gc, d_pc, n, 0.0, d_w, st);
  if (!status) {
    k_tps_eval<<<(unsigned)((nf + 127) / 128), 128, 0, st>>>(d_w, d_gc, d_pc, n, S.d_grel, S.d_prel, ng, np,
                                                              S.d_f0rel);
    if (cudaGetLastError() != cudaSuccess) status = ALPS_E_CUDA;
  }
  if (!status) {
    double dgamma = S.grel[2] - S.grel[1], dpb = S.prel[2] - S.prel[1];
    k_rel_norm<<<1, 256, 0, st>>>(S.d_f0rel, S.d_grel, ng, np, 2.0 * ALPS_PI * dgamma * dpb * cube(ms / vA));
    k_rel_deriv<<<(unsigned)((nf + 127) / 128), 128, 0, st>>>(S.d_f0rel, S.d_grel, S.d_prel, ng, np, S.d_dfr1,
                                                                S.d_dfr2);
    k_rel_cone<<<(ng + 1 + 127) / 128, 128, 0, st>>>(S.d_f0rel, ng, np, S.d_cone);
    double* d_ee = nullptr;
    cudaMalloc(&d_ee, sizeof(double));
    double scale = 2.0 * ALPS_PI * S.sp.qs / (ms) * dgamma * dpb * 0.25 * cube(ms / vA);
    k_rel_ee<<<1, 256, 0, st>>>(S.d_f0rel, S.d_dfr2, S.d_prel, ng, np, scale, d_ee);
    if (cudaGetLastError() != cudaSuccess) status = ALPS_E_CUDA;
    double ee = 0.0;
    cudaMemcpyAsync(&ee, d_ee, sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    cudaFree(d_ee);
    S.int_ee_rel = ee;
  }
  cudaFree(d_gc);
  cudaFree(d_pc);
  cudaFree(d_w);
  return status;
}

// ===========================================================================
// The interpolation tool (interpolation/interpolation.f90): thin-plate
// spline of log f through scattered samples, on a fine tensor grid,
// optionally normalised.
extern "C" int alps_interpolate(const double* pperp_c, const double* ppar_c, const double* f_c, int n,
                                const alps_interp_params* p, double* pperp_out, double* ppar_out, double* f_out) {
  if (!pperp_c || !ppar_c || !f_c || !p || n < 1 || p->nperp < 2 || p->npar < 2) return ALPS_E_INVALID;
  for (int k = 0; k < n; ++k)
    if (!(f_c[k] > 0.0)) return ALPS_E_INVALID;  // log f
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return ALPS_E_NO_DEVICE;
  const int nperp = p->nperp, npar = p->npar, m = n + 3;
  const size_t nf = (size_t)(nperp + 1) * (npar + 1);
  // the fine grid, as the reference forms it
  std::vector<double> pp(nperp + 1), pl(npar + 1);
  for (int i = 0; i <= nperp; ++i) pp[i] = p->pperp_min + (p->pperp_max - p->pperp_min) * i / (1.0 * nperp);
  for (int j = 0; j <= npar; ++j) pl[j] = p->ppar_min + (p->ppar_max - p->ppar_min) * j / (1.0 * npar);
  cudaStream_t st = nullptr;
  ALPS_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  double *d_gc = nullptr, *d_pc = nullptr, *d_f = nullptr, *d_w = nullptr, *d_pp = nullptr, *d_pl = nullptr;
  double *d_g = nullptr, *d_out = nullptr;
  int status = ALPS_OK;
  if (cudaMalloc(&d_gc, n * sizeof(double)) != cudaSuccess || cudaMalloc(&d_pc, n * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&d_f, n * sizeof(double)) != cudaSuccess || cudaMalloc(&d_w, m * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&d_pp, (nperp + 1) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&d_pl, (npar + 1) * sizeof(double)) != cudaSuccess || cudaMalloc(&d_g, nf * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&d_out, nf * sizeof(double)) != cudaSuccess)
    status = ALPS_E_OOM;
  if (!status) {
    cudaMemcpyAsync(d_gc, pperp_c, n * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_pc, ppar_c, n * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_f, f_c, n * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_pp, pp.data(), (nperp + 1) * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_pl, pl.data(), (npar + 1) * sizeof(double), cudaMemcpyHostToDevice, st);
    k_tps_rhs<<<(m + 127) / 128, 128, 0, st>>>(d_f, n, d_w);
    if (cudaGetLastError() != cudaSuccess) status = ALPS_E_CUDA;
  }
  if (!status) status = tps_solve_device(d_gc, d_pc, n, p->smoothing, d_w, st);
  if (!status) {
    k_tps_eval_grid<<<(unsigned)((nf + 127) / 128), 128, 0, st>>>(d_w, d_gc, d_pc, n, d_pp, d_pl, nperp, npar, d_g);
    // dpperp = pperp(2,1) - pperp(1,1), dppar = ppar(1,2) - ppar(1,1)
    k_interp_finish<<<1, 256, 0, st>>>(d_g, d_pp, nperp, npar, pp[2] - pp[1], pl[2] - pl[1], p->do_normalize,
                                       p->mult_f, d_out);
    if (cudaGetLastError() != cudaSuccess) status = ALPS_E_CUDA;
  }
  if (!status && f_out && cudaMemcpyAsync(f_out, d_out, nf * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    status = ALPS_E_CUDA;
  if (!status && cudaStreamSynchronize(st) != cudaSuccess) status = ALPS_E_CUDA;
  if (!status)
    for (int i = 0; i <= nperp; ++i)
      for (int j = 0; j <= npar; ++j) {
        if (pperp_out) pperp_out[(size_t)i * (npar + 1) + j] = pp[i];
        if (ppar_out) ppar_out[(size_t)i * (npar + 1) + j] = pl[j];
      }
  cudaFree(d_gc);
  cudaFree(d_pc);
  cudaFree(d_f);
  cudaFree(d_w);
  cudaFree(d_pp);
  cudaFree(d_pl);
  cudaFree(d_g);
  cudaFree(d_out);
  cudaStreamDestroy(st);
  return status;
}

int launch_rel_bessel(alps_ctx* c, int is, double kperp) {
  SpeciesHost& S = c->spec[is];
  int ng = c->sys.ngamma, np = c->sys.npparbar, nrows = S.nmax + 2;
  size_t need = (size_t)nrows * (ng + 1) * (np + 1);
  if (need > S.jrel_cap || !S.d_jrel) {
    if (S.d_jrel) cudaFree(S.d_jrel);
    S.d_jrel = nullptr;
    ALPS_CUDA_TRY(cudaMalloc(&S.d_jrel, need * sizeof(double)));
    S.jrel_cap = need;
  }
  double zfac = kperp * S.sp.ms / (c->sys.vA * S.sp.qs);
  k_rel_jtab<<<(unsigned)((need + 127) / 128), 128, 0, c->stream>>>(S.d_grel, S.d_prel, ng, np, nrows, zfac,
                                                                     S.d_jrel);
  ALPS_CUDA_TRY(cudaGetLastError());
  return ALPS_OK;
}

// ===========================================================================
// omega batch
// ===========================================================================
namespace {

struct RelArgs {
  SysDev sys;
  SpecDev sp[ALPS_MAX_SPECIES];
  int relcap;
};

// six int_T entries with the factors i (entry 4) and -i (entry 6) left out;
// they are applied once to the finished sums (multiplying by i is exact)
struct C6 {
  double2 v[6];
};

__device__ inline void c6_zero(C6& a) {
#pragma unroll
  for (int e = 0; e < 6; ++e) a.v[e] = cmk(0.0, 0.0);
}

// sum over the 32 lanes of a warp, the same butterfly on every lane (the
// result, on all lanes, does not depend on timing)
__device__ inline void c6_warp_sum(C6& a) {
#pragma unroll
  for (int e = 0; e < 6; ++e)
    for (int o = 16; o > 0; o >>= 1) {
      a.v[e].x += __shfl_xor_sync(0xffffffffu, a.v[e].x, o);
      a.v[e].y += __shfl_xor_sync(0xffffffffu, a.v[e].y, o);
    }
}

// Bessel pair of signed order m from J(k), k >= 0 (int_T_rel :1297-1329)
template <typename T, typename F>
__device__ inline void bessel_pair_m(int m, F J, T& b, T& bp) {
  auto sgn = [](int k) { return (k % 2 == 0) ? 1.0 : -1.0; };
  if (m < 0) b = J(-m) * sgn(m);
  else b = J(m);
  if (m >= 1) bp = (J(m - 1) - J(m + 1)) * 0.5;
  else if (m < -1) bp = (J(-(m - 1)) * sgn(m - 1) - J(-(m + 1)) * sgn(m + 1)) * 0.5;
  else if (m == 0) bp = J(1) * -1.0;
  else bp = (J(2) - J(0)) * 0.5;
}

// int_T_rel entries at node (ig, ip) (src/ALPS_fns_rel.f90:1256-1369)
__device__ inline void t_node_rel(const SpecDev& S, const SysDev& sy, int m, int ig, int ip, double t[6]) {
  const double ms = S.ms, qs = S.qs, vA = sy.vA, kperp = sy.kperp;
  const bool kn = sy.kperp_norm != 0;
  const double g = S.grel[ig], pb = S.prel[ip];
  const double pperpbar = sqrt(g * g - 1.0 - pb * pb);
  const double zbar = kn ? kperp * ms / (vA * qs) : ms / (vA * qs);
  const size_t plane = (size_t)(S.ng + 1) * (S.np + 1);
  const double* J0 = S.jrel + (size_t)ig * (S.np + 1) + ip;
  auto J = [&](int k) { return J0[(size_t)k * plane]; };
  double b, bp;
  bessel_pair_m(m, J, b, bp);
  const double kf = kn ? 1.0 : kperp, kf2 = kn ? 1.0 : kperp * kperp;
  t[0] = 1.0 * (m * m) * b * b / (zbar * zbar);
  t[1] = kf2 * bp * bp * pperpbar * pperpbar;
  t[2] = kf2 * b * b * (pb * pb);
  t[3] = (1.0 * m) * kf * b * bp * pperpbar / zbar;
  t[4] = (1.0 * m) * kf * b * b * pb / zbar;
  t[5] = kf2 * b * bp * pb * pperpbar;
}

// fit_function for the Gamma rows, fit types 4 and 5 (src/ALPS_analyt.f90:244-258)
__device__ inline double2 eval_fit_rel(const SpecDev& S, int ig, double2 p) {
  double2 ff = cmk(0.0, 0.0);
  const double g = S.grel[ig];
  const int nf = S.nf;
  for (int f = 0; f < nf; ++f) {
    const double* P = S.fit + (size_t)ig * 5 * nf + f;
    const double pc = S.perp_corr[f];
    if (S.fit_type[f] == 4) {
      ff = cadd(ff, cmk(P[0] * exp(-pc * g), 0.0));
    } else {
      double2 d = csub(p, cmk(P[2 * nf], 0.0));
      double2 d2 = cmul(d, d);
      ff = cadd(ff, cscale(cexp_d(cscale(d2, -P[nf])), P[0] * exp(-pc * g)));
    }
  }
  return ff;
}

// the reference's Lanczos Gamma (src/ALPS_fns_rel.f90:1738-1791)
__device__ inline double gamma_lanczos(double xx) {
  const double cof[6] = {76.18009173, -86.50532033, 24.01409822, -1.231739516, 0.120858003e-2, -0.536382e-5};
  double x = xx - 1.0;
  double tmp = x + 5.5;
  tmp = (x + 0.5) * log(tmp) - tmp;
  double ser = 1.0;
  for (int j = 0; j < 6; ++j) {
    x = x + 1.0;
    ser = ser + cof[j] / x;
  }
  return exp(tmp + log(2.50662827465 * ser));
}

__device__ inline double2 cpowi_d(double2 x, int n) {
  double2 pw = cmk(1.0, 0.0);
  if (n == 0) return pw;
  unsigned u = (unsigned)(n < 0 ? -n : n);
  for (;;) {
    if (u & 1) pw = cmul(pw, x);
    u >>= 1;
    if (u) x = cmul(x, x);
    else break;
  }
  if (n < 0) pw = cdiv(cmk(1.0, 0.0), pw);
  return pw;
}

// CBESSJ (src/ALPS_fns_rel.f90:1502-1553): 21-term power series
__device__ double2 cbessj_d(double2 z, int nu) {
  double2 sum = cmk(0.0, 0.0);
  double2 q = cscale(cmul(cneg(z), z), 0.25);
  double fk = 1.0;
  for (int k = 0; k <= 20; ++k) {
    if (k >= 2) fk = fk * (1.0 * k);
    double2 t = cpowi_d(q, k);
    t = cmk(t.x / fk, t.y / fk);
    double gm = gamma_lanczos(1.0 * (nu + k + 1));
    t = cmk(t.x / gm, t.y / gm);
    sum = cadd(sum, t);
  }
  return cmul(cpowi_d(cscale(z, 0.5), nu), sum);
}

struct cwrap {  // complex value with the arithmetic bessel_pair_m needs
  double2 v;
  __device__ cwrap operator*(double s) const { return cwrap{cscale(v, s)}; }
  __device__ cwrap operator-(const cwrap& o) const { return cwrap{csub(v, o.v)}; }
};

// int_T_res_rel entries (src/ALPS_fns_rel.f90:1374-1495)
__device__ void t_res_rel(const SpecDev& S, const SysDev& sy, int m, int ig, double2 pr, double2 t[6]) {
  const double ms = S.ms, qs = S.qs, vA = sy.vA, kperp = sy.kperp;
  const bool kn = sy.kperp_norm != 0;
  const double g = S.grel[ig];
  double2 pperpbar = csqrt_d(csub(cmk(g * g - 1.0, 0.0), cmul(pr, pr)));
  double2 z = cscale(pperpbar, kperp * ms / (vA * qs));
  const double zbar = kn ? kperp * ms / (vA * qs) : ms / (vA * qs);
  cwrap b, bp;
  bessel_pair_m(m, [&](int k) { return cwrap{cbessj_d(z, k)}; }, b, bp);
  const double kf = kn ? 1.0 : kperp, kf2 = kn ? 1.0 : kperp * kperp;
  double2 bb = cmul(b.v, b.v), bbp = cmul(b.v, bp.v);
  t[0] = cscale(bb, 1.0 * (m * m) / (zbar * zbar));
  t[1] = cscale(cmul(cmul(bp.v, bp.v), cmul(pperpbar, pperpbar)), kf2);
  t[2] = cscale(cmul(bb, cmul(pr, pr)), kf2);
  t[3] = cscale(cmul(bbp, pperpbar), (1.0 * m) * kf / zbar);
  t[4] = cscale(cmul(bb, pr), (1.0 * m) * kf / zbar);
  t[5] = cscale(cmul(bbp, cmul(pr, pperpbar)), kf2);
}

__device__ inline double fr_at(const SpecDev& S, int ig, int ip) {
  if (ip < 0 || ip > S.np || ig < 0 || ig > S.ng) return -1.0;
  return S.f0rel[(size_t)ig * (S.np + 1) + ip];
}

struct RowCtx {
  const SpecDev& S;
  const SysDev& sy;
  double2 om;
  int m, ig;
  double Kc;  // -2 pi (ms/vA)^3 q vA / (k_par m)
};

// integrand of funct_g_rel at a node, six entries
__device__ inline void h_node_rel(const RowCtx& r, int ip, double2 h[6]) {
  const SpecDev& S = r.S;
  size_t k = (size_t)r.ig * (S.np + 1) + ip;
  double2 A = cadd(cscale(r.om, S.dfr1[k]), cmk((r.sy.kpar / r.sy.vA) * S.dfr2[k], 0.0));
  A = cscale(A, r.Kc);
  double t[6];
  t_node_rel(S, r.sy, r.m, r.ig, ip, t);
#pragma unroll
  for (int e = 0; e < 6; ++e) h[e] = cscale(A, t[e]);
}

// funct_g_rel (src/ALPS_fns_rel.f90:918-999)
__device__ void funct_g_rel_d(const RowCtx& r, double pp, double2 G[6]) {
  const SpecDev& S = r.S;
  const int np = S.np;
  const double* pb = S.prel;
  const double dpb = pb[2] - pb[1];
  int close = -2;
  if (pp >= pb[0] && pp < pb[np]) {
    // the last k in 0..np-1 with pb[k] <= pp: the uniform grid's index,
    // moved by the grid values themselves where rounding put it one off
    int k = (int)floor((pp - pb[0]) * ((double)np / (pb[np] - pb[0])));
    k = max(0, min(np - 1, k));
    while (k > 0 && pb[k] > pp) --k;
    while (k < np - 1 && pb[k + 1] <= pp) ++k;
    close = k;
  }
  if (fr_at(S, r.ig, close + 1) <= -1.0) close = close - 1;
  if (fr_at(S, r.ig, close - 1) <= -1.0) close = close + 1;
  if (pp == pb[np]) close = np - 2;
  if (close >= (np - 1)) close = np - 2;
  if (close <= 1) close = 2;
  double2 hp[6], hm[6];
  h_node_rel(r, close + 1, hp);
  h_node_rel(r, close - 1, hm);
  h_node_rel(r, close, G);
  double dx = pp - pb[close];
#pragma unroll
  for (int e = 0; e < 6; ++e) G[e] = cadd(G[e], cscale(cscale(csub(hp[e], hm[e]), 1.0 / dpb), 0.5 * dx));
}

// principal_integral_rel (src/ALPS_fns_rel.f90:724-913), by the 32 lanes of
// a warp: the sample points are spread over the lanes and the lanes' sums
// are added by a warp reduction; out (on every lane) receives the window's
// contribution
__device__ void principal_rel_d(const RowCtx& r, int ipres, int upperlimit, C6& out, int lane) {
  const SpecDev& S = r.S;
  const SysDev& sy = r.sy;
  const double ms = S.ms, qs = S.qs, vA = sy.vA, kpar = sy.kpar;
  const int M_I = sy.M_I, M_P = sy.M_P;
  const double* pb = S.prel;
  const double dpb = pb[2] - pb[1];
  const double g = S.grel[r.ig];
  double2 t1 = cscale(cscale(r.om, g), vA);
  t1 = cmk(t1.x / kpar, t1.y / kpar);
  const double denomR = t1.x - (1.0 * r.m) * (qs / ms) * vA / kpar;
  const double denomI = t1.y;
  const double capDelta = denomR - pb[ipres - M_I];
  const double smdelta = capDelta / (1.0 * M_P);
  C6 pi;
  c6_zero(pi);
  double2 Ga[6], Gb[6];
  const double2 dIp = cmk(0.0, -denomI), dIm = cmk(0.0, denomI);
  // sum += w*(G(pp)/(pp-dR-i dI) - G(2dR-pp)/(pp-dR+i dI))
  auto pair = [&](double pp, double w) {
    funct_g_rel_d(r, pp, Ga);
    funct_g_rel_d(r, 2.0 * denomR - pp, Gb);
    double2 da = cadd(cmk(pp - denomR, 0.0), dIp), db = cadd(cmk(pp - denomR, 0.0), dIm);
#pragma unroll
    for (int e = 0; e < 6; ++e) {
      pi.v[e] = cadd(pi.v[e], cdiv(cscale(Ga[e], w), da));
      pi.v[e] = csub(pi.v[e], cdiv(cscale(Gb[e], w), db));
    }
  };
  if (fabs(denomI) > sy.Tlim) {
    if (lane == 0) pair(denomR, 1.0);
    if (lane == 1) pair(denomR + capDelta, 1.0);
    // sample points rounded as the reference writes them (no FMA): a point
    // can fall on a node, where funct_g_rel's choice of node depends on it
    for (int ip = 1 + lane; ip <= M_P - 1; ip += 32) pair(__dadd_rn(denomR, __dmul_rn(smdelta, (double)ip)), 2.0);
  } else {
    funct_g_rel_d(r, denomR + dpb, Ga);
    funct_g_rel_d(r, denomR - dpb, Gb);
    double2 gp[6];
#pragma unroll
    for (int e = 0; e < 6; ++e) {
      gp[e] = csub(Ga[e], Gb[e]);
      gp[e] = cmk(gp[e].x / (2.0 * dpb), gp[e].y / (2.0 * dpb));
    }
    auto lor = [&](double pp, double w) {
      double d = pp - denomR;
      double f = (d * d) / ((d * d) + denomI * denomI);
#pragma unroll
      for (int e = 0; e < 6; ++e) pi.v[e] = cadd(pi.v[e], cscale(cscale(gp[e], w), f));
    };
    if (lane == 0) lor(denomR + capDelta, 2.0);
    for (int ip = 1 + lane; ip <= M_P - 1; ip += 32) lor(__dadd_rn(denomR, __dmul_rn(smdelta, (double)ip)), 4.0);
    if (denomI != 0.0 && lane == 0) {
      funct_g_rel_d(r, denomR, Ga);
      double sgn = denomI > 0.0 ? 1.0 : -1.0;
#pragma unroll
      for (int e = 0; e < 6; ++e) {
        double2 q = cscale(Ga[e], 2.0 * ALPS_PI / smdelta);
        pi.v[e] = cadd(pi.v[e], cmk(-sgn * q.y, sgn * q.x));  // +- i q
      }
    }
  }
  int ntiny = (int)((pb[upperlimit] - denomR - capDelta) / smdelta);
  if (ntiny > 0) {
    double correction = ((pb[upperlimit] - denomR - capDelta) / (1.0 * ntiny)) / smdelta;
    auto tail = [&](double pp, double w) {
      funct_g_rel_d(r, pp, Ga);
      double2 da = cmk(pp - denomR, -denomI);
#pragma unroll
      for (int e = 0; e < 6; ++e) pi.v[e] = cadd(pi.v[e], cscale(cdiv(Ga[e], da), w * correction));
    };
    if (lane == 0) tail(denomR + capDelta, 1.0);
    auto tp = [&](int ip) {
      return __dadd_rn(__dadd_rn(denomR, capDelta), __dmul_rn(__dmul_rn(correction, smdelta), (double)ip));
    };
    if (lane == 1) tail(tp(ntiny), 1.0);
    for (int ip = 1 + lane; ip <= ntiny - 1; ip += 32) tail(tp(ip), 2.0);
  }
  c6_warp_sum(pi);
#pragma unroll
  for (int e = 0; e < 6; ++e) out.v[e] = cadd(out.v[e], cscale(pi.v[e], smdelta));
}

// integrate_resU_rel for one Gamma row (src/ALPS_fns_rel.f90:516-719), by
// the 32 lanes of a warp: the window decisions on every lane, the nodes and
// the principal-value samples spread over the lanes; out (on every lane)
// receives the row's integral
__device__ void row_rel_d(const RowCtx& r, C6& out, bool& err, int lane) {
  const SpecDev& S = r.S;
  const SysDev& sy = r.sy;
  const double ms = S.ms, qs = S.qs, vA = sy.vA, kpar = sy.kpar;
  const int M_I = sy.M_I, np = S.np;
  const double* pb = S.prel;
  const double dpb = pb[2] - pb[1];
  const double g = S.grel[r.ig];
  c6_zero(out);
  // the resonance and its window decided as the reference rounds them (no FMA)
  const double x = __ddiv_rn(__dmul_rn(__dsub_rn(__dmul_rn(g, r.om.x), __ddiv_rn(__dmul_rn(1.0 * r.m, qs), ms)), vA), kpar);
  int ipres = 0;
  bool found = false;
  if (__dmul_rn(x, x) <= __dsub_rn(__dmul_rn(g, g), 1.0)) {
    // the ip in 1..np-2 with pb[ip] <= x < pb[ip+1]
    int lo = 1, hi = np - 2;
    if (np - 2 >= 1 && pb[1] <= x) {
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (pb[mid] <= x) lo = mid;
        else hi = mid - 1;
      }
      if (pb[lo + 1] > x) {
        ipres = lo;
        found = true;
      }
    }
  }
  for (int ip = 0; ip <= M_I; ++ip) {
    if ((x >= __dsub_rn(pb[0], __dmul_rn(dpb, (double)ip))) && (x < __dsub_rn(pb[0], __dmul_rn(dpb, (double)(ip - 1))))) {
      ipres = -ip;
      found = true;
    }
    if ((x >= __dadd_rn(pb[np - 1], __dmul_rn(dpb, (double)ip))) &&
        (x < __dadd_rn(pb[np - 1], __dmul_rn(dpb, (double)(ip + 1))))) {
      ipres = np - 1 + ip;
      found = true;
    }
  }
  const int2 cn = S.cone[r.ig];
  const int lowerC = cn.x, upperC = cn.y;
  int int_start, int_end, lowerlimit, upperlimit;
  if (found) {
    int_start = lowerC;
    int_end = upperC;
    lowerlimit = ipres - M_I;
    upperlimit = ipres + M_I + 1;
    if ((ipres >= 0) && (ipres <= np))
      if (fabs(x - pb[ipres]) > (0.5 * dpb)) upperlimit = upperlimit + 1;
    if ((lowerlimit < lowerC) && (upperlimit > upperC)) {
      err = true;
      return;
    } else if (lowerlimit <= lowerC) {
      int_start = 1;
      lowerlimit = 0;
      upperlimit = lowerC;
    } else if (upperlimit >= upperC) {
      lowerlimit = upperC;
      upperlimit = np;
      int_end = np - 1;
    }
  } else {
    int_start = lowerC;
    lowerlimit = upperC;
    int_end = np - 1;
    upperlimit = np;
  }
  // trapezoid over the nodes away from the pole
  double2 gom = cscale(cscale(r.om, g), vA);
  gom = cmk(gom.x / kpar, gom.y / kpar);
  const double nq = (1.0 * r.m) * qs * vA / (kpar * ms);
  auto term = [&](int ip, double w) {
    double2 h[6];
    h_node_rel(r, ip, h);
    double2 den = cadd(csub(cmk(pb[ip], 0.0), gom), cmk(nq, 0.0));
#pragma unroll
    for (int e = 0; e < 6; ++e) out.v[e] = cadd(out.v[e], cscale(cdiv(h[e], den), w));
  };
  if (lane == 0 && int_start <= lowerlimit) term(int_start, 1.0);
  for (int ip = int_start + 1 + lane; ip <= lowerlimit - 1; ip += 32) term(ip, 2.0);
  if (lane == 1 && int_start < lowerlimit) term(lowerlimit, 1.0);
  if (lane == 2 && upperlimit <= int_end) term(upperlimit, 1.0);
  for (int ip = upperlimit + 1 + lane; ip <= int_end - 1; ip += 32) term(ip, 2.0);
  if (lane == 3 && upperlimit < int_end) term(int_end, 1.0);
  c6_warp_sum(out);
#pragma unroll
  for (int e = 0; e < 6; ++e) out.v[e] = cscale(out.v[e], dpb);
  if (found && (lowerlimit >= int_start) && (upperlimit <= int_end)) principal_rel_d(r, ipres, upperlimit, out, lane);
}

// one Landau row of landau_integrate_rel (src/ALPS_fns_rel.f90:1005-1092)
__device__ void landau_row_rel_d(const RowCtx& r, C6& acc) {
  const SpecDev& S = r.S;
  const SysDev& sy = r.sy;
  const double ms = S.ms, qs = S.qs, vA = sy.vA, kpar = sy.kpar;
  const int ig = r.ig;
  const double g = S.grel[ig];
  const double dg = S.grel[2] - S.grel[1], dpb = S.prel[2] - S.prel[1];
  double2 pr = cscale(cscale(r.om, g), vA);
  pr = cmk(pr.x / kpar - (1.0 * r.m) * qs * vA / (kpar * ms), pr.y / kpar);
  // inside the subluminal cone, decided as the reference rounds it (no FMA)
  if (!(__dmul_rn(pr.x, pr.x) <= __dsub_rn(__dmul_rn(g, g), 1.0))) return;
  double h = (ig == S.ng - 1) ? 0.5 : 1.0;
  double2 dfg;
  if (ig == 1) {
    dfg = csub(eval_fit_rel(S, ig + 1, pr), eval_fit_rel(S, ig, pr));
    dfg = cmk(dfg.x / dg, dfg.y / dg);
  } else {
    dfg = csub(eval_fit_rel(S, ig + 1, pr), eval_fit_rel(S, ig - 1, pr));
    dfg = cmk(dfg.x / (2.0 * dg), dfg.y / (2.0 * dg));
  }
  double2 dfp = csub(eval_fit_rel(S, ig, cadd(pr, cmk(dpb, 0.0))), eval_fit_rel(S, ig, csub(pr, cmk(dpb, 0.0))));
  dfp = cmk(dfp.x / (2.0 * dpb), dfp.y / (2.0 * dpb));
  double2 coef = cscale(cadd(cmul(r.om, dfg), cscale(dfp, kpar / vA)), h);
  double2 t[6];
  t_res_rel(S, sy, r.m, ig, pr, t);
#pragma unroll
  for (int e = 0; e < 6; ++e) acc.v[e] = csub(acc.v[e], cmul(coef, t[e]));
}

// deterministic block sum of 12 doubles per thread (blockDim.x = 128)
// sum over the block's threads (REL_THREADS), in warp order
__device__ void block_sum12(double v[12], double* sh /* [REL_THREADS/32][12] */) {
#pragma unroll
  for (int q = 0; q < 12; ++q)
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int q = 0; q < 12; ++q) sh[warp * 12 + q] = v[q];
  __syncthreads();
  if (threadIdx.x == 0)
    for (int q = 0; q < 12; ++q) {
      double t = sh[q];
      for (int k = 1; k < REL_THREADS / 32; ++k) t += sh[k * 12 + q];
      v[q] = t;
    }
  __syncthreads();
}

// One block per (omega, species, signed order, row block): the REL_RB row
// blocks of an order each take every REL_RB-th group of Gamma rows (a warp
// per row) or every REL_RB-th stretch of the regular grid, and write their
// partial sums to their own slot; k_finalize adds the slots in order.
__global__ void __launch_bounds__(REL_THREADS) k_rel_orders(RelArgs a, const double2* __restrict__ om, int n_om,
                                                            double2* __restrict__ out, int* flags) {
  __shared__ double sh[(REL_THREADS / 32) * 12];
  const int w = blockIdx.x, s = blockIdx.z;
  const int rb = blockIdx.y % REL_RB, ord = blockIdx.y / REL_RB;
  const int n = ord >> 1, sg = ord & 1;
  const SpecDev& S = a.sp[s];
  if (w >= n_om || !S.relat || n > S.nmax || n >= a.relcap || (n == 0 && sg == 1)) return;
  const SysDev& sy = a.sys;
  const int m = sg ? -n : n;
  const double2 o = om[w];
  const double ms = S.ms, qs = S.qs, vA = sy.vA, kpar = sy.kpar, kperp = sy.kperp;
  const int N = S.N, M = S.M, L = M + 1;
  // determine_resonances, relativistic branch (src/ALPS_fns.f90:680-702)
  bool res = false;
  for (int t = threadIdx.x; t < (N + 1) * M; t += blockDim.x) {
    int i = t / M, j = t % M;
    double p1 = S.pperp[i], p2 = S.ppar[j];
    // the decision rounds as the reference's expression does (no FMA)
    const double gamma = __dsqrt_rn(__dadd_rn(
        __ddiv_rn(__dmul_rn(__dadd_rn(__dmul_rn(p1, p1), __dmul_rn(p2, p2)), __dmul_rn(vA, vA)), __dmul_rn(ms, ms)),
        1.0));
    const double pr = __ddiv_rn(__dsub_rn(__dmul_rn(__dmul_rn(gamma, ms), o.x), __dmul_rn(1.0 * m, qs)), kpar);
    if ((S.ppar[j] <= pr) && (S.ppar[j + 1] > pr)) res = true;
  }
  res = __syncthreads_or(res) != 0;
  double v[12];
  C6 r6;
  if (!res) {
    // integrate with the Lorentz factor in resU (src/ALPS_fns.f90:799-864,
    // 1560-1596), rows 1..N-1 and columns 1..M-1
    const bool kn = sy.kperp_norm != 0;
    const double z = kn ? kperp / qs : 1.0 / qs;
    const double kf = kn ? 1.0 : kperp, kf2 = kn ? 1.0 : kperp * kperp;
    c6_zero(r6);
    const int LB = N + 1;
    for (int t = rb * blockDim.x + threadIdx.x; t < (N - 1) * (M - 1); t += REL_RB * blockDim.x) {
      int i = 1 + t / (M - 1), j = 1 + t % (M - 1);
      double wi = (i == N - 1) ? 1.0 : 2.0;
      if (i == 1 && N - 1 == 1) wi = 3.0;
      double wj = (j == 1 || j == M - 1) ? 1.0 : 2.0;
      if (M - 1 == 1) wj = 2.0;
      size_t k = (size_t)i * L + j;
      double p1 = S.pperp[i], p2 = S.ppar[j];
      double gamma = sqrt((p1 * p1 + p2 * p2) * (vA * vA) / (ms * ms) + 1.0);
      double2 num = cadd(cscale(o, S.g1[k]), cmk((kpar / (gamma * ms)) * S.g2[k], 0.0));
      num = cscale(num, qs);
      double2 den = cmk(gamma * ms * o.x - kpar * p2 - (1.0 * m) * qs, gamma * ms * o.y);
      double2 rU = cdiv(num, den);
      auto J = [&](int kk) { return S.bessel[(size_t)(kk + 1) * LB + i]; };
      double b, bp;
      bessel_pair_m(m, J, b, bp);
      double tt[6];
      tt[0] = 1.0 * (m * m) * b * b / (z * z);
      tt[1] = kf2 * (p1 * p1) * bp * bp;
      tt[2] = kf2 * b * b * (p2 * p2);
      tt[3] = kf * p1 * (1.0 * m) * b * bp / z;
      tt[4] = (1.0 * m) * kf * b * b * p2 / z;
      tt[5] = kf2 * b * bp * p2 * p1;
#pragma unroll
      for (int e = 0; e < 6; ++e) r6.v[e] = cadd(r6.v[e], cscale(rU, wi * wj * tt[e]));
    }
    for (int e = 0; e < 6; ++e) {
      v[2 * e] = r6.v[e].x;
      v[2 * e + 1] = r6.v[e].y;
    }
    block_sum12(v, sh);
    if (threadIdx.x == 0) {
      double f = 2.0 * ALPS_PI * S.dpperp * S.dppar_abs * 0.25;
      for (int e = 0; e < 6; ++e) r6.v[e] = cscale(cmk(v[2 * e], v[2 * e + 1]), f);
    }
  } else {
    // integrate_res_rel + landau_integrate_rel over the Gamma rows
    const double Kc = -2.0 * ALPS_PI * cube(ms / vA) * (qs * vA / (kpar * ms));
    C6 acc, lacc;
    c6_zero(acc);
    c6_zero(lacc);
    bool err = false;
    const double lw = (o.y > 0.0) ? 0.0 : ((o.y < 0.0) ? 2.0 : 1.0);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int ig = 1 + rb * nw + warp; ig <= S.ng - 1; ig += REL_RB * nw) {
      RowCtx rc{S, sy, o, m, ig, Kc};
      C6 row;
      row_rel_d(rc, row, err, lane);
      double wr = (ig <= S.ng - 2) ? 2.0 : 1.0;
      if (lane == 0) {
#pragma unroll
        for (int e = 0; e < 6; ++e) acc.v[e] = cadd(acc.v[e], cscale(row.v[e], wr));
        if (lw != 0.0) landau_row_rel_d(rc, lacc);
      }
    }
    if (err) atomicOr(flags, 2);
    for (int e = 0; e < 6; ++e) {
      v[2 * e] = acc.v[e].x;
      v[2 * e + 1] = acc.v[e].y;
    }
    block_sum12(v, sh);
    double dg = S.grel[2] - S.grel[1];
    if (threadIdx.x == 0)
      for (int e = 0; e < 6; ++e) r6.v[e] = cscale(cscale(cmk(v[2 * e], v[2 * e + 1]), dg), 0.25);
    for (int e = 0; e < 6; ++e) {
      v[2 * e] = lacc.v[e].x;
      v[2 * e + 1] = lacc.v[e].y;
    }
    block_sum12(v, sh);
    if (threadIdx.x == 0 && lw != 0.0) {
      double f = dg * ALPS_PI * 2.0 * ALPS_PI * (qs * vA / (kpar * ms)) * cube(ms / vA);
      for (int e = 0; e < 6; ++e) {
        double2 l = cmk(v[2 * e], v[2 * e + 1]);
        l = cmk(-l.y, l.x);  // * i
        r6.v[e] = cadd(r6.v[e], cscale(cscale(l, f), lw));
      }
    }
  }
  if (threadIdx.x == 0) {
    r6.v[3] = cmk(-r6.v[3].y, r6.v[3].x);  // * i
    r6.v[5] = cmk(r6.v[5].y, -r6.v[5].x);  // * -i
    double2* dst = out + (((((size_t)w * sy.nspec + s) * a.relcap + n) * 2 + sg) * REL_RB + rb) * 6;
    for (int e = 0; e < 6; ++e) dst[e] = r6.v[e];
  }
}

}  // namespace

int launch_rel_orders(const SysDev& sys, const SpecDev* sp, int relcap, int n, const double2* d_om, double2* d_out,
                      int* d_flags, cudaStream_t st) {
  RelArgs a;
  a.sys = sys;
  bool any = false;
  for (int s = 0; s < sys.nspec; ++s) {
    a.sp[s] = sp[s];
    any = any || sp[s].relat;
  }
  a.relcap = relcap;
  if (!any || n <= 0) return ALPS_OK;
  k_rel_orders<<<dim3(n, 2 * relcap * REL_RB, sys.nspec), REL_THREADS, 0, st>>>(a, d_om, n, d_out, d_flags);
  ALPS_CUDA_TRY(cudaGetLastError());
  return ALPS_OK;
}
