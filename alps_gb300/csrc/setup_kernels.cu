// setup_kernels.cu -- per-run and per-wavevector device preprocessing.
//
//   k_derivatives     derivative_f0 (src/ALPS_fns.f90:103-115), plus the
//                     second RHS vector pperp*df/dppar - ppar*df/dpperp of resU
//   k_int_ee          int_ee (src/ALPS_fns.f90:1457-1555)
//   k_lm_fit          determine_param_fit + LM_nonlinear_fit
//                     (src/ALPS_analyt.f90:365-728, 1183-1636)
//   k_nmax            determine_nmax (src/ALPS_fns.f90:3971-4075)
//   k_bessel_table    determine_bessel_array (src/ALPS_fns.f90:4214-4255)
//   k_bessel_rows     weighted Bessel-product rows of the p_perp contraction
//   k_dgemm           FP64 tiled GEMM for the contraction
//   k_fold_reduced    reduced vectors V[n][j][12] of the omega pass
#include <cmath>
#include <cstring>
#include <cstdio>

#include "alps_internal.cuh"
#include "tc_gemm.cuh"
#include "device_math.cuh"

namespace {

__global__ void k_derivatives(const double* __restrict__ f0, const double* __restrict__ pperp,
                              const double* __restrict__ ppar, int N, int M, double* g1, double* g2,
                              double* G) {
  int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  int i = blockIdx.y + 1;
  if (i > N - 1 || j > M - 1) return;
  int L = M + 1;
  double df1 = __ddiv_rn(__dsub_rn(f0[(i + 1) * L + j], f0[(i - 1) * L + j]),
                         __dsub_rn(pperp[i + 1], pperp[i - 1]));
  double df2 = __ddiv_rn(__dsub_rn(f0[i * L + j + 1], f0[i * L + j - 1]),
                         __dsub_rn(ppar[j + 1], ppar[j - 1]));
  double gg2 = __dsub_rn(__dmul_rn(pperp[i], df2), __dmul_rn(ppar[j], df1));
  g1[i * L + j] = df1;
  g2[i * L + j] = gg2;
  // contraction RHS, row-major [(i-1)][g*(M-1) + (j-1)]
  size_t row = (size_t)(i - 1) * 2 * (M - 1);
  G[row + (j - 1)] = df1;
  G[row + (M - 1) + (j - 1)] = gg2;
}

// ee term; weights w_perp(i) * w_par(j) of the reference's trapezoid.
__global__ void k_int_ee(const double* __restrict__ g2, const double* __restrict__ ppar, int N, int M,
                         double scale, double* out) {
  __shared__ double red[256];
  double acc = 0.0;
  int L = M + 1;
  long total = (long)(N - 1) * (M - 1);
  for (long t = threadIdx.x; t < total; t += blockDim.x) {
    int i = (int)(t / (M - 1)) + 1, j = (int)(t % (M - 1)) + 1;
    double wperp = (i <= N - 2) ? 2.0 : 1.0;
    double wpar = (j == 1 || j == M - 1) ? 1.0 : 2.0;
    acc += wperp * wpar * (ppar[j] * g2[i * L + j]);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0] * scale;
}

// ---------------------------------------------------------------------------
// Levenberg-Marquardt fit of the analytic continuation.  One warp walks the
// iperp rows of one species in order (each row starts from the previous
// result, src/ALPS_analyt.f90:518); within a row the lanes share the points
// and the entries of J^T J, and every sum keeps the reference's order.
// ---------------------------------------------------------------------------
struct FitArgs {
  int N, M, nf, log_fit;
  int fit_type[ALPS_MAX_FITS];
  double pc[ALPS_MAX_FITS];
  double ms, vA;
  int maxsteps;
  double lambda0, lambdafac, eps;
  // relativistic species: rows of the (Gamma, pparbar) grid
  int rel, ng, np;
  const double* f0rel;  // [(ng+1)*(np+1)]
  const double* grel;   // [ng+1]
  const double* prel;   // [np+1]
};

__device__ int fit_nparams(const FitArgs& a, int t) {
  return (t == 1 || t == 3 || t == 5) ? 3 : (t == 2 ? 5 : (t == 6 ? 4 : 1));
}

// fit_function (src/ALPS_analyt.f90:185-266) at real ppar
__device__ double fit_value_real(const FitArgs& a, const double* params, double pperp, double ppar) {
  double ff = 0.0;
  int par_ind = 0;
  for (int ifit = 1; ifit <= a.nf; ++ifit) {
    int t = a.fit_type[ifit - 1];
    double pc = a.pc[ifit - 1];
    const double* p = params + (ifit + par_ind) - 1;
    double d = ppar - p[2];
    if (t == 1) {
      ff = ff + (p[0] * exp(-pc * (pperp * pperp))) * exp(-p[1] * (d * d));
      par_ind += 2;
    } else if (t == 2) {
      double kp = 1.0 + p[1] * (d * d) + pc * p[4] * (pperp * pperp);
      ff = ff + p[0] * exp(p[3] * log(kp));
      par_ind += 4;
    } else if (t == 3) {
      double sq = sqrt(1.0 + ((pperp * pperp) + d * d) * a.vA * a.vA / (a.ms * a.ms));
      ff = ff + p[0] * exp(-p[1] * sq);
      par_ind += 2;
    } else if (t == 4) {
      ff = ff + p[0] * exp(-pc * pperp);
    } else if (t == 5) {
      ff = ff + p[0] * exp(-pc * pperp) * exp(-p[1] * (d * d));
      par_ind += 2;
    } else if (t == 6) {
      double q = p[3] * pc * (pperp * pperp) + p[1] * (d * d);
      ff = ff + p[0] * exp(0.5 * (q - exp(q)));
      par_ind += 3;
    }
  }
  return ff;
}

// determine_JT (src/ALPS_analyt.f90:1183-1389) for one ppar node
__device__ void fit_jacobian(const FitArgs& a, const double* params, int iperp, double pperp, double ppar,
                             double* J /* nJT */) {
  int par_ind = 0, JT_ind = 0;
  for (int ifit = 1; ifit <= a.nf; ++ifit) {
    int t = a.fit_type[ifit - 1];
    double pc = a.pc[ifit - 1];
    const double* p = params + (ifit + par_ind) - 1;
    double* Jp = J + (ifit + JT_ind) - 1;
    double d = ppar - p[2];
    if (t == 1) {
      double e = exp(-p[1] * (d * d) - pc * (pperp * pperp));
      Jp[0] = e;
      Jp[1] = -((d * d)) * p[0] * e;
      Jp[2] = 2.0 * p[1] * d * p[0] * e;
      par_ind += 2;
      JT_ind += 2;
    } else if (t == 2) {
      double kp = 1.0 + p[1] * (d * d) + pc * p[4] * (pperp * pperp);
      double kpm = pow(kp, p[3] - 1.0);
      Jp[0] = pow(kp, p[3]);
      Jp[1] = p[0] * p[3] * kpm * (d * d);
      Jp[2] = p[0] * p[3] * kpm * 2.0 * p[1] * (p[2] - ppar);
      Jp[3] = log(kp) * p[0] * pow(kp, p[3]);
      if (iperp == 0) {
        JT_ind += 3;
      } else {
        Jp[4] = p[0] * p[3] * kpm * pc * (pperp * pperp);
        JT_ind += 4;
      }
      par_ind += 4;
    } else if (t == 3) {
      double sq = sqrt(1.0 + ((pperp * pperp) + d * d) * a.vA * a.vA / (a.ms * a.ms));
      Jp[0] = exp(-p[1] * sq);
      Jp[1] = -p[0] * exp(-p[1] * sq) * sq;
      Jp[2] = p[0] * exp(-p[1] * sq) * (p[1] / sq) * d * a.vA * a.vA / (a.ms * a.ms);
      par_ind += 2;
      JT_ind += 2;
    } else if (t == 4) {
      Jp[0] = exp(-pc * pperp);
    } else if (t == 5) {
      double e = exp(-p[1] * (d * d)) * exp(-pc * pperp);
      Jp[0] = e;
      Jp[1] = -p[0] * e * (d * d);
      Jp[2] = 2.0 * p[0] * d * p[1] * e;
      par_ind += 2;
      JT_ind += 2;
    } else if (t == 6) {
      double q = p[3] * pc * (pperp * pperp) + p[1] * (d * d);
      double e = exp(0.5 * (q - exp(q)));
      Jp[0] = e;
      Jp[1] = p[0] * e * 0.5 * (d * d) * (1.0 - exp(q));
      Jp[2] = p[0] * e * p[1] * (p[2] - ppar) * (1.0 - exp(q));
      if (iperp == 0) {
        JT_ind += 2;
      } else {
        Jp[3] = p[0] * e * 0.5 * pc * (pperp * pperp) * (1.0 - exp(q));
        JT_ind += 3;
      }
      par_ind += 3;
    }
  }
}

#define FIT_MAXP (5 * ALPS_MAX_FITS)

// One species' fit: fit[(i*5+ip)*nf + ifit] holds the seeds at row 0 on
// entry and the fitted rows on exit.  scratch: (M+1)*(FIT_MAXP+1), with M
// the largest row length.  Rows are the iperp rows of the f0 table, or for a
// relativistic species the Gamma rows of f0_rel restricted to the subluminal
// cone (src/ALPS_analyt.f90:546-607).
// One species' fit, run by one warp: the points of a row are spread over
// the lanes; the scalar control flow (LM step, LU, parameter update) runs
// identically in every lane, and every sum over points runs in the
// reference's order.  Am_sh / jr_sh: the warp's shared scratch.
__device__ void lm_fit_body(const FitArgs& a, const double* __restrict__ f0, const double* __restrict__ pperp,
                            const double* __restrict__ ppar, double* fit, double* scratch, int* status,
                            double* Am_sh, double* jr_sh) {
  const int lane = threadIdx.x & 31;
  int nf = a.nf, N = a.rel ? a.ng : a.N;
  int n_params = 0;
  for (int f = 0; f < nf; ++f) n_params += fit_nparams(a, a.fit_type[f]);
  double params[FIT_MAXP];
  bool mask[FIT_MAXP];
  double* JT = scratch;                         // [(npts)][FIT_MAXP]
  int maxpts = a.rel ? a.np : a.M;
  double* resid = scratch + (size_t)(maxpts + 1) * FIT_MAXP;
  if (!a.rel && (1 + a.M) < n_params) {
    if (lane == 0) *status = ALPS_E_FIT_POINTS;
    return;
  }
  for (int iperp = 0; iperp <= N; ++iperp) {
    if (iperp != 0 && lane == 0)
      for (int ip = 0; ip < 5; ++ip)
        for (int f = 0; f < nf; ++f) fit[(iperp * 5 + ip) * nf + f] = fit[((iperp - 1) * 5 + ip) * nf + f];
    __syncwarp();
    int par_ind = 0, nJT = 0;
    for (int k = 0; k < n_params; ++k) mask[k] = true;
    for (int ifit = 1; ifit <= nf; ++ifit) {
      int t = a.fit_type[ifit - 1];
      int np = fit_nparams(a, t);
      for (int k = 0; k < np; ++k) params[ifit + par_ind + k - 1] = fit[(iperp * 5 + k) * nf + ifit - 1];
      if (t == 2 && iperp == 0) { nJT -= 1; mask[ifit + par_ind + 4 - 1] = false; }
      if (t == 6 && iperp == 0) { nJT -= 1; mask[ifit + par_ind + 3 - 1] = false; }
      par_ind += np - 1;
    }
    nJT += n_params;
    // points of this row: coordinates and fitted values
    int npts, off = 0;
    double xperp;
    if (a.rel) {
      const double* fr = a.f0rel + (size_t)iperp * (a.np + 1);
      bool fl = false, fu = false;
      int lower = 1, upper = a.np - 1;
      for (int ip = 1; ip <= a.np - 1; ++ip) {
        if (!fl && fr[ip - 1] <= -1.0 && fr[ip] > -1.0) { lower = ip; fl = true; }
        if (!fu && fr[ip] > -1.0 && fr[ip + 1] <= -1.0) { upper = ip; fu = true; }
      }
      xperp = a.grel[iperp];
      if ((upper - lower) <= 2) {
        int pi2 = 0;
        for (int ifit = 1; ifit <= nf; ++ifit) {
          params[ifit + pi2 - 1] = fr[(upper + lower) / 2] / exp(-a.pc[ifit - 1] * a.grel[iperp]);
          if (a.fit_type[ifit - 1] == 5) {
            params[ifit + pi2] = 1.0e-12;
            params[ifit + pi2 + 1] = 0.0;
            pi2 += 2;
          }
        }
        npts = -1;
      } else {
        npts = upper - lower;
        off = lower;
      }
    } else {
      npts = a.M;
      xperp = pperp[iperp];
    }
    auto xpar = [&](int j) { return a.rel ? a.prel[off + j] : ppar[j]; };
    auto gval = [&](int j) {
      double v = a.rel ? a.f0rel[(size_t)iperp * (a.np + 1) + off + j] : f0[iperp * (a.M + 1) + j];
      return a.log_fit ? log(v) : v;
    };
    if (npts >= 0) {
      double lambda_fit = a.lambda0, LSQ = 0.0, LSQnew;
      int counter = 0;
      bool converged = false;
      while (!converged) {
        counter++;
        for (int j = lane; j <= npts; j += 32) {
          double* Jc = JT + (size_t)j * FIT_MAXP;
          fit_jacobian(a, params, iperp, xperp, xpar(j), Jc);
          double fv = fit_value_real(a, params, xperp, xpar(j));
          if (a.log_fit) {
            for (int k = 0; k < nJT; ++k) Jc[k] = Jc[k] / fv;
            resid[j] = gval(j) - log(fv);
          } else {
            resid[j] = gval(j) - fv;
          }
        }
        __syncwarp();
        LSQ = 0.0;
        for (int j = 0; j <= npts; ++j) LSQ = LSQ + resid[j] * resid[j];
        double Am[FIT_MAXP * FIT_MAXP], jr[FIT_MAXP];
        for (int t = lane; t < nJT * nJT + nJT; t += 32) {
          double acc = 0.0;
          if (t < nJT * nJT) {
            int k = t % nJT, l = t / nJT;
            for (int j = 0; j <= npts; ++j) acc += JT[(size_t)j * FIT_MAXP + k] * JT[(size_t)j * FIT_MAXP + l];
            Am_sh[t] = acc;
          } else {
            int k = t - nJT * nJT;
            for (int j = 0; j <= npts; ++j) acc += JT[(size_t)j * FIT_MAXP + k] * resid[j];
            jr_sh[k] = acc;
          }
        }
        __syncwarp();
        for (int t = 0; t < nJT * nJT; ++t) Am[t] = Am_sh[t];
        for (int k = 0; k < nJT; ++k) jr[k] = jr_sh[k];
        __syncwarp();
        for (int k = 0; k < nJT; ++k) Am[k + nJT * k] = Am[k + nJT * k] + lambda_fit * Am[k + nJT * k];
        // LU with partial pivoting (dgetrf), then inverse (dgetri) times JT*r
        int piv[FIT_MAXP];
        bool singular = false;
        for (int k = 0; k < nJT && !singular; ++k) {
          int p = k;
          double mx = fabs(Am[k + nJT * k]);
          for (int i = k + 1; i < nJT; ++i)
            if (fabs(Am[i + nJT * k]) > mx) { mx = fabs(Am[i + nJT * k]); p = i; }
          piv[k] = p;
          if (Am[p + nJT * k] == 0.0) { singular = true; break; }
          if (p != k)
            for (int jj = 0; jj < nJT; ++jj) {
              double tmp = Am[k + nJT * jj];
              Am[k + nJT * jj] = Am[p + nJT * jj];
              Am[p + nJT * jj] = tmp;
            }
          for (int i = k + 1; i < nJT; ++i) {
            Am[i + nJT * k] /= Am[k + nJT * k];
            for (int jj = k + 1; jj < nJT; ++jj) Am[i + nJT * jj] -= Am[i + nJT * k] * Am[k + nJT * jj];
          }
        }
        if (singular) {
          if (lane == 0) *status = ALPS_E_SINGULAR;
          return;
        }
        double inv[FIT_MAXP * FIT_MAXP];
        for (int cc = 0; cc < nJT; ++cc) {
          double x[FIT_MAXP];
          for (int i = 0; i < nJT; ++i) x[i] = (i == cc) ? 1.0 : 0.0;
          for (int k = 0; k < nJT; ++k) {
            double tmp = x[k];
            x[k] = x[piv[k]];
            x[piv[k]] = tmp;
          }
          for (int i = 0; i < nJT; ++i)
            for (int k = 0; k < i; ++k) x[i] -= Am[i + nJT * k] * x[k];
          for (int i = nJT - 1; i >= 0; --i) {
            for (int k = i + 1; k < nJT; ++k) x[i] -= Am[i + nJT * k] * x[k];
            x[i] /= Am[i + nJT * i];
          }
          for (int i = 0; i < nJT; ++i) inv[i + nJT * cc] = x[i];
        }
        double delta[FIT_MAXP];
        for (int k = 0; k < nJT; ++k) {
          double acc = 0.0;
          for (int l = 0; l < nJT; ++l) acc += inv[k + nJT * l] * jr[l];
          delta[k] = acc;
        }
        int l = 0;
        for (int k = 0; k < n_params; ++k)
          if (mask[k]) params[k] = params[k] + delta[l++];
        for (int j = lane; j <= npts; j += 32) {
          double fv = fit_value_real(a, params, xperp, xpar(j));
          resid[j] = a.log_fit ? gval(j) - log(fv) : gval(j) - fv;
        }
        __syncwarp();
        LSQnew = 0.0;
        for (int j = 0; j <= npts; ++j) LSQnew = LSQnew + resid[j] * resid[j];
        __syncwarp();
        if (LSQnew > LSQ) {
          l = 0;
          for (int k = 0; k < n_params; ++k)
            if (mask[k]) params[k] = params[k] - delta[l++];
          lambda_fit = lambda_fit * a.lambdafac;
        } else {
          lambda_fit = lambda_fit / a.lambdafac;
        }
        if (fabs(LSQnew - LSQ) < a.eps) converged = true;
        if (counter == a.maxsteps) converged = true;
      }
    }
    par_ind = 0;
    for (int ifit = 1; ifit <= nf && lane == 0; ++ifit) {
      int np = fit_nparams(a, a.fit_type[ifit - 1]);
      for (int k = 0; k < np; ++k) fit[(iperp * 5 + k) * nf + ifit - 1] = params[ifit + par_ind + k - 1];
      par_ind += np - 1;
    }
    __syncwarp();
  }
}

__global__ void k_lm_fit(FitArgs a, const double* __restrict__ f0, const double* __restrict__ pperp,
                         const double* __restrict__ ppar, double* fit, double* scratch, int* status) {
  if (blockIdx.x != 0) return;
  __shared__ double Am_sh[FIT_MAXP * FIT_MAXP], jr_sh[FIT_MAXP];
  lm_fit_body(a, f0, pperp, ppar, fit, scratch, status, Am_sh, jr_sh);
}

}  // namespace

// the fit of one (context, species) in a batched launch
struct FitJob {
  FitArgs a;
  const double *f0, *pperp, *ppar;
  double *fit, *scratch;
  int* status;
};

namespace {

// every job of the batch, one warp each: fits of different plasmas are
// independent; within a fit the reference's warm start orders the rows
__global__ void k_lm_fit_many(const FitJob* __restrict__ jobs, int n) {
  const int j = blockIdx.x;
  if (j >= n) return;
  __shared__ double Am_sh[FIT_MAXP * FIT_MAXP], jr_sh[FIT_MAXP];
  const FitJob& J = jobs[j];
  lm_fit_body(J.a, J.f0, J.pperp, J.ppar, J.fit, J.scratch, J.status, Am_sh, jr_sh);
}

// determine_nmax for one species: the smallest n >= 1 with
// max_i |J_n(z_i)| <= Bessel_zero, z_i = k_perp pperp_i / q, or n = limit.
// The maximum exceeds the cutoff exactly when some node's |J_n| does.  The
// orders go in chunks of NMAX_CHUNK: first one thread per order tests the
// node nearest J_n's largest maximum (z = n + 0.81 n^(1/3); for orders past
// the grid's last z that is the last node, where |J_n| is largest), which
// settles nearly every order below the answer with one alps_bessj call;
// then the unsettled orders, in increasing order, test every node with the
// whole block, and the first with none above the cutoff is the answer.
// Each order's decision is the reference's: the same alps_bessj values
// against the same cutoff.  (The FP64 pipe is narrow on this part: one
// call of order n costs about 5 (n + sqrt(40 n)) FP64 operations.)
#define NMAX_CHUNK 128
__device__ void nmax_body(const double* __restrict__ pperp, int N, double kperp, double qs, double bzero, int limit,
                          int* nmax_out, unsigned* settled) {
  const int t = threadIdx.x;
  const double zs = fabs(qs) / kperp, dp = pperp[1] - pperp[0];
  auto above = [&](int nn, int i) {
    const double z = __ddiv_rn(__dmul_rn(kperp, pperp[i]), qs);
    return fabs(alps_bessj(nn, z)) > bzero;
  };
  for (int base = 1;; base += NMAX_CHUNK) {
    if (t < NMAX_CHUNK) {  // whole warps (NMAX_CHUNK is a multiple of 32)
      const int nn = base + t;
      bool hit = false;
      if (nn < limit) {
        const double u = ((nn + 0.81 * cbrt((double)nn)) * zs - pperp[0]) / dp;
        const int i0 = (u >= 0.0 && u <= (double)N) ? (int)rint(u) : ((u > 0.0 || u != u) ? N : 0);
        hit = above(nn, i0);
      }
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      if ((t & 31) == 0) settled[t >> 5] = m;
    }
    __syncthreads();
    for (int k = 0; k < NMAX_CHUNK; ++k) {
      const int nn = base + k;
      if (nn >= limit) {
        if (t == 0) *nmax_out = limit;
        return;
      }
      if ((settled[k >> 5] >> (k & 31)) & 1u) continue;
      bool hit = false;
      for (int i = t; i <= N && !hit; i += blockDim.x) hit = above(nn, i);
      if (!__syncthreads_or(hit)) {
        if (t == 0) *nmax_out = nn;
        return;
      }
    }
    __syncthreads();  // settled[] is rewritten by the next chunk
  }
}

__global__ void k_nmax(const double* __restrict__ pperp, int N, double kperp, double qs, double bzero,
                       int limit, int* nmax_out) {
  __shared__ unsigned settled[NMAX_CHUNK / 32];
  nmax_body(pperp, N, kperp, qs, bzero, limit, nmax_out, settled);
}

}  // namespace

// determine_nmax of one (context, species) in a batched launch
struct NmaxJob {
  const double* pperp;
  int N;
  double kperp, qs, bzero;
  int* out;
};

namespace {

__global__ void k_nmax_many(const NmaxJob* __restrict__ jobs, int n, int limit) {
  __shared__ unsigned settled[NMAX_CHUNK / 32];
  if ((int)blockIdx.x >= n) return;
  const NmaxJob& J = jobs[blockIdx.x];
  nmax_body(J.pperp, J.N, J.kperp, J.qs, J.bzero, limit, J.out, settled);
}

// bessel[(n+1)*(N+1)+i] = J_n(k_perp pperp_i / q), n = -1 .. nmax+1
__global__ void k_bessel_table(const double* __restrict__ pperp, int N, int nmax, double kperp, double qs,
                               double* bessel) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int n = (int)blockIdx.y - 1;
  if (i > N || n > nmax + 1) return;
  double z = __ddiv_rn(__dmul_rn(kperp, pperp[i]), qs);
  bessel[(size_t)(n + 1) * (N + 1) + i] = (n == -1) ? -alps_bessj(1, z) : alps_bessj(n, z);
}

// Rw[(F*(nmax+1) + n)*(N-1) + (i-1)] = w_perp(i) * R_F(n,i), F = 0: J_n^2,
// 1: pperp^2 J_n'^2, 2: pperp J_n J_n' (the three Bessel-product families of
// int_T), w_perp = 2 for i < N-1 and 1 at i = N-1.
__global__ void k_bessel_rows(const double* __restrict__ bessel, const double* __restrict__ pperp, int N,
                              int nmax, double* Rw) {
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  int n = blockIdx.y;
  if (i > N - 1 || n > nmax) return;
  const double* B = bessel;
  int L = N + 1;
  double J = B[(size_t)(n + 1) * L + i];
  double Jp = (n == 0) ? -B[(size_t)2 * L + i] : 0.5 * (B[(size_t)n * L + i] - B[(size_t)(n + 2) * L + i]);
  double w = (i <= N - 2) ? 2.0 : 1.0;
  double p = pperp[i];
  size_t stride = (size_t)(nmax + 1) * (N - 1);
  size_t o = (size_t)n * (N - 1) + (i - 1);
  Rw[o] = w * (J * J);
  Rw[stride + o] = w * ((p * p) * Jp * Jp);
  Rw[2 * stride + o] = w * (p * J * Jp);
}

// C[m][n] = sum_k A[m][k] B[k][n], row-major, FP64, 32x32 tiles, 2x2 per thread.
__global__ void k_dgemm(int Mr, int Nc, int K, const double* __restrict__ A, const double* __restrict__ B,
                        double* C) {
  __shared__ double As[32][17];
  __shared__ double Bs[16][33];
  int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  int row0 = blockIdx.y * 32, col0 = blockIdx.x * 32;
  double acc[2][2] = {{0, 0}, {0, 0}};
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int t = threadIdx.x; t < 32 * 16; t += 256) {
      int r = t / 16, kk = t % 16;
      int gr = row0 + r, gk = k0 + kk;
      As[r][kk] = (gr < Mr && gk < K) ? A[(size_t)gr * K + gk] : 0.0;
    }
    for (int t = threadIdx.x; t < 16 * 32; t += 256) {
      int kk = t / 32, cc = t % 32;
      int gk = k0 + kk, gc = col0 + cc;
      Bs[kk][cc] = (gk < K && gc < Nc) ? B[(size_t)gk * Nc + gc] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      double a0 = As[ty * 2][kk], a1 = As[ty * 2 + 1][kk];
      double b0 = Bs[kk][tx * 2], b1 = Bs[kk][tx * 2 + 1];
      acc[0][0] = fma(a0, b0, acc[0][0]);
      acc[0][1] = fma(a0, b1, acc[0][1]);
      acc[1][0] = fma(a1, b0, acc[1][0]);
      acc[1][1] = fma(a1, b1, acc[1][1]);
    }
    __syncthreads();
  }
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      int r = row0 + ty * 2 + a, cidx = col0 + tx * 2 + b;
      if (r < Mr && cidx < Nc) C[(size_t)r * Nc + cidx] = acc[a][b];
    }
}

// V[((n*(M-1)) + (j-1))*12 + 2*e + g] = 2 * c_e(j) * A[F(e)][n][g][j],
// entries e = xx, yy, zz, xy, xz, yz; c = 1, 1, ppar^2, 1, ppar, ppar.
// V of order n (block n) as float pairs scaled by 2^-e, e the exponent of
// max |V[n]|: x 2^-e = hi + lo, hi = float(x 2^-e), lo = float(x 2^-e - hi)
__global__ void k_split_df(const double* __restrict__ V, int M, double* scale, float* Vh, float* Vl) {
  __shared__ double red[256];
  const size_t len = (size_t)(M - 1) * 12;
  const double* v = V + (size_t)blockIdx.x * len;
  double mx = 0.0;
  for (size_t t = threadIdx.x; t < len; t += blockDim.x) mx = fmax(mx, fabs(v[t]));
  red[threadIdx.x] = mx;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  const int e = (red[0] > 0.0) ? ilogb(red[0]) : 0;
  const double down = ldexp(1.0, -e);
  if (threadIdx.x == 0) scale[blockIdx.x] = ldexp(1.0, e);
  for (size_t t = threadIdx.x; t < len; t += blockDim.x) {
    const double x = v[t] * down;
    const float h = __double2float_rn(x);
    Vh[(size_t)blockIdx.x * len + t] = h;
    Vl[(size_t)blockIdx.x * len + t] = __double2float_rn(x - (double)h);
  }
}

// ppar as float pairs
__global__ void k_split_pp(const double* __restrict__ ppar, int M, float* ph, float* pl) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j > M) return;
  const float h = __double2float_rn(ppar[j]);
  ph[j] = h;
  pl[j] = __double2float_rn(ppar[j] - (double)h);
}

__global__ void k_fold_reduced(const double* __restrict__ A, const double* __restrict__ ppar, int M, int nmax,
                               double* V) {
  int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  int n = blockIdx.y;
  if (j > M - 1 || n > nmax) return;
  size_t ncol = 2 * (size_t)(M - 1);
  auto Aat = [&](int F, int g) { return A[((size_t)F * (nmax + 1) + n) * ncol + (size_t)g * (M - 1) + (j - 1)]; };
  double p = ppar[j];
  double* v = V + ((size_t)n * (M - 1) + (j - 1)) * 12;
  for (int g = 0; g < 2; ++g) {
    double a0 = Aat(0, g), a1 = Aat(1, g), a2 = Aat(2, g);
    v[0 + g] = 2.0 * a0;
    v[2 + g] = 2.0 * a1;
    v[4 + g] = 2.0 * ((p * p) * a0);
    v[6 + g] = 2.0 * a2;
    v[8 + g] = 2.0 * (p * a0);
    v[10 + g] = 2.0 * (p * a2);
  }
}

// X[(j-1)*ALPS_KFAR + k] = x_j^k with x_j = (ppar_j - pcen)/prad, j = 1..M-1
__global__ void k_powers(const double* __restrict__ ppar, int M, double pcen, double prad, double* X) {
  int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > M - 1) return;
  double x = (ppar[j] - pcen) / prad;
  double p = 1.0;
  double* o = X + (size_t)(j - 1) * ALPS_KFAR;
  for (int k = 0; k < ALPS_KFAR; ++k) {
    o[k] = p;
    p *= x;
  }
}

// Laurent moments of the full-range trapezoid pole sum:
// mom[(n*ALPS_KFAR + k)*12 + q] = sum_j f_j V[n][j][q] x_j^k, f_j = 1/2 at
// j = 1, M-1 and 1 inside (the reduced vectors carry the interior weight 2).
// For a pole p far from the grid, sum_j f_j V_j / (p - ppar_j) =
//   (1/d) sum_k mom_k (prad/d)^k,  d = p - pcen.
// Also written: momf = mom rounded to FP32, and mom / Vscale[n] as float
// pairs (momh + moml, the per-order scale of the reduced vectors' pairs).
__global__ void k_moments(const double* __restrict__ V, const double* __restrict__ X, int M, int nmax,
                          const double* __restrict__ Vscale, double* mom, float* momf, float* momh, float* moml) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int total = (nmax + 1) * ALPS_KFAR * 12;
  if (t >= total) return;
  int q = t % 12, k = (t / 12) % ALPS_KFAR, n = t / (12 * ALPS_KFAR);
  const double* v = V + (size_t)n * (M - 1) * 12 + q;
  double acc = 0.0;
  for (int j = 1; j <= M - 1; ++j) {
    double f = (j == 1 || j == M - 1) ? 0.5 : 1.0;
    acc = fma(f * v[(size_t)(j - 1) * 12], X[(size_t)(j - 1) * ALPS_KFAR + k], acc);
  }
  mom[t] = acc;
  momf[t] = (float)acc;
  const double x = acc * (1.0 / Vscale[n]);  // a power of 2: exact
  const float h = __double2float_rn(x);
  momh[t] = h;
  moml[t] = __double2float_rn(x - (double)h);
}

// Base tables of the fast path's pole sums.  The six T-tensor entries use
// three Bessel families, F1 = J^2 (xx, xz, zz), F2 = pperp^2 J'^2 (yy) and
// F3 = pperp J J' (xy, yz), with the p_par factors 1, p_par, p_par^2.  With
// R_j = 1 / (k_par (zeta - p_j)), zeta the complex resonance momentum,
//   p_j R_j = zeta R_j - 1/k_par,
// so the p_par-weighted sums follow from the family sums and the
// omega-independent sums of the family vectors themselves:
//   sum w F p R   = zeta sum w F R - (1/k_par) sum w F,
//   sum w F p^2 R = zeta sum w F p R - (1/k_par) sum w F p.
// A node or Laurent term then feeds 6 real vectors instead of 12.  The
// vectors are V's q = 0, 1 (F1), 2, 3 (F2), 6, 7 (F3), scaled by
// 1/Vscale[n] (a power of two) and split into float pairs.
__device__ __forceinline__ int base_q(int b) { return b < 4 ? b : b + 2; }

// Bt and mBt: hi parts at [rec*12 + b], lo parts at [rec*12 + 6 + b]
__global__ void k_base_pairs(const double* __restrict__ V, const double* __restrict__ mom,
                             const double* __restrict__ Vscale, int M, int nmax, float* Bt, float* mBt) {
  const size_t nv = (size_t)(nmax + 1) * (M - 1) * 6, nm = (size_t)(nmax + 1) * ALPS_KFAR * 6;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nv + nm) return;
  const bool isv = t < nv;
  const size_t u = isv ? t : t - nv;
  const size_t rec = u / 6;
  const int b = (int)(u % 6);
  const int n = isv ? (int)(rec / (M - 1)) : (int)(rec / ALPS_KFAR);
  const double x = (isv ? V[rec * 12 + base_q(b)] : mom[rec * 12 + base_q(b)]) * (1.0 / Vscale[n]);
  const float h = __double2float_rn(x), l = __double2float_rn(x - (double)h);
  float* o = isv ? Bt : mBt;
  o[rec * 12 + b] = h;
  o[rec * 12 + 6 + b] = l;
}

// Pre[(n*M + j)*6 + c] = sum_{i=1..j} X_c(i), X = V[q]/Vscale[n] for
// q = 0, 1 (F1), 6, 7 (F3), 8, 9 (p_par F1), compensated (two-sum) so that
// each stored prefix is the exact sum rounded once; Cfull[n*6 + c] = the
// trapezoid sum over j = 1..M-1 (ends at weight 1/2).  One thread per (n, c).
__global__ void k_base_consts(const double* __restrict__ V, const double* __restrict__ Vscale, int M, int nmax,
                              double* Pre, double* Cfull) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (nmax + 1) * 6) return;
  const int n = t / 6, c = t % 6;
  const int q = (c < 2) ? c : c + 4;
  const double sc = 1.0 / Vscale[n];
  const double* v = V + (size_t)n * (M - 1) * 12 + q;
  double* P = Pre + (size_t)n * M * 6 + c;
  double s = 0.0, e = 0.0;
  P[0] = 0.0;
  for (int j = 1; j <= M - 1; ++j) {
    const double x = v[(size_t)(j - 1) * 12] * sc;
    const double y = s + x, bb = y - s;
    e += (s - (y - bb)) + (x - bb);
    s = y;
    P[(size_t)j * 6] = s + e;
  }
  const double x1 = v[0] * sc, xe = v[(size_t)(M - 2) * 12] * sc;
  Cfull[t] = (s + e) - 0.5 * (x1 + xe);
}

// Escale[e] = 2^E, E the exponent of max_n |C0 v_e(n) Vscale[n]|, and
// bfac[(n*6 + e)*2 + {0,1}] = C0 v_e(n) Vscale[n] / Escale[e] as a float
// pair (v_e of order n >= 0; xy and xz flip sign for -n).  One warp.
__global__ void k_base_fac(int nmax, double z, double kperp, int kperp_norm, double C0,
                           const double* __restrict__ Vscale, double* Escale, float* bfac) {
  const int e = threadIdx.x;
  if (e >= 6) return;
  double mx = 0.0;
  for (int n = 0; n <= nmax; ++n) mx = fmax(mx, fabs(fused_factor(n, e, z, kperp, kperp_norm, C0) * Vscale[n]));
  const double sc = (mx > 0.0 && isfinite(mx)) ? ldexp(1.0, ilogb(mx)) : 1.0;
  Escale[e] = sc;
  for (int n = 0; n <= nmax; ++n) {
    const double x = fused_factor(n, e, z, kperp, kperp_norm, C0) * Vscale[n] * (1.0 / sc);
    const float h = __double2float_rn(x);
    bfac[((size_t)n * 6 + e) * 2] = h;
    bfac[((size_t)n * 6 + e) * 2 + 1] = __double2float_rn(x - (double)h);
  }
}

// omega-independent factors of Maxwellian continuation terms, per row and
// fit: a0 = p1 exp(-pc pperp^2) (the reference's left-to-right product),
// p2, p3, exp(-p2 dppar^2)
__global__ void k_fit_aux(const double* __restrict__ fit, const double* __restrict__ pperp, int N, int nf,
                          double pc0, double pc1, double pc2, double pc3, double dppar, double* aux) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > N) return;
  double pcs[4] = {pc0, pc1, pc2, pc3};
  double p = pperp[i];
  for (int f = 0; f < nf; ++f) {
    double p1 = fit[(i * 5 + 0) * nf + f], p2 = fit[(i * 5 + 1) * nf + f], p3 = fit[(i * 5 + 2) * nf + f];
    double* o = aux + ((size_t)i * nf + f) * 4;
    o[0] = p1 * exp(-pcs[f] * (p * p));
    o[1] = p2;
    o[2] = p3;
    o[3] = exp(-p2 * (dppar * dppar));
  }
}

// Moments of the factorised Landau sums (one Maxwellian term per row,
// f(i,p) = a0_i exp(u_r(p)) exp(delta_i(p)), delta_i = a_i p^2 + b_i p + c_i,
// exp(delta) ~ 1 + delta + delta^2/2 = sum_m kappa_{i,m} p^m, m = 0..4):
//   w = 0: sum_i h_i R_F(n,i) pperp_i a0_i kappa_{i,m}   (the dfpar sum)
//   w = 1: sum_i c_i a0_i kappa_{i,m}, c = the transpose of landau_integrate's
//          p_perp difference operator applied to h_i R_F(n,i)  (the dfperp sum)
// h_i = 1/2 at i = 0, N-1, N and 1 otherwise (src/ALPS_fns.f90:1389-1444).
__global__ void k_landau_moments(const double* __restrict__ bessel, const double* __restrict__ pperp,
                                 const double* __restrict__ aux, int N, int nmax, double dpperp, double* lmom,
                                 float* lmomf) {
  // one warp per (n, F): lanes over the rows, then a warp sum
  const int t = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (t >= (nmax + 1) * 3) return;
  const int n = t / 3, F = t % 3;
  const int L = N + 1;
  auto Rw = [&](int i) {
    double J = bessel[(size_t)(n + 1) * L + i];
    double Jp = (n == 0) ? -bessel[(size_t)2 * L + i]
                         : 0.5 * (bessel[(size_t)n * L + i] - bessel[(size_t)(n + 2) * L + i]);
    double p = pperp[i];
    double h = (i == 0 || i == N - 1 || i == N) ? 0.5 : 1.0;
    double R = (F == 0) ? J * J : (F == 1 ? (p * p) * Jp * Jp : p * J * Jp);
    return h * R;
  };
  const double p2r = aux[1], p3r = aux[2];
  const double i2d = 1.0 / (2.0 * dpperp), i1d = 1.0 / dpperp;
  double m0[5] = {0, 0, 0, 0, 0}, m1[5] = {0, 0, 0, 0, 0};
  for (int i = lane; i <= N; i += 32) {
    const double* ai = aux + (size_t)i * 4;
    double a0 = ai[0], p2 = ai[1], p3 = ai[2];
    double a = -(p2 - p2r), b = 2.0 * (p2 * p3 - p2r * p3r), c = -(p2 * p3 * p3 - p2r * p3r * p3r);
    double k[5] = {1.0 + c + 0.5 * c * c, b * (1.0 + c), a + 0.5 * b * b + a * c, a * b, 0.5 * a * a};
    double w0 = Rw(i) * pperp[i];
    double cc = 0.0;  // transpose of the difference operator at i
    if (i - 1 >= 1 && i - 1 <= N - 1) cc += Rw(i - 1) * i2d;
    if (i + 1 >= 1 && i + 1 <= N - 1) cc -= Rw(i + 1) * i2d;
    if (i == 1) cc += Rw(0) * i1d;
    if (i == 0) cc -= Rw(0) * i1d;
    if (i == N) cc += Rw(N) * i1d;
    if (i == N - 1) cc -= Rw(N) * i1d;
    for (int m = 0; m < 5; ++m) {
      m0[m] += w0 * a0 * k[m];
      m1[m] += cc * a0 * k[m];
    }
  }
  for (int m = 0; m < 5; ++m)
    for (int off = 16; off > 0; off >>= 1) {
      m0[m] += __shfl_xor_sync(0xffffffffu, m0[m], off);
      m1[m] += __shfl_xor_sync(0xffffffffu, m1[m], off);
    }
  if (lane == 0) {
    double* o = lmom + (size_t)t * 10;
    for (int m = 0; m < 5; ++m) {
      o[m] = m0[m];
      o[5 + m] = m1[m];
    }
    // the fast path's copy: float pairs scaled by 2^-e, e the exponent of
    // the largest of the ten (hi at 0..9, lo at 10..19, e at 20)
    double mx = 0.0;
    for (int m = 0; m < 10; ++m) mx = fmax(mx, fabs(o[m]));
    const int e = (mx > 0.0 && isfinite(mx)) ? ilogb(mx) : 0;
    float* f = lmomf + (size_t)t * 24;
    for (int m = 0; m < 10; ++m) {
      const double x = ldexp(o[m], -e);
      const float h = __double2float_rn(x);
      f[m] = h;
      f[10 + m] = __double2float_rn(x - (double)h);
    }
    f[20] = (float)e;
    f[21] = f[22] = f[23] = 0.0f;
  }
}

// grows a table to at least n elements; a regrown table gets a quarter
// more, so a k scan whose nmax rises step by step reallocates (and pays
// cudaFree's device-wide wait) only now and then
template <typename T>
int ensure(T*& ptr, size_t& cap, size_t n) {
  if (n <= cap && ptr) return ALPS_OK;
  const size_t want = ptr ? n + n / 4 : n;
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  cap = 0;
  ALPS_CUDA_TRY(cudaMalloc(&ptr, want * sizeof(T)));
  cap = want;
  return ALPS_OK;
}

// ---------------------------------------------------------------------------
// Chebyshev continuation (ACmethod 2): set_polynomial_basis + determine_GLLS
// + least_squares_fit (src/ALPS_analyt.f90:731-889).  The basis on the
// uniform p_par nodes, and so the normal matrix A^T A, is the same on every
// p_perp row: it is built and LU-factored once (partial pivoting, dgetrf);
// each row then only forms A^T b and back-substitutes.  Sums run over p_par
// in ascending order without contraction.
// ---------------------------------------------------------------------------
__global__ void k_glls_basis(int M, int np, double* A /* [(M+1)][(np+1)] */) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j > M) return;
  double yy = __dadd_rn(-1.0, __dmul_rn((double)j, 2.0 / M));
  double* a = A + (size_t)j * (np + 1);
  a[0] = 1.0;
  if (np >= 1) a[1] = yy;
  for (int n = 2; n <= np; ++n) a[n] = __dsub_rn(__dmul_rn(__dmul_rn(2.0, yy), a[n - 1]), a[n - 2]);
}

// alpha = A^T A (column-major m x m), then its LU in place; one block
__global__ void k_glls_normal(const double* __restrict__ A, int M, int np, double* alpha, int* piv, int* status) {
  const int m = np + 1;
  for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
    int k = t % m, l = t / m;
    double acc = 0.0;
    for (int j = 0; j <= M; ++j) acc = __dadd_rn(acc, __dmul_rn(A[(size_t)j * m + k], A[(size_t)j * m + l]));
    alpha[t] = acc;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int k = 0; k < m; ++k) {
    int p = k;
    double mx = fabs(alpha[k + m * k]);
    for (int i = k + 1; i < m; ++i)
      if (fabs(alpha[i + m * k]) > mx) {
        mx = fabs(alpha[i + m * k]);
        p = i;
      }
    piv[k] = p;
    if (alpha[p + m * k] == 0.0) {
      *status = ALPS_E_SINGULAR;
      return;
    }
    if (p != k)
      for (int j = 0; j < m; ++j) {
        double tmp = alpha[k + m * j];
        alpha[k + m * j] = alpha[p + m * j];
        alpha[p + m * j] = tmp;
      }
    double dk = alpha[k + m * k];
    for (int i = k + 1; i < m; ++i) alpha[i + m * k] = __ddiv_rn(alpha[i + m * k], dk);
    for (int j = k + 1; j < m; ++j) {
      double f = alpha[k + m * j];
      if (f == 0.0) continue;
      for (int i = k + 1; i < m; ++i) alpha[i + m * j] = __dsub_rn(alpha[i + m * j], __dmul_rn(alpha[i + m * k], f));
    }
  }
}

// one block per p_perp row: b = log10 f0 (zeros replaced by 0.01 x the
// smallest positive value of the row) or f0, w = A^T b, LU solve
__global__ void k_glls_rows(const double* __restrict__ f0, const double* __restrict__ A,
                            const double* __restrict__ alpha, const int* __restrict__ piv, int M, int np, int log_fit,
                            const int* status, double* coeffs) {
  extern __shared__ double sm[];
  double* b = sm;            // [M+1]
  double* w = sm + (M + 1);  // [np+1]
  __shared__ double smin[128], spos[128];
  if (*status) return;
  const int i = blockIdx.x, m = np + 1;
  const double* row = f0 + (size_t)i * (M + 1);
  for (int j = threadIdx.x; j <= M; j += blockDim.x) b[j] = row[j];
  __syncthreads();
  if (log_fit) {
    double mn = 1.0e308, mp = 1.0e308;
    for (int j = threadIdx.x; j <= M; j += blockDim.x) {
      mn = fmin(mn, b[j]);
      if (b[j] > 0.0) mp = fmin(mp, b[j]);
    }
    smin[threadIdx.x] = mn;
    spos[threadIdx.x] = mp;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + s]);
        spos[threadIdx.x] = fmin(spos[threadIdx.x], spos[threadIdx.x + s]);
      }
      __syncthreads();
    }
    const bool fix = !(smin[0] > 0.0);
    const double repl = 0.01 * (spos[0] < 1.0e308 ? spos[0] : 1.0e-40);
    for (int j = threadIdx.x; j <= M; j += blockDim.x) b[j] = log10((fix && b[j] == 0.0) ? repl : b[j]);
    __syncthreads();
  }
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j <= M; ++j) acc = __dadd_rn(acc, __dmul_rn(A[(size_t)j * m + k], b[j]));
    w[k] = acc;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int k = 0; k < m; ++k) {
    double t = w[k];
    w[k] = w[piv[k]];
    w[piv[k]] = t;
  }
  for (int j = 0; j < m; ++j)
    for (int r = j + 1; r < m; ++r) w[r] = __dsub_rn(w[r], __dmul_rn(alpha[r + m * j], w[j]));
  for (int j = m - 1; j >= 0; --j) {
    w[j] = __ddiv_rn(w[j], alpha[j + m * j]);
    for (int r = 0; r < j; ++r) w[r] = __dsub_rn(w[r], __dmul_rn(alpha[r + m * j], w[j]));
  }
  for (int k = 0; k < m; ++k) coeffs[(size_t)i * m + k] = w[k];
}

}  // namespace

// ---------------------------------------------------------------------------
int launch_prepare_species(alps_ctx* c, int is) {
  SpeciesHost& S = c->spec[is];
  S.aux_ready = false;  // a new fit: its continuation factors and bounds follow at the next set_k
  if (S.sp.use_bM) return ALPS_OK;  // closed form: nothing to derive or fit
  int N = c->sys.nperp, M = c->sys.npar;
  cudaStream_t st = c->stream;
  size_t nn = (size_t)(N + 1) * (M + 1);
  if (!S.d_g1) ALPS_CUDA_TRY(cudaMalloc(&S.d_g1, nn * sizeof(double)));
  if (!S.d_g2) ALPS_CUDA_TRY(cudaMalloc(&S.d_g2, nn * sizeof(double)));
  if (!S.d_G) ALPS_CUDA_TRY(cudaMalloc(&S.d_G, (size_t)(N - 1) * 2 * (M - 1) * sizeof(double)));
  ALPS_CUDA_TRY(cudaMemsetAsync(S.d_g1, 0, nn * sizeof(double), st));
  ALPS_CUDA_TRY(cudaMemsetAsync(S.d_g2, 0, nn * sizeof(double), st));
  dim3 grid((M - 1 + 127) / 128, N - 1);
  k_derivatives<<<grid, 128, 0, st>>>(S.d_f0, S.d_pperp, S.d_ppar, N, M, S.d_g1, S.d_g2, S.d_G);
  ALPS_CUDA_TRY(cudaGetLastError());
  // ee term: int_ee * 2*pi*q/m * dpperp*dppar/4
  double dpperp = S.pperp[2] - S.pperp[1];
  double dppar = std::fabs(S.ppar[2] - S.ppar[1]);
  double scale = 2.0 * ALPS_PI * S.sp.qs / S.sp.ms * dpperp * dppar * 0.25;
  // per-species device words and fit scratch are kept with the species: a
  // cudaFree here would wait for the whole device, and contexts prepared on
  // several host threads would run one after another
  if (!S.d_words) ALPS_CUDA_TRY(cudaMalloc(&S.d_words, 2 * sizeof(double)));
  double* d_ee = S.d_words;
  int* d_status = reinterpret_cast<int*>(S.d_words + 1);
  k_int_ee<<<1, 256, 0, st>>>(S.d_g2, S.d_ppar, N, M, scale, d_ee);
  ALPS_CUDA_TRY(cudaGetLastError());
  // relativistic species: (Gamma, pparbar) grid, f0_rel and its derivatives
  int st_fit = ALPS_OK;
  if (S.sp.relat) st_fit = launch_rel_prepare(c, is);
  // Chebyshev continuation (ACmethod 2)
  if (S.sp.ac_method == 2 && st_fit == ALPS_OK) st_fit = launch_glls(c, is);
  // LM fit of the analytic continuation (ACmethod 1)
  if (S.sp.ac_method == 1 && st_fit == ALPS_OK) {
    FitArgs a;
    a.N = N;
    a.M = M;
    a.nf = S.sp.n_fits;
    a.log_fit = S.sp.log_fit;
    for (int f = 0; f < ALPS_MAX_FITS; ++f) {
      a.fit_type[f] = S.sp.fit_type[f];
      a.pc[f] = S.sp.perp_correction[f];
    }
    a.ms = S.sp.ms;
    a.vA = c->sys.vA;
    a.maxsteps = c->sys.maxsteps_fit;
    a.lambda0 = c->sys.lambda_initial_fit;
    a.lambdafac = c->sys.lambdafac_fit;
    a.eps = c->sys.epsilon_fit;
    a.rel = S.sp.relat ? 1 : 0;
    a.ng = c->sys.ngamma;
    a.np = c->sys.npparbar;
    a.f0rel = S.d_f0rel;
    a.grel = S.d_grel;
    a.prel = S.d_prel;
    int maxpts = a.rel ? a.np : M;
    int rc;
    if ((rc = ensure(S.d_fit_scratch, S.fit_scratch_cap, (size_t)(maxpts + 1) * (FIT_MAXP + 1)))) return rc;
    ALPS_CUDA_TRY(cudaMemsetAsync(d_status, 0, sizeof(int), st));
    k_lm_fit<<<1, 32, 0, st>>>(a, S.d_f0, S.d_pperp, S.d_ppar, S.d_fit, S.d_fit_scratch, d_status);
    ALPS_CUDA_TRY(cudaGetLastError());
    ALPS_CUDA_TRY(cudaMemcpyAsync(&st_fit, d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    ALPS_CUDA_TRY(cudaStreamSynchronize(st));
  }
  double ee = 0.0;
  ALPS_CUDA_TRY(cudaMemcpyAsync(&ee, d_ee, sizeof(double), cudaMemcpyDeviceToHost, st));
  ALPS_CUDA_TRY(cudaStreamSynchronize(st));
  S.int_ee = ee;
  return st_fit;
}

// ---------------------------------------------------------------------------
// Batched preparation of many contexts (alps_prepare_many): the derivative
// and ee kernels of every context on a few streams, then the
// Levenberg-Marquardt fits of every (context, species) in one launch, one
// warp each, then one synchronisation.  Relativistic species and the
// Chebyshev continuation take the per-context path.
// ---------------------------------------------------------------------------
static FitArgs fit_args_of(const alps_ctx* c, const SpeciesHost& S) {
  FitArgs a;
  a.N = c->sys.nperp;
  a.M = c->sys.npar;
  a.nf = S.sp.n_fits;
  a.log_fit = S.sp.log_fit;
  for (int f = 0; f < ALPS_MAX_FITS; ++f) {
    a.fit_type[f] = S.sp.fit_type[f];
    a.pc[f] = S.sp.perp_correction[f];
  }
  a.ms = S.sp.ms;
  a.vA = c->sys.vA;
  a.maxsteps = c->sys.maxsteps_fit;
  a.lambda0 = c->sys.lambda_initial_fit;
  a.lambdafac = c->sys.lambdafac_fit;
  a.eps = c->sys.epsilon_fit;
  a.rel = S.sp.relat ? 1 : 0;
  a.ng = c->sys.ngamma;
  a.np = c->sys.npparbar;
  a.f0rel = S.d_f0rel;
  a.grel = S.d_grel;
  a.prel = S.d_prel;
  return a;
}

bool ctx_batch_preparable(const alps_ctx* c) {
  for (const SpeciesHost& S : c->spec)
    if (!S.loaded || S.sp.relat || (!S.sp.use_bM && S.sp.ac_method != 1)) return false;
  return true;
}

int prepare_contexts(alps_ctx* const* ctx, int n, int* status) {
  const int NS = 8;
  cudaStream_t st[NS];
  for (int q = 0; q < NS; ++q) ALPS_CUDA_TRY(cudaStreamCreateWithFlags(&st[q], cudaStreamNonBlocking));
  std::vector<FitJob> jobs;
  std::vector<std::pair<int, int>> who;  // (context, species) of each job
  int rc = ALPS_OK;
  for (int i = 0; i < n && !rc; ++i) {
    alps_ctx* c = ctx[i];
    cudaStream_t s = st[i % NS];
    const int N = c->sys.nperp, M = c->sys.npar;
    const size_t nn = (size_t)(N + 1) * (M + 1);
    for (int is = 0; is < c->sys.nspec && !rc; ++is) {
      SpeciesHost& S = c->spec[is];
      S.aux_ready = false;
      if (S.sp.use_bM) continue;
      auto fail = [&](cudaError_t e) {
        if (e != cudaSuccess) rc = (e == cudaErrorMemoryAllocation) ? ALPS_E_OOM : ALPS_E_CUDA;
      };
      if (!S.d_g1) fail(cudaMalloc(&S.d_g1, nn * sizeof(double)));
      if (!S.d_g2 && !rc) fail(cudaMalloc(&S.d_g2, nn * sizeof(double)));
      if (!S.d_G && !rc) fail(cudaMalloc(&S.d_G, (size_t)(N - 1) * 2 * (M - 1) * sizeof(double)));
      if (!S.d_words && !rc) fail(cudaMalloc(&S.d_words, 2 * sizeof(double)));
      if (!rc && (rc = ensure(S.d_fit_scratch, S.fit_scratch_cap, (size_t)(M + 1) * (FIT_MAXP + 1)))) break;
      if (rc) break;
      fail(cudaMemsetAsync(S.d_g1, 0, nn * sizeof(double), s));
      fail(cudaMemsetAsync(S.d_g2, 0, nn * sizeof(double), s));
      fail(cudaMemsetAsync(S.d_words + 1, 0, sizeof(double), s));
      dim3 grid((M - 1 + 127) / 128, N - 1);
      k_derivatives<<<grid, 128, 0, s>>>(S.d_f0, S.d_pperp, S.d_ppar, N, M, S.d_g1, S.d_g2, S.d_G);
      const double dpperp = S.pperp[2] - S.pperp[1], dppar = std::fabs(S.ppar[2] - S.ppar[1]);
      const double scale = 2.0 * ALPS_PI * S.sp.qs / S.sp.ms * dpperp * dppar * 0.25;
      k_int_ee<<<1, 256, 0, s>>>(S.d_g2, S.d_ppar, N, M, scale, S.d_words);
      fail(cudaGetLastError());
      FitJob j;
      j.a = fit_args_of(c, S);
      j.f0 = S.d_f0;
      j.pperp = S.d_pperp;
      j.ppar = S.d_ppar;
      j.fit = S.d_fit;
      j.scratch = S.d_fit_scratch;
      j.status = reinterpret_cast<int*>(S.d_words + 1);
      jobs.push_back(j);
      who.push_back({i, is});
    }
  }
  FitJob* d_jobs = nullptr;
  for (int q = 0; q < NS && !rc; ++q)
    if (cudaStreamSynchronize(st[q]) != cudaSuccess) rc = ALPS_E_CUDA;
  if (!rc && !jobs.empty()) {
    if (cudaMalloc(&d_jobs, jobs.size() * sizeof(FitJob)) != cudaSuccess) rc = ALPS_E_OOM;
    if (!rc && cudaMemcpyAsync(d_jobs, jobs.data(), jobs.size() * sizeof(FitJob), cudaMemcpyHostToDevice, st[0]) !=
                   cudaSuccess)
      rc = ALPS_E_CUDA;
    if (!rc) {
      k_lm_fit_many<<<(unsigned)jobs.size(), 32, 0, st[0]>>>(d_jobs, (int)jobs.size());
      if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st[0]) != cudaSuccess) rc = ALPS_E_CUDA;
    }
  }
  // ee terms and fit statuses, then the continuation factors (asynchronous)
  for (size_t k = 0; k < who.size() && !rc; ++k) {
    alps_ctx* c = ctx[who[k].first];
    SpeciesHost& S = c->spec[who[k].second];
    double w[2];
    if (cudaMemcpy(w, S.d_words, 2 * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
      rc = ALPS_E_CUDA;
      break;
    }
    S.int_ee = w[0];
    int fst = 0;
    memcpy(&fst, &w[1], sizeof(int));
    if (fst && status && !status[who[k].first]) status[who[k].first] = fst;
  }
  for (int q = 0; q < NS; ++q) cudaStreamDestroy(st[q]);
  cudaFree(d_jobs);
  return rc;
}

// determine_nmax of every (non-closed-form) species of every context in one
// launch; nm[i][s] receives the results (closed-form species get 1)
int nmax_contexts(alps_ctx* const* ctx, int n, const double* kperp, std::vector<std::vector<int>>& nm) {
  std::vector<NmaxJob> jobs;
  nm.assign(n, {});
  size_t tot = 0;
  for (int i = 0; i < n; ++i) tot += ctx[i]->sys.nspec;
  // the results and the job table in one stream-ordered allocation on a
  // stream of its own: nothing here waits for other work on the device
  const size_t ob = ((tot ? tot : 1) * sizeof(int) + 15) / 16 * 16;
  size_t njobs = 0;
  for (int i = 0; i < n; ++i)
    for (int is = 0; is < ctx[i]->sys.nspec; ++is) njobs += ctx[i]->spec[is].sp.use_bM ? 0 : 1;
  cudaStream_t st;
  ALPS_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  unsigned char* d_buf = nullptr;
  int rc = ALPS_OK;
  if (cudaMallocAsync(&d_buf, ob + (njobs ? njobs : 1) * sizeof(NmaxJob), st) != cudaSuccess) rc = ALPS_E_OOM;
  int* d_out = reinterpret_cast<int*>(d_buf);
  NmaxJob* d_jobs = reinterpret_cast<NmaxJob*>(d_buf + ob);
  size_t k = 0;
  for (int i = 0; i < n; ++i) {
    nm[i].assign(ctx[i]->sys.nspec, 1);
    for (int is = 0; is < ctx[i]->sys.nspec; ++is, ++k) {
      const SpeciesHost& S = ctx[i]->spec[is];
      if (S.sp.use_bM) continue;
      jobs.push_back(NmaxJob{S.d_pperp, ctx[i]->sys.nperp, kperp[i], S.sp.qs, ctx[i]->sys.Bessel_zero, d_out + k});
    }
  }
  std::vector<int> out(tot ? tot : 1, 0);
  if (!rc && !jobs.empty()) {
    if (cudaMemcpyAsync(d_jobs, jobs.data(), jobs.size() * sizeof(NmaxJob), cudaMemcpyHostToDevice, st) !=
        cudaSuccess)
      rc = ALPS_E_CUDA;
    if (!rc) {
      k_nmax_many<<<(unsigned)jobs.size(), 256, 0, st>>>(d_jobs, (int)jobs.size(), 2000);
      if (cudaGetLastError() != cudaSuccess) rc = ALPS_E_CUDA;
    }
    if (!rc && cudaMemcpyAsync(out.data(), d_out, tot * sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
      rc = ALPS_E_CUDA;
  }
  if (d_buf) cudaFreeAsync(d_buf, st);
  if (cudaStreamSynchronize(st) != cudaSuccess && !rc) rc = ALPS_E_CUDA;
  cudaStreamDestroy(st);
  k = 0;
  for (int i = 0; i < n && !rc; ++i)
    for (int is = 0; is < ctx[i]->sys.nspec; ++is, ++k)
      if (!ctx[i]->spec[is].sp.use_bM) {
        if (out[k] >= 2000) rc = ALPS_E_INVALID;  // orders beyond 2000 are outside the supported range
        nm[i][is] = out[k];
      }
  return rc;
}

int launch_glls(alps_ctx* c, int is) {
  SpeciesHost& S = c->spec[is];
  const int N = c->sys.nperp, M = c->sys.npar, np = S.sp.poly_order, m = np + 1;
  cudaStream_t st = c->stream;
  double *d_A = nullptr, *d_alpha = nullptr;
  int *d_piv = nullptr, *d_status = nullptr;
  ALPS_CUDA_TRY(cudaMalloc(&d_A, (size_t)(M + 1) * m * sizeof(double)));
  ALPS_CUDA_TRY(cudaMalloc(&d_alpha, (size_t)m * m * sizeof(double)));
  ALPS_CUDA_TRY(cudaMalloc(&d_piv, m * sizeof(int)));
  ALPS_CUDA_TRY(cudaMalloc(&d_status, sizeof(int)));
  ALPS_CUDA_TRY(cudaMemsetAsync(d_status, 0, sizeof(int), st));
  k_glls_basis<<<(M + 1 + 127) / 128, 128, 0, st>>>(M, np, d_A);
  k_glls_normal<<<1, 256, 0, st>>>(d_A, M, np, d_alpha, d_piv, d_status);
  size_t smem = (size_t)(M + 1 + m) * sizeof(double);
  if (smem > 48 * 1024) ALPS_CUDA_TRY(cudaFuncSetAttribute(k_glls_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_glls_rows<<<N + 1, 128, smem, st>>>(S.d_f0, d_A, d_alpha, d_piv, M, np, S.sp.log_fit, d_status, S.d_fit);
  ALPS_CUDA_TRY(cudaGetLastError());
  int status = 0;
  ALPS_CUDA_TRY(cudaMemcpyAsync(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  ALPS_CUDA_TRY(cudaStreamSynchronize(st));
  cudaFree(d_A);
  cudaFree(d_alpha);
  cudaFree(d_piv);
  cudaFree(d_status);
  return status;
}

int launch_set_k_species(alps_ctx* c, int is, double kperp, int* nmax_out) {
  SpeciesHost& S = c->spec[is];
  if (S.sp.use_bM) {  // determine_nmax gives a bi-Maxwellian species 1 (src/ALPS_fns.f90:4012-4014)
    *nmax_out = 1;
    return ALPS_OK;
  }
  // a device word kept with the species: no allocation (and no cudaFree,
  // which would wait for the whole device) per k step
  if (!S.d_nmax) ALPS_CUDA_TRY(cudaMalloc(&S.d_nmax, sizeof(int)));
  k_nmax<<<1, 256, 0, c->stream>>>(S.d_pperp, c->sys.nperp, kperp, S.sp.qs, c->sys.Bessel_zero, 2000, S.d_nmax);
  ALPS_CUDA_TRY(cudaGetLastError());
  int nm = 0;
  ALPS_CUDA_TRY(cudaMemcpyAsync(&nm, S.d_nmax, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  ALPS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (nm >= 2000) return ALPS_E_INVALID;  // orders beyond 2000 are outside the supported range
  *nmax_out = nm;
  return ALPS_OK;
}

int launch_build_bessel_and_reduced(alps_ctx* c, int is, double kperp) {
  SpeciesHost& S = c->spec[is];
  int N = c->sys.nperp, M = c->sys.npar, nmax = S.nmax;
  cudaStream_t st = c->stream;
  int rc;
  if ((rc = ensure(S.d_bessel, S.bessel_cap, (size_t)(nmax + 3) * (N + 1)))) return rc;
  if ((rc = ensure(S.d_Rw, S.Rw_cap, (size_t)3 * (nmax + 1) * (N - 1)))) return rc;
  if ((rc = ensure(S.d_A, S.A_cap, (size_t)3 * (nmax + 1) * 2 * (M - 1)))) return rc;
  if ((rc = ensure(S.d_V, S.V_cap, (size_t)(nmax + 1) * (M - 1) * 12))) return rc;
  k_bessel_table<<<dim3((N + 1 + 127) / 128, nmax + 3), 128, 0, st>>>(S.d_pperp, N, nmax, kperp, S.sp.qs,
                                                                       S.d_bessel);
  ALPS_CUDA_TRY(cudaGetLastError());
  k_bessel_rows<<<dim3((N - 1 + 127) / 128, nmax + 1), 128, 0, st>>>(S.d_bessel, S.d_pperp, N, nmax, S.d_Rw);
  ALPS_CUDA_TRY(cudaGetLastError());
  int Mr = 3 * (nmax + 1), Nc = 2 * (M - 1), K = N - 1;
  S.tc_used = 0;
  S.tc_fixed = 0;
  if (c->precision == ALPS_PREC_MIXED && K <= 256) {
    // mixed path: the contraction on the tensor cores, FP64-accurate per
    // entry (tc_product_checked recomputes in FP64 whatever its bound does
    // not cover)
    const size_t need = tc_checked_workspace_bytes(Mr, Nc, K);
    if (need > S.tcws_cap) {
      if (S.d_tcws) cudaFree(S.d_tcws);
      S.d_tcws = nullptr;
      S.tcws_cap = 0;
      ALPS_CUDA_TRY(cudaMalloc(&S.d_tcws, need));
      S.tcws_cap = need;
    }
    // (a batched set_k defers the count of FP64-recomputed entries: no sync here)
    if ((rc = tc_product_checked(S.d_Rw, S.d_G, S.d_A, Mr, Nc, K, S.d_tcws, c->defer_sync ? nullptr : &S.tc_fixed,
                                 st)))
      return rc;
    S.tc_used = 1;
  } else {
    k_dgemm<<<dim3((Nc + 31) / 32, (Mr + 31) / 32), 256, 0, st>>>(Mr, Nc, K, S.d_Rw, S.d_G, S.d_A);
    ALPS_CUDA_TRY(cudaGetLastError());
  }
  k_fold_reduced<<<dim3((M - 1 + 127) / 128, nmax + 1), 128, 0, st>>>(S.d_A, S.d_ppar, M, nmax, S.d_V);
  ALPS_CUDA_TRY(cudaGetLastError());
  {
    // the FP32 test for orders far from resonance (both paths' classify):
    // the resonance interval of determine_resonances with a margin of 1e-5
    // of its extent
    const double mi = c->sys.positions_principal * (S.ppar[2] - S.ppar[1]);
    const double rlo = std::min(S.ppar[1] - mi, S.ppar[1]), rhi = std::max(S.ppar[M], S.ppar[M - 1] + mi);
    const double mg = 1e-5 * (std::fabs(rlo) + std::fabs(rhi));
    S.qlo = (float)(rlo - mg);
    S.qhi = (float)(rhi + mg);
    S.qlo_in = (float)(rlo + mg);
    S.qhi_in = (float)(rhi - mg);
  }
  // the plain path sums nodes in FP64 on V alone; the float pairs, Laurent
  // moments and order-fused tables below serve the mixed path only (a
  // change of path rebuilds the k tables)
  if (c->precision == ALPS_PREC_FP64) return ALPS_OK;
  const size_t nvf = (size_t)(nmax + 1) * (M - 1) * 12;
  if ((rc = ensure(S.d_Vh, S.Vf_cap, 2 * nvf))) return rc;  // hi, then lo
  S.d_Vl = S.d_Vh + nvf;
  if ((rc = ensure(S.d_Vscale, S.Vs_cap, (size_t)(nmax + 1)))) return rc;
  k_split_df<<<nmax + 1, 256, 0, st>>>(S.d_V, M, S.d_Vscale, S.d_Vh, S.d_Vl);
  ALPS_CUDA_TRY(cudaGetLastError());
  if (!S.d_pph) {
    ALPS_CUDA_TRY(cudaMalloc(&S.d_pph, (M + 1) * sizeof(float)));
    ALPS_CUDA_TRY(cudaMalloc(&S.d_ppl, (M + 1) * sizeof(float)));
  }
  k_split_pp<<<(M + 1 + 127) / 128, 128, 0, st>>>(S.d_ppar, M, S.d_pph, S.d_ppl);
  ALPS_CUDA_TRY(cudaGetLastError());
  double pcen = 0.5 * (S.ppar[1] + S.ppar[M - 1]), prad = 0.5 * (S.ppar[M - 1] - S.ppar[1]);
  if (!S.d_X) ALPS_CUDA_TRY(cudaMalloc(&S.d_X, (size_t)(M - 1) * ALPS_KFAR * sizeof(double)));
  if ((rc = ensure(S.d_mom, S.mom_cap, (size_t)(nmax + 1) * ALPS_KFAR * 12))) return rc;
  const size_t nmo = (size_t)(nmax + 1) * ALPS_KFAR * 12;
  if ((rc = ensure(S.d_momf, S.momf_cap, 3 * nmo))) return rc;  // momf, then the pairs' hi and lo
  S.d_momh = S.d_momf + nmo;
  S.d_moml = S.d_momf + 2 * nmo;
  k_powers<<<(M - 1 + 127) / 128, 128, 0, st>>>(S.d_ppar, M, pcen, prad, S.d_X);
  ALPS_CUDA_TRY(cudaGetLastError());
  int tot = (nmax + 1) * ALPS_KFAR * 12;
  k_moments<<<(tot + 127) / 128, 128, 0, st>>>(S.d_V, S.d_X, M, nmax, S.d_Vscale, S.d_mom, S.d_momf, S.d_momh,
                                               S.d_moml);
  ALPS_CUDA_TRY(cudaGetLastError());
  // base tables of the fast path's pole sums
  {
    const double z = c->sys.kperp_norm ? kperp / S.sp.qs : 1.0 / S.sp.qs;
    const double dpperp = S.pperp[2] - S.pperp[1], dppar_abs = std::fabs(S.ppar[2] - S.ppar[1]);
    const double C0 = 2.0 * ALPS_PI * dpperp * dppar_abs * 0.25 * S.sp.qs;
    const size_t nm = (size_t)(nmax + 1);
    if ((rc = ensure(S.d_Bt, S.Bt_cap, nvf + nmo + nm * 12))) return rc;  // Bt, mBt, bfac
    if ((rc = ensure(S.d_Bd, S.Bd_cap, 8 + nm * 6 + nm * (size_t)M * 6))) return rc;  // Escale, Cfull, Pre
    const size_t np = (nvf + nmo) / 2;
    k_base_pairs<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(S.d_V, S.d_mom, S.d_Vscale, M, nmax, S.d_Bt,
                                                              S.d_Bt + nvf);
    ALPS_CUDA_TRY(cudaGetLastError());
    k_base_consts<<<(unsigned)((nm * 6 + 127) / 128), 128, 0, st>>>(S.d_V, S.d_Vscale, M, nmax,
                                                                      S.d_Bd + 8 + nm * 6, S.d_Bd + 8);
    ALPS_CUDA_TRY(cudaGetLastError());
    k_base_fac<<<1, 32, 0, st>>>(nmax, z, kperp, c->sys.kperp_norm, C0, S.d_Vscale, S.d_Bd, S.d_Bt + nvf + nmo);
    ALPS_CUDA_TRY(cudaGetLastError());
  }
  return ALPS_OK;
}

int launch_fit_aux(alps_ctx* c, int is) {
  SpeciesHost& S = c->spec[is];
  if (S.aux_ready) return ALPS_OK;  // built for the current fit already
  bool maxw = S.sp.ac_method == 1 && !S.sp.use_bM;
  for (int f = 0; f < S.sp.n_fits && maxw; ++f) maxw = S.sp.fit_type[f] == 1;
  if (!maxw) {
    if (S.d_fit_aux) cudaFree(S.d_fit_aux);
    S.d_fit_aux = nullptr;
    return ALPS_OK;
  }
  int N = c->sys.nperp, nf = S.sp.n_fits;
  if (!S.d_fit_aux) ALPS_CUDA_TRY(cudaMalloc(&S.d_fit_aux, (size_t)(N + 1) * ALPS_MAX_FITS * 4 * sizeof(double)));
  double dppar = std::fabs(S.ppar[2] - S.ppar[1]);
  k_fit_aux<<<(N + 1 + 127) / 128, 128, 0, c->stream>>>(S.d_fit, S.d_pperp, N, nf, S.sp.perp_correction[0],
                                                         S.sp.perp_correction[1], S.sp.perp_correction[2],
                                                         S.sp.perp_correction[3], dppar, S.d_fit_aux);
  ALPS_CUDA_TRY(cudaGetLastError());
  return ALPS_OK;
}

// Factorised Landau moments for species whose continuation is one Maxwellian
// term; the per-item validity bound uses max |a_i|, |b_i|, |c_i| (host).
int launch_landau_moments(alps_ctx* c, int is) {
  SpeciesHost& S = c->spec[is];
  if (S.aux_ready) {
    // the bounds belong to the fit, not to k: only the moments are per k,
    // and only the mixed path reads them
    if (!S.lfact || c->precision == ALPS_PREC_FP64) return ALPS_OK;
    int rc;
    if ((rc = ensure(S.d_lmom, S.lmom_cap, (size_t)(S.nmax + 1) * (30 + 36)))) return rc;  // FP64, then the pairs
    const int tot = (S.nmax + 1) * 3;
    k_landau_moments<<<(tot + 3) / 4, 128, 0, c->stream>>>(S.d_bessel, S.d_pperp, S.d_fit_aux, c->sys.nperp,
                                                           S.nmax, S.pperp[2] - S.pperp[1], S.d_lmom,
                                                           reinterpret_cast<float*>(S.d_lmom + (size_t)(S.nmax + 1) * 30));
    ALPS_CUDA_TRY(cudaGetLastError());
    return ALPS_OK;
  }
  S.aux_ready = true;
  S.lfact = false;
  if (!S.d_fit_aux || S.sp.n_fits != 1 || !S.d_bessel) return ALPS_OK;
  int N = c->sys.nperp, nmax = S.nmax;
  std::vector<double> aux((size_t)(N + 1) * 4);
  ALPS_CUDA_TRY(cudaMemcpyAsync(aux.data(), S.d_fit_aux, aux.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                c->stream));
  ALPS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  double p2r = aux[1], p3r = aux[2], la = 0, lb = 0, lc = 0, mina0 = 1e308;
  for (int i = 0; i <= N; ++i) {
    double p2 = aux[i * 4 + 1], p3 = aux[i * 4 + 2];
    la = std::max(la, std::fabs(p2 - p2r));
    lb = std::max(lb, std::fabs(2.0 * (p2 * p3 - p2r * p3r)));
    lc = std::max(lc, std::fabs(p2 * p3 * p3 - p2r * p3r * p3r));
    if (i >= 1) mina0 = std::min(mina0, std::fabs(aux[i * 4 + 0]));
    if (!std::isfinite(p2) || !std::isfinite(p3) || !std::isfinite(aux[i * 4])) return ALPS_OK;
  }
  S.p2r = p2r;
  S.p3r = p3r;
  S.la = la;
  S.lb = lb;
  S.lc = lc;
  S.min_a0 = mina0;
  S.lfact = true;
  if (c->precision == ALPS_PREC_FP64) return ALPS_OK;
  int rc;
  if ((rc = ensure(S.d_lmom, S.lmom_cap, (size_t)(nmax + 1) * (30 + 36)))) return rc;  // FP64, then the pairs
  int tot = (nmax + 1) * 3;
  double dpperp = S.pperp[2] - S.pperp[1];
  k_landau_moments<<<(tot + 3) / 4, 128, 0, c->stream>>>(S.d_bessel, S.d_pperp, S.d_fit_aux, N, nmax, dpperp,
                                                         S.d_lmom,
                                                         reinterpret_cast<float*>(S.d_lmom + (size_t)(nmax + 1) * 30));
  ALPS_CUDA_TRY(cudaGetLastError());
  return ALPS_OK;
}
