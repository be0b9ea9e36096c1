// nhds_kernels.cu -- bi-Maxwellian and cold species in closed form
// (src/ALPS_NHDS.f90, used for species with use_bM = T; dispatched at
// src/ALPS_fns.f90:338-360).
//
// Per k (launch_nhds_bessel): z = (k_perp v_th / Omega)^2 alpha / 2 depends
// on k_perp only, so exp(-z) I_n(z) for every order the sum needs is one
// small table, and the order range (the first n with n >= bM_nmaxs or
// exp(-z) I_n(z) < bM_Bessel_zeros, calc_chi :131-140) is read back once.
// Per omega batch (launch_nhds): one block per (omega, species); threads take
// the Bessel orders of Stix's Y tensor (calc_ypsilon :244-367), each through
// the plasma dispersion function of the Faddeeva function w (WOFZ :537-711),
// and a fixed-order block reduction forms chi and chi_low (calc_chi
// :59-238); a cold species (beta = 0) takes calc_chi_cold (:371-455).
#include <cmath>

#include "alps_internal.cuh"
#include "device_math.cuh"

namespace {

// BESSI0 / BESSI1 (:806-862): exp(-|x|) I_0(x), exp(-|x|) I_1(x)
__device__ double bessi0_s(double x) {
  const double P1 = 1.0, P2 = 3.5156229, P3 = 3.0899424, P4 = 1.2067492, P5 = 0.2659732, P6 = 0.360768e-1,
               P7 = 0.45813e-2;
  const double Q1 = 0.39894228, Q2 = 0.1328592e-1, Q3 = 0.225319e-2, Q4 = -0.157565e-2, Q5 = 0.916281e-2,
               Q6 = -0.2057706e-1, Q7 = 0.2635537e-1, Q8 = -0.1647633e-1, Q9 = 0.392377e-2;
  double ax = fabs(x);
  if (ax < 3.75) {
    double y = (x / 3.75) * (x / 3.75);
    return (P1 + y * (P2 + y * (P3 + y * (P4 + y * (P5 + y * (P6 + y * P7)))))) * exp(-ax);
  }
  double y = 3.75 / ax, bx = 1.0 / sqrt(ax);
  ax = Q1 + y * (Q2 + y * (Q3 + y * (Q4 + y * (Q5 + y * (Q6 + y * (Q7 + y * (Q8 + y * Q9)))))));
  return ax * bx;
}

__device__ double bessi1_s(double x) {
  const double P1 = 0.5, P2 = 0.87890594, P3 = 0.51498869, P4 = 0.15084934, P5 = 0.2658733e-1, P6 = 0.301532e-2,
               P7 = 0.32411e-3;
  const double Q1 = 0.39894228, Q2 = -0.3988024e-1, Q3 = -0.362018e-2, Q4 = 0.163801e-2, Q5 = -0.1031555e-1,
               Q6 = 0.2282967e-1, Q7 = -0.2895312e-1, Q8 = 0.1787654e-1, Q9 = -0.420059e-2;
  double ax = fabs(x);
  if (ax < 3.75) {
    double y = (x / 3.75) * (x / 3.75);
    return x * (P1 + y * (P2 + y * (P3 + y * (P4 + y * (P5 + y * (P6 + y * P7)))))) * exp(-ax);
  }
  double y = 3.75 / ax, bx = 1.0 / sqrt(ax);
  ax = Q1 + y * (Q2 + y * (Q3 + y * (Q4 + y * (Q5 + y * (Q6 + y * (Q7 + y * (Q8 + y * Q9)))))));
  return ax * bx;
}

// BESSI (:760-801): Miller's downward recurrence from 2(n + sqrt(40 n)),
// rescaled by 2^-512 whenever the binary exponent passes 512
__device__ double bessi_s(int n, double x) {
  if (n == 0) return bessi0_s(x);
  if (n == 1) return bessi1_s(x);
  if (x == 0.0) return 0.0;
  const int IBIGNO = 512;
  double tox = 2.0 / x, bip = 0.0, bi = 1.0, r = 0.0;
  int m = 2 * (n + (int)sqrtf((float)(40 * n)));
  for (int j = m; j >= 1; --j) {
    double bim = bip + (double)j * tox * bi;
    bip = bi;
    bi = bim;
    int e = 0;
    if (bi != 0.0) frexp(bi, &e);
    if (e > IBIGNO) {
      bi = ldexp(bi, -IBIGNO);
      bip = ldexp(bip, -IBIGNO);
      r = ldexp(r, -IBIGNO);
    }
    if (j == n) r = bip;
  }
  return bessi0_s(x) * (r / bi);
}

__device__ double powi_d(double x, int m) {
  unsigned n = m < 0 ? -(unsigned)m : (unsigned)m;
  double y = (n % 2) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2) y = y * x;
  }
  return m < 0 ? 1.0 / y : y;
}

// Faddeeva function, algorithm 680 (Poppe and Wijers, ACM TOMS 16, 47, 1990),
// with the reference's single-precision literals kept as such
__device__ double2 wofz_d(double XI, double YI) {
  const double FACTOR = 1.12837916709551257388, RMAXREAL = 0.5e154, RMAXEXP = 708.503061461606,
               RMAXGONI = 3.53711887601422e15;
  double U = 0.0, V = 0.0;
  double XABS = fabs(XI), YABS = fabs(YI);
  double X = XABS / (double)6.3f, Y = YABS / (double)4.4f;
  if ((XABS > RMAXREAL) || (YABS > RMAXREAL)) return cmk(U, V);
  double QRHO = X * X + Y * Y;
  double XABSQ = XABS * XABS;
  double XQUAD = XABSQ - YABS * YABS;
  double YQUAD = 2 * XABS * YABS;
  bool A = QRHO < 0.085264;
  double U2 = 0.0, V2 = 0.0;
  if (A) {
    QRHO = (1 - (double)0.85f * Y) * sqrt(QRHO);
    int N = (int)llround(6 + 72 * QRHO);
    int J = 2 * N + 1;
    double XSUM = (double)(1.0f / (float)J);
    double YSUM = 0.0;
    for (int I = N; I >= 1; --I) {
      J = J - 2;
      double XAUX = (XSUM * XQUAD - YSUM * YQUAD) / I;
      YSUM = (XSUM * YQUAD + YSUM * XQUAD) / I;
      XSUM = XAUX + (double)(1.0f / (float)J);
    }
    double U1 = -FACTOR * (XSUM * YABS + YSUM * XABS) + 1.0;
    double V1 = FACTOR * (XSUM * XABS - YSUM * YABS);
    double DAUX = exp(-XQUAD);
    U2 = DAUX * cos(YQUAD);
    V2 = -DAUX * sin(YQUAD);
    U = U1 * U2 - V1 * V2;
    V = U1 * V2 + V1 * U2;
  } else {
    double H, H2 = 0.0, QLAMBDA = 0.0;
    int KAPN, NU;
    if (QRHO > 1.0) {
      H = 0.0;
      KAPN = 0;
      QRHO = sqrt(QRHO);
      NU = (int)(3 + (1442 / (26 * QRHO + 77)));
    } else {
      QRHO = (1 - Y) * sqrt(1 - QRHO);
      H = (double)1.88f * QRHO;
      H2 = 2 * H;
      KAPN = (int)llround(7 + 34 * QRHO);
      NU = (int)llround(16 + 26 * QRHO);
    }
    bool B = (H > 0.0);
    if (B) QLAMBDA = powi_d(H2, KAPN);
    double RX = 0.0, RY = 0.0, SX = 0.0, SY = 0.0;
    for (int N = NU; N >= 0; --N) {
      int NP1 = N + 1;
      double TX = YABS + H + NP1 * RX;
      double TY = XABS - NP1 * RY;
      double C = 0.5 / (TX * TX + TY * TY);
      RX = C * TX;
      RY = C * TY;
      if (B && (N <= KAPN)) {
        TX = QLAMBDA + SX;
        SX = RX * TX - RY * SY;
        SY = RY * TX + RX * SY;
        QLAMBDA = QLAMBDA / H2;
      }
    }
    if (H == 0.0) {
      U = FACTOR * RX;
      V = FACTOR * RY;
    } else {
      U = FACTOR * SX;
      V = FACTOR * SY;
    }
    if (YABS == 0.0) U = exp(-(XABS * XABS));
  }
  if (YI < 0.0) {
    if (A) {
      U2 = 2 * U2;
      V2 = 2 * V2;
    } else {
      XQUAD = -XQUAD;
      if ((YQUAD > RMAXGONI) || (XQUAD > RMAXEXP)) return cmk(U, V);
      double W1 = 2 * exp(XQUAD);
      U2 = W1 * cos(YQUAD);
      V2 = -W1 * sin(YQUAD);
    }
    U = U2 - U;
    V = V2 - V;
    if (XI > 0.0) V = -V;
  } else {
    if (XI < 0.0) V = -V;
  }
  return cmk(U, V);
}

// plasma dispersion function (dispfunct :487-531): Z = i sqrt(pi) w(zeta)
__device__ double2 dispfunct_d(double2 zeta, bool kpos) {
  const double sp = sqrt(ALPS_PI);
  if (kpos) {
    double2 w = wofz_d(zeta.x, zeta.y);
    return cmk(-sp * w.y, sp * w.x);
  }
  double2 w = wofz_d(-zeta.x, -zeta.y);
  return cmk(sp * w.y, -sp * w.x);
}

struct BM {
  double Omega, ell, vtherm, vdrift, alpha;
};

__device__ BM bm_of(const SpecDev& S) {
  BM b;
  b.Omega = S.qs / S.ms;
  b.ell = sqrt(S.ms / (S.ns * S.qs * S.qs));
  b.vtherm = sqrt(S.bm_beta / (S.ns * S.ms));
  b.vdrift = S.bm_pdrift / S.ms;
  b.alpha = S.bm_alpha;
  return b;
}

// entries 11 22 33 12 13 23 of Stix's Y tensor of order n (calc_ypsilon)
__device__ void ypsilon6(const SpecDev& S, const SysDev& sy, const BM& b, int n, double2 x, double2 Y[6]) {
  const double kz = sy.kpar, kperp = sy.kperp;
  const bool kpos = !(kz < 0.0), kn = sy.kperp_norm != 0;
  const double Omega = b.Omega, vth = b.vtherm, vd = b.vdrift, al = b.alpha;
  const double nO = 1.0 * n * Omega;
  double2 resfac = cmk(x.x - kz * vd - nO, x.y);
  double2 zeta = cmk(resfac.x / (kz * vth), resfac.y / (kz * vth));
  const double z = 0.5 * (kperp * vth / Omega) * (kperp * vth / Omega) * al;
  const double zp = 0.5 * (vth / Omega) * (vth / Omega) * al;
  double2 Z = dispfunct_d(zeta, kpos);
  double2 t = cadd(cscale(resfac, al), cmk(nO, 0.0));
  double2 An = cadd(cmk(al - 1.0, 0.0), cmul(cscale(t, 1.0 / (kz * vth)), Z));
  double2 xn = cmk(x.x - nO, x.y);
  double2 Bn = cscale(csub(cscale(xn, al), cmk(kz * vd - nO, 0.0)), 1.0 / kz);
  Bn = cadd(Bn, cmul(cscale(cmul(xn, t), 1.0 / (kz * kz * vth)), Z));
  const int an = n < 0 ? -n : n;
  const double BI = S.bmI[an];
  const double dB = 5.0e-1 * (S.bmI[(n + 1) < 0 ? -(n + 1) : (n + 1)] + S.bmI[(n - 1) < 0 ? -(n - 1) : (n - 1)]);
  const double nn = (double)(n * n), d = BI - dB;
  if (kn) {
    Y[0] = cscale(An, nn * BI / z);
    Y[1] = cscale(An, nn * BI / z + 2.0 * z * BI - 2.0 * z * dB);
    Y[2] = cscale(cmul(xn, Bn), 2.0 * BI / (kz * vth * vth * al));
    double2 a = cscale(An, -(double)n * d);                          // -i n (I - I') An
    Y[3] = cmk(-a.y, a.x);
    Y[4] = cscale(Bn, kperp * n * BI / (Omega * z));
    double2 c = cscale(Bn, kperp * d / Omega);                       // i kperp (I - I') Bn / Omega
    Y[5] = cmk(-c.y, c.x);
  } else {
    const double k2 = kperp * kperp;
    Y[0] = cscale(An, nn * BI / zp);
    Y[1] = cscale(An, nn * BI / zp + k2 * 2.0 * z * BI - k2 * 2.0 * z * dB);
    Y[2] = cscale(cmul(xn, Bn), k2 * 2.0 * BI / (kz * vth * vth * al));
    double2 a = cscale(An, -(double)n * d * k2);
    Y[3] = cmk(-a.y, a.x);
    Y[4] = cscale(Bn, kperp * n * BI / (Omega * zp));
    double2 c = cscale(Bn, k2 * kperp * d / Omega);
    Y[5] = cmk(-c.y, c.x);
  }
}

// calc_chi_cold, entries 11 22 33 12 13 23
__device__ void chi_cold6(const SpecDev& S, const SysDev& sy, const BM& b, double2 x, double2 c[6]) {
  const double kz = sy.kpar, kperp = sy.kperp, Omega = b.Omega, vd = b.vdrift;
  const double il2 = 1.0 / (b.ell * b.ell);
  double2 d = cmk(x.x - kz * vd, x.y);
  double2 R = cscale(cdiv(d, cmk(d.x + Omega, d.y)), -il2);
  double2 L = cscale(cdiv(d, cmk(d.x - Omega, d.y)), -il2);
  double2 d2 = cmul(d, d);
  double2 den = cmk(d2.x - Omega * Omega, d2.y);
  double2 P = cadd(cdiv(cmul(x, x), d2), cdiv(cmk((kperp * vd) * (kperp * vd), 0.0), den));
  P = cscale(P, -il2);
  double2 J = cscale(cdiv(d, den), -il2 * kperp * vd);
  double2 Mi = cscale(cdiv(cmk(1.0, 0.0), den), il2 * kperp * vd * Omega);  // dispM / i
  double2 sum = cscale(cadd(R, L), 0.5), dif = cscale(csub(R, L), 0.5);
  c[0] = sum;
  c[1] = sum;
  c[2] = P;
  c[3] = cmk(dif.y, -dif.x);  // -i (R - L) / 2
  c[4] = J;
  c[5] = cmk(-Mi.y, Mi.x);    // i (...)
}

// exp(-z) I_n(z) for n = 0..nmax+1, then the order range
__global__ void k_nhds_bessel(double z, int nmax, double bzero, double* bI, int* nrun) {
  for (int n = threadIdx.x; n <= nmax + 1; n += blockDim.x) bI[n] = bessi_s(n, z);
  __syncthreads();
  if (threadIdx.x == 0) {
    int n = 0;
    while (!((n >= nmax) || (bI[n] < bzero))) n = n + 1;
    *nrun = n;
  }
}

__device__ void block_sum(double* v, int nv, double* sh) {
  for (int q = 0; q < nv; ++q)
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int q = 0; q < nv; ++q) sh[warp * nv + q] = v[q];
  __syncthreads();
  if (threadIdx.x == 0)
    for (int q = 0; q < nv; ++q) v[q] = ((sh[q] + sh[nv + q]) + sh[2 * nv + q]) + sh[3 * nv + q];
  __syncthreads();
}

struct NhdsArgs {
  SysDev sys;
  SpecDev sp[ALPS_MAX_SPECIES];
};

// one block (128 threads) per (omega, species)
__global__ void __launch_bounds__(128) k_nhds(NhdsArgs a, const double2* __restrict__ om, int n_om,
                                              double2* __restrict__ out) {
  __shared__ double sh[4 * 12];
  __shared__ double2 ylow[3][6];
  const int w = blockIdx.x, s = blockIdx.y;
  const SpecDev& S = a.sp[s];
  if (w >= n_om || !S.bm) return;
  const double2 x = om[w];
  const BM b = bm_of(S);
  double2* dst = out + ((size_t)w * a.sys.nspec + s) * 24;
  if (S.bm_beta == 0.0) {  // cold species: no chi_low
    if (threadIdx.x == 0) {
      double2 c[6];
      chi_cold6(S, a.sys, b, x, c);
      for (int e = 0; e < 6; ++e) dst[e] = c[e];
      for (int e = 6; e < 24; ++e) dst[e] = cmk(0.0, 0.0);
    }
    return;
  }
  const int nr = S.bm_nrun;
  double v[12];
  for (int q = 0; q < 12; ++q) v[q] = 0.0;
  for (int n = -nr + (int)threadIdx.x; n <= nr; n += blockDim.x) {
    double2 Y[6];
    ypsilon6(S, a.sys, b, n, x, Y);
    for (int e = 0; e < 6; ++e) {
      v[2 * e] += Y[e].x;
      v[2 * e + 1] += Y[e].y;
    }
    if (n >= -1 && n <= 1)
      for (int e = 0; e < 6; ++e) ylow[n + 1][e] = Y[e];
  }
  if (nr == 0) {
    // only n = 0 ran; the n = +-1 parts are zero
    if (threadIdx.x == 0)
      for (int e = 0; e < 6; ++e) ylow[0][e] = ylow[2][e] = cmk(0.0, 0.0);
  }
  __syncthreads();
  block_sum(v, 12, sh);
  if (threadIdx.x == 0) {
    const double l2 = b.ell * b.ell;
    const double kperp = a.sys.kperp, kz = a.sys.kpar;
    double2 drift = cscale(x, 2.0 * b.vdrift / (l2 * kz * b.vtherm * b.vtherm * b.alpha));
    if (!a.sys.kperp_norm) drift = cscale(drift, kperp * kperp);
    for (int e = 0; e < 6; ++e) dst[e] = cmk(v[2 * e] / l2, v[2 * e + 1] / l2);
    dst[2] = cadd(drift, dst[2]);
    for (int l = 0; l < 3; ++l)
      for (int e = 0; e < 6; ++e) dst[6 + 6 * l + e] = cmk(ylow[l][e].x / l2, ylow[l][e].y / l2);
    dst[6 + 6 + 2] = cadd(dst[6 + 6 + 2], drift);
  }
}

}  // namespace

int launch_nhds_bessel(alps_ctx* c, int is, double kperp) {
  SpeciesHost& S = c->spec[is];
  const alps_species& sp = S.sp;
  S.bm_nrun = 0;
  if (sp.bM_betas == 0.0) return ALPS_OK;
  double Omega = sp.qs / sp.ms, vth = std::sqrt(sp.bM_betas / (sp.ns * sp.ms));
  double z = 0.5 * (kperp * vth / Omega) * (kperp * vth / Omega) * sp.bM_alphas;
  int nmax = std::max(sp.bM_nmaxs, 0);
  if (S.d_bmI) cudaFree(S.d_bmI);
  S.d_bmI = nullptr;
  ALPS_CUDA_TRY(cudaMalloc(&S.d_bmI, (size_t)(nmax + 2) * sizeof(double)));
  int* d_n = nullptr;
  ALPS_CUDA_TRY(cudaMalloc(&d_n, sizeof(int)));
  k_nhds_bessel<<<1, 256, 0, c->stream>>>(z, nmax, sp.bM_Bessel_zeros, S.d_bmI, d_n);
  ALPS_CUDA_TRY(cudaGetLastError());
  int nr = 0;
  ALPS_CUDA_TRY(cudaMemcpyAsync(&nr, d_n, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  ALPS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  cudaFree(d_n);
  S.bm_nrun = nr;
  return ALPS_OK;
}

int launch_nhds(const SysDev& sys, const SpecDev* sp, int n, const double2* d_om, double2* d_out, cudaStream_t st) {
  NhdsArgs a;
  a.sys = sys;
  bool any = false;
  for (int s = 0; s < sys.nspec; ++s) {
    a.sp[s] = sp[s];
    any = any || sp[s].bm;
  }
  if (!any || n <= 0) return ALPS_OK;
  k_nhds<<<dim3(n, sys.nspec), 128, 0, st>>>(a, d_om, n, d_out);
  ALPS_CUDA_TRY(cudaGetLastError());
  return ALPS_OK;
}
