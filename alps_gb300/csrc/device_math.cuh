// device_math.cuh -- device restatements of the reference's special
// functions and of its exactly-rounded index arithmetic.
//
// The Bessel recurrences and the resonance tests are written with explicit
// round-to-nearest intrinsics (__dmul_rn, __dadd_rn, ...) so that the compiler
// cannot contract them into FMAs: the reference (gfortran, no FMA) makes its
// nmax and resonance decisions from exactly these roundings.
#pragma once
#include "alps_internal.cuh"

// J0, J1: rational approximations of src/ALPS_fns_rel.f90:1651-1735
// (Hart / Abramowitz-Stegun coefficients as printed there).  The
// single-precision literals of the reference (8., 2.35619491) are kept.
__device__ inline double alps_bessj0(double x) {
  const double P1 = 1.0, P2 = -.1098628627e-2, P3 = .2734510407e-4, P4 = -.2073370639e-5,
               P5 = .2093887211e-6;
  const double Q1 = -.1562499995e-1, Q2 = .1430488765e-3, Q3 = -.6911147651e-5, Q4 = .7621095161e-6,
               Q5 = -.9349451520e-7;
  const double R1 = 57568490574.0, R2 = -13362590354.0, R3 = 651619640.7, R4 = -11214424.18,
               R5 = 77392.33017, R6 = -184.9052456;
  const double S1 = 57568490411.0, S2 = 1029532985.0, S3 = 9494680.718, S4 = 59272.64853,
               S5 = 267.8532712, S6 = 1.0;
  if (x == 0.0) return 1.0;
  double ax = fabs(x);
  if (ax < 8.0) {
    double y = __dmul_rn(x, x);
    double fr = __dadd_rn(R1, __dmul_rn(y, __dadd_rn(R2, __dmul_rn(y, __dadd_rn(R3, __dmul_rn(y,
                __dadd_rn(R4, __dmul_rn(y, __dadd_rn(R5, __dmul_rn(y, R6))))))))));
    double fs = __dadd_rn(S1, __dmul_rn(y, __dadd_rn(S2, __dmul_rn(y, __dadd_rn(S3, __dmul_rn(y,
                __dadd_rn(S4, __dmul_rn(y, __dadd_rn(S5, __dmul_rn(y, S6))))))))));
    return __ddiv_rn(fr, fs);
  }
  double z = __ddiv_rn(8.0, ax);
  double y = __dmul_rn(z, z);
  double xx = __dsub_rn(ax, .785398164);
  double fp = __dadd_rn(P1, __dmul_rn(y, __dadd_rn(P2, __dmul_rn(y, __dadd_rn(P3, __dmul_rn(y,
              __dadd_rn(P4, __dmul_rn(y, P5))))))));
  double fq = __dadd_rn(Q1, __dmul_rn(y, __dadd_rn(Q2, __dmul_rn(y, __dadd_rn(Q3, __dmul_rn(y,
              __dadd_rn(Q4, __dmul_rn(y, Q5))))))));
  return __dmul_rn(sqrt(__ddiv_rn(.636619772, ax)),
                   __dsub_rn(__dmul_rn(fp, cos(xx)), __dmul_rn(__dmul_rn(z, fq), sin(xx))));
}

__device__ inline double alps_bessj1(double x) {
  const double P1 = 1.0, P2 = .183105e-2, P3 = -.3516396496e-4, P4 = .2457520174e-5,
               P5 = -.240337019e-6, P6 = .636619772;
  const double Q1 = .04687499995, Q2 = -.2002690873e-3, Q3 = .8449199096e-5, Q4 = -.88228987e-6,
               Q5 = .105787412e-6;
  const double R1 = 72362614232.0, R2 = -7895059235.0, R3 = 242396853.1, R4 = -2972611.439,
               R5 = 15704.48260, R6 = -30.16036606;
  const double S1 = 144725228442.0, S2 = 2300535178.0, S3 = 18583304.74, S4 = 99447.43394,
               S5 = 376.9991397, S6 = 1.0;
  double ax = fabs(x);
  if (ax < 8.0) {
    double y = __dmul_rn(x, x);
    double fr = __dadd_rn(R1, __dmul_rn(y, __dadd_rn(R2, __dmul_rn(y, __dadd_rn(R3, __dmul_rn(y,
                __dadd_rn(R4, __dmul_rn(y, __dadd_rn(R5, __dmul_rn(y, R6))))))))));
    double fs = __dadd_rn(S1, __dmul_rn(y, __dadd_rn(S2, __dmul_rn(y, __dadd_rn(S3, __dmul_rn(y,
                __dadd_rn(S4, __dmul_rn(y, __dadd_rn(S5, __dmul_rn(y, S6))))))))));
    return __dmul_rn(x, __ddiv_rn(fr, fs));
  }
  double z = __ddiv_rn(8.0, ax);
  double y = __dmul_rn(z, z);
  double xx = __dsub_rn(ax, (double)2.35619491f);
  double fp = __dadd_rn(P1, __dmul_rn(y, __dadd_rn(P2, __dmul_rn(y, __dadd_rn(P3, __dmul_rn(y,
              __dadd_rn(P4, __dmul_rn(y, P5))))))));
  double fq = __dadd_rn(Q1, __dmul_rn(y, __dadd_rn(Q2, __dmul_rn(y, __dadd_rn(Q3, __dmul_rn(y,
              __dadd_rn(Q4, __dmul_rn(y, Q5))))))));
  double r = __dmul_rn(sqrt(__ddiv_rn(P6, ax)),
                       __dsub_rn(__dmul_rn(cos(xx), fp), __dmul_rn(__dmul_rn(z, sin(xx)), fq)));
  return x < 0.0 ? -r : r;
}

// BESSJ (src/ALPS_fns_rel.f90:1575-1646): upward recurrence for x > n,
// Miller's downward recurrence with renormalisation otherwise.
__device__ inline double alps_bessj(int n, double x) {
  if (n == 0) return alps_bessj0(x);
  if (n == 1) return alps_bessj1(x);
  if (x == 0.0) return 0.0;
  double tox = __ddiv_rn(2.0, x);
  if (x > (double)(float)n) {
    double bjm = alps_bessj0(x), bj = alps_bessj1(x), bjp;
    for (int j = 1; j <= n - 1; ++j) {
      bjp = __dsub_rn(__dmul_rn(__dmul_rn((double)j, tox), bj), bjm);
      bjm = bj;
      bj = bjp;
    }
    return bj;
  }
  int m = 2 * ((n + (int)sqrtf((float)(40 * n))) / 2);
  double res = 0.0, sum = 0.0, bjp = 0.0, bj = 1.0, bjm;
  int jsum = 0;
  for (int j = m; j >= 1; --j) {
    bjm = __dsub_rn(__dmul_rn(__dmul_rn((double)j, tox), bj), bjp);
    bjp = bj;
    bj = bjm;
    if (fabs(bj) > 1.0e10) {
      bj = __dmul_rn(bj, 1.0e-10);
      bjp = __dmul_rn(bjp, 1.0e-10);
      res = __dmul_rn(res, 1.0e-10);
      sum = __dmul_rn(sum, 1.0e-10);
    }
    if (jsum != 0) sum = __dadd_rn(sum, bj);
    jsum = 1 - jsum;
    if (j == n) res = bjp;
  }
  sum = __dsub_rn(__dmul_rn(2.0, sum), bj);
  return __ddiv_rn(res, sum);
}

// ---------------------------------------------------------------------------
// complex elementary functions (FP64)
// ---------------------------------------------------------------------------
__device__ inline double2 cexp_d(double2 z) {
  double e = exp(z.x), s, c;
  sincos(z.y, &s, &c);
  return cmk(e * c, e * s);
}
__device__ inline double2 clog_d(double2 z) { return cmk(log(hypot(z.x, z.y)), atan2(z.y, z.x)); }
__device__ inline double2 csqrt_d(double2 z) {
  double r = hypot(z.x, z.y);
  if (r == 0.0) return cmk(0.0, 0.0);
  double t = sqrt(0.5 * (r + fabs(z.x)));
  if (z.x >= 0.0) return cmk(t, 0.5 * z.y / t);
  return cmk(0.5 * fabs(z.y) / t, z.y >= 0.0 ? t : -t);
}

// ---------------------------------------------------------------------------
// Double-float arithmetic: x = h + l with |l| <= ulp(h)/2, about 48 bits,
// on the FP32 pipes (64 times the FP64 rate on this part).  Error-free
// transformations: two_sum (Knuth), the FMA product error; every operation
// explicitly rounded so that nothing is contracted.
// ---------------------------------------------------------------------------
struct dflt {
  float h, l;
};
__device__ __forceinline__ dflt df_of(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ double df_val(dflt a) { return (double)a.h + (double)a.l; }
__device__ __forceinline__ dflt df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ dflt df_quick(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dflt df_add(dflt a, dflt b) {
  const dflt s = df_two_sum(a.h, b.h);
  return df_quick(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ dflt df_mul(dflt a, dflt b) {
  const float p = __fmul_rn(a.h, b.h);
  const float e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, __fmaf_rn(a.h, b.h, -p)));
  return df_quick(p, e);
}
__device__ __forceinline__ dflt df_neg(dflt a) { return {-a.h, -a.l}; }
__device__ __forceinline__ dflt df_scale(dflt a, float s) { return {__fmul_rn(a.h, s), __fmul_rn(a.l, s)}; }  // s a power of 2
// 1/a: one Newton step from the FP32 reciprocal, r = r0 + r0 (1 - a r0)
__device__ __forceinline__ dflt df_rcp(dflt a) {
  const float r0 = __frcp_rn(a.h);
  const dflt e = df_add({1.0f, 0.0f}, df_neg(df_mul(a, {r0, 0.0f})));
  return df_add({r0, 0.0f}, df_mul({r0, 0.0f}, e));
}
// 1/a from the FP32 approximate reciprocal r0 (within 1 ulp):
// d = 1 - a r0 (|d| <= 2^-22; 1 - a.h r0 is exact in one FMA), and
// 1/a = r0 (1 + d + d^2 + ...), so 1/a = r0 + r0 (d + d^2) with an error of
// about 2^-45 relative (d^3 <= 2^-66; three roundings of 2^-24 of terms
// below 2^-22).  The pair is returned unnormalised (|l| <= 2^-21 |h|), which
// df_mul and df_add accept.  a must be a normal float pair.
__device__ __forceinline__ dflt df_rcp_approx(dflt a) {
  float r0;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(a.h));
  const float d = __fmaf_rn(-a.l, r0, __fmaf_rn(-a.h, r0, 1.0f));
  return {r0, __fmul_rn(r0, __fmaf_rn(d, d, d))};
}
// acc += c, the low part unnormalised until the end
__device__ __forceinline__ void df_acc(dflt& acc, dflt c) {
  const dflt s = df_two_sum(acc.h, c.h);
  acc.h = s.h;
  acc.l = __fadd_rn(acc.l, __fadd_rn(s.l, c.l));
}
// acc += (vh + vl)(rh + rl), the low parts unnormalised until the end
__device__ __forceinline__ void df_mac(dflt& acc, float vh, float vl, dflt r) {
  const float p = __fmul_rn(vh, r.h);
  const float pl = __fmaf_rn(vh, r.l, __fmaf_rn(vl, r.h, __fmaf_rn(vh, r.h, -p)));
  const dflt s = df_two_sum(acc.h, p);
  acc.h = s.h;
  acc.l = __fadd_rn(acc.l, __fadd_rn(s.l, pl));
}

// 1/j! as float pairs (hi, lo), j = 0..18: the Taylor coefficients of
// df_exp_scaled and df_cis
__constant__ float c_inv_fact[19][2] = {
    {1.0f, 0.0f}, {1.0f, 0.0f}, {0.5f, 0.0f},
    {0.1666666716337204f, -4.967053879312289e-09f}, {0.0416666679084301f, -1.2417634698280722e-09f},
    {0.008333333767950535f, -4.34617203337595e-10f}, {0.0013888889225199819f, -3.3631094437103215e-11f},
    {0.00019841270113829523f, -2.725596874933456e-12f}, {2.4801587642286904e-05f, -3.40699609366682e-13f},
    {2.7557318844628753e-06f, 3.793571224297229e-14f}, {2.755731998149713e-07f, -7.575112209051195e-15f},
    {2.5052107943679403e-08f, 4.4176230446483665e-16f}, {2.0876755879584152e-09f, 1.1082839147459852e-16f},
    {1.6059044372074283e-10f, -5.352526511562726e-18f}, {1.147074536050896e-11f, 2.372207689231238e-19f},
    {7.647163609812713e-13f, 1.2200710471178288e-20f}, {4.7794772561329454e-14f, 7.62544404448643e-22f},
    {2.8114573589663704e-15f, -1.0462084739763658e-22f}, {1.5619206814541513e-16f, 1.5404471465941993e-24f}};
__device__ __forceinline__ dflt inv_fact(int j) { return {c_inv_fact[j][0], c_inv_fact[j][1]}; }

// exp(x) = 2^k m for a double x, |x| <= 1000, with m a float pair in
// [0.70, 1.42] (relative error about 2^-47, tested against FP64 on the CPU):
// k = rint(x / ln 2) and r = x - k ln 2 in FP64 (Cody and Waite: ln 2 in two
// parts, k ln2_hi exact for |k| < 2^21), then the Taylor polynomial of
// degree 13 of exp(r), |r| <= 0.347 (truncation below 2^-57), in
// double-float.
__device__ __forceinline__ dflt df_exp_scaled(double x, int& k) {
  const double kd = rint(x * 1.4426950408889634);
  double r = fma(-kd, 0.6931471803691238, x);
  r = fma(-kd, 1.9082149292705877e-10, r);
  k = (int)kd;
  const dflt q = df_of(r);
  dflt p = inv_fact(13);
#pragma unroll
  for (int j = 12; j >= 0; --j) p = df_add(df_mul(p, q), inv_fact(j));
  return p;
}

// cos(y) + i sin(y) for a double y, |y| < 1e6 (absolute error about 2^-46):
// q = rint(y 2/pi) and r = y - q pi/2 in FP64 (Cody and Waite: pi/2 in three
// parts, the first two products exact for |q| < 2^20), then with s = r^2,
// |r| <= pi/4, sin r = r sum_j (-s)^j / (2j+1)! and cos r = sum_j (-s)^j /
// (2j)!, j <= 8 (truncation below 2^-58), in double-float; q mod 4 picks
// the signs and the order.
__device__ __forceinline__ void df_cis(double y, dflt& c, dflt& sn) {
  const double qd = rint(y * 0.6366197723675814);
  double r = fma(-qd, 1.5707963267341256, y);
  r = fma(-qd, 6.077100506303966e-11, r);
  r = fma(-qd, 2.0222662487959506e-21, r);
  const dflt rd = df_of(r), sq = df_mul(rd, rd);
  const dflt ms = df_neg(sq);
  dflt ps = inv_fact(17), pc = inv_fact(16);
#pragma unroll
  for (int j = 7; j >= 0; --j) {
    ps = df_add(df_mul(ps, ms), inv_fact(2 * j + 1));
    pc = df_add(df_mul(pc, ms), inv_fact(2 * j));
  }
  const dflt sv = df_mul(ps, rd);
  const int qm = (int)((long long)qd & 3);
  c = (qm == 0) ? pc : ((qm == 1) ? df_neg(sv) : ((qm == 2) ? df_neg(pc) : sv));
  sn = (qm == 0) ? sv : ((qm == 1) ? pc : ((qm == 2) ? df_neg(sv) : df_neg(pc)));
}

// Fast FP64 reciprocal: PTX rcp.approx seed + two Newton steps (<= 1 ulp).
__device__ __forceinline__ double rcp_fast(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  return r;
}

// ---------------------------------------------------------------------------
// Resonance geometry of order nn at omega (determine_resonances,
// src/ALPS_fns.f90:641-745, and the index logic of integrate_res, :870-1000).
// ---------------------------------------------------------------------------
struct ResGeom {
  int res;          // resonance flag of determine_resonances
  int kind;         // 0 plain, 1 early "integrate(ipar_res+M_I, npar-1)",
                    // 2 early "integrate(1, ipar_res-M_I)", 3 principal value
  int lo1, hi1, lo2, hi2;   // j ranges of the trapezoid pole sums
  int ipar_res, lower, upper;
  double pr, pi;    // complex resonance momentum
};

__device__ inline double pres_real(const SpecDev& S, double omr, int nn, double kpar) {
  return __ddiv_rn(__dsub_rn(__dmul_rn(S.ms, omr), __dmul_rn((double)nn, S.qs)), kpar);
}

__device__ inline ResGeom res_geometry(const SpecDev& S, int M_I, double2 om, int nn, double kpar) {
  ResGeom g;
  const double* pp = S.ppar;
  int M = S.M;
  double x = pres_real(S, om.x, nn, kpar);
  g.pr = x;
  g.pi = __ddiv_rn(__dmul_rn(S.ms, om.y), kpar);
  double dpp = S.dppar;
  double mi_dpp = __dmul_rn((double)M_I, dpp);
  bool res = (pp[1] <= x) && (x < pp[M]);
  if ((x < pp[1]) && (x >= __dsub_rn(pp[1], mi_dpp))) res = true;
  if ((x >= pp[M - 1]) && (x < __dadd_rn(pp[M - 1], mi_dpp))) res = true;
  g.res = res;
  g.lo2 = 1;
  g.hi2 = 0;
  g.ipar_res = 0;
  g.lower = g.upper = 0;
  if (!res) {
    g.kind = 0;
    g.lo1 = 1;
    g.hi1 = M - 1;
    return g;
  }
  int ipar_res = 0;
  if ((x >= pp[1]) && (x < pp[M - 1])) {
    // largest i in [1, M-2] with pp[i] <= x: the uniform grid gives the
    // index to within one, and the comparisons settle it
    int i = 1 + (int)floor((x - pp[1]) * S.idppar);
    i = (i < 1) ? 1 : ((i > M - 2) ? M - 2 : i);
    while (i < M - 2 && pp[i + 1] <= x) ++i;
    while (i > 1 && pp[i] > x) --i;
    ipar_res = i;
  }
  for (int ip = 0; ip <= M_I; ++ip) {
    if ((x >= __dsub_rn(pp[0], __dmul_rn(dpp, (double)ip))) &&
        (x < __dsub_rn(pp[0], __dmul_rn(dpp, (double)(ip - 1)))))
      ipar_res = -ip;
    if ((x >= __dadd_rn(pp[M - 1], __dmul_rn(dpp, (double)ip))) &&
        (x < __dadd_rn(pp[M - 1], __dmul_rn(dpp, (double)(ip + 1)))))
      ipar_res = M - 1 + ip;
  }
  g.ipar_res = ipar_res;
  if ((ipar_res - M_I) <= 2) {
    g.kind = 1;
    g.lo1 = ipar_res + M_I;
    g.hi1 = M - 1;
    return g;
  }
  if ((ipar_res + M_I) >= (M - 2)) {
    g.kind = 2;
    g.lo1 = 1;
    g.hi1 = ipar_res - M_I;
    return g;
  }
  g.kind = 3;
  g.lower = ipar_res - M_I;
  if (fabs(__dsub_rn(x, pp[ipar_res])) < __dmul_rn(0.5, dpp)) g.upper = ipar_res + M_I + 1;
  else g.upper = ipar_res + M_I + 2;
  g.lo1 = 1;
  g.hi1 = g.lower;
  g.lo2 = g.upper;
  g.hi2 = M - 1;
  return g;
}

// Prefactors of the T-tensor entries (int_T, src/ALPS_fns.f90:1601-1707)
// after the Bessel and momentum factors have been moved into the reduced
// vectors.  Entry order: xx, yy, zz, xy, xz, yz.
__device__ inline void t_prefactors(int nn, double z, double kperp, int kperp_norm, double2 pref[6]) {
  double dn = (double)nn;
  double k2 = kperp_norm ? 1.0 : kperp * kperp;
  double k1 = kperp_norm ? 1.0 : kperp;
  pref[0] = cmk(dn * dn / (z * z), 0.0);
  pref[1] = cmk(k2, 0.0);
  pref[2] = cmk(k2, 0.0);
  pref[3] = cmk(0.0, k1 * dn / z);
  pref[4] = cmk(k1 * dn / z, 0.0);
  pref[5] = cmk(0.0, -k2);
}

// C0 v_e(n) of the order-fused tables: C0 times the nonzero part of
// prefactor e of order n >= 0 (imaginary for xy and yz, else real)
__device__ __forceinline__ double fused_factor(int n, int e, double z, double kperp, int kperp_norm, double C0) {
  double2 pref[6];
  t_prefactors(n, z, kperp, kperp_norm, pref);
  return C0 * ((e == 3 || e == 5) ? pref[e].y : pref[e].x);
}
