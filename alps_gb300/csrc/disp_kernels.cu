// disp_kernels.cu -- the omega pass: det D(omega, k) for a batch of
// frequencies (disp, src/ALPS_fns.f90:252-636).
//
// For fixed k the reference's double loop
//     sum_{i,j} w_i w_j resU(i,j) int_T(n,i,j,mode)
// factorises: resU's denominator depends on ppar_j only and its numerator is
// linear in omega, so the p_perp sum was done once per k into the reduced
// vectors V[n][j][12] (setup_kernels.cu).  What is left per omega is a 1-D
// pole sum over ppar per Bessel order:
//     S_{e,g}(n) = sum_j (w_j/2) V_{e,g}(n,j) / (m omega - k_par ppar_j - n q)
// plus, for resonant orders, the principal-value window and the Landau term.
//
// Kernels of one batch (launched on one stream, in this order), each over
// a table of jobs (one per context; a lone batch is one job):
//   k_stage             a lone batch's arguments and job to device memory
//   k_classify_multi    resonant orders of each (omega, species) into
//                       fixed slots, one warp per (omega, species)
//   k_pole_sums_multi   the pole sums over all orders: order chunks x omega
//                       tiles x node slices.  Plain path in FP64; fast path
//                       (pole_fused) in double-float on the FP32 pipes, all
//                       orders of a chunk in one set of sums
//   k_resonant_multi    principal value + Landau per resonant (omega,
//                       species, n): occupied slots gathered into batches
//                       of 32; scalar work one item per lane, vector work
//                       one item per warp (fast path: pv_fast, double-float)
//   k_finalize_multi    chi, epsilon, wave tensor and det, one thread (or
//                       warp) per omega; sums in a fixed order, so results
//                       do not depend on timing or on the other jobs.
//
// Double-float (fast path): a value is a pair of floats h + l (about 46-48
// bits) handled with error-free transformations (device_math.cuh); GB300
// runs FP32 at 64 times its FP64 rate.  Resonance decisions, windows and
// sample points are the reference's on both paths.
#include <algorithm>
#include <array>
#include <atomic>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>

#include "alps_internal.cuh"
#include "device_math.cuh"

// what the kernels read of one context (the plasma at its current k)
struct __align__(16) DispArgs {
  SysDev sys;
  SpecDev sp[ALPS_MAX_SPECIES];
  int rcap;      // max resonant slots over species
  int relcap;    // order slots per relativistic species (max nmax + 1), 0 if none
  int has_bm;    // some species go through the NHDS closed form
};

// the shape of one batch: the order chunks of the pole sums and the items
// per warp of k_resonant.  It follows from the batch size and the context
// alone, so a batch sums in the same order wherever it runs.
struct DispShape {
  int nchunk;    // order chunks per species
  int csize;     // orders per chunk
  int ipw;       // resonant-item slots per warp of k_resonant (1..256)
};

namespace {

// ---------------------------------------------------------------------------
// One warp per (omega, species): the lanes test the orders -nmax..nmax
// and a ballot prefix gives every resonant order its slot in increasing nn,
// so the slot order does not depend on the launch shape.
__device__ __forceinline__ void classify_body(const DispArgs& a, const double2* __restrict__ om, int n_om,
                                              int* count, int* slot_nn, int* flags, long wid) {
  const int lane = threadIdx.x & 31;
  const int S_ = a.sys.nspec;
  if (wid >= (long)n_om * S_) return;
  const int t = (int)(wid / S_), s = (int)(wid % S_);
  const SpecDev& S = a.sp[s];
  if (S.relat || S.bm) {  // relativistic orders run in k_rel_orders, NHDS species in k_nhds
    if (lane == 0) count[(size_t)t * S_ + s] = 0;
    return;
  }
  const double2 o = om[t];
  int* slots = slot_nn + ((size_t)t * S_ + s) * a.rcap;
  int cnt = 0;
  const float ikp32 = (float)a.sys.ikpar;
  for (int base = -S.nmax; base <= S.nmax; base += 32) {
    const int nn = base + lane;
    bool res = false;
    if (nn <= S.nmax) {
      // an FP32 estimate of Re p_res settles the orders clearly outside or
      // inside the resonance interval (its bounds carry a margin of 1e-5 of
      // its extent, the estimate's error is below 2^-22 |p|); the FP64 test
      // decides near the interval's ends
      const float x32 = (float)(S.ms * o.x - (double)nn * S.qs) * ikp32;
      const float mg = 9.5367431640625e-7f * fabsf(x32);
      if (x32 < S.qlo - mg || x32 > S.qhi + mg) res = false;
      else if (x32 > S.qlo_in + mg && x32 < S.qhi_in - mg) res = true;
      else res = res_geometry(S, a.sys.M_I, o, nn, a.sys.kpar).res;
    }
    const unsigned m = __ballot_sync(0xffffffffu, res);
    const int at = cnt + __popc(m & ((1u << lane) - 1u));
    if (res && at < a.rcap) slots[at] = nn;
    cnt += __popc(m);
  }
  if (lane == 0) {
    if (cnt > a.rcap) {
      atomicOr(flags, 1);
      cnt = a.rcap;
    }
    count[(size_t)t * S_ + s] = cnt;
  }
}

// ---------------------------------------------------------------------------
// Pole sums.  Block = TW omegas x JS slices of j.  grid = (omega tiles,
// species, order chunks).  Each thread accumulates the six chi entries of its
// omega over the orders of its chunk (and the n = -1,0,1 parts for chi_low).
// ---------------------------------------------------------------------------
// Complex double-float helpers of the order-fused pole sums
__device__ __forceinline__ void df_cmul2(dflt ax, dflt ay, dflt bx, dflt by, dflt& rx, dflt& ry) {
  const dflt x = df_add(df_mul(ax, bx), df_neg(df_mul(ay, by)));
  ry = df_add(df_mul(ax, by), df_mul(ay, bx));
  rx = x;
}

// complex double-float values and the combinations of the base sums
struct cdf {
  dflt x, y;
};
__device__ __forceinline__ cdf cdf_mul(cdf a, cdf b) {
  cdf r;
  df_cmul2(a.x, a.y, b.x, b.y, r.x, r.y);
  return r;
}
__device__ __forceinline__ cdf cdf_add(cdf a, cdf b) { return {df_add(a.x, b.x), df_add(a.y, b.y)}; }
__device__ __forceinline__ cdf cdf_rmul(cdf a, dflt s) { return {df_mul(a.x, s), df_mul(a.y, s)}; }
// omega v1 + kappa v2 (v1, v2 complex)
__device__ __forceinline__ cdf om_comb(cdf o, dflt kap, cdf v1, cdf v2) {
  const cdf r = cdf_mul(o, v1);
  return {df_add(r.x, df_mul(kap, v2.x)), df_add(r.y, df_mul(kap, v2.y))};
}
// omega c1 + kappa c2 (c1, c2 real)
__device__ __forceinline__ cdf om_combr(cdf o, dflt kap, dflt c1, dflt c2) {
  return {df_add(df_mul(o.x, c1), df_mul(kap, c2)), df_mul(o.y, c1)};
}

// ---------------------------------------------------------------------------
// Fast path of the pole sums (no chi_low), on the base tables: per (omega,
// signed order) the sums of the three Bessel families against g1 and g2
// (6 real vectors, complex weights), in double-float on the FP32 pipes:
//   * node sums Q = sum_j w_j F_j R_j, R_j = 1/(A - k_par p_j + i D), the
//     p_par-weighted entries from zeta Q - (1/k_par) sum w F (the sums of
//     the family vectors over the summed ranges: full-range table, or FP64
//     prefix sums where a resonance window is cut out);
//   * far poles: the Laurent series Q = f sum_k mom_k t^k, d = p_res - pcen,
//     t = prad/d, f = 1/(k_par d); with T = f sum_{k>=1}, U = f sum_{k>=2}:
//     sum F p R = pcen Q + d T, sum F p^2 R = pcen^2 Q + 2 pcen d T + d^2 U
//     (no cancellation for far poles); the terms from K32 on in FP32.
// An FP32 test settles orders far from resonance (the FP64 geometry decides
// the rest).  Each order's entries X_e = omega S_{e,1} + kappa S_{e,2} are
// added, times the order factor C0 v_e(n) (sign of -n for xy, xz), to one
// double-float sum per entry; the phase (i for xy, yz) and the entry scale
// are applied once per chunk in FP64.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pole_fused(const SysDev& sys, const SpecDev& S, double2 o, int js, int js_count,
                                           int n_begin, int n_end, double2* acc_out) {
  const int M = S.M;
  const double kpar = sys.kpar;
  dflt acc[12];
#pragma unroll
  for (int q = 0; q < 12; ++q) acc[q] = {0.0f, 0.0f};
  const dflt oxd = df_of(o.x), oyd = df_of(o.y), msd = df_of(S.ms), qsd = df_of(S.qs);
  const cdf omd = {oxd, oyd};
  const dflt kap = {S.kaph, S.kapl};
  const dflt kd = df_of(kpar), ikd = df_of(sys.ikpar), pcd = df_of(S.pcen), prd = df_of(S.prad);
  const dflt Dd = df_mul(msd, oyd);  // m omega_i
  const dflt D2 = df_mul(Dd, Dd);
  const dflt dyd = df_mul(Dd, ikd);  // Im p_res
  const dflt mox = df_mul(msd, oxd);
  const float ikp32 = (float)sys.ikpar;
  const int k0 = (js >= 2) ? js : js + js_count * ((2 - js + js_count - 1) / js_count);  // first k >= 2
  for (int n = n_begin; n < n_end; ++n) {
    const float* __restrict__ Bn = S.Bt + (size_t)n * (M - 1) * 12;
    const float* __restrict__ mBn = S.mBt + (size_t)n * ALPS_KFAR * 12;
    for (int sg = 0; sg < (n == 0 ? 1 : 2); ++sg) {
      const int nn = sg ? -n : n;
      // A = m omega_r - nn q, the pole's real part times k_par
      const dflt Ad = df_add(mox, df_neg(df_mul({(float)nn, 0.0f}, qsd)));
      const float x32 = Ad.h * ikp32;
      const float mg = 9.5367431640625e-7f * fabsf(x32);  // 2^-20 |x|
      ResGeom g;
      float ddf;  // |p_res - pcen|^2 (in FP32 alone for orders far from resonance)
      if (x32 < S.qlo - mg || x32 > S.qhi + mg) {
        g.res = 0;
        g.lo1 = 1;
        g.hi1 = M - 1;
        g.lo2 = 1;
        g.hi2 = 0;
        const float dx = x32 - S.pcen32;
        ddf = fmaf(dx, dx, dyd.h * dyd.h);
      } else {
        g = res_geometry(S, sys.M_I, o, nn, kpar);
        const double2 dfar = cmk(g.pr - S.pcen, g.pi);
        ddf = (float)(dfar.x * dfar.x + dfar.y * dfar.y);
      }
      int K = S.kfar + 1, K32 = K;
      // the series is used up to rho^2 < 0.58, where its K <= kfar terms
      // (checked below) cost less than the node sum
      if (!g.res && S.prad32 * S.prad32 < 0.58f * ddf) {
        const float rho = S.prad32 * rsqrtf(ddf);
        const float lr = -__logf(rho), l1 = log1pf(-rho);
        K = (int)ceilf((36.7368006f - l1) / lr) + 1;    // 53 ln 2
        K32 = (int)ceilf((22.8738570f - l1) / lr) + 1;  // 33 ln 2
      }
      // the double-float values stay normal floats: |f| = 1/(k_par |d|) for
      // the series, |A - k_par p_j|^2 + D^2 at the summed ranges' ends for
      // the node sum (zero if the pole lies inside a summed range)
      if (K <= S.kfar) {
        const float fm = fabsf(ikp32) * rsqrtf(ddf);
        if (!(fm >= 1e-30f && fm <= 1e30f)) K = K32 = S.kfar + 1;
      }
      bool nodes_df = true;
      if (K > S.kfar) {
        float lo = 3.0e38f, hi = 0.0f;
        const int ends[4] = {g.lo1, g.hi1, g.lo2, g.hi2};
        for (int r2 = 0; r2 < 2; ++r2) {
          const int j0 = max(1, ends[2 * r2]), j1 = min(M - 1, ends[2 * r2 + 1]);
          if (j0 > j1) continue;
          const float d0 = Ad.h - kd.h * S.pph[j0], d1 = Ad.h - kd.h * S.pph[j1];
          lo = ((d0 < 0.0f) != (d1 < 0.0f)) ? 0.0f : fminf(lo, fminf(fabsf(d0), fabsf(d1)));
          hi = fmaxf(hi, fmaxf(fabsf(d0), fabsf(d1)));
        }
        const float d2 = D2.h;
        nodes_df = d2 + lo * lo >= 1e-30f && d2 + hi * hi <= 1e30f;
      }
      cdf X[6];  // the order's entries (xx yy zz xy xz yz), scaled by 1/Vscale[n]
      if (K > S.kfar && !nodes_df) {
        // FP64 node sum of this order over V, X_e = omega S_e1 + kappa S_e2
        const double* __restrict__ Vn = S.V + (size_t)n * (M - 1) * 12;
        const double Ar = S.ms * o.x - (double)nn * S.qs, Di = S.ms * o.y;
        double2 Sx[12];
#pragma unroll
        for (int q = 0; q < 12; ++q) Sx[q] = cmk(0.0, 0.0);
        auto nd = [&](int j, double wgt) {
          const double dr = fma(-kpar, S.ppar[j], Ar);
          const double rr = wgt / fma(dr, dr, Di * Di);
          const double* v = Vn + (size_t)(j - 1) * 12;
#pragma unroll
          for (int q = 0; q < 12; ++q) {
            Sx[q].x = fma(v[q], dr * rr, Sx[q].x);
            Sx[q].y = fma(v[q], -Di * rr, Sx[q].y);
          }
        };
        for (int j = 1 + js; j <= M - 1; j += js_count)
          if ((j >= g.lo1 && j <= g.hi1) || (j >= g.lo2 && j <= g.hi2)) nd(j, 1.0);
        const int ends[4] = {g.lo1, g.hi1, g.lo2, g.hi2};
        for (int r2 = 0; r2 < 2; ++r2) {
          const int lo = ends[2 * r2], hi = ends[2 * r2 + 1];
          if (lo >= hi) continue;
          for (int side = 0; side < 2; ++side) {
            const int j = side ? hi : lo;
            if (j >= 1 && j <= M - 1 && ((j - 1) % js_count) == js) nd(j, -0.5);
          }
        }
        const double isc = 1.0 / S.Vscale[n], kapd = S.kappa;
#pragma unroll
        for (int e = 0; e < 6; ++e) {
          const double2 t = cscale(cadd(cmul(o, Sx[2 * e]), cscale(Sx[2 * e + 1], kapd)), isc);
          X[e] = {df_of(t.x), df_of(t.y)};
        }
      } else if (K <= S.kfar) {
        // Laurent series: d = p_res - pcen, t = prad/d, f = 1/(k_par d)
        const cdf d = {df_add(df_mul(Ad, ikd), df_neg(pcd)), dyd};
        const dflt r = df_rcp_approx(df_add(df_mul(d.x, d.x), df_mul(d.y, d.y)));
        const cdf iv = {df_mul(d.x, r), df_neg(df_mul(d.y, r))};
        const cdf t1 = cdf_rmul(iv, prd), f = cdf_rmul(iv, ikd);
        // U = f sum_{k >= 2} mom_k t^k over this slice's k: powers from f t^k0,
        // step t^js_count (both by squaring)
        cdf tp = f, st = t1;
        {
          cdf pw = t1;
          for (int q = k0; q; q >>= 1) {
            if (q & 1) tp = cdf_mul(tp, pw);
            pw = cdf_mul(pw, pw);
          }
          for (int q = js_count; q > 1; q >>= 1) st = cdf_mul(st, st);
        }
        dflt U[12];
        float Uf[12];
#pragma unroll
        for (int q = 0; q < 12; ++q) {
          U[q] = {0.0f, 0.0f};
          Uf[q] = 0.0f;
        }
        int k = k0;
        for (; k < K32; k += js_count) {
          const float4* m4 = reinterpret_cast<const float4*>(mBn + (size_t)k * 12);
          const float4 a0 = __ldg(m4), a1 = __ldg(m4 + 1), a2 = __ldg(m4 + 2);
          const float hb[6] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y}, lb[6] = {a1.z, a1.w, a2.x, a2.y, a2.z, a2.w};
#pragma unroll
          for (int b = 0; b < 6; ++b) {
            df_mac(U[2 * b], hb[b], lb[b], tp.x);
            df_mac(U[2 * b + 1], hb[b], lb[b], tp.y);
          }
          tp = cdf_mul(tp, st);
        }
        if (k < K) {
          // the tail: terms below 2^-33 of the bound, in FP32
          float fx = tp.x.h + tp.x.l, fy = tp.y.h + tp.y.l;
          const float gx = st.x.h + st.x.l, gy = st.y.h + st.y.l;
          for (; k < K; k += js_count) {
            const float4* m4 = reinterpret_cast<const float4*>(mBn + (size_t)k * 12);
            const float4 a0 = __ldg(m4);
            const float2 a1 = __ldg(reinterpret_cast<const float2*>(m4 + 1));
            const float hb[6] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y};
#pragma unroll
            for (int b = 0; b < 6; ++b) {
              Uf[2 * b] = fmaf(hb[b], fx, Uf[2 * b]);
              Uf[2 * b + 1] = fmaf(hb[b], fy, Uf[2 * b + 1]);
            }
            const float nx = fx * gx - fy * gy;
            fy = fx * gy + fy * gx;
            fx = nx;
          }
        }
        // per family F1, F2, F3: omega U_{F,g1} + kappa U_{F,g2}
        cdf Uw[3];
#pragma unroll
        for (int fm = 0; fm < 3; ++fm) {
          const int b1 = 2 * fm, b2 = 2 * fm + 1;
          const cdf u1 = {df_add(U[2 * b1], {Uf[2 * b1], 0.0f}), df_add(U[2 * b1 + 1], {Uf[2 * b1 + 1], 0.0f})};
          const cdf u2 = {df_add(U[2 * b2], {Uf[2 * b2], 0.0f}), df_add(U[2 * b2 + 1], {Uf[2 * b2 + 1], 0.0f})};
          Uw[fm] = om_comb(omd, kap, u1, u2);
        }
        // T = f mom_1 t + U, Q = f mom_0 + T on the slices that own k = 1, 0
        cdf T[3] = {Uw[0], Uw[1], Uw[2]};
        auto mterm = [&](int kk, cdf w, cdf* out) {
          const float* m = mBn + (size_t)kk * 12;
#pragma unroll
          for (int fm = 0; fm < 3; ++fm) {
            const cdf mw = om_combr(omd, kap, {m[2 * fm], m[6 + 2 * fm]}, {m[2 * fm + 1], m[6 + 2 * fm + 1]});
            out[fm] = cdf_add(out[fm], cdf_mul(w, mw));
          }
        };
        if (js == 1 % js_count) mterm(1, cdf_mul(f, t1), T);
        cdf Q[3] = {T[0], T[1], T[2]};
        if (js == 0) mterm(0, f, Q);
        X[0] = Q[0];
        X[1] = Q[1];
        X[3] = Q[2];
        X[4] = cdf_mul(d, T[0]);
        X[5] = cdf_mul(d, T[2]);
        if (S.pcen32 != 0.0f) {
          // sum F p R = pcen Q + d T, sum F p^2 R = pcen (sum F p R) + d (pcen T + d U)
          X[4] = cdf_add(cdf_rmul(Q[0], pcd), X[4]);
          X[5] = cdf_add(cdf_rmul(Q[2], pcd), X[5]);
          X[2] = cdf_add(cdf_rmul(X[4], pcd), cdf_mul(d, cdf_add(cdf_rmul(T[0], pcd), cdf_mul(d, Uw[0]))));
        } else {
          X[2] = cdf_mul(d, cdf_mul(d, Uw[0]));
        }
      } else {
        // node sum in double-float: Q_b = sum_j w_j B_b(j) / (A - k_par p_j + i D)
        dflt Qs[12];
#pragma unroll
        for (int q = 0; q < 12; ++q) Qs[q] = {0.0f, 0.0f};
        // node j's terms; the trapezoid ends enter again at weight -1/2
        auto node = [&](int j, bool end) {
          const dflt dr = df_add(Ad, df_neg(df_mul(kd, {S.pph[j], S.ppl[j]})));
          const dflt r = df_rcp_approx(df_add(df_mul(dr, dr), D2));
          dflt Rr = df_mul(dr, r), Ri = df_neg(df_mul(Dd, r));
          if (end) {
            Rr = df_scale(Rr, -0.5f);
            Ri = df_scale(Ri, -0.5f);
          }
          const float4* b4 = reinterpret_cast<const float4*>(Bn + (size_t)(j - 1) * 12);
          const float4 a0 = __ldg(b4), a1 = __ldg(b4 + 1), a2 = __ldg(b4 + 2);
          const float hb[6] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y}, lb[6] = {a1.z, a1.w, a2.x, a2.y, a2.z, a2.w};
#pragma unroll
          for (int b = 0; b < 6; ++b) {
            df_mac(Qs[2 * b], hb[b], lb[b], Rr);
            df_mac(Qs[2 * b + 1], hb[b], lb[b], Ri);
          }
        };
        const int ends[4] = {g.lo1, g.hi1, g.lo2, g.hi2};
        // the summed ranges (disjoint), each over this slice's nodes
        // j = 1 + js (mod js_count)
#pragma unroll
        for (int r2 = 0; r2 < 2; ++r2) {
          const int lo = max(1, ends[2 * r2]), hi = min(M - 1, ends[2 * r2 + 1]);
          const int j0 = lo + (((js - (lo - 1)) % js_count) + js_count) % js_count;
          for (int j = j0; j <= hi; j += js_count) node(j, false);
        }
        // trapezoid end weights
#pragma unroll
        for (int r2 = 0; r2 < 2; ++r2) {
          const int lo = ends[2 * r2], hi = ends[2 * r2 + 1];
          if (lo >= hi) continue;
#pragma unroll
          for (int side = 0; side < 2; ++side) {
            const int j = side ? hi : lo;
            if (j >= 1 && j <= M - 1 && ((j - 1) % js_count) == js) node(j, true);
          }
        }
        cdf P[3];
#pragma unroll
        for (int fm = 0; fm < 3; ++fm)
          P[fm] = om_comb(omd, kap, {Qs[4 * fm], Qs[4 * fm + 1]}, {Qs[4 * fm + 2], Qs[4 * fm + 3]});
        const cdf zeta = {df_mul(Ad, ikd), dyd};
        X[0] = P[0];
        X[1] = P[1];
        X[3] = P[2];
        cdf xz = cdf_mul(zeta, P[0]), yz = cdf_mul(zeta, P[2]);
        cdf cp = {{0.0f, 0.0f}, {0.0f, 0.0f}};
        if (js == 0) {
          // (1/k_par) times the omega-combined sums of F1, F3 and p_par F1
          // over the summed ranges (slice 0 adds them once)
          double C[6];
          const double* __restrict__ Cf = S.Cfull + (size_t)n * 6;
          if (!g.res) {
#pragma unroll
            for (int c = 0; c < 6; ++c) C[c] = Cf[c];
          } else {
            const double* __restrict__ P0 = S.Pre + (size_t)n * M * 6;
            const double* __restrict__ Vn = S.V + (size_t)n * (M - 1) * 12;
            const double isc = 1.0 / S.Vscale[n];
#pragma unroll
            for (int c = 0; c < 6; ++c) C[c] = 0.0;
            for (int r2 = 0; r2 < 2; ++r2) {
              const int lo = max(1, ends[2 * r2]), hi = min(M - 1, ends[2 * r2 + 1]);
              if (lo > hi) continue;
              const bool trap = ends[2 * r2] < ends[2 * r2 + 1];
#pragma unroll
              for (int c = 0; c < 6; ++c) {
                const int q = (c < 2) ? c : c + 4;
                double v = P0[(size_t)hi * 6 + c] - P0[(size_t)(lo - 1) * 6 + c];
                if (trap) v -= 0.5 * (Vn[(size_t)(lo - 1) * 12 + q] + Vn[(size_t)(hi - 1) * 12 + q]) * isc;
                C[c] += v;
              }
            }
          }
          const dflt ik = ikd;
          const cdf c1 = cdf_rmul(om_combr(omd, kap, df_of(C[0]), df_of(C[1])), ik);
          const cdf c3 = cdf_rmul(om_combr(omd, kap, df_of(C[2]), df_of(C[3])), ik);
          cp = cdf_rmul(om_combr(omd, kap, df_of(C[4]), df_of(C[5])), ik);
          xz = {df_add(xz.x, df_neg(c1.x)), df_add(xz.y, df_neg(c1.y))};
          yz = {df_add(yz.x, df_neg(c3.x)), df_add(yz.y, df_neg(c3.y))};
        }
        const cdf zz = cdf_mul(zeta, xz);
        X[2] = {df_add(zz.x, df_neg(cp.x)), df_add(zz.y, df_neg(cp.y))};
        X[4] = xz;
        X[5] = yz;
      }
      // add the order's entries with its factors C0 v_e(n) (xy and xz odd in n)
      const float* __restrict__ fac = S.bfac + (size_t)n * 12;
#pragma unroll
      for (int e = 0; e < 6; ++e) {
        dflt fe = {fac[2 * e], fac[2 * e + 1]};
        if (nn < 0 && (e == 3 || e == 4)) fe = df_neg(fe);
        df_acc(acc[2 * e], df_mul(fe, X[e].x));
        df_acc(acc[2 * e + 1], df_mul(fe, X[e].y));
      }
    }
  }
  // rescale and apply the phase (i for xy and yz)
#pragma unroll
  for (int e = 0; e < 6; ++e) {
    const double sc = S.Escale[e];
    const double2 t = cmk(df_val(acc[2 * e]) * sc, df_val(acc[2 * e + 1]) * sc);
    acc_out[e] = (e == 3 || e == 5) ? cmk(-t.y, t.x) : t;
  }
}

// The double-float node sum keeps |A - k_par p_j|^2 + D^2 a normal float:
// its smallest value (at a summed range's end, or zero if the pole lies
// inside a summed range) at least 1e-30, its largest at most 1e30.
__device__ __forceinline__ bool df_node_range(const SpecDev& S, const ResGeom& g, double Ar, double kpar,
                                              double Di) {
  double lo = 1e300, hi = 0.0;
  const int ends[4] = {g.lo1, g.hi1, g.lo2, g.hi2};
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int j0 = max(1, ends[2 * r]), j1 = min(S.M - 1, ends[2 * r + 1]);
    if (j0 > j1) continue;
    const double d0 = Ar - kpar * S.ppar[j0], d1 = Ar - kpar * S.ppar[j1];
    lo = ((d0 < 0.0) != (d1 < 0.0)) ? 0.0 : fmin(lo, fmin(fabs(d0), fabs(d1)));
    hi = fmax(hi, fmax(fabs(d0), fabs(d1)));
  }
  return Di * Di + lo * lo >= 1e-30 && Di * Di + hi * hi <= 1e30;
}

template <bool LOW>
__device__ __forceinline__ void pole_body(const SysDev& sys, const SpecDev& S, const DispShape& sh, const double2* __restrict__ om,
                                          int n_om, int js_count, double2* part, double2* low, int tile, int s,
                                          int chunk) {
  const int n_begin = chunk * sh.csize;
  const int n_end = (S.relat || S.bm) ? n_begin : min(S.nmax + 1, n_begin + sh.csize);
  // the js_count slices of an omega are adjacent threads, so an omega's
  // per-order set-up is one warp instruction for all its slices
  const int TW = blockDim.x / js_count;
  const int wl = threadIdx.x / js_count, js = threadIdx.x % js_count;
  const int w = tile * TW + wl;
  const bool active = (w < n_om);
  const double2 o = active ? om[w] : cmk(0.0, 0.0);
  const int M = S.M;
  const double kpar = sys.kpar;
  const double kappa = kpar / S.ms;
  const double C0 = 2.0 * ALPS_PI * S.dpperp * S.dppar_abs * 0.25 * S.qs;
  const double z = sys.kperp_norm ? sys.kperp / S.qs : 1.0 / S.qs;
  const double Di = S.ms * o.y;
  const double Di2 = Di * Di;
  const double* __restrict__ pp = S.ppar;
  double2 acc[6];
  double2 lacc[LOW ? 3 : 1][6];
#pragma unroll
  for (int e = 0; e < 6; ++e) {
    acc[e] = cmk(0.0, 0.0);
#pragma unroll
    for (int q = 0; q < (LOW ? 3 : 1); ++q) lacc[q][e] = cmk(0.0, 0.0);
  }
  if (active && !LOW && S.df_sums && S.Bt && n_end > n_begin) {
    pole_fused(sys, S, o, js, js_count, n_begin, n_end, acc);
  } else if (active) {
    for (int n = n_begin; n < n_end; ++n) {
      const double* __restrict__ Vn = S.V + (size_t)n * (M - 1) * 12;
      for (int sg = 0; sg < (n == 0 ? 1 : 2); ++sg) {
        const int nn = sg ? -n : n;
        ResGeom g = res_geometry(S, sys.M_I, o, nn, kpar);
        const double Ar = S.ms * o.x - (double)nn * S.qs;
        double2 Sx[12];
#pragma unroll
        for (int q = 0; q < 12; ++q) Sx[q] = cmk(0.0, 0.0);
        // Laurent series for a pole far outside the grid: truncation
        // rho^K <= 2^-53 (1 - rho), rho = prad/|p_res - pcen|.  With
        // |mom_k| <= sum_j |V_j|, the terms from K32 on (rho^K32 <= 2^-33
        // (1 - rho)) add at most 2^-33 of that bound, so they are summed in
        // FP32: their rounding stays below 2^-53 of it.
        int K = S.kfar + 1, K32 = K;
        double2 d = cmk(g.pr - S.pcen, g.pi);
        double dd = d.x * d.x + d.y * d.y;
        if (!g.res && S.prad * S.prad < 0.5 * dd) {
          // term counts from FP32 logarithms, one term added to each for
          // their rounding (rho < 0.71 here, so the counts are below 110)
          const float rho = (float)(S.prad * rsqrt(dd));
          const float lr = -__logf(rho), l1 = log1pf(-rho);
          K = (int)ceilf((36.7368006f - l1) / lr) + 1;    // 53 ln 2
          K32 = (int)ceilf((22.8738570f - l1) / lr) + 1;  // 33 ln 2
        }
        if (K <= S.kfar) {
          const double* __restrict__ mom = S.mom + (size_t)n * ALPS_KFAR * 12;
          double idd = 1.0 / dd;
          double2 inv = cmk(d.x * idd, -d.y * idd);
          double2 t = cscale(inv, S.prad);
          double2 tk = cmk(1.0, 0.0), step = t;
          // tk = t^js, step = t^js_count by squaring (js_count is a power of 2)
          double2 pw = t;
          for (int q = js; q; q >>= 1) {
            if (q & 1) tk = cmul(tk, pw);
            pw = cmul(pw, pw);
          }
          for (int q = js_count; q > 1; q >>= 1) step = cmul(step, step);
          int k = js;
          if (S.df_sums) {
            // fast path: the leading terms in double-float arithmetic on the
            // FP32 pipes (moments as pairs scaled by 2^-e per order)
            const float* __restrict__ mh = S.momh + (size_t)n * ALPS_KFAR * 12;
            const float* __restrict__ ml = S.moml + (size_t)n * ALPS_KFAR * 12;
            dflt tx = df_of(tk.x), ty = df_of(tk.y);
            const dflt sx = df_of(step.x), sy = df_of(step.y);
            dflt sacc[24];
#pragma unroll
            for (int q = 0; q < 24; ++q) sacc[q] = {0.0f, 0.0f};
            for (; k < K32; k += js_count) {
              const float4* h4 = reinterpret_cast<const float4*>(mh + (size_t)k * 12);
              const float4* l4 = reinterpret_cast<const float4*>(ml + (size_t)k * 12);
#pragma unroll
              for (int q = 0; q < 3; ++q) {
                const float4 h = __ldg(h4 + q), l = __ldg(l4 + q);
                df_mac(sacc[8 * q + 0], h.x, l.x, tx);
                df_mac(sacc[8 * q + 1], h.x, l.x, ty);
                df_mac(sacc[8 * q + 2], h.y, l.y, tx);
                df_mac(sacc[8 * q + 3], h.y, l.y, ty);
                df_mac(sacc[8 * q + 4], h.z, l.z, tx);
                df_mac(sacc[8 * q + 5], h.z, l.z, ty);
                df_mac(sacc[8 * q + 6], h.w, l.w, tx);
                df_mac(sacc[8 * q + 7], h.w, l.w, ty);
              }
              const dflt nx = df_add(df_mul(tx, sx), df_neg(df_mul(ty, sy)));
              ty = df_add(df_mul(tx, sy), df_mul(ty, sx));
              tx = nx;
            }
            const double sc = S.Vscale[n];
#pragma unroll
            for (int q = 0; q < 12; ++q) Sx[q] = cmk(df_val(sacc[2 * q]) * sc, df_val(sacc[2 * q + 1]) * sc);
            tk = cmk(df_val(tx), df_val(ty));
          }
          for (; k < K32; k += js_count) {
            const double2* m2 = reinterpret_cast<const double2*>(mom + (size_t)k * 12);
#pragma unroll
            for (int q = 0; q < 6; ++q) {
              double2 m = __ldg(m2 + q);
              Sx[2 * q].x = fma(m.x, tk.x, Sx[2 * q].x);
              Sx[2 * q].y = fma(m.x, tk.y, Sx[2 * q].y);
              Sx[2 * q + 1].x = fma(m.y, tk.x, Sx[2 * q + 1].x);
              Sx[2 * q + 1].y = fma(m.y, tk.y, Sx[2 * q + 1].y);
            }
            tk = cmul(tk, step);
          }
          if (k < K) {
            const float* __restrict__ momf = S.momf + (size_t)n * ALPS_KFAR * 12;
            float2 tf = make_float2((float)tk.x, (float)tk.y);
            const float2 sf = make_float2((float)step.x, (float)step.y);
            float2 Sf[12];
#pragma unroll
            for (int q = 0; q < 12; ++q) Sf[q] = make_float2(0.0f, 0.0f);
            for (; k < K; k += js_count) {
              const float4* m4 = reinterpret_cast<const float4*>(momf + (size_t)k * 12);
#pragma unroll
              for (int q = 0; q < 3; ++q) {
                const float4 m = __ldg(m4 + q);
                Sf[4 * q].x = fmaf(m.x, tf.x, Sf[4 * q].x);
                Sf[4 * q].y = fmaf(m.x, tf.y, Sf[4 * q].y);
                Sf[4 * q + 1].x = fmaf(m.y, tf.x, Sf[4 * q + 1].x);
                Sf[4 * q + 1].y = fmaf(m.y, tf.y, Sf[4 * q + 1].y);
                Sf[4 * q + 2].x = fmaf(m.z, tf.x, Sf[4 * q + 2].x);
                Sf[4 * q + 2].y = fmaf(m.z, tf.y, Sf[4 * q + 2].y);
                Sf[4 * q + 3].x = fmaf(m.w, tf.x, Sf[4 * q + 3].x);
                Sf[4 * q + 3].y = fmaf(m.w, tf.y, Sf[4 * q + 3].y);
              }
              tf = make_float2(tf.x * sf.x - tf.y * sf.y, tf.x * sf.y + tf.y * sf.x);
            }
#pragma unroll
            for (int q = 0; q < 12; ++q) {
              Sx[q].x += (double)Sf[q].x;
              Sx[q].y += (double)Sf[q].y;
            }
          }
          // S = (1/(k_par d)) sum_k mom_k t^k
          double2 f = cscale(inv, sys.ikpar);
#pragma unroll
          for (int q = 0; q < 12; ++q) Sx[q] = cmul(Sx[q], f);
        } else if (S.df_sums && df_node_range(S, g, Ar, kpar, Di)) {
          // fast path: the node sum in double-float arithmetic on the FP32
          // pipes (about 46 bits; V in pairs scaled by 2^-e per order)
          const float* __restrict__ Vh = S.Vh + (size_t)n * (M - 1) * 12;
          const float* __restrict__ Vl = S.Vl + (size_t)n * (M - 1) * 12;
          const dflt Ad = df_of(Ar), kd = df_of(kpar), Dd = df_of(Di);
          const dflt D2 = df_mul(Dd, Dd);
          dflt sacc[24];
#pragma unroll
          for (int q = 0; q < 24; ++q) sacc[q] = {0.0f, 0.0f};
          auto node = [&](int j, float wgt) {
            const dflt dr = df_add(Ad, df_neg(df_mul(kd, {S.pph[j], S.ppl[j]})));
            const dflt r = df_rcp_approx(df_add(df_mul(dr, dr), D2));
            const dflt Rr = df_scale(df_mul(dr, r), wgt), Ri = df_scale(df_neg(df_mul(Dd, r)), wgt);
            const float4* vh4 = reinterpret_cast<const float4*>(Vh + (size_t)(j - 1) * 12);
            const float4* vl4 = reinterpret_cast<const float4*>(Vl + (size_t)(j - 1) * 12);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
              const float4 h = __ldg(vh4 + q), l = __ldg(vl4 + q);
              df_mac(sacc[8 * q + 0], h.x, l.x, Rr);
              df_mac(sacc[8 * q + 1], h.x, l.x, Ri);
              df_mac(sacc[8 * q + 2], h.y, l.y, Rr);
              df_mac(sacc[8 * q + 3], h.y, l.y, Ri);
              df_mac(sacc[8 * q + 4], h.z, l.z, Rr);
              df_mac(sacc[8 * q + 5], h.z, l.z, Ri);
              df_mac(sacc[8 * q + 6], h.w, l.w, Rr);
              df_mac(sacc[8 * q + 7], h.w, l.w, Ri);
            }
          };
          for (int j = 1 + js; j <= M - 1; j += js_count) {
            bool in = (j >= g.lo1 && j <= g.hi1) || (j >= g.lo2 && j <= g.hi2);
            if (in) node(j, 1.0f);
          }
          // trapezoid end weights, as below
          int ends[4] = {g.lo1, g.hi1, g.lo2, g.hi2};
#pragma unroll
          for (int r2 = 0; r2 < 2; ++r2) {
            int lo = ends[2 * r2], hi = ends[2 * r2 + 1];
            if (lo >= hi) continue;
#pragma unroll
            for (int side = 0; side < 2; ++side) {
              int j = side ? hi : lo;
              if (((j - 1) % js_count) == js) node(j, -0.5f);
            }
          }
          const double sc = S.Vscale[n];
#pragma unroll
          for (int q = 0; q < 12; ++q) Sx[q] = cmk(df_val(sacc[2 * q]) * sc, df_val(sacc[2 * q + 1]) * sc);
        } else {
          for (int j = 1 + js; j <= M - 1; j += js_count) {
            bool in = (j >= g.lo1 && j <= g.hi1) || (j >= g.lo2 && j <= g.hi2);
            if (!in) continue;
            double dr = fma(-kpar, pp[j], Ar);
            double r = rcp_fast(fma(dr, dr, Di2));
            double Rr = dr * r, Ri = -Di * r;
            const double2* v2 = reinterpret_cast<const double2*>(Vn + (size_t)(j - 1) * 12);
#pragma unroll
            for (int q = 0; q < 6; ++q) {
              double2 v = __ldg(v2 + q);
              Sx[2 * q].x = fma(v.x, Rr, Sx[2 * q].x);
              Sx[2 * q].y = fma(v.x, Ri, Sx[2 * q].y);
              Sx[2 * q + 1].x = fma(v.y, Rr, Sx[2 * q + 1].x);
              Sx[2 * q + 1].y = fma(v.y, Ri, Sx[2 * q + 1].y);
            }
          }
          // trapezoid end weights: the range ends carry half weight unless the
          // range is a single node (integrate(a,a) weighs it fully)
          int ends[4] = {g.lo1, g.hi1, g.lo2, g.hi2};
#pragma unroll
          for (int r2 = 0; r2 < 2; ++r2) {
            int lo = ends[2 * r2], hi = ends[2 * r2 + 1];
            if (lo >= hi) continue;
#pragma unroll
            for (int side = 0; side < 2; ++side) {
              int j = side ? hi : lo;
              if (((j - 1) % js_count) != js) continue;
              double dr = fma(-kpar, pp[j], Ar);
              double r = rcp_fast(fma(dr, dr, Di2));
              double Rr = -0.5 * dr * r, Ri = 0.5 * Di * r;
              const double* v = Vn + (size_t)(j - 1) * 12;
#pragma unroll
              for (int q = 0; q < 12; ++q) {
                Sx[q].x = fma(v[q], Rr, Sx[q].x);
                Sx[q].y = fma(v[q], Ri, Sx[q].y);
              }
            }
          }
        }
        double2 pref[6];
        t_prefactors(nn, z, sys.kperp, sys.kperp_norm, pref);
#pragma unroll
        for (int e = 0; e < 6; ++e) {
          if (n == 0 && (e == 0 || e == 3 || e == 4)) continue;
          // integrate = C0 * pref * (omega S_e1 + kappa S_e2)
          double2 t1 = cadd(cmul(o, Sx[2 * e]), cscale(Sx[2 * e + 1], kappa));
          double2 val = cscale(cmul(pref[e], t1), C0);
          acc[e] = cadd(acc[e], val);
          if (LOW && nn >= -1 && nn <= 1) lacc[LOW ? nn + 1 : 0][e] = cadd(lacc[LOW ? nn + 1 : 0][e], val);
        }
      }
    }
  }
  // reduce over the j slices: they are adjacent lanes of one warp (js_count
  // divides 32), so a butterfly over the lane offsets below js_count
  auto slice_sum = [&](double2& v) {
    for (int off = js_count >> 1; off > 0; off >>= 1) {
      v.x += __shfl_xor_sync(0xffffffffu, v.x, off);
      v.y += __shfl_xor_sync(0xffffffffu, v.y, off);
    }
  };
  if (js_count > 1) {
    for (int e = 0; e < 6; ++e) slice_sum(acc[e]);
    if (LOW)
      for (int l = 0; l < 3; ++l)
        for (int e = 0; e < 6; ++e) slice_sum(lacc[LOW ? l : 0][e]);
  }
  if (js == 0 && active) {
    size_t base = ((size_t)w * sys.nspec + s) * sh.nchunk + chunk;
    for (int e = 0; e < 6; ++e) part[base * 6 + e] = acc[e];
    if (LOW)
      for (int l = 0; l < 3; ++l)
        for (int e = 0; e < 6; ++e) low[(base * 3 + l) * 6 + e] = lacc[LOW ? l : 0][e];
  }
}



// ---------------------------------------------------------------------------
// Analytic continuation f(pperp_i, complex ppar) (eval_fit,
// src/ALPS_analyt.f90:32-181; fit_function :185-266).
// ---------------------------------------------------------------------------
// fit_function_poly (src/ALPS_analyt.f90:268-363): Chebyshev series in
// t = (p - centre)/half-width, zero for |t| > 1; with log_fit the series is
// log10 f, cut to zero beyond +-poly_log_max
__device__ double2 eval_fit_poly(const SpecDev& S, int iperp, double2 p) {
  const int np = S.poly_order;
  const double* c = S.fit + (size_t)iperp * (np + 1);
  const double n1 = 5.0e-1 * (S.ppar_hi + S.ppar_lo), n2 = 5.0e-1 * (S.ppar_hi - S.ppar_lo);
  double2 t = cmk((p.x - n1) / n2, p.y / n2);
  if (cabs_(t) > 1.0) return cmk(0.0, 0.0);
  double2 b0 = cmk(1.0, 0.0), b1 = t;
  double2 f = cadd(cscale(b0, c[0]), cscale(b1, c[1]));
  for (int n = 2; n <= np; ++n) {
    double2 b2 = csub(cmul(cscale(t, 2.0), b1), b0);
    f = cadd(f, cscale(b2, c[n]));
    b0 = b1;
    b1 = b2;
  }
  if (S.log_fit) {
    const double L = S.poly_log_max;
    if ((f.x < -L) || (f.y < -L) || (f.x > L) || (f.y > L)) return cmk(0.0, 0.0);
    f = cexp_d(cscale(f, 2.302585092994045684));  // 10^f = exp(f ln 10)
  }
  return f;
}

__device__ double2 eval_fit_d(const SpecDev& S, double vA, int iperp, double2 p) {
  if (S.ac_method == 2) return eval_fit_poly(S, iperp, p);
  double pperp = S.pperp[iperp];
  if (S.ac_method == 0) {
    // distribution_analyt (distribution/distribution_analyt.f90:59-79)
    double ms;
    if (S.species_index == 1) ms = 1.0;
    else if (S.species_index == 2) ms = 1.0 / 1836.0;
    else return cmk(0.0, 0.0);
    double norm = pow(ALPS_PI, -1.5) / pow(ms * 1.0, 1.5);
    double2 p2 = cmul(p, p);
    double2 arg = cmk(-(p2.x / ms + (pperp * pperp) / ms), -(p2.y / ms));
    return cscale(cexp_d(arg), norm);
  }
  double2 ff = cmk(0.0, 0.0);
  const double* fit = S.fit;
  int nf = S.nf;
  for (int f = 0; f < nf; ++f) {
    int t = S.fit_type[f];
    double pc = S.perp_corr[f];
    auto P = [&](int k) { return fit[(iperp * 5 + k) * nf + f]; };
    double2 d = csub(p, cmk(P(2), 0.0));
    double2 d2 = cmul(d, d);
    if (t == 1) {
      double a0 = P(0) * exp(-pc * (pperp * pperp));
      ff = cadd(ff, cscale(cexp_d(cscale(d2, -P(1))), a0));
    } else if (t == 2) {
      double2 kp = cadd(cmk(1.0 + pc * P(4) * (pperp * pperp), 0.0), cscale(d2, P(1)));
      kp = cadd(cmk(1.0, 0.0), cadd(cscale(d2, P(1)), cmk(pc * P(4) * (pperp * pperp), 0.0)));
      ff = cadd(ff, cscale(cexp_d(cscale(clog_d(kp), P(3))), P(0)));
    } else if (t == 3) {
      double2 in = cadd(cmk(1.0, 0.0), cscale(cadd(cmk(pperp * pperp, 0.0), d2), vA * vA / (S.ms * S.ms)));
      double2 sq = csqrt_d(in);
      ff = cadd(ff, cscale(cexp_d(cscale(sq, -P(1))), P(0)));
    } else if (t == 6) {
      double2 q = cadd(cmk(P(3) * pc * (pperp * pperp), 0.0), cscale(d2, P(1)));
      double2 arg = cscale(csub(q, cexp_d(q)), 0.5);
      ff = cadd(ff, cscale(cexp_d(arg), P(0)));
    }
  }
  return ff;
}

// h_e(j) = omega V_{e,1}(j) + kappa V_{e,2}(j)
__device__ inline double2 h_node(const double* Vn, int j, int e, double2 o, double kappa) {
  const double* v = Vn + (size_t)(j - 1) * 12 + 2 * e;
  return cmk(o.x * v[0] + kappa * v[1], o.y * v[0]);
}

// ---------------------------------------------------------------------------
// Resonant items: the principal-value part of integrate_res
// (src/ALPS_fns.f90:1000-1236) and landau_integrate (:1327-1452) for one
// (omega, species, n).  One warp per item.
//
// Principal value: summed over iperp, funct_g (:1243-1321) is the linear
// interpolation H_e(p) = h_e(jc) + s_e(jc) (p - ppar_jc) on the node values
// h_e(j) = omega V_{e,1}(j) + kappa V_{e,2}(j) with the centred slope
// s_e(j) = (h_e(j+1) - h_e(j-1)) / (2 dppar); both are staged per window node
// in shared memory.  Landau: for Maxwellian fit terms the three continuation
// values a row needs share one Gaussian, exp(-p2 (d +- D)^2) =
// exp(-p2 d^2) exp(-+2 p2 D d) exp(-p2 D^2), so a row costs two complex
// exponentials; the omega-independent factors come from k_fit_aux.
// ---------------------------------------------------------------------------
#define RES_WARPS 4
#define RES_WIN 32  // largest node window staged in shared memory
// principal-value piece records per warp, in double2: (group, lane, slot)
// sums A, B; run sums A, B; then the int tables (group, lane, slot) piece
// and run start lane, slot, group, piece
#define PV_GROUPS 3
#define PV_RECV (PV_GROUPS * 32 * 2 * 2)
#define PV_RUNV (32 * 2)
#define PV_INTS (PV_GROUPS * 64 + 4 * 32)
#define PV_SMEM (PV_RECV + PV_RUNV + (PV_INTS + 3) / 4)
// record planes: sum ab (0 A, 1 B) of slot sl of (group gi, lane L); lanes
// are adjacent within a plane, so a warp's record stores and loads touch
// consecutive 16-byte words (no bank conflicts)
__host__ __device__ inline int rec_at(int gi, int L, int sl, int ab) { return ((sl * 2 + ab) * PV_GROUPS + gi) * 32 + L; }
__host__ __device__ inline int recj_at(int gi, int L, int sl) { return (sl * PV_GROUPS + gi) * 32 + L; }

// node window of the principal-value sum: nodes lower-2 .. upper+2
__host__ __device__ inline int res_win(int M_I) { return (2 * M_I + 8 < RES_WIN) ? 2 * M_I + 8 : RES_WIN; }

// what the warp phase of k_resonant needs of one item
struct __align__(16) ResItem {
  double pr, pim;     // complex resonance momentum
  double smdelta;     // principal-value sample spacing (integrate_res's smdelta)
  int lower, upper;   // principal-value window
  int nn, work;       // signed order; bit 0 principal value, bit 1 Landau rows, lf << 2
  int w, s;           // omega, species
  long long slot;     // the item's slot (its output row)
  // the fast path's principal-value constants, formed one item per lane:
  int ntiny, pvdf;    // sample points of the tiny rest; pv_fast applies
  float u0, du, ut0, dut;  // FP32 piece estimates of the sample points
  float smd[2], capd[2], pimd[2], pim2[2], csd[2], cord[2];  // double-float pairs
  double pref[6];     // T-tensor prefactors: imaginary for xy and yz, else real
};
// prefactor e of an item as the complex number t_prefactors gives
__device__ __forceinline__ double2 item_pref(const ResItem& it, int e) {
  return (e == 3 || e == 5) ? cmk(0.0, it.pref[e]) : cmk(it.pref[e], 0.0);
}

// The principal-value constants of a resonant item (integrate_res,
// src/ALPS_fns.f90:1000-1040: capDelta, smdelta, the tiny rest's ntiny and
// corr), and for the fast path their double-float pairs and FP32 piece
// estimates, formed in the one-item-per-lane phase so that the warp phase
// starts from them.  pvdf = 0 leaves the item to the FP64 code: a spacing,
// window or |p_im| outside 1e-12 .. 1e12 would leave the normal floats.
__device__ __forceinline__ void pv_constants(const DispArgs& a, const SpecDev& S, const ResGeom& g, ResItem& it) {
  it.smdelta = 0.0;
  it.ntiny = 0;
  it.pvdf = 0;
  if (g.kind != 3) return;
  const double pr = g.pr, pim = g.pi;
  const double capDelta = pr - S.ppar[g.lower];
  const double smdelta = capDelta / (1.0 * a.sys.M_P);
  const int ntiny = (int)((S.ppar[g.upper] - pr - capDelta) / smdelta);
  const double corr = (ntiny > 0) ? ((S.ppar[g.upper] - pr - capDelta) / (1.0 * ntiny)) / smdelta : 0.0;
  it.smdelta = smdelta;
  it.ntiny = ntiny;
  if (!S.df_sums) return;
  const bool sym = fabs(pim) > a.sys.Tlim;
  auto inr = [](double x) { return x >= 1e-12 && x <= 1e12; };
  if (!(inr(smdelta) && inr(capDelta) && fabs(pim) <= 1e12 && (!sym || inr(fabs(pim))) &&
        (ntiny <= 0 || inr(corr * smdelta))))
    return;
  it.pvdf = 1;
  it.u0 = (float)(1.0 + (pr - S.ppar[1]) * S.idppar);
  it.du = (float)(smdelta * S.idppar);
  it.ut0 = (float)(1.0 + (pr + capDelta - S.ppar[1]) * S.idppar);
  it.dut = (float)(corr * smdelta * S.idppar);
  auto put2 = [](float* d, double x) {
    const dflt v = df_of(x);
    d[0] = v.h;
    d[1] = v.l;
  };
  put2(it.smd, smdelta);
  put2(it.capd, capDelta);
  put2(it.pimd, pim);
  put2(it.pim2, pim * pim);
  put2(it.csd, __dmul_rn(corr, smdelta));
  put2(it.cord, corr);
}

// the region used first by the principal-value records, then by the Landau
// rows, in double2
__host__ __device__ inline size_t res_region(int N) {
  const size_t rows = 3 * (size_t)(N + 1);
  return rows > PV_SMEM ? rows : (size_t)PV_SMEM;
}

// per-warp shared memory in double2: the window (h, s), the records / rows
// region, the warp's 32 items, 6 values handed to lanes 0-5 and the queue of
// occupied slots (64 ints)
__host__ __device__ inline size_t res_warp_smem(int N, int W) {
  return (size_t)W * 12 + res_region(N) + 32 * (sizeof(ResItem) / sizeof(double2)) + 6 + 16;
}

// Slots per warp: a warp gathers the occupied slots of its range into
// batches of up to 32 items, does the per-item scalar work one item per
// lane, then the vector work of the batch's items one after another.  Large
// batches take up to 256 slots per warp (about 7 waves of resident warps on
// the map lattice); small ones spread their items over more warps (a single
// omega's few resonant orders run side by side, as latency wants).
inline int res_items_per_warp(long nslots, int warps_per_sm = 12) {
  const long warps_wanted = 152L * warps_per_sm;  // SMs x resident warps of k_resonant
  long ipw = nslots / warps_wanted;
  return (int)(ipw < 1 ? 1 : (ipw > 256 ? 256 : ipw));
}

__device__ inline double2 crcp(double2 z) {
  double r = 1.0 / (z.x * z.x + z.y * z.y);
  return cmk(z.x * r, -z.y * r);
}

// ---------------------------------------------------------------------------
// Fast path of one item's principal-value window: the same sums as the FP64
// code in resonant_body (sample points, pieces, per-piece sums A and C, the
// merge in lane order, h A + s B per (run, entry), the Tlim branch), all in
// double-float arithmetic on the FP32 pipes, on the reduced vectors' float
// pairs (scaled by 2^-e for order n; the result is rescaled at the end).
// The pieces are still chosen from the FP64 sample points wherever the FP32
// estimate lies within its error bound of a half-way point.  Returns false,
// with nothing written to out, when the item's constants were not formed
// (a range would leave the normal floats) or the merge does not apply (the
// caller then runs the FP64 code); otherwise adds the item's
// principal-value part to out (entry e: pref_e T_e times the window scale).
// ---------------------------------------------------------------------------
struct PvSlotF {
  int jd, jc;  // finished piece (-1: none), current piece
  dflt Adx, Ady, Bdx, Bdy, Acx, Acy, Bcx, Bcy;
};

__device__ __forceinline__ float4 f4_of(dflt x, dflt y) { return make_float4(x.h, x.l, y.h, y.l); }
__device__ __forceinline__ dflt f4x(float4 v) { return {v.x, v.y}; }
__device__ __forceinline__ dflt f4y(float4 v) { return {v.z, v.w}; }
// (ax + i ay)(bx + i by), real and imaginary parts
__device__ __forceinline__ void df_cmul(dflt ax, dflt ay, dflt bx, dflt by, dflt& rx, dflt& ry) {
  rx = df_add(df_mul(ax, bx), df_neg(df_mul(ay, by)));
  ry = df_add(df_mul(ax, by), df_mul(ay, bx));
}

__device__ __noinline__ bool pv_fast(const DispArgs& a, const SpecDev& S, const ResItem& it, double2 o, int n,
                                     int W, float4* win, double2* pvv, double2* out) {
  if (!it.pvdf) return false;
  const int lane = threadIdx.x & 31;
  const int M = S.M;
  const double pr = it.pr, pim = it.pim;
  const double smdelta = it.smdelta;
  const bool sym = fabs(pim) > a.sys.Tlim;
  const int NP = a.sys.M_P + 1;
  const int ntiny = it.ntiny;
  const int jw0 = max(1, it.lower - 2), jw1 = min(M - 1, it.upper + 2);
  const int nw = jw1 - jw0 + 1;
  const float* __restrict__ Vh = S.Vh + (size_t)n * (M - 1) * 12;
  const float* __restrict__ Vl = S.Vl + (size_t)n * (M - 1) * 12;
  const dflt oxd = df_of(o.x), oyd = df_of(o.y), kad = {S.kaph, S.kapl}, hid = {S.hidh, S.hidl};
  // node value h_e(j) = omega V_{e,1}(j) + kappa V_{e,2}(j), scaled
  auto hnode = [&](int j, int e, dflt& hx, dflt& hy) {
    const size_t b = (size_t)(j - 1) * 12 + 2 * e;
    const dflt v1 = {Vh[b], Vl[b]}, v2 = {Vh[b + 1], Vl[b + 1]};
    hx = df_add(df_mul(oxd, v1), df_mul(kad, v2));
    hy = df_mul(oyd, v1);
  };
  float4* wh = win;           // h at window nodes
  float4* ws = win + W * 6;   // centred slopes
  for (int t = lane; t < nw * 6; t += 32) {
    const int jj = t / 6, e = t % 6;
    dflt hx, hy;
    hnode(jw0 + jj, e, hx, hy);
    wh[jj * 6 + e] = f4_of(hx, hy);
  }
  __syncwarp();
  for (int t = lane; t < nw * 6; t += 32) {
    const int jj = t / 6, e = t % 6;
    if (jj >= 1 && jj + 1 < nw) {
      const float4 u = wh[(jj + 1) * 6 + e], d = wh[(jj - 1) * 6 + e];
      ws[jj * 6 + e] = f4_of(df_mul(df_add(f4x(u), df_neg(f4x(d))), hid), df_mul(df_add(f4y(u), df_neg(f4y(d))), hid));
    }
  }
  __syncwarp();
  // node value and slope of entry e at piece jc (window, or from the pairs)
  auto node1 = [&](int jc, int e, dflt& hx, dflt& hy, dflt& sx, dflt& sy) {
    if (jc - 1 >= jw0 && jc + 1 <= jw1) {
      const float4 h = wh[(jc - jw0) * 6 + e], s = ws[(jc - jw0) * 6 + e];
      hx = f4x(h);
      hy = f4y(h);
      sx = f4x(s);
      sy = f4y(s);
    } else {
      dflt ux, uy, dx, dy;
      hnode(jc, e, hx, hy);
      hnode(jc + 1, e, ux, uy);
      hnode(jc - 1, e, dx, dy);
      sx = df_mul(df_add(ux, df_neg(dx)), hid);
      sy = df_mul(df_add(uy, df_neg(dy)), hid);
    }
  };
  // pieces, as in resonant_body: the last node in 1..M-1 within half a
  // spacing of p (funct_g's search), clamped to 2..M-2
  const double idpa = fabs(S.idppar), half = 0.5 * S.dppar_abs;
  auto piece_raw = [&](double p) {
    int jr = 0;
    double jd = floor((p - S.ppar[0]) * idpa + 0.5);
    if (jd > -10.0 && jd < (double)M + 10.0) {
      int j0 = (int)jd;
      int hi = min(j0 + 2, M - 1), lo = max(j0 - 2, 1);
      for (int jj = hi; jj >= lo; --jj)
        if (fabs(S.ppar[jj] - p) <= half) {
          jr = jj;
          break;
        }
    }
    return jr;
  };
  auto clampj = [&](int jr) { return (jr >= M - 1) ? M - 2 : ((jr <= 1) ? 2 : jr); };
  // the FP32 estimates u (node j at u = j) are within 2^-23 (M + 20) of a
  // spacing (two roundings of numbers below M + 10) and the nodes within
  // 1e-6 of a spacing of their uniform positions: farther than four times
  // that from a half-way point, the nearest node is the search's answer
  const float hthr = 0.5f - (4.0f * 1.1920929e-7f * (float)(M + 20) + 4.0e-6f);
  auto off_half = [&](float u) { return fabsf(u - rintf(u)) < hthr; };
  auto node_of = [&](float u) {
    const int j = (int)rintf(u);
    return (j >= 1 && j <= M - 1) ? j : 0;
  };
  const dflt prd = df_of(pr);
  auto ppd = [&](int j) { return dflt{S.pph[j], S.ppl[j]}; };
  // the FP64 sample points as integrate_res writes them (for the search
  // near half-way points only)
  auto sym_p = [&](int k) {
    const double capDelta = pr - S.ppar[it.lower];
    return (k == 0) ? pr : ((k == a.sys.M_P) ? __dadd_rn(pr, capDelta) : __dadd_rn(pr, __dmul_rn(smdelta, (double)k)));
  };
  auto tiny_p = [&](int k) {
    const double capDelta = pr - S.ppar[it.lower];
    const double corr = ((S.ppar[it.upper] - pr - capDelta) / (1.0 * ntiny)) / smdelta;
    return (k == 0) ? __dadd_rn(pr, capDelta)
                    : __dadd_rn(__dadd_rn(pr, capDelta), __dmul_rn(__dmul_rn(corr, smdelta), (double)k));
  };
  bool bad = false;
  const dflt z0 = {0.0f, 0.0f};
  auto putf = [&](PvSlotF& q, int j, dflt dx, dflt cx, dflt cy, int dir) {
    if (j != q.jc) {
      if (q.jc >= 0) {
        if (q.jd >= 0 || (dir > 0 ? j < q.jc : j > q.jc)) bad = true;
        q.jd = q.jc;
        q.Adx = q.Acx;
        q.Ady = q.Acy;
        q.Bdx = q.Bcx;
        q.Bdy = q.Bcy;
      }
      q.jc = j;
      q.Acx = q.Acy = q.Bcx = q.Bcy = z0;
    }
    df_acc(q.Acx, cx);
    df_acc(q.Acy, cy);
    df_mac(q.Bcx, cx.h, cx.l, dx);
    df_mac(q.Bcy, cy.h, cy.l, dx);
  };
  // records: (group, lane, slot) sums A, B as float4 pairs; run tables as in
  // resonant_body
  float4* recv = reinterpret_cast<float4*>(pvv);
  float4* runv = reinterpret_cast<float4*>(pvv + PV_RECV);
  int* recj = reinterpret_cast<int*>(pvv + PV_RECV + PV_RUNV);
  int* runL = recj + PV_GROUPS * 64;
  int* runS = runL + 32;
  int* runG = runS + 32;
  int* runJ = runG + 32;
  int nruns = 0, nl[PV_GROUPS] = {0, 0, 0};
  const unsigned lt = (1u << lane) - 1u;
  auto records = [&](int gi, const PvSlotF& q, int dir) {
    const bool two = q.jd >= 0;
    const int j0 = two ? q.jd : q.jc, j1 = two ? q.jc : -1;
    recj[recj_at(gi, lane, 0)] = j0;
    recj[recj_at(gi, lane, 1)] = j1;
    recv[rec_at(gi, lane, 0, 0)] = two ? f4_of(q.Adx, q.Ady) : f4_of(q.Acx, q.Acy);
    recv[rec_at(gi, lane, 0, 1)] = two ? f4_of(q.Bdx, q.Bdy) : f4_of(q.Bcx, q.Bcy);
    recv[rec_at(gi, lane, 1, 0)] = two ? f4_of(q.Acx, q.Acy) : f4_of(z0, z0);
    recv[rec_at(gi, lane, 1, 1)] = two ? f4_of(q.Bcx, q.Bcy) : f4_of(z0, z0);
    const int last = (j1 >= 0) ? j1 : j0;
    const int prev = __shfl_up_sync(0xffffffffu, last, 1);
    const bool st0 = (j0 >= 0) && (lane == 0 || j0 != prev);
    const bool st1 = (j1 >= 0);
    if (j0 >= 0 && lane > 0 && (prev < 0 || (dir > 0 ? j0 < prev : j0 > prev))) bad = true;
    const unsigned m0 = __ballot_sync(0xffffffffu, st0), m1 = __ballot_sync(0xffffffffu, st1);
    const int nr = __popc(m0) + __popc(m1);
    if (nruns + nr <= 32) {
      const int id0 = nruns + __popc(m0 & lt) + __popc(m1 & lt), id1 = id0 + (st0 ? 1 : 0);
      if (st0) {
        runL[id0] = lane;
        runS[id0] = 0;
        runG[id0] = gi;
      }
      if (st1) {
        runL[id1] = lane;
        runS[id1] = 1;
        runG[id1] = gi;
      }
    }
    nruns += nr;
    nl[gi] = __popc(__ballot_sync(0xffffffffu, j0 >= 0));
  };
  const dflt pimd = {it.pimd[0], it.pimd[1]}, pim2 = {it.pim2[0], it.pim2[1]};
  const dflt smd = {it.smd[0], it.smd[1]}, capd = {it.capd[0], it.capd[1]};
  dflt Tlx = z0, Tly = z0;  // the Tlim part of entry e on lane e
  if (sym) {
    const int per = (NP + 31) / 32;
    const int k0 = lane * per, k1 = min(NP, k0 + per);
    PvSlotF su{-1, -1, z0, z0, z0, z0, z0, z0, z0, z0}, sd = su;
    const float u0 = it.u0, du = it.du;
    for (int k = k0; k < k1; ++k) {
      // K = w (dx, p_im) / (dx^2 + p_im^2), dx = p_k - p_res
      const dflt dx = (k == a.sys.M_P) ? capd : df_mul(smd, {(float)k, 0.0f});
      const dflt r = df_scale(df_rcp_approx(df_add(df_mul(dx, dx), pim2)), (k == 0 || k == a.sys.M_P) ? 1.0f : 2.0f);
      const dflt Kx = df_mul(dx, r), Ky = df_mul(pimd, r);
      const float uu = fmaf((float)k, du, u0), ud = fmaf(-(float)k, du, u0);
      int cu, cd;
      if (off_half(uu)) cu = node_of(uu);
      else cu = piece_raw(sym_p(k));
      if (off_half(ud)) cd = node_of(ud);
      else cd = piece_raw(2.0 * pr - sym_p(k));
      putf(su, clampj(cu), dx, Kx, Ky, 1);
      putf(sd, clampj(cd), df_neg(dx), Kx, df_neg(Ky), -1);
    }
    records(0, su, 1);
    records(1, sd, -1);
  } else {
    // Tlim branch: g' sum_k w_k dx^2/(dx^2 + p_im^2) + sign(p_im) i pi G(p_res)/smdelta
    dflt frd = z0;
    for (int k = 1 + lane; k <= a.sys.M_P; k += 32) {
      const dflt dx = (k == a.sys.M_P) ? capd : df_mul(smd, {(float)k, 0.0f});
      const dflt d2 = df_mul(dx, dx);
      const dflt q = df_mul(d2, df_rcp_approx(df_add(d2, pim2)));
      df_acc(frd, df_scale(q, (k == a.sys.M_P) ? 1.0f : 2.0f));
    }
    for (int off = 16; off > 0; off >>= 1)
      frd = df_add(frd, {__shfl_xor_sync(0xffffffffu, frd.h, off), __shfl_xor_sync(0xffffffffu, frd.l, off)});
    if (lane < 6) {
      const int e = lane;
      const double dps = S.dppar;
      // H at p_res + side dppar: u = u0 + side, dx = p - pp(jc) in double-float
      auto Hc1 = [&](int side, dflt& Hx, dflt& Hy) {
        const float u = it.u0 + (float)side;
        int jc;
        if (off_half(u)) jc = node_of(u);
        else jc = piece_raw(side > 0 ? pr + dps : (side < 0 ? pr - dps : pr));
        jc = clampj(jc);
        dflt hx, hy, sx, sy;
        node1(jc, e, hx, hy, sx, sy);
        const dflt dx = df_add(df_add(prd, df_scale({S.dpph, S.dppl}, (float)side)), df_neg(ppd(jc)));
        Hx = df_add(hx, df_mul(sx, dx));
        Hy = df_add(hy, df_mul(sy, dx));
      };
      dflt H1x, H1y, H2x, H2y, H0x, H0y;
      Hc1(1, H1x, H1y);
      Hc1(-1, H2x, H2y);
      Hc1(0, H0x, H0y);
      // g' 2 fr = (H1 - H2) fr / dppar;  i sign(p_im) 2 pi / smdelta, smdelta = capDelta / M_P
      const float sgn = (pim > 0.0) ? 1.0f : ((pim < 0.0) ? -1.0f : 0.0f);
      const dflt c1 = df_mul(frd, {S.idph, S.idpl});
      const dflt c2 = df_scale(df_mul({S.tpmh, S.tpml}, df_rcp_approx(capd)), sgn);
      Tlx = df_add(df_mul(df_add(H1x, df_neg(H2x)), c1), df_neg(df_mul(c2, H0y)));
      Tly = df_add(df_mul(df_add(H1y, df_neg(H2y)), c1), df_mul(c2, H0x));
    }
  }
  if (ntiny > 0) {
    const int per = (ntiny + 1 + 31) / 32;
    const int k0 = lane * per, k1 = min(ntiny + 1, k0 + per);
    PvSlotF sq{-1, -1, z0, z0, z0, z0, z0, z0, z0, z0};
    const float ut0 = it.ut0, dut = it.dut;
    const dflt csd = {it.csd[0], it.csd[1]}, cord = {it.cord[0], it.cord[1]};
    for (int k = k0; k < k1; ++k) {
      // K = w corr (dx, p_im) / (dx^2 + p_im^2)
      const dflt dx = (k == 0) ? capd : df_add(capd, df_mul(csd, {(float)k, 0.0f}));
      const dflt r = df_scale(df_mul(df_rcp_approx(df_add(df_mul(dx, dx), pim2)), cord),
                              (k == 0 || k == ntiny) ? 1.0f : 2.0f);
      const dflt Kx = df_mul(dx, r), Ky = df_mul(pimd, r);
      const float ut = fmaf((float)k, dut, ut0);
      int ct;
      if (off_half(ut)) ct = node_of(ut);
      else ct = piece_raw(tiny_p(k));
      putf(sq, clampj(ct), dx, Kx, Ky, 1);
    }
    records(2, sq, 1);
  }
  if (__any_sync(0xffffffffu, bad) || nruns > 32) return false;
  dflt accd = z0;  // component c = lane (< 12) of T: xx.re, xx.im, yy.re, ...
  if (nruns > 0) {
    __syncwarp();
    // run totals in (lane, slot) order
    if (lane < nruns) {
      const int L = runL[lane], sl = runS[lane], gi = runG[lane];
      int Ln = nl[gi], sn = 0;
      if (lane + 1 < nruns && runG[lane + 1] == gi) {
        Ln = runL[lane + 1];
        sn = runS[lane + 1];
      }
      float4 A4 = recv[rec_at(gi, L, sl, 0)], B4 = recv[rec_at(gi, L, sl, 1)];
      dflt Ax = f4x(A4), Ay = f4y(A4), Bx = f4x(B4), By = f4y(B4);
      for (int L2 = L + 1; L2 < Ln || (L2 == Ln && sn == 1); ++L2) {
        const float4 a2 = recv[rec_at(gi, L2, 0, 0)], b2 = recv[rec_at(gi, L2, 0, 1)];
        Ax = df_add(Ax, f4x(a2));
        Ay = df_add(Ay, f4y(a2));
        Bx = df_add(Bx, f4x(b2));
        By = df_add(By, f4y(b2));
      }
      runJ[lane] = recj[recj_at(gi, L, sl)];
      runv[lane * 2] = f4_of(Ax, Ay);
      runv[lane * 2 + 1] = f4_of(Bx, By);
    }
    __syncwarp();
    // (run, entry) pairs: h A + s B with B = C + (p_res - pp(jc)) A,
    // mirrored runs with the minus sign
    float4* contrib = recv;
    for (int q = lane; q < nruns * 6; q += 32) {
      const int rho = q / 6, e = q % 6;
      const int jc = runJ[rho];
      dflt hx, hy, sx, sy;
      node1(jc, e, hx, hy, sx, sy);
      const float4 A4 = runv[rho * 2], C4 = runv[rho * 2 + 1];
      const dflt Ax = f4x(A4), Ay = f4y(A4);
      const dflt del = df_add(prd, df_neg(ppd(jc)));
      const dflt Bx = df_add(f4x(C4), df_mul(Ax, del)), By = df_add(f4y(C4), df_mul(Ay, del));
      dflt t1x, t1y, t2x, t2y;
      df_cmul(hx, hy, Ax, Ay, t1x, t1y);
      df_cmul(sx, sy, Bx, By, t2x, t2y);
      dflt tx = df_add(t1x, t2x), ty = df_add(t1y, t2y);
      if (runG[rho] == 1) {
        tx = df_neg(tx);
        ty = df_neg(ty);
      }
      contrib[q] = f4_of(tx, ty);
    }
    __syncwarp();
    // component c of T: the runs in order
    if (lane < 12) {
      const int e = lane >> 1;
      dflt s = z0;
      for (int rho = 0; rho < nruns; ++rho) {
        const float4 c = contrib[rho * 6 + e];
        s = df_add(s, (lane & 1) ? f4y(c) : f4x(c));
      }
      accd = s;
    }
  }
  {
    // plus the Tlim part of component c (entry c/2 sits on lane c/2)
    const int src = (lane < 12) ? (lane >> 1) : 0;
    const float xh = __shfl_sync(0xffffffffu, Tlx.h, src), xl = __shfl_sync(0xffffffffu, Tlx.l, src);
    const float yh = __shfl_sync(0xffffffffu, Tly.h, src), yl = __shfl_sync(0xffffffffu, Tly.l, src);
    accd = df_add(accd, (lane & 1) ? dflt{yh, yl} : dflt{xh, xl});
  }
  // out_e += pref_e T_e scale: scale = 2 pi smdelta dpperp/4 (-q/(2 k_par))
  // and the pairs' 2^e; an imaginary prefactor (xy, yz) maps (x, y) to
  // pe (-y, x)
  const double v = df_val(accd) * (S.Vscale[n] * it.smdelta * S.pvc);
  const double w = __shfl_xor_sync(0xffffffffu, v, 1);
  if (lane < 12) {
    const int e = lane >> 1;
    if (!(n == 0 && (e == 0 || e == 3 || e == 4))) {
      const double pe = it.pref[e];
      double* o2 = reinterpret_cast<double*>(out + e);
      o2[lane & 1] += (e == 3 || e == 5) ? ((lane & 1) ? pe * w : -pe * w) : pe * v;
    }
  }
  __syncwarp();
  return true;
}

__device__ __forceinline__ void resonant_body(const DispArgs& a, const DispShape& sh, const double2* __restrict__ om,
                                              int n_om, const int* __restrict__ count,
                                              const int* __restrict__ slot_nn, double2* items, long block) {
  extern __shared__ double2 sm[];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int S_ = a.sys.nspec;
  const int N = a.sp[0].N;  // every species has the same p_perp grid
  const int W = res_win(a.sys.M_I);
  double2* wh = sm + (size_t)warp * res_warp_smem(N, W);  // node values h
  double2* ws = wh + W * 6;                                // node slopes s
  double2* pvv = ws + W * 6;                               // principal-value records
  double2* frow = pvv;                                     // f(i, p_res), after them
  double2* fpr = frow + (N + 1);                           // f(i, p_res + dppar)
  double2* fmr = fpr + (N + 1);                            // f(i, p_res - dppar)
  ResItem* ri = reinterpret_cast<ResItem*>(pvv + res_region(N));
  double2* tb = reinterpret_cast<double2*>(ri + 32);      // values handed to lanes 0-5
  int* queue = reinterpret_cast<int*>(tb + 6);            // occupied slots, offsets from slot0
  const long total = (long)n_om * S_ * a.rcap;
  // this warp's slots: slot0 .. slot0 + sh.ipw - 1.  Most slots of a large
  // batch are empty (an (omega, species) fills count of its rcap slots), so
  // the occupied ones are gathered, in slot order, into batches of up to 32
  // items; each batch runs the per-item phase one item per lane and then
  // the per-warp phase.  Which batch or lane an item lands on does not
  // change its result.
  const long slot0 = (block * RES_WARPS + warp) * (long)sh.ipw;
  if (slot0 >= total) return;
  const unsigned lt = (1u << lane) - 1u;
  int qn = 0;
  for (int c0 = 0; c0 < sh.ipw; c0 += 32) {
    {
      const long sl = slot0 + c0 + lane;
      bool occ = false;
      if (c0 + lane < sh.ipw && sl < total) {
        const int r = (int)(sl % a.rcap);
        const int s = (int)((sl / a.rcap) % S_);
        const int w = (int)(sl / ((long)a.rcap * S_));
        occ = r < count[(size_t)w * S_ + s];
      }
      const unsigned m = __ballot_sync(0xffffffffu, occ);
      if (occ) queue[qn + __popc(m & lt)] = c0 + lane;
      qn += __popc(m);
      __syncwarp();
    }
    const bool last = c0 + 32 >= sh.ipw;
    while (qn >= 32 || (last && qn > 0)) {
  const int nb = qn < 32 ? qn : 32;
  const long item = (lane < nb) ? slot0 + queue[lane] : total;

  // ---- one item per thread: geometry, prefactors, factorised Landau rows ----
  int work = 0;
  if (item < total) {
    const int r = (int)(item % a.rcap);
    const int s = (int)((item / a.rcap) % S_);
    const int w = (int)(item / ((long)a.rcap * S_));
    {
      const SpecDev& S = a.sp[s];
      const int nn = slot_nn[((size_t)w * S_ + s) * a.rcap + r];
      const int n = nn < 0 ? -nn : nn;
      const double2 o = om[w];
      const double kpar = a.sys.kpar;
      const double z = a.sys.kperp_norm ? a.sys.kperp / S.qs : 1.0 / S.qs;
      double2 pref[6];
      t_prefactors(nn, z, a.sys.kperp, a.sys.kperp_norm, pref);
      const ResGeom g = res_geometry(S, a.sys.M_I, o, nn, kpar);
      double2 res[6];
      for (int e = 0; e < 6; ++e) res[e] = cmk(0.0, 0.0);
      const int lf = (o.y < 0.0) ? 2 : ((o.y == 0.0) ? 1 : 0);
      bool rows = lf > 0;
      if (lf > 0 && S.lmom) {
        // factorised rows: valid when the row deviation |delta_i(p')| <= 1e-5
        // for p' = p, p +- dppar (second-order remainder <= 1.7e-16); the
        // bound in FP32 with a margin (an item just inside it takes the rows)
        const double2 p = cmk(g.pr, g.pi);
        const float ap = sqrtf(fmaf((float)p.x, (float)p.x, (float)p.y * (float)p.y)) * 1.00001f + (float)S.dppar_abs;
        const float bound = fmaf(fmaf(S.la32, ap, S.lb32), ap, S.lc32);
        if (bound <= 0.999e-5f) {
          rows = false;
          // Row Gaussian G(x) = exp(-p2r (x - p3r)^2) at x = p, p +- dppar:
          // G(p +- pd) = lgc G(p) X^{+-1}, X = exp(-2 p2r pd (p - p3r)).  In
          // double-float with powers of two kept apart: G(p) = 2^k0 g0,
          // X = 2^kx xm.  With P_F, Q_F the moment polynomials of family F,
          //   Spar  = (G(p+pd) P_F(p+pd) - G(p-pd) P_F(p-pd)) / (2 pd)
          //         = lgc/(2 pd) G(p) (X P_F(p+pd) - X^-1 P_F(p-pd)),
          //   Sperp = G(p) Q_F(p),
          //   sum_F = (q/|k_par|) (kappa Spar + (omega - kappa p) Sperp).
          const double dx = p.x - S.p3r, dy = p.y;
          int k0, kx;
          dflt c0, s0, cx, sx;
          const dflt m0 = df_exp_scaled(-S.p2r * ((dx - dy) * (dx + dy)), k0);
          df_cis(-2.0 * S.p2r * dx * dy, c0, s0);
          const dflt mx = df_exp_scaled(S.lcx * dx, kx);
          df_cis(S.lcx * dy, cx, sx);
          // an underflowing Gaussian (|G| min_a0 below the FP64 range at any
          // of the three points) leaves the term zero, as in FP64
          const int akx = kx < 0 ? -kx : kx;
          const bool zero = (k0 + S.lze < -1072) || (k0 - akx + S.lge + S.lze < -1072);
          if (!zero) {
            const cdf g0 = {df_mul(m0, c0), df_mul(m0, s0)};
            const cdf xm = {df_mul(mx, cx), df_mul(mx, sx)};
            const dflt ixm = df_rcp_approx(mx);
            const cdf xi = {df_mul(ixm, cx), df_neg(df_mul(ixm, sx))};
            // X P+ - X^-1 P- = 2^|kx| (a P+ - b P-): (a, b) = (xm, 2^-2kx xi)
            // for kx >= 0, (2^2kx xm, xi) otherwise (a term below 2^-126 of
            // the other is dropped)
            const int sh = 2 * akx;
            const float sc = sh <= 126 ? ldexpf(1.0f, -sh) : 0.0f;
            const cdf fa = kx >= 0 ? xm : cdf{df_scale(xm.x, sc), df_scale(xm.y, sc)};
            const cdf fb = kx >= 0 ? cdf{df_scale(xi.x, sc), df_scale(xi.y, sc)} : xi;
            const cdf pz = {df_of(p.x), df_of(p.y)};
            const dflt pdd = df_of(S.dppar_abs);
            // powers 1..4 of p + pd, p - pd and p
            cdf zp[3][5];
            zp[0][1] = {df_add(pz.x, pdd), pz.y};
            zp[1][1] = {df_add(pz.x, df_neg(pdd)), pz.y};
            zp[2][1] = pz;
#pragma unroll
            for (int u = 0; u < 3; ++u) {
              zp[u][2] = cdf_mul(zp[u][1], zp[u][1]);
              zp[u][3] = cdf_mul(zp[u][2], zp[u][1]);
              zp[u][4] = cdf_mul(zp[u][2], zp[u][2]);
            }
            // sum_m c_m z^m, c real (float pairs at c[m], c[10 + m])
            auto poly = [&](const float* c, int u) {
              cdf acc = {{c[0], c[10]}, {0.0f, 0.0f}};
#pragma unroll
              for (int m = 1; m < 5; ++m) {
                const dflt cm = {c[m], c[10 + m]};
                acc = cdf_add(acc, cdf_rmul(zp[u][m], cm));
              }
              return acc;
            };
            const cdf omd = {df_of(o.x), df_of(o.y)};
            // q / |k_par| (the sign of the charge stays)
            const dflt kapd = df_of(S.kappa), qld = df_of(kpar < 0.0 ? -S.qk : S.qk);
            const cdf wk = {df_add(omd.x, df_neg(df_mul(kapd, pz.x))), df_add(omd.y, df_neg(df_mul(kapd, pz.y)))};
            // lgc / (2 pd) and the factor 2^-|kx| of Sperp against Spar
            const dflt lgd = df_mul({S.lgch, S.lgcl}, df_rcp_approx(df_scale(pdd, 2.0f)));
            const float sp = akx <= 126 ? ldexpf(1.0f, -akx) : 0.0f;
            cdf sumF[3];
            int eF[3];
#pragma unroll
            for (int F = 0; F < 3; ++F) {
              const float* lm = S.lmomf + ((size_t)n * 3 + F) * 24;
              const cdf Pp = poly(lm, 0), Pm = poly(lm, 1);
              const cdf Qp = poly(lm + 5, 2);
              const cdf br = {df_add(cdf_mul(fa, Pp).x, df_neg(cdf_mul(fb, Pm).x)),
                              df_add(cdf_mul(fa, Pp).y, df_neg(cdf_mul(fb, Pm).y))};
              const cdf spar = cdf_rmul(cdf_mul(g0, br), lgd);
              const cdf sperp = cdf_mul(cdf_mul(g0, Qp), wk);
              const cdf t = {df_add(df_mul(spar.x, kapd), df_scale(sperp.x, sp)),
                             df_add(df_mul(spar.y, kapd), df_scale(sperp.y, sp))};
              sumF[F] = cdf_rmul(t, qld);
              eF[F] = k0 + akx + (int)lm[20];
            }
            // res_e = pref_e c_e sum_F(e) ifac, c_e = 1, p or p^2; ifac =
            // -i dpperp 2 pi^2 lf, pref_e real (imaginary for xy, yz)
            const cdf p2 = cdf_mul(pz, pz);
            const double fi = -S.dpperp * ALPS_PI * 2.0 * ALPS_PI * (double)lf;
#pragma unroll
            for (int e = 0; e < 6; ++e) {
              const int fam = (e == 1) ? 1 : ((e == 3 || e == 5) ? 2 : 0);
              cdf v = sumF[fam];
              if (e == 2) v = cdf_mul(v, p2);
              else if (e == 4 || e == 5) v = cdf_mul(v, pz);
              // pref ifac: real pref -> i (pref fi); imaginary i pref.y -> -(pref.y fi)
              const bool im = (e == 3 || e == 5);
              const dflt f = df_of(im ? -pref[e].y * fi : pref[e].x * fi);
              const double vx = df_val(df_mul(v.x, f)), vy = df_val(df_mul(v.y, f));
              // multiply by i for a real prefactor: (x, y) -> (-y, x)
              res[e] = im ? cmk(ldexp(vx, eF[fam]), ldexp(vy, eF[fam])) : cmk(ldexp(-vy, eF[fam]), ldexp(vx, eF[fam]));
            }
          }
        }
      }
      work = ((g.kind == 3) ? 1 : 0) | (rows ? 2 : 0);
      double2* out = items + item * 6;
      for (int e = 0; e < 6; ++e) {
        const bool skip = (n == 0 && (e == 0 || e == 3 || e == 4));
        out[e] = skip ? cmk(0.0, 0.0) : res[e];
      }
      ResItem& it = ri[lane];
      it.pr = g.pr;
      it.pim = g.pi;
      it.lower = g.lower;
      it.upper = g.upper;
      it.nn = nn;
      it.work = work | (lf << 2);
      it.w = w;
      it.s = s;
      it.slot = item;
      for (int e = 0; e < 6; ++e) it.pref[e] = (e == 3 || e == 5) ? pref[e].y : pref[e].x;
      pv_constants(a, S, g, it);
    }
  }
  __syncwarp();

  // ---- one item per warp: the principal-value sums and the Landau rows ----
  unsigned pend = __ballot_sync(0xffffffffu, work != 0);
  while (pend) {
    const int il = __ffs(pend) - 1;
    pend &= pend - 1;
    const ResItem& it = ri[il];
    const int s = it.s, w = it.w, nn = it.nn;
    const int n = nn < 0 ? -nn : nn;
    const int wk = it.work & 3, lf = it.work >> 2;
    const SpecDev& S = a.sp[s];
    const double2 o = om[w];
    const int M = S.M;
    const double kpar = a.sys.kpar, kappa = S.kappa;
    const double* Vn = S.V + (size_t)n * (M - 1) * 12;
    double2* out = items + it.slot * 6;

    // ---- principal value window (case 3) ----
    if (wk & 1) {
      const double pr = it.pr, pim = it.pim;
      const double dpa = S.dppar_abs, dps = S.dppar;
      const int jw0 = max(1, it.lower - 2), jw1 = min(M - 1, it.upper + 2);
      const int nw = jw1 - jw0 + 1;
      const bool winok = nw <= W;
      double2 T[6];
      for (int e = 0; e < 6; ++e) T[e] = cmk(0.0, 0.0);
      // the fast path's double-float sums; the FP64 code below otherwise
      const bool fast = S.df_sums && winok && pv_fast(a, S, it, o, n, W, reinterpret_cast<float4*>(wh), pvv, out);
      if (!fast) {
      if (winok) {
        for (int t = lane; t < nw * 6; t += 32) {
          int jj = t / 6, e = t % 6;
          wh[jj * 6 + e] = h_node(Vn, jw0 + jj, e, o, kappa);
        }
        __syncwarp();
        for (int t = lane; t < nw * 6; t += 32) {
          int jj = t / 6, e = t % 6;
          if (jj >= 1 && jj + 1 < nw) ws[jj * 6 + e] = cscale(csub(wh[(jj + 1) * 6 + e], wh[(jj - 1) * 6 + e]), S.hidpa);
        }
      }
      __syncwarp();
      // funct_g summed over iperp (src/ALPS_fns.f90:1243-1321): the node whose
      // interpolant serves p is "the last ipar in 1..npar-1 with
      // |pp(ipar) - p| <= dppar/2", clamped to 2..npar-2
      const double idpa = fabs(S.idppar), half = 0.5 * dpa;
      // last node in 1..M-1 within half a spacing of p, or 0 (the search of
      // funct_g before its clamp); the candidates bracket the nearest node
      auto piece_raw = [&](double p) {
        int jr = 0;
        double jd = floor((p - S.ppar[0]) * idpa + 0.5);
        if (jd > -10.0 && jd < (double)M + 10.0) {
          int j0 = (int)jd;
          int hi = min(j0 + 2, M - 1), lo = max(j0 - 2, 1);
          for (int jj = hi; jj >= lo; --jj)
            if (fabs(S.ppar[jj] - p) <= half) { jr = jj; break; }
        }
        return jr;
      };
      auto clampj = [&](int jr) { return (jr >= M - 1) ? M - 2 : ((jr <= 1) ? 2 : jr); };
      // the same search from u, an FP32 estimate of p in node units (node j
      // at u = j).  Away from the half-way points between nodes by more than
      // 1e-3 of a spacing, the nearest node is the search's answer: u's
      // rounding is below 1e-4 of a spacing, and alps_set_species admits
      // only grids whose steps agree to 1e-9, so a node is within 1e-6 of a
      // spacing of its uniform position.  Nearer the half-way points the
      // FP64 search decides.
      auto off_half = [&](float u) { return fabsf(u - rintf(u)) < 0.499f; };
      auto node_of = [&](float u) {
        const int j = (int)rintf(u);
        return (j >= 1 && j <= M - 1) ? j : 0;
      };
      auto piece = [&](double p) { return clampj(piece_raw(p)); };
      // the same index for p increasing (up) or decreasing (down) from a known
      // raw index: |pp(j) - p| is monotone in p, so the last valid node moves
      // by single steps
      auto piece_up = [&](int jr, double p) {
        if (jr == 0) return piece_raw(p);
        while (jr < M - 1 && fabs(S.ppar[jr + 1] - p) <= half) ++jr;
        return (fabs(S.ppar[jr] - p) <= half) ? jr : piece_raw(p);
      };
      auto piece_down = [&](int jr, double p) {
        if (jr == 0) return piece_raw(p);
        while (jr >= 1 && !(fabs(S.ppar[jr] - p) <= half)) --jr;
        return (jr >= 1) ? jr : piece_raw(p);
      };
      // node value h and centred slope s of entry e at node jc
      auto node1 = [&](int jc, int e, double2& h, double2& sl) {
        if (winok && jc - 1 >= jw0 && jc + 1 <= jw1) {
          h = wh[(jc - jw0) * 6 + e];
          sl = ws[(jc - jw0) * 6 + e];
        } else {
          h = h_node(Vn, jc, e, o, kappa);
          sl = cscale(csub(h_node(Vn, jc + 1, e, o, kappa), h_node(Vn, jc - 1, e, o, kappa)), S.hidpa);
        }
      };
      auto node = [&](int jc, double2* h, double2* sl) {
  #pragma unroll
        for (int e = 0; e < 6; ++e) node1(jc, e, h[e], sl[e]);
      };
      const double capDelta = pr - S.ppar[it.lower];
      const double smdelta = capDelta / (1.0 * a.sys.M_P);
      const bool sym = fabs(pim) > a.sys.Tlim;
      const int NP = a.sys.M_P + 1;
      // tiny rest between pr + capDelta and ppar[upper]
      const int ntiny = (int)((S.ppar[it.upper] - pr - capDelta) / smdelta);
      const double corr = (ntiny > 0) ? ((S.ppar[it.upper] - pr - capDelta) / (1.0 * ntiny)) / smdelta : 0.0;
      // the sample points: k in 0..M_P of the symmetric sum (group 0 direct,
      // group 1 mirrored), k in 0..ntiny of the tiny rest (group 2).  Their
      // coordinates are rounded as integrate_res writes them, without fused
      // multiply-adds: a point can sit exactly on a piece boundary
      // pp(j) + dppar/2, and its piece must be the reference's.
      auto sym_point = [&](int k, double& p, double& dx, double2& K) {
        p = (k == 0) ? pr
                     : ((k == a.sys.M_P) ? __dadd_rn(pr, capDelta) : __dadd_rn(pr, __dmul_rn(smdelta, (double)k)));
        double wk = (k == 0 || k == a.sys.M_P) ? 1.0 : 2.0;
        dx = p - pr;
        double rr = wk * rcp_fast(fma(dx, dx, pim * pim));
        K = cmk(dx * rr, pim * rr);
      };
      auto tiny_point = [&](int k, double& p, double& dx, double2& K) {
        p = (k == 0) ? __dadd_rn(pr, capDelta)
                     : __dadd_rn(__dadd_rn(pr, capDelta), __dmul_rn(__dmul_rn(corr, smdelta), (double)k));
        double wk = (k == 0 || k == ntiny) ? 1.0 : 2.0;
        dx = p - pr;
        double rr = wk * corr * rcp_fast(fma(dx, dx, pim * pim));
        K = cmk(dx * rr, pim * rr);
      };

      // Sum_k c_k H(p_k) with H linear on each piece jc needs, per piece, only
      // A = Sum c_k and B = Sum c_k (p_k - pp(jc)) = C + (p_res - pp(jc)) A,
      // C = Sum c_k (p_k - p_res); the piece adds h A + s B.
      // Each lane walks a run of consecutive k and keeps the sums of at most
      // two pieces (pieces are M_P/(M_I+1) or more points wide, far wider
      // than a lane's run); the lanes' piece sums are merged per piece in
      // shared memory in lane order, and each (piece, entry) pair is then one
      // thread's h A + s B.  A lane that meets a third piece, or indices that
      // are not monotone in k, send the item to the per-lane flush below.
      struct PvSlot {
        int jd, jc;          // finished piece (-1: none), current piece
        double2 Ad, Bd, Ac, Bc;  // A and C of each
      };
      bool bad = false;
      auto put = [&](PvSlot& q, int j, double dx, double2 c, int dir) {
        if (j != q.jc) {
          if (q.jc >= 0) {
            if (q.jd >= 0 || (dir > 0 ? j < q.jc : j > q.jc)) bad = true;
            q.jd = q.jc;
            q.Ad = q.Ac;
            q.Bd = q.Bc;
          }
          q.jc = j;
          q.Ac = q.Bc = cmk(0.0, 0.0);
        }
        q.Ac = cadd(q.Ac, c);
        q.Bc = cmk(fma(c.x, dx, q.Bc.x), fma(c.y, dx, q.Bc.y));
      };
      int* recj = reinterpret_cast<int*>(pvv + PV_RECV + PV_RUNV);  // (group, lane, slot) piece
      int* runL = recj + PV_GROUPS * 64;                               // run start lane
      int* runS = runL + 32;                                           // run start slot
      int* runG = runS + 32;                                           // run group
      int* runJ = runG + 32;                                           // run piece
      double2* recv = pvv;                                             // (group, lane, slot) A, B
      double2* runv = pvv + PV_RECV;                                   // run A, B
      int nruns = 0, nl[PV_GROUPS] = {0, 0, 0};
      // a lane's two pieces to shared memory; run starts get ids in
      // (lane, slot) order after the runs of the earlier groups
      auto records = [&](int gi, const PvSlot& q, int dir) {
        const int j0 = (q.jd >= 0) ? q.jd : q.jc, j1 = (q.jd >= 0) ? q.jc : -1;
        recj[recj_at(gi, lane, 0)] = j0;
        recj[recj_at(gi, lane, 1)] = j1;
        recv[rec_at(gi, lane, 0, 0)] = (q.jd >= 0) ? q.Ad : q.Ac;
        recv[rec_at(gi, lane, 0, 1)] = (q.jd >= 0) ? q.Bd : q.Bc;
        recv[rec_at(gi, lane, 1, 0)] = (q.jd >= 0) ? q.Ac : cmk(0.0, 0.0);
        recv[rec_at(gi, lane, 1, 1)] = (q.jd >= 0) ? q.Bc : cmk(0.0, 0.0);
        const int last = (j1 >= 0) ? j1 : j0;
        const int prev = __shfl_up_sync(0xffffffffu, last, 1);
        const bool st0 = (j0 >= 0) && (lane == 0 || j0 != prev);
        const bool st1 = (j1 >= 0);
        if (j0 >= 0 && lane > 0 && (prev < 0 || (dir > 0 ? j0 < prev : j0 > prev))) bad = true;
        const unsigned m0 = __ballot_sync(0xffffffffu, st0), m1 = __ballot_sync(0xffffffffu, st1);
        const unsigned lt = (1u << lane) - 1u;
        const int nr = __popc(m0) + __popc(m1);
        if (nruns + nr <= 32) {
          const int id0 = nruns + __popc(m0 & lt) + __popc(m1 & lt), id1 = id0 + (st0 ? 1 : 0);
          if (st0) {
            runL[id0] = lane;
            runS[id0] = 0;
            runG[id0] = gi;
          }
          if (st1) {
            runL[id1] = lane;
            runS[id1] = 1;
            runG[id1] = gi;
          }
        }
        nruns += nr;
        nl[gi] = __popc(__ballot_sync(0xffffffffu, j0 >= 0));
      };
      // Fast path: the sample sums in double-float arithmetic on the FP32
      // pipes (about 46 bits; the pieces are still found from the FP64
      // sample points).  Used where every pair stays a normal float: spacing,
      // window and |p_im| within 1e-12 .. 1e12.
      auto inr = [](double x) { return x >= 1e-12 && x <= 1e12; };
      const bool dfsym = S.df_sums && inr(smdelta) && inr(capDelta) && inr(fabs(pim));
      const bool dftiny = S.df_sums && inr(capDelta) && inr(corr * smdelta) && fabs(pim) <= 1e12;
      struct PvSlotF {
        int jd, jc;
        dflt Adx, Ady, Bdx, Bdy, Acx, Acy, Bcx, Bcy;
      };
      const dflt z0 = {0.0f, 0.0f};
      auto putf = [&](PvSlotF& q, int j, dflt dx, dflt cx, dflt cy, int dir) {
        if (j != q.jc) {
          if (q.jc >= 0) {
            if (q.jd >= 0 || (dir > 0 ? j < q.jc : j > q.jc)) bad = true;
            q.jd = q.jc;
            q.Adx = q.Acx;
            q.Ady = q.Acy;
            q.Bdx = q.Bcx;
            q.Bdy = q.Bcy;
          }
          q.jc = j;
          q.Acx = q.Acy = q.Bcx = q.Bcy = z0;
        }
        df_acc(q.Acx, cx);
        df_acc(q.Acy, cy);
        df_mac(q.Bcx, cx.h, cx.l, dx);
        df_mac(q.Bcy, cy.h, cy.l, dx);
      };
      auto to64 = [&](const PvSlotF& q) {
        PvSlot r;
        r.jd = q.jd;
        r.jc = q.jc;
        r.Ad = cmk(df_val(q.Adx), df_val(q.Ady));
        r.Bd = cmk(df_val(q.Bdx), df_val(q.Bdy));
        r.Ac = cmk(df_val(q.Acx), df_val(q.Acy));
        r.Bc = cmk(df_val(q.Bcx), df_val(q.Bcy));
        return r;
      };
      // the sample points as integrate_res writes them (for the FP64 search)
      auto sym_p = [&](int k) {
        return (k == 0) ? pr
                        : ((k == a.sys.M_P) ? __dadd_rn(pr, capDelta) : __dadd_rn(pr, __dmul_rn(smdelta, (double)k)));
      };
      auto tiny_p = [&](int k) {
        return (k == 0) ? __dadd_rn(pr, capDelta)
                        : __dadd_rn(__dadd_rn(pr, capDelta), __dmul_rn(__dmul_rn(corr, smdelta), (double)k));
      };
      if (sym && dfsym) {
        const int per = (NP + 31) / 32;
        const int k0 = lane * per, k1 = min(NP, k0 + per);
        PvSlotF su{-1, -1, z0, z0, z0, z0, z0, z0, z0, z0}, sd = su;
        const float u0 = (float)(1.0 + (pr - S.ppar[1]) * S.idppar), du = (float)(smdelta * S.idppar);
        const dflt smd = df_of(smdelta), capd = df_of(capDelta), pimd = df_of(pim), pim2 = df_of(pim * pim);
        for (int k = k0; k < k1; ++k) {
          // K = w (dx, p_im) / (dx^2 + p_im^2), dx = p_k - p_res
          const dflt dx = (k == a.sys.M_P) ? capd : df_mul(smd, {(float)k, 0.0f});
          const dflt r = df_scale(df_rcp_approx(df_add(df_mul(dx, dx), pim2)),
                                  (k == 0 || k == a.sys.M_P) ? 1.0f : 2.0f);
          const dflt Kx = df_mul(dx, r), Ky = df_mul(pimd, r);
          const float uu = fmaf((float)k, du, u0), ud = fmaf(-(float)k, du, u0);
          const int cu = clampj(off_half(uu) ? node_of(uu) : piece_raw(sym_p(k)));
          const int cd = clampj(off_half(ud) ? node_of(ud) : piece_raw(2.0 * pr - sym_p(k)));
          putf(su, cu, dx, Kx, Ky, 1);
          putf(sd, cd, df_neg(dx), Kx, df_neg(Ky), -1);
        }
        records(0, to64(su), 1);
        records(1, to64(sd), -1);
      } else if (sym) {
        const int per = (NP + 31) / 32;
        const int k0 = lane * per, k1 = min(NP, k0 + per);
        PvSlot su{-1, -1, cmk(0, 0), cmk(0, 0), cmk(0, 0), cmk(0, 0)}, sd = su;
        const float u0 = (float)(1.0 + (pr - S.ppar[1]) * S.idppar), du = (float)(smdelta * S.idppar);
        for (int k = k0; k < k1; ++k) {
          double p, dx;
          double2 K;
          sym_point(k, p, dx, K);
          const float uu = fmaf((float)k, du, u0), ud = fmaf(-(float)k, du, u0);
          const int cu = clampj(off_half(uu) ? node_of(uu) : piece_raw(p));
          const int cd = clampj(off_half(ud) ? node_of(ud) : piece_raw(2.0 * pr - p));
          put(su, cu, dx, K, 1);
          put(sd, cd, -dx, cmk(K.x, -K.y), -1);
        }
        records(0, su, 1);
        records(1, sd, -1);
      } else {
        // Tlim branch: g' * sum_k w_k (p-pr)^2/((p-pr)^2+pim^2) + sign(pim) i pi G(pr)/smdelta
        double fr = 0.0;
        for (int k = 1 + lane; k <= a.sys.M_P; k += 32) {
          double p = (k == a.sys.M_P) ? __dadd_rn(pr, capDelta) : __dadd_rn(pr, __dmul_rn(smdelta, (double)k));
          double wk = (k == a.sys.M_P) ? 1.0 : 2.0;
          double d = p - pr;
          fr += wk * ((d * d) / (d * d + pim * pim));
        }
        for (int off = 16; off > 0; off >>= 1) fr += __shfl_xor_sync(0xffffffffu, fr, off);
        // entry e on lane e, then T (on lane 0, as the other branches leave it)
        double2 Te = cmk(0.0, 0.0);
        if (lane < 6) {
          const int e = lane;
          auto Hc1 = [&](double p) {
            const int jc = piece(p);
            double2 h, sl;
            node1(jc, e, h, sl);
            const double dx = p - S.ppar[jc];
            return cmk(fma(sl.x, dx, h.x), fma(sl.y, dx, h.y));
          };
          const double2 H1 = Hc1(pr + dps), H2 = Hc1(pr - dps), H0 = Hc1(pr);
          double sgn = (pim > 0.0) ? 1.0 : ((pim < 0.0) ? -1.0 : 0.0);
          double2 gp = cscale(csub(H1, H2), 1.0 / (2.0 * dps));
          Te = cadd(cscale(gp, 2.0 * fr), cmul(cmk(0.0, sgn * 2.0 * ALPS_PI / smdelta), H0));
        }
  #pragma unroll
        for (int e = 0; e < 6; ++e) {
          const double tx = __shfl_sync(0xffffffffu, Te.x, e), ty = __shfl_sync(0xffffffffu, Te.y, e);
          if (lane == 0) T[e] = cmk(tx, ty);
        }
      }
      if (ntiny > 0 && dftiny) {
        const int per = (ntiny + 1 + 31) / 32;
        const int k0 = lane * per, k1 = min(ntiny + 1, k0 + per);
        PvSlotF sq{-1, -1, z0, z0, z0, z0, z0, z0, z0, z0};
        const float ut0 = (float)(1.0 + (pr + capDelta - S.ppar[1]) * S.idppar), dut = (float)(corr * smdelta * S.idppar);
        const dflt capd = df_of(capDelta), csd = df_of(__dmul_rn(corr, smdelta)), cord = df_of(corr),
                   pimd = df_of(pim), pim2 = df_of(pim * pim);
        for (int k = k0; k < k1; ++k) {
          // K = w corr (dx, p_im) / (dx^2 + p_im^2)
          const dflt dx = (k == 0) ? capd : df_add(capd, df_mul(csd, {(float)k, 0.0f}));
          const dflt r = df_scale(df_mul(df_rcp_approx(df_add(df_mul(dx, dx), pim2)), cord),
                                  (k == 0 || k == ntiny) ? 1.0f : 2.0f);
          const dflt Kx = df_mul(dx, r), Ky = df_mul(pimd, r);
          const float ut = fmaf((float)k, dut, ut0);
          const int ct = clampj(off_half(ut) ? node_of(ut) : piece_raw(tiny_p(k)));
          putf(sq, ct, dx, Kx, Ky, 1);
        }
        records(2, to64(sq), 1);
      } else if (ntiny > 0) {
        const int per = (ntiny + 1 + 31) / 32;
        const int k0 = lane * per, k1 = min(ntiny + 1, k0 + per);
        PvSlot sq{-1, -1, cmk(0, 0), cmk(0, 0), cmk(0, 0), cmk(0, 0)};
        const float ut0 = (float)(1.0 + (pr + capDelta - S.ppar[1]) * S.idppar), dut = (float)(corr * smdelta * S.idppar);
        for (int k = k0; k < k1; ++k) {
          double p, dx;
          double2 K;
          tiny_point(k, p, dx, K);
          const float ut = fmaf((float)k, dut, ut0);
          const int ct = clampj(off_half(ut) ? node_of(ut) : piece_raw(p));
          put(sq, ct, dx, K, 1);
        }
        records(2, sq, 1);
      }
      const bool merged = !__any_sync(0xffffffffu, bad) && nruns <= 32;
      if (merged && nruns > 0) {
        __syncwarp();
        // run totals in (lane, slot) order: the run's first slot, then slot 0
        // of the following lanes up to the next run start of its group
        if (lane < nruns) {
          const int L = runL[lane], sl = runS[lane], gi = runG[lane];
          int Ln = nl[0], sn = 0;
          if (gi == 1) Ln = nl[1];
          if (gi == 2) Ln = nl[2];
          if (lane + 1 < nruns && runG[lane + 1] == gi) {
            Ln = runL[lane + 1];
            sn = runS[lane + 1];
          }
          double2 A = recv[rec_at(gi, L, sl, 0)], B = recv[rec_at(gi, L, sl, 1)];
          for (int L2 = L + 1; L2 < Ln || (L2 == Ln && sn == 1); ++L2) {
            A = cadd(A, recv[rec_at(gi, L2, 0, 0)]);
            B = cadd(B, recv[rec_at(gi, L2, 0, 1)]);
          }
          runJ[lane] = recj[recj_at(gi, L, sl)];
          runv[lane * 2] = A;
          runv[lane * 2 + 1] = B;
        }
        __syncwarp();
        // (run, entry) pairs: h A + s B, mirrored runs with the minus sign;
        // the products overwrite the lane records
        double2* contrib = recv;
        for (int q = lane; q < nruns * 6; q += 32) {
          const int rho = q / 6, e = q % 6;
          const int jc = runJ[rho];
          double2 h, sl;
          node1(jc, e, h, sl);
          const double2 A = runv[rho * 2];
          const double2 B = cadd(runv[rho * 2 + 1], cscale(A, pr - S.ppar[jc]));
          double2 t = cadd(cmul(h, A), cmul(sl, B));
          contrib[q] = (runG[rho] == 1) ? cmk(-t.x, -t.y) : t;
        }
        __syncwarp();
        // component c of T: the runs in order
        double acc = 0.0;
        if (lane < 12) {
          const int e = lane >> 1;
          for (int rho = 0; rho < nruns; ++rho) acc += (lane & 1) ? contrib[rho * 6 + e].y : contrib[rho * 6 + e].x;
        }
  #pragma unroll
        for (int e = 0; e < 6; ++e) {
          const double tx = __shfl_sync(0xffffffffu, acc, 2 * e), ty = __shfl_sync(0xffffffffu, acc, 2 * e + 1);
          T[e] = cadd(T[e], cmk(tx, ty));
        }
      } else if (!merged) {
        // per-lane piece sums flushed as the piece changes, then a warp sum
        struct Acc {
          int jc;
          double2 A, B;
        };
        auto flush = [&](Acc& q, double sign) {
          if (q.jc < 0) return;
          double2 h[6], sl[6];
          node(q.jc, h, sl);
  #pragma unroll
          for (int e = 0; e < 6; ++e) {
            double2 t = cadd(cmul(h[e], q.A), cmul(sl[e], q.B));
            T[e] = cmk(fma(sign, t.x, T[e].x), fma(sign, t.y, T[e].y));
          }
          q.A = q.B = cmk(0.0, 0.0);
        };
        auto add = [&](Acc& q, int jc, double p, double2 c, double sign) {
          if (jc != q.jc) {
            flush(q, sign);
            q.jc = jc;
          }
          double dx = p - S.ppar[jc];
          q.A = cadd(q.A, c);
          q.B = cmk(fma(c.x, dx, q.B.x), fma(c.y, dx, q.B.y));
        };
        if (sym) {
          const int per = (NP + 31) / 32;
          const int k0 = lane * per, k1 = min(NP, k0 + per);
          Acc up{-1, cmk(0, 0), cmk(0, 0)}, dn{-1, cmk(0, 0), cmk(0, 0)};
          int ju = -1, jd = -1;
          for (int k = k0; k < k1; ++k) {
            double p, dx;
            double2 K;
            sym_point(k, p, dx, K);
            const double pm = 2.0 * pr - p;
            ju = (ju < 0) ? piece_raw(p) : piece_up(ju, p);
            jd = (jd < 0) ? piece_raw(pm) : piece_down(jd, pm);
            add(up, clampj(ju), p, K, 1.0);
            add(dn, clampj(jd), pm, cmk(K.x, -K.y), -1.0);
          }
          flush(up, 1.0);
          flush(dn, -1.0);
        }
        if (ntiny > 0) {
          const int per = (ntiny + 1 + 31) / 32;
          const int k0 = lane * per, k1 = min(ntiny + 1, k0 + per);
          Acc q{-1, cmk(0, 0), cmk(0, 0)};
          int jt = -1;
          for (int k = k0; k < k1; ++k) {
            double p, dx;
            double2 K;
            tiny_point(k, p, dx, K);
            jt = (jt < 0) ? piece_raw(p) : piece_up(jt, p);
            add(q, clampj(jt), p, K, 1.0);
          }
          flush(q, 1.0);
        }
        for (int e = 0; e < 6; ++e)
          for (int off = 16; off > 0; off >>= 1) {
            T[e].x += __shfl_xor_sync(0xffffffffu, T[e].x, off);
            T[e].y += __shfl_xor_sync(0xffffffffu, T[e].y, off);
          }
      }
      // G = K_e H with K_e = -(q/kpar) pref_e / 2; result 2 pi T smdelta dpperp/4
      double scale = 2.0 * ALPS_PI * smdelta * S.dpperp * 0.25 * (-S.qk * 0.5);
      // lane 0 holds the whole T; lanes 0-5 add entry e
      if (lane == 0)
        for (int e = 0; e < 6; ++e) tb[e] = T[e];
      __syncwarp();
      if (lane < 6 && !(n == 0 && (lane == 0 || lane == 3 || lane == 4)))
        out[lane] = cadd(out[lane], cscale(cmul(item_pref(it, lane), tb[lane]), scale));
      __syncwarp();
      }  // FP64 code
    }

    if (wk & 2) {
      const double2 p = cmk(it.pr, it.pim);
      const double pd = S.dppar_abs, dpp = S.dpperp;
      const double vA = a.sys.vA;
      if (S.fit_aux) {
        // Maxwellian terms: f = sum_f a0 exp(-p2 (p - p3)^2)
        const int nf = S.nf;
        for (int i = lane; i <= N; i += 32) {
          double2 f0 = cmk(0, 0), fp = cmk(0, 0), fm = cmk(0, 0);
          for (int f = 0; f < nf; ++f) {
            const double* aux = S.fit_aux + ((size_t)i * nf + f) * 4;  // a0, p2, p3, exp(-p2 D^2)
            double p2 = aux[1];
            double2 d = cmk(p.x - aux[2], p.y);
            double2 E0 = cexp_d(cscale(cmul(d, d), -p2));
            double2 G = cscale(E0, aux[0]);
            double2 ax = cscale(d, -2.0 * p2 * pd);
            double2 X, Xi;
            if (fabs(ax.x) < 600.0) {
              X = cexp_d(ax);
              Xi = crcp(X);
              double2 Gc = cscale(G, aux[3]);
              fp = cadd(fp, cmul(Gc, X));
              fm = cadd(fm, cmul(Gc, Xi));
            } else {
              double2 dp = cadd(d, cmk(pd, 0.0)), dm = csub(d, cmk(pd, 0.0));
              fp = cadd(fp, cscale(cexp_d(cscale(cmul(dp, dp), -p2)), aux[0]));
              fm = cadd(fm, cscale(cexp_d(cscale(cmul(dm, dm), -p2)), aux[0]));
            }
            f0 = cadd(f0, G);
          }
          frow[i] = f0;
          fpr[i] = fp;
          fmr[i] = fm;
        }
      } else {
        for (int i = lane; i <= N; i += 32) {
          frow[i] = eval_fit_d(S, vA, i, p);
          fpr[i] = eval_fit_d(S, vA, i, cadd(p, cmk(pd, 0.0)));
          fmr[i] = eval_fit_d(S, vA, i, csub(p, cmk(pd, 0.0)));
        }
      }
      __syncwarp();
      bool zero = false;
      double2 sums[3] = {cmk(0, 0), cmk(0, 0), cmk(0, 0)};
      const double ql = S.qs / fabs(kpar);
      const int L = N + 1;
      for (int i = lane; i <= N; i += 32) {
        double2 fpi = fpr[i], fpf = fmr[i];
        double2 dfperp, dfpar;
        double h;
        if (i == 0) {
          dfperp = cscale(csub(frow[1], frow[0]), 1.0 / dpp);
          h = 0.5;
        } else if (i == N) {
          dfperp = cscale(csub(frow[N], frow[N - 1]), 1.0 / dpp);
          h = 0.5;
        } else {
          if (cabs_(fpi) == 0.0 || cabs_(fpf) == 0.0 || cabs_(frow[i + 1]) == 0.0) zero = true;
          dfperp = cscale(csub(frow[i + 1], frow[i - 1]), 1.0 / (2.0 * dpp));
          h = (i == N - 1) ? 0.5 : 1.0;
        }
        dfpar = cscale(csub(fpi, fpf), 1.0 / (2.0 * pd));
        double pp_i = S.pperp[i];
        // (q/|kpar|) ((pperp dfpar - p dfperp) kpar/m + omega dfperp)
        double2 Lv = cscale(cadd(cscale(csub(cscale(dfpar, pp_i), cmul(p, dfperp)), kpar / S.ms), cmul(o, dfperp)),
                            ql);
        double J = S.bessel[(size_t)(n + 1) * L + i];
        double Jp = (n == 0) ? -S.bessel[(size_t)2 * L + i]
                             : 0.5 * (S.bessel[(size_t)n * L + i] - S.bessel[(size_t)(n + 2) * L + i]);
        sums[0] = cadd(sums[0], cscale(Lv, h * (J * J)));
        sums[1] = cadd(sums[1], cscale(Lv, h * ((pp_i * pp_i) * Jp * Jp)));
        sums[2] = cadd(sums[2], cscale(Lv, h * (pp_i * J * Jp)));
      }
      zero = __any_sync(0xffffffffu, zero);
      for (int F = 0; F < 3; ++F)
        for (int off = 16; off > 0; off >>= 1) {
          sums[F].x += __shfl_xor_sync(0xffffffffu, sums[F].x, off);
          sums[F].y += __shfl_xor_sync(0xffffffffu, sums[F].y, off);
        }
      if (!zero) {
        // landau_e = -pref_e c_e(p) Sigma_F(e) * i dpperp 2 pi^2, lanes 0-5
        if (lane == 0)
          for (int F = 0; F < 3; ++F) tb[F] = sums[F];
        __syncwarp();
        if (lane < 6 && !(n == 0 && (lane == 0 || lane == 3 || lane == 4))) {
          const int e = lane;
          const double2 ce = (e == 2) ? cmul(p, p) : ((e == 4 || e == 5) ? p : cmk(1.0, 0.0));
          const int fam = (e == 1) ? 1 : ((e == 3 || e == 5) ? 2 : 0);
          const double2 ifac = cmk(0.0, -dpp * ALPS_PI * 2.0 * ALPS_PI * (double)lf);
          const double2 land = cmul(cmul(item_pref(it, e), ce), tb[fam]);
          out[e] = cadd(out[e], cmul(land, ifac));
        }
        __syncwarp();
      }
    }
    __syncwarp();  // the next item reuses the window and the records
  }
      // the items beyond this batch move to the front of the queue
      const int rest = qn - nb;
      const int keep = (lane < rest) ? queue[nb + lane] : 0;
      __syncwarp();
      if (lane < rest) queue[lane] = keep;
      __syncwarp();
      qn = rest;
    }
  }
}

// ---------------------------------------------------------------------------
// chi, epsilon, wave tensor, det (src/ALPS_fns.f90:500-626)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void finalize_body(const DispArgs& a, const DispShape& sh, const double2* __restrict__ om,
                                              int n_om, const double2* __restrict__ part,
                                              const double2* __restrict__ low, const int* __restrict__ count,
                                              const int* __restrict__ slot_nn, const double2* __restrict__ items,
                                              const double2* __restrict__ rel, const double2* __restrict__ bmres,
                                              double2* D, double2* ext, int w, bool warp_mode) {
  if (w >= n_om) return;
  // warp_mode: the 32 lanes of a warp share one omega; they split the sums
  // over order chunks and run the rest redundantly, lane 0 writes
  const int lane = threadIdx.x & 31, lstep = warp_mode ? 32 : 1, l0 = warp_mode ? lane : 0;
  auto wsum = [&](double2& v) {
    if (warp_mode)
      for (int off = 16; off > 0; off >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, off);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, off);
      }
  };
  const int S_ = a.sys.nspec;
  const double2 o = om[w];
  double2 eps[6];
  for (int e = 0; e < 6; ++e) eps[e] = cmk(0.0, 0.0);
  const double kperp = a.sys.kperp, kpar = a.sys.kpar, vA = a.sys.vA;
  double2 denom = cmul(o, o);
  denom = a.sys.kperp_norm ? cscale(cscale(denom, vA), vA) : cscale(cscale(cscale(cscale(denom, vA), vA), kperp), kperp);
  for (int s = 0; s < S_; ++s) {
    const SpecDev& S = a.sp[s];
    double2 chi[6], cl[3][6];
    for (int e = 0; e < 6; ++e) {
      chi[e] = cmk(0.0, 0.0);
      for (int l = 0; l < 3; ++l) cl[l][e] = cmk(0.0, 0.0);
    }
    size_t base = ((size_t)w * S_ + s) * sh.nchunk;
    // small batches leave one partial per order: unrolled, so that the
    // loads of several chunks are in flight at once
#pragma unroll 4
    for (int ch = l0; ch < sh.nchunk; ch += lstep)
      for (int e = 0; e < 6; ++e) chi[e] = cadd(chi[e], part[(base + ch) * 6 + e]);
    if (ext && low)
      for (int ch = l0; ch < sh.nchunk; ch += lstep)
        for (int l = 0; l < 3; ++l)
          for (int e = 0; e < 6; ++e) cl[l][e] = cadd(cl[l][e], low[((base + ch) * 3 + l) * 6 + e]);
    int cnt = count[(size_t)w * S_ + s];
    for (int r = l0; r < cnt; r += lstep) {
      size_t ib = ((size_t)w * S_ + s) * a.rcap + r;
      int nn = slot_nn[ib];
      for (int e = 0; e < 6; ++e) {
        double2 v = items[ib * 6 + e];
        chi[e] = cadd(chi[e], v);
        if (nn == -1) cl[0][e] = cadd(cl[0][e], v);
        if (nn == 0) cl[1][e] = cadd(cl[1][e], v);
        if (nn == 1) cl[2][e] = cadd(cl[2][e], v);
      }
    }
    // warp mode: each lane summed its share of the chunks and items
    for (int e = 0; e < 6; ++e) wsum(chi[e]);
    if (ext)
      for (int l = 0; l < 3; ++l)
        for (int e = 0; e < 6; ++e) wsum(cl[l][e]);
    if (S.bm) {
      // NHDS chi, divided by n q before the common normalisation as in disp
      // (src/ALPS_fns.f90:344-358); no ee term
      const double2* b = bmres + ((size_t)w * S_ + s) * 24;
      const double nq = S.ns * S.qs;
      for (int e = 0; e < 6; ++e) chi[e] = cadd(chi[e], cmk(b[e].x / nq, b[e].y / nq));
      for (int l = 0; l < 3; ++l)
        for (int e = 0; e < 6; ++e) cl[l][e] = cmk(b[6 + 6 * l + e].x / nq, b[6 + 6 * l + e].y / nq);
    } else if (S.relat) {
      // orders in the reference's order; n = 0 adds yy, zz, yz only, and the
      // ee term goes into chi alone (src/ALPS_fns.f90:461-497)
      for (int n = 0; n <= S.nmax; ++n) {
        // the row blocks' partial sums of +n and -n, added in order
        const double2* base = rel + ((((size_t)w * S_ + s) * a.relcap + n) * 2 + 0) * REL_RB * 6;
        double2 pl[6], mi[6];
        for (int e = 0; e < 6; ++e) {
          pl[e] = base[e];
          mi[e] = base[REL_RB * 6 + e];
          for (int q = 1; q < REL_RB; ++q) {
            pl[e] = cadd(pl[e], base[q * 6 + e]);
            mi[e] = cadd(mi[e], base[(REL_RB + q) * 6 + e]);
          }
        }
        if (n == 0) {
          const int e0[3] = {1, 2, 5};
          for (int q = 0; q < 3; ++q) {
            chi[e0[q]] = cadd(chi[e0[q]], pl[e0[q]]);
            cl[1][e0[q]] = pl[e0[q]];
          }
        } else {
          for (int e = 0; e < 6; ++e) {
            if (n == 1) {
              cl[2][e] = pl[e];
              cl[0][e] = mi[e];
              chi[e] = cadd(chi[e], cadd(pl[e], mi[e]));
            } else {
              chi[e] = cadd(cadd(chi[e], pl[e]), mi[e]);
            }
          }
        }
      }
      double ee = a.sys.kperp_norm ? S.int_ee_rel : kperp * kperp * S.int_ee_rel;
      chi[2] = cadd(chi[2], cmk(ee, 0.0));
    } else {
      double ee = a.sys.kperp_norm ? S.int_ee : kperp * kperp * S.int_ee;
      chi[2] = cadd(chi[2], cmk(ee, 0.0));
      cl[1][2] = cadd(cl[1][2], cmk(ee, 0.0));
    }
    double norm = S.ns * S.qs;
    for (int e = 0; e < 6; ++e) {
      chi[e] = cscale(chi[e], norm);
      for (int l = 0; l < 3; ++l) cl[l][e] = cscale(cl[l][e], norm);
      eps[e] = cadd(eps[e], chi[e]);
    }
    if (ext && l0 == 0) {
      // chi0 (S x 3 x 3) then chi0_low (S x 3 x 3 x 3), then wave (9)
      double2* c0 = ext + (size_t)w * (S_ * 36 + 9) + s * 9;
      const int ii[6] = {0, 1, 2, 0, 0, 1}, jj[6] = {0, 1, 2, 1, 2, 2};
      double2 t[9];
      for (int e = 0; e < 6; ++e) t[3 * ii[e] + jj[e]] = cdiv(chi[e], denom);
      t[3] = cneg(t[1]);
      t[6] = t[2];
      t[7] = cneg(t[5]);
      for (int q = 0; q < 9; ++q) c0[q] = t[q];
      double2* c1 = ext + (size_t)w * (S_ * 36 + 9) + S_ * 9 + s * 27;
      for (int l = 0; l < 3; ++l) {
        double2 u[9];
        for (int e = 0; e < 6; ++e) u[3 * ii[e] + jj[e]] = cdiv(cl[l][e], denom);
        u[3] = cneg(u[1]);
        u[6] = u[2];
        u[7] = cneg(u[5]);
        for (int q = 0; q < 9; ++q) c1[l * 9 + q] = u[q];
      }
    }
  }
  // eps entries: xx yy zz xy xz yz
  double2 unit = a.sys.kperp_norm ? cmul(cscale(o, vA), cscale(o, vA))
                                  : cmul(cscale(cscale(o, kperp), vA), cscale(cscale(o, kperp), vA));
  double enx2, enz2, enxnz;
  if (a.sys.kperp_norm) {
    enx2 = kperp * kperp;
    enz2 = kpar * kpar;
    enxnz = kpar * kperp;
  } else {
    enx2 = kperp * kperp * kperp * kperp;
    enz2 = kpar * kpar * kperp * kperp;
    enxnz = kpar * kperp * kperp * kperp;
  }
  double2 w11 = csub(cadd(eps[0], unit), cmk(enz2, 0.0));
  double2 w22 = csub(csub(cadd(eps[1], unit), cmk(enz2, 0.0)), cmk(enx2, 0.0));
  double2 w33 = csub(cadd(eps[2], unit), cmk(enx2, 0.0));
  double2 w13 = cadd(eps[4], cmk(enxnz, 0.0));
  double2 w12 = eps[3];
  double2 w23 = eps[5];
  double2 det = cadd(cadd(csub(cadd(cmul(w11, cadd(cmul(w22, w33), cmul(w23, w23))),
                                    cscale(cmul(cmul(w12, w23), w13), 2.0)),
                               cmul(cmul(w13, w13), w22)),
                          cmul(cmul(w12, w12), w33)),
                     cmk(0.0, 0.0));
  if (l0 == 0) D[w] = det;
  if (ext && l0 == 0) {
    double2* wv = ext + (size_t)w * (S_ * 36 + 9) + S_ * 36;
    wv[0] = w11;
    wv[1] = w12;
    wv[2] = w13;
    wv[3] = cneg(w12);
    wv[4] = w22;
    wv[5] = w23;
    wv[6] = w13;
    wv[7] = cneg(w23);
    wv[8] = w33;
  }
}


// ---------------------------------------------------------------------------
// Jobs.  Every batch, of one context or fused over many, runs the same four
// kernels over a table of jobs in device memory: each kernel's grid is the
// concatenation of the jobs' own grids, and a block finds its job by the
// first block of each job.  A job's arguments (the context at its k) and its
// launch shape are those of a lone batch of its size, and one compiled
// kernel serves every case, so a context's results do not depend on what it
// was batched with, bit for bit.
// ---------------------------------------------------------------------------
struct DispJob {
  const DispArgs* a;  // the context's arguments (device copy)
  DispShape sh;
  int n, js, tiles, S;
  long blk[4];        // first block of the job in classify, pole sums, resonant, finalize
  const double2* om;
  double2* D;
  double2* part;
  int* count;
  int* slot_nn;
  double2* items;
  int* flags;
  double2* low;       // chi_low partials (calc_eigen) or null
  double2* ext;       // chi0, chi0_low, wave per omega, or null
  const double2* rel; // relativistic orders, or null
  const double2* bm;  // closed-form species, or null
};

// stores a lone batch's arguments and job where its kernels read them
__global__ void k_stage(DispArgs a, DispJob j, DispArgs* da, DispJob* dj) {
  const int4* src = reinterpret_cast<const int4*>(&a);
  int4* dst = reinterpret_cast<int4*>(da);
  for (int q = threadIdx.x; q < (int)(sizeof(DispArgs) / sizeof(int4)); q += blockDim.x) dst[q] = src[q];
  if (threadIdx.x == 0) {
    j.a = da;
    *dj = j;
  }
}

__device__ __forceinline__ const DispJob& job_of(const DispJob* jobs, int nj, long b, int k) {
  int lo = 0, hi = nj - 1;  // last job whose first block is <= b
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].blk[k] <= b) lo = mid;
    else hi = mid - 1;
  }
  return jobs[lo];
}

// k_finalize: one warp per omega when a batch leaves many order chunks
// (small batches), one thread per omega otherwise
__host__ __device__ inline bool fin_warp_mode(const DispShape& sh) { return sh.nchunk >= 8; }
__host__ __device__ inline long fin_blocks(const DispShape& sh, int n) {
  return fin_warp_mode(sh) ? (n + 3) / 4 : (n + 127) / 128;
}

// A block's job is one context: its arguments go to shared memory once, and
// every thread reads them there.
__device__ __forceinline__ const DispArgs& stage_args(const DispArgs* src, DispArgs& dst) {
  const int4* s4 = reinterpret_cast<const int4*>(src);
  int4* d4 = reinterpret_cast<int4*>(&dst);
  for (int q = threadIdx.x; q < (int)(sizeof(DispArgs) / sizeof(int4)); q += blockDim.x) d4[q] = s4[q];
  __syncthreads();
  return dst;
}

#define CLS_PER_WARP 8
// blocks of 128 threads of k_classify_multi for n omegas and S species
__host__ __device__ inline long cls_blocks(long n, int S_) { return (n * S_ + 4 * CLS_PER_WARP - 1) / (4 * CLS_PER_WARP); }

__global__ void k_classify_multi(const DispJob* __restrict__ jobs, int nj) {
  __shared__ DispArgs sa;
  const DispJob& J = job_of(jobs, nj, blockIdx.x, 0);
  const DispArgs& a = stage_args(J.a, sa);
  const long lb = (long)blockIdx.x - J.blk[0];
  // CLS_PER_WARP (omega, species) pairs per warp: the block's argument
  // staging is shared by more pairs
  const long w0 = ((lb * blockDim.x + threadIdx.x) >> 5) * CLS_PER_WARP;
  for (int q = 0; q < CLS_PER_WARP; ++q) classify_body(a, J.om, J.n, J.count, J.slot_nn, J.flags, w0 + q);
}

// copies n bytes (a multiple of 16) from global to shared memory
__device__ __forceinline__ void stage_bytes(const void* src, void* dst, int n) {
  const int4* s4 = reinterpret_cast<const int4*>(src);
  int4* d4 = reinterpret_cast<int4*>(dst);
  for (int q = threadIdx.x; q < n / 16; q += blockDim.x) d4[q] = s4[q];
}

// A pole-sums block works on one species: it stages the system constants
// and that species' constants only (an eighth of DispArgs), which matters
// when a fused round has many small jobs, each of many small blocks.
template <bool LOW>
__global__ void __launch_bounds__(128, 3) k_pole_sums_multi(const DispJob* __restrict__ jobs, int nj) {
  __shared__ __align__(16) SysDev ssys;
  __shared__ __align__(16) SpecDev sspec;
  const DispJob& J = job_of(jobs, nj, blockIdx.x, 1);
  const long lb = (long)blockIdx.x - J.blk[1];
  const int tile = (int)(lb % J.tiles), s = (int)((lb / J.tiles) % J.S), chunk = (int)(lb / ((long)J.tiles * J.S));
  stage_bytes(&J.a->sys, &ssys, sizeof(SysDev));
  stage_bytes(&J.a->sp[s], &sspec, sizeof(SpecDev));
  __syncthreads();
  pole_body<LOW>(ssys, sspec, J.sh, J.om, J.n, J.js, J.part, J.low, tile, s, chunk);
}

__global__ void __launch_bounds__(RES_WARPS * 32, 3) k_resonant_multi(const DispJob* __restrict__ jobs, int nj) {
  __shared__ DispArgs sa;
  const DispJob& J = job_of(jobs, nj, blockIdx.x, 2);
  const DispArgs& a = stage_args(J.a, sa);
  resonant_body(a, J.sh, J.om, J.n, J.count, J.slot_nn, J.items, (long)blockIdx.x - J.blk[2]);
}

__global__ void k_finalize_multi(const DispJob* __restrict__ jobs, int nj) {
  __shared__ DispArgs sa;
  const DispJob& J = job_of(jobs, nj, blockIdx.x, 3);
  const DispArgs& a = stage_args(J.a, sa);
  const long lb = (long)blockIdx.x - J.blk[3];
  const bool wm = fin_warp_mode(J.sh);
  const long w = wm ? lb * (blockDim.x / 32) + threadIdx.x / 32 : lb * blockDim.x + threadIdx.x;
  finalize_body(a, J.sh, J.om, J.n, J.part, J.low, J.count, J.slot_nn, J.items, J.rel, J.bm, J.D, J.ext, (int)w,
                wm);
}

template <typename T>
int ensure_buf(T*& ptr, size_t& cap, size_t n) {
  if (n <= cap && ptr) return ALPS_OK;
  // a buffer that grows again grows by half its size at least: each
  // regrowth frees the old buffer, and cudaFree waits for the whole device
  // (in the request server, for every request in flight)
  const size_t want = ptr ? std::max(n, cap + cap / 2) : n;
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  cap = 0;
  ALPS_CUDA_TRY(cudaMalloc(&ptr, (want ? want : 1) * sizeof(T)));
  cap = want;
  return ALPS_OK;
}

}  // namespace

void fill_sys_dev(const alps_ctx* c, SysDev* o) {
  o->nspec = c->sys.nspec;
  o->kperp_norm = c->sys.kperp_norm;
  o->M_I = c->sys.positions_principal;
  o->M_P = c->sys.n_resonance_interval;
  o->Tlim = c->sys.Tlim;
  o->vA = c->sys.vA;
  o->kperp = c->kperp;
  o->kpar = c->kpar;
  o->ikpar = 1.0 / c->kpar;
}

void fill_spec_dev(const alps_ctx* c, int is, SpecDev* o) {
  const SpeciesHost& S = c->spec[is];
  o->N = c->sys.nperp;
  o->M = c->sys.npar;
  o->nmax = S.nmax;
  o->nf = S.sp.ac_method == 1 ? S.sp.n_fits : 1;
  o->ac_method = S.sp.ac_method;
  o->log_fit = S.sp.log_fit;
  for (int f = 0; f < ALPS_MAX_FITS; ++f) {
    o->fit_type[f] = S.sp.fit_type[f];
    o->perp_corr[f] = S.sp.perp_correction[f];
  }
  o->qs = S.sp.qs;
  o->ms = S.sp.ms;
  o->ns = S.sp.ns;
  const bool bm = S.sp.use_bM != 0;
  o->dpperp = bm ? 0.0 : S.pperp[2] - S.pperp[1];
  o->dppar = bm ? 0.0 : S.ppar[2] - S.ppar[1];
  o->dppar_abs = std::fabs(o->dppar);
  o->idppar = bm ? 0.0 : 1.0 / o->dppar;
  o->hidpa = bm ? 0.0 : 0.5 / o->dppar_abs;
  o->qk = S.sp.qs / c->kpar;
  o->species_index = is + 1;
  o->int_ee = S.int_ee;
  o->pperp = S.d_pperp;
  o->ppar = S.d_ppar;
  o->f0 = S.d_f0;
  o->g1 = S.d_g1;
  o->g2 = S.d_g2;
  o->fit = S.d_fit;
  o->bessel = S.d_bessel;
  o->V = S.d_V;
  o->mom = S.d_mom;
  o->momf = S.d_momf;
  o->momh = S.d_momh;
  o->moml = S.d_moml;
  o->Vh = S.d_Vh;
  o->Vl = S.d_Vl;
  o->Vscale = S.d_Vscale;
  o->pph = S.d_pph;
  o->ppl = S.d_ppl;
  o->df_sums = (c->precision != ALPS_PREC_FP64 && S.d_Vh) ? 1 : 0;
  {
    const size_t nm = (size_t)(S.nmax + 1), M = (size_t)c->sys.npar;
    const size_t nvf = nm * (M - 1) * 12, nmo = nm * ALPS_KFAR * 12;
    const bool fz = S.d_Bt != nullptr && S.d_Bd != nullptr;
    o->Bt = fz ? S.d_Bt : nullptr;
    o->mBt = fz ? S.d_Bt + nvf : nullptr;
    o->bfac = fz ? S.d_Bt + nvf + nmo : nullptr;
    o->Escale = fz ? S.d_Bd : nullptr;
    o->Cfull = fz ? S.d_Bd + 8 : nullptr;
    o->Pre = fz ? S.d_Bd + 8 + nm * 6 : nullptr;
    o->qlo = S.qlo;
    o->qhi = S.qhi;
    o->qlo_in = S.qlo_in;
    o->qhi_in = S.qhi_in;
  }
  {
    const double kap = c->kpar / S.sp.ms;
    o->kaph = (float)kap;  // round to nearest, as __double2float_rn
    o->kapl = (float)(kap - (double)o->kaph);
    o->hidh = (float)o->hidpa;
    o->hidl = (float)(o->hidpa - (double)o->hidh);
    o->kappa = kap;
    o->dpph = (float)o->dppar;
    o->dppl = (float)(o->dppar - (double)o->dpph);
    o->idph = (float)o->idppar;
    o->idpl = (float)(o->idppar - (double)o->idph);
    const double tpm = 2.0 * ALPS_PI * c->sys.n_resonance_interval;
    o->tpmh = (float)tpm;
    o->tpml = (float)(tpm - (double)o->tpmh);
    o->pvc = 2.0 * ALPS_PI * o->dpperp * 0.25 * (-o->qk * 0.5);
  }
  o->pcen = bm ? 0.0 : 0.5 * (S.ppar[1] + S.ppar[c->sys.npar - 1]);
  o->prad = bm ? 0.0 : 0.5 * (S.ppar[c->sys.npar - 1] - S.ppar[1]);
  o->pcen32 = (float)o->pcen;
  o->prad32 = (float)o->prad;
  // the series is used only where it is cheaper than the node sum
  o->kfar = (c->precision == ALPS_PREC_FP64) ? 0 : std::min(ALPS_KFAR, (int)(0.8 * (c->sys.npar - 1)));
  o->rcap = S.rcap;
  o->fit_aux = S.d_fit_aux;
  o->lmom = (S.lfact && c->precision != ALPS_PREC_FP64) ? S.d_lmom : nullptr;
  o->p2r = S.p2r;
  o->p3r = S.p3r;
  o->la = S.la;
  o->lb = S.lb;
  o->lc = S.lc;
  o->min_a0 = S.min_a0;
  o->lgc = std::exp(-S.p2r * o->dppar * o->dppar);  // dppar is 0 for closed-form species (no grid)
  o->lmomf = o->lmom ? reinterpret_cast<const float*>(S.d_lmom + (size_t)(S.nmax + 1) * 30) : nullptr;
  o->la32 = (float)S.la;
  o->lb32 = (float)S.lb;
  o->lc32 = (float)S.lc;
  o->lgch = (float)o->lgc;
  o->lgcl = (float)(o->lgc - (double)o->lgch);
  o->lcx = -2.0 * S.p2r * o->dppar_abs;
  o->lze = (S.min_a0 > 0.0 && std::isfinite(S.min_a0)) ? std::ilogb(S.min_a0) : 0;
  o->lge = (o->lgc > 0.0) ? std::ilogb(o->lgc) : -2000;
  o->relat = S.sp.relat ? 1 : 0;
  o->ng = c->sys.ngamma;
  o->np = c->sys.npparbar;
  o->grel = S.d_grel;
  o->prel = S.d_prel;
  o->f0rel = S.d_f0rel;
  o->dfr1 = S.d_dfr1;
  o->dfr2 = S.d_dfr2;
  o->jrel = S.d_jrel;
  o->cone = S.d_cone;
  o->int_ee_rel = S.int_ee_rel;
  o->poly_order = S.sp.poly_order;
  o->poly_log_max = S.sp.poly_log_max;
  o->ppar_lo = bm ? 0.0 : S.ppar[0];
  o->ppar_hi = bm ? 0.0 : S.ppar[c->sys.npar];
  o->bm = bm ? 1 : 0;
  o->bm_nrun = S.bm_nrun;
  o->bm_beta = S.sp.bM_betas;
  o->bm_alpha = S.sp.bM_alphas;
  o->bm_pdrift = S.sp.bM_pdrifts;
  o->bmI = S.d_bmI;
}

bool any_bm(const alps_ctx* c) {
  for (int s = 0; s < c->sys.nspec; ++s)
    if (c->spec[s].sp.use_bM) return true;
  return false;
}

// order slots of the relativistic per-order results (0 when no species is)
int rel_capacity(const alps_ctx* c) {
  int cap = 0;
  for (int s = 0; s < c->sys.nspec; ++s)
    if (c->spec[s].sp.relat) cap = std::max(cap, c->spec[s].nmax + 1);
  return cap;
}

int collect_profile(alps_ctx* c) {
  for (auto& ev : c->ev_pending) {
    ALPS_CUDA_TRY(cudaEventSynchronize(ev[4]));
    for (int q = 0; q < 4; ++q) {
      float ms = 0.f;
      ALPS_CUDA_TRY(cudaEventElapsedTime(&ms, ev[q], ev[q + 1]));
      c->prof_ms[q] += ms;
    }
    c->prof_batches++;
    for (auto e : ev) c->ev_pool.push_back(e);
  }
  c->ev_pending.clear();
  return ALPS_OK;
}

// Runs the four kernels of one batch on stream st.
// the arguments of one context at its current k; *maxn = largest nmax
void build_disp_args(const alps_ctx* c, DispArgs* a, int* maxn) {
  fill_sys_dev(c, &a->sys);
  int mx = 0, rc = 1;
  for (int s = 0; s < c->sys.nspec; ++s) {
    fill_spec_dev(c, s, &a->sp[s]);
    mx = std::max(mx, c->spec[s].nmax);
    rc = std::max(rc, c->spec[s].rcap);
  }
  a->rcap = rc;
  a->relcap = rel_capacity(c);
  a->has_bm = any_bm(c) ? 1 : 0;
  *maxn = mx;
}

// ---------------------------------------------------------------------------
// Launch-shape table of the autotuner (alps_autotune).  Per bucket of
// (N_perp, N_par, nmax + 1, batch size), each rounded up to a power of two,
// species count and precision path: the tuned j slices per omega, pole-sum
// blocks per SM and resonant warps per SM.  Batches outside the table take
// the default rule of batch_geom.  A change of the table moves the tuning
// epoch, which retires the server's captured graphs.
// ---------------------------------------------------------------------------
namespace {
std::mutex g_tune_mu;
std::map<std::array<int, 6>, TuneShape> g_tune;
std::atomic<uint64_t> g_tune_epoch{0};
thread_local const TuneShape* t_tune_force = nullptr;  // the autotuner's candidate
int ceil_log2(long v) {
  int b = 0;
  while ((1L << b) < v) ++b;
  return b;
}
std::array<int, 6> tune_key(const alps_ctx* c, int n, int maxn) {
  return {ceil_log2(c->sys.nperp), ceil_log2(c->sys.npar), ceil_log2(maxn + 1), ceil_log2(n), c->sys.nspec,
          c->precision};
}
TuneShape tune_lookup(const alps_ctx* c, int n, int maxn) {
  if (t_tune_force) return *t_tune_force;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (g_tune.empty()) return TuneShape{};
  auto it = g_tune.find(tune_key(c, n, maxn));
  return it == g_tune.end() ? TuneShape{} : it->second;
}
}  // namespace

uint64_t tune_epoch() { return g_tune_epoch.load(); }

// launch shape of a batch of n omegas on a context: j slices and order
// chunks give small batches more pole-sum blocks, up to about four per SM
// (default rule), or the autotuner's shape for the batch's bucket.  The
// shape depends on n, the context and the table only: the slices and
// chunks fix the summation order.
struct BatchGeom {
  int js, tiles;
  size_t nslots;
  DispShape sh;
};
BatchGeom batch_geom(const alps_ctx* c, int n, int S_, int maxn, int rcap) {
  BatchGeom b;
  const TuneShape ts = tune_lookup(c, n, maxn);
  b.js = ts.js ? ts.js : ((n < 32) ? 32 : ((n < 64) ? 4 : ((n < 128) ? 2 : 1)));
  const int TW = 128 / b.js;
  b.tiles = (n + TW - 1) / TW;
  const int want_blocks = 152 * (ts.blocks_per_sm ? ts.blocks_per_sm : 4);
  const int nchunk = std::max(1, std::min(maxn + 1, (want_blocks + b.tiles * S_ - 1) / (b.tiles * S_)));
  b.sh.csize = (maxn + 1 + nchunk - 1) / nchunk;
  // a batch of a few frequencies gives each block at least about 16
  // (frequency, order) pairs: alone it still spreads over enough blocks, and
  // in a fused round of thousands of such batches (the uneven batch, the
  // server) the blocks stay worth their set-up
  if (n < 32) b.sh.csize = std::max(b.sh.csize, std::min(maxn + 1, 16 / std::max(1, n)));
  b.sh.nchunk = (maxn + 1 + b.sh.csize - 1) / b.sh.csize;
  b.nslots = (size_t)n * S_ * rcap;
  b.sh.ipw = res_items_per_warp((long)b.nslots, ts.warps_per_sm ? ts.warps_per_sm : 12);
  return b;
}

namespace {

// the job of a lone batch (first blocks at 0)
DispJob lone_job(const DispShape& sh, int n, int js, int tiles, int S_, const double2* om, double2* D, double2* part,
                 int* count, int* slots, double2* items, int* flags) {
  DispJob j;
  j.a = nullptr;
  j.sh = sh;
  j.n = n;
  j.js = js;
  j.tiles = tiles;
  j.S = S_;
  for (int k = 0; k < 4; ++k) j.blk[k] = 0;
  j.om = om;
  j.D = D;
  j.part = part;
  j.count = count;
  j.slot_nn = slots;
  j.items = items;
  j.flags = flags;
  j.low = nullptr;
  j.ext = nullptr;
  j.rel = nullptr;
  j.bm = nullptr;
  return j;
}

// dynamic shared memory of k_resonant_multi for a context, and the opt-in
// above 48 KB (per kernel, once per size)
size_t res_smem(const alps_ctx* c) {
  return (size_t)RES_WARPS * res_warp_smem(c->sys.nperp, res_win(c->sys.positions_principal)) * sizeof(double2);
}
std::mutex g_res_smem_mu;
size_t g_res_smem_set = 0;
int res_smem_optin(size_t smem) {
  if (smem <= 48 * 1024) return ALPS_OK;
  std::lock_guard<std::mutex> lk(g_res_smem_mu);
  if (g_res_smem_set < smem) {
    ALPS_CUDA_TRY(cudaFuncSetAttribute(k_resonant_multi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    g_res_smem_set = smem;
  }
  return ALPS_OK;
}

}  // namespace

int launch_disp_batch(alps_ctx* c, int n, const double2* d_om, double2* d_D, double2* d_ext, cudaStream_t st) {
  if (n <= 0) return ALPS_OK;
  const int S_ = c->sys.nspec;
  DispArgs a;
  int maxn = 0;
  build_disp_args(c, &a, &maxn);
  const BatchGeom bg = batch_geom(c, n, S_, maxn, a.rcap);
  const DispShape sh = bg.sh;
  const int js = bg.js, tiles = bg.tiles;
  const size_t nslots = bg.nslots;
  int rcode;
  const void* before[8] = {c->d_part, c->d_count, c->d_slot_nn, c->d_items, c->d_low, c->d_rel, c->d_bm, c->d_flags};
  if ((rcode = ensure_buf(c->d_part, c->part_cap, (size_t)n * S_ * sh.nchunk * 6))) return rcode;
  if ((rcode = ensure_buf(c->d_count, c->count_cap, (size_t)n * S_))) return rcode;
  if (nslots * 6 > c->items_cap || !c->d_slot_nn) {
    // the slot table holds items_cap / 6 entries (one per item row of six)
    if ((rcode = ensure_buf(c->d_items, c->items_cap, nslots * 6))) return rcode;
    if (c->d_slot_nn) cudaFree(c->d_slot_nn);
    c->d_slot_nn = nullptr;
    ALPS_CUDA_TRY(cudaMalloc(&c->d_slot_nn, (c->items_cap / 6) * sizeof(int)));
  }
  bool want_low = d_ext != nullptr;
  if (want_low)
    if ((rcode = ensure_buf(c->d_low, c->low_cap, (size_t)n * S_ * sh.nchunk * 18))) return rcode;
  if (a.relcap)
    if ((rcode = ensure_buf(c->d_rel, c->rel_cap, (size_t)n * S_ * a.relcap * 2 * REL_RB * 6))) return rcode;
  if (a.has_bm)
    if ((rcode = ensure_buf(c->d_bm, c->bm_cap, (size_t)n * S_ * 24))) return rcode;
  if (!c->d_flags) ALPS_CUDA_TRY(cudaMalloc(&c->d_flags, sizeof(int)));
  const void* after[8] = {c->d_part, c->d_count, c->d_slot_nn, c->d_items, c->d_low, c->d_rel, c->d_bm, c->d_flags};
  for (int q = 0; q < 8; ++q)
    if (before[q] != after[q]) c->gen++;  // buffer addresses changed: cached graphs are stale
  ALPS_CUDA_TRY(cudaMemsetAsync(c->d_flags, 0, sizeof(int), st));

  std::vector<cudaEvent_t> ev;
  if (c->profiling) {
    for (int q = 0; q < 5; ++q) {
      cudaEvent_t e;
      if (!c->ev_pool.empty()) {
        e = c->ev_pool.back();
        c->ev_pool.pop_back();
      } else {
        ALPS_CUDA_TRY(cudaEventCreate(&e));
      }
      ev.push_back(e);
    }
    ALPS_CUDA_TRY(cudaEventRecord(ev[0], st));
  }
  if (!c->d_args) {
    ALPS_CUDA_TRY(cudaMalloc(&c->d_args, sizeof(DispArgs)));
    ALPS_CUDA_TRY(cudaMallocHost(&c->h_args, sizeof(DispArgs)));
  }
  if (!c->d_job) ALPS_CUDA_TRY(cudaMalloc(&c->d_job, sizeof(DispJob)));
  DispJob job = lone_job(sh, n, js, tiles, S_, d_om, d_D, c->d_part, c->d_count, c->d_slot_nn, c->d_items, c->d_flags);
  job.low = want_low ? c->d_low : nullptr;
  job.ext = d_ext;
  job.rel = a.relcap ? c->d_rel : nullptr;
  job.bm = a.has_bm ? c->d_bm : nullptr;
  const DispJob* dj = static_cast<const DispJob*>(c->d_job);
  k_stage<<<1, 128, 0, st>>>(a, job, static_cast<DispArgs*>(c->d_args), static_cast<DispJob*>(c->d_job));
  ALPS_CUDA_TRY(cudaGetLastError());
  c->args_gen = c->gen;  // the device copy is the context at its current state
  c->args_maxn = maxn;
  c->args_rcap = a.rcap;
  k_classify_multi<<<(unsigned)cls_blocks(n, S_), 128, 0, st>>>(dj, 1);
  ALPS_CUDA_TRY(cudaGetLastError());
  if (c->profiling) ALPS_CUDA_TRY(cudaEventRecord(ev[1], st));
  const unsigned g2 = (unsigned)((long)tiles * S_ * sh.nchunk);
  const size_t smem = res_smem(c);
  if ((rcode = res_smem_optin(smem))) return rcode;
  long blocks = ((long)nslots + RES_WARPS * sh.ipw - 1) / (RES_WARPS * sh.ipw);
  if (want_low)
    k_pole_sums_multi<true><<<g2, 128, 0, st>>>(dj, 1);
  else
    k_pole_sums_multi<false><<<g2, 128, 0, st>>>(dj, 1);
  ALPS_CUDA_TRY(cudaGetLastError());
  if (c->profiling) ALPS_CUDA_TRY(cudaEventRecord(ev[2], st));
  k_resonant_multi<<<(unsigned)blocks, RES_WARPS * 32, smem, st>>>(dj, 1);
  ALPS_CUDA_TRY(cudaGetLastError());
  if (a.relcap && (rcode = launch_rel_orders(a.sys, a.sp, a.relcap, n, d_om, c->d_rel, c->d_flags, st)))
    return rcode;
  if (a.has_bm && (rcode = launch_nhds(a.sys, a.sp, n, d_om, c->d_bm, st))) return rcode;
  if (c->profiling) ALPS_CUDA_TRY(cudaEventRecord(ev[3], st));
  k_finalize_multi<<<(unsigned)fin_blocks(sh, n), 128, 0, st>>>(dj, 1);
  ALPS_CUDA_TRY(cudaGetLastError());
  if (c->profiling) {
    ALPS_CUDA_TRY(cudaEventRecord(ev[4], st));
    c->ev_pending.push_back(ev);
  }
  c->stats.n_eval = n;
  c->stats.n_eval_total += n;
  c->stats.kernels_launched = 5 + (a.relcap ? 1 : 0) + (a.has_bm ? 1 : 0);  // k_stage and the four
  return ALPS_OK;
}

// ---------------------------------------------------------------------------
// Fused batches of several contexts (the request server's rounds)
// ---------------------------------------------------------------------------
struct MultiScratch {
  DispJob* d_jobs = nullptr;
  DispJob* h_jobs = nullptr;  // pinned
  size_t jobs_cap = 0;
  double2* part = nullptr;
  size_t part_cap = 0;
  int* count = nullptr;
  size_t count_cap = 0;
  int* slots = nullptr;
  size_t slots_cap = 0;
  double2* items = nullptr;
  size_t items_cap = 0;
};

void multi_scratch_free(MultiScratch* m) {
  if (!m) return;
  cudaFree(m->d_jobs);
  cudaFreeHost(m->h_jobs);
  cudaFree(m->part);
  cudaFree(m->count);
  cudaFree(m->slots);
  cudaFree(m->items);
  delete m;
}

bool ctx_fusable(const alps_ctx* c) { return !rel_capacity(c) && !any_bm(c) && !c->profiling; }

namespace {

// the context's kernel arguments on the device, rebuilt when the plasma, k,
// precision or a table moved (alps_ctx::gen)
int ctx_device_args(alps_ctx* c, cudaStream_t st, const DispArgs** out) {
  if (!c->d_args) {
    ALPS_CUDA_TRY(cudaMalloc(&c->d_args, sizeof(DispArgs)));
    ALPS_CUDA_TRY(cudaMallocHost(&c->h_args, sizeof(DispArgs)));
    c->args_gen = 0;
  }
  if (c->args_gen != c->gen) {
    DispArgs* h = static_cast<DispArgs*>(c->h_args);
    build_disp_args(c, h, &c->args_maxn);
    c->args_rcap = h->rcap;
    ALPS_CUDA_TRY(cudaMemcpyAsync(c->d_args, h, sizeof(DispArgs), cudaMemcpyHostToDevice, st));
    c->args_gen = c->gen;
  }
  *out = static_cast<const DispArgs*>(c->d_args);
  return ALPS_OK;
}

}  // namespace

int launch_disp_multi(alps_ctx* const* ctx, const int* n, int nj, const double2* d_om, double2* d_D, int* d_flags,
                      MultiScratch** scratch, cudaStream_t st) {
  if (nj <= 0) return ALPS_OK;
  MultiLaunch ml;
  int rc = prepare_disp_multi(ctx, n, nj, d_om, d_D, d_flags, scratch, st, &ml);
  if (rc) return rc;
  return run_disp_multi(ml, st);
}

int prepare_disp_multi(alps_ctx* const* ctx, const int* n, int nj, const double2* d_om, double2* d_D, int* d_flags,
                       MultiScratch** scratch, cudaStream_t st, MultiLaunch* out) {
  MultiScratch* m = *scratch;
  if (!m) *scratch = m = new MultiScratch();
  if ((size_t)nj > m->jobs_cap) {
    cudaFree(m->d_jobs);
    cudaFreeHost(m->h_jobs);
    m->d_jobs = nullptr;
    m->h_jobs = nullptr;
    m->jobs_cap = 0;
    ALPS_CUDA_TRY(cudaMalloc(&m->d_jobs, (size_t)nj * sizeof(DispJob)));
    ALPS_CUDA_TRY(cudaMallocHost(&m->h_jobs, (size_t)nj * sizeof(DispJob)));
    m->jobs_cap = nj;
  }
  // shapes, grid offsets and scratch offsets of every job
  std::vector<size_t> o_part(nj), o_count(nj), o_slots(nj);
  size_t part_n = 0, count_n = 0, slots_n = 0, om_off = 0, smem = 0;
  long blk[4] = {0, 0, 0, 0};
  for (int j = 0; j < nj; ++j) {
    alps_ctx* c = ctx[j];
    const DispArgs* da = nullptr;
    int rcode = ctx_device_args(c, st, &da);
    if (rcode) return rcode;
    const int S_ = c->sys.nspec;
    const BatchGeom bg = batch_geom(c, n[j], S_, c->args_maxn, c->args_rcap);
    DispJob& J = m->h_jobs[j];
    J.a = da;
    J.sh = bg.sh;
    J.n = n[j];
    J.js = bg.js;
    J.tiles = bg.tiles;
    J.S = S_;
    J.blk[0] = blk[0];
    blk[0] += cls_blocks(n[j], S_);
    J.blk[1] = blk[1];
    blk[1] += (long)bg.tiles * S_ * bg.sh.nchunk;
    J.blk[2] = blk[2];
    blk[2] += ((long)bg.nslots + RES_WARPS * bg.sh.ipw - 1) / (RES_WARPS * bg.sh.ipw);
    J.blk[3] = blk[3];
    blk[3] += fin_blocks(bg.sh, n[j]);
    J.om = d_om + om_off;
    J.D = d_D + om_off;
    J.flags = d_flags + j;
    J.low = nullptr;
    J.ext = nullptr;
    J.rel = nullptr;
    J.bm = nullptr;
    om_off += n[j];
    o_part[j] = part_n;
    part_n += (size_t)n[j] * S_ * bg.sh.nchunk * 6;
    o_count[j] = count_n;
    count_n += (size_t)n[j] * S_;
    o_slots[j] = slots_n;
    slots_n += bg.nslots;
    smem = std::max(smem, res_smem(c));
  }
  // items per warp of k_resonant from the whole round (it does not change sums)
  const int ipw = res_items_per_warp((long)slots_n);
  blk[2] = 0;
  for (int j = 0; j < nj; ++j) {
    DispJob& J = m->h_jobs[j];
    J.sh.ipw = ipw;
    J.blk[2] = blk[2];
    const long nsl = (long)((j + 1 < nj ? o_slots[j + 1] : slots_n) - o_slots[j]);
    blk[2] += (nsl + RES_WARPS * ipw - 1) / (RES_WARPS * ipw);
  }
  int rcode;
  if ((rcode = ensure_buf(m->part, m->part_cap, part_n))) return rcode;
  if ((rcode = ensure_buf(m->count, m->count_cap, count_n))) return rcode;
  if ((rcode = ensure_buf(m->slots, m->slots_cap, slots_n))) return rcode;
  if ((rcode = ensure_buf(m->items, m->items_cap, slots_n * 6))) return rcode;
  for (int j = 0; j < nj; ++j) {
    DispJob& J = m->h_jobs[j];
    J.part = m->part + o_part[j];
    J.count = m->count + o_count[j];
    J.slot_nn = m->slots + o_slots[j];
    J.items = m->items + o_slots[j] * 6;
  }
  ALPS_CUDA_TRY(cudaMemcpyAsync(m->d_jobs, m->h_jobs, (size_t)nj * sizeof(DispJob), cudaMemcpyHostToDevice, st));
  if ((rcode = res_smem_optin(smem))) return rcode;
  out->jobs = m->d_jobs;
  out->nj = nj;
  for (int k = 0; k < 4; ++k) out->blocks[k] = blk[k];
  out->smem = smem;
  out->flags = d_flags;
  return ALPS_OK;
}

// Where a job's frequency count sits in the device job table: a caller that
// lowers it between launches (alps_solve_many: roots asking for one
// frequency, or finished) makes the kernels skip the other slots, while the
// job's launch shape, and so its sums, stay those of the prepared size.
void disp_job_layout(size_t* stride, size_t* n_offset) {
  *stride = sizeof(DispJob);
  *n_offset = offsetof(DispJob, n);
}

// The kernels of a prepared fused batch (no host work: capturable, also
// inside a conditional graph body).
int run_disp_multi(const MultiLaunch& ml, cudaStream_t st) {
  const DispJob* jobs = static_cast<const DispJob*>(ml.jobs);
  ALPS_CUDA_TRY(cudaMemsetAsync(ml.flags, 0, (size_t)ml.nj * sizeof(int), st));
  k_classify_multi<<<(unsigned)ml.blocks[0], 128, 0, st>>>(jobs, ml.nj);
  ALPS_CUDA_TRY(cudaGetLastError());
  k_pole_sums_multi<false><<<(unsigned)ml.blocks[1], 128, 0, st>>>(jobs, ml.nj);
  ALPS_CUDA_TRY(cudaGetLastError());
  k_resonant_multi<<<(unsigned)ml.blocks[2], RES_WARPS * 32, ml.smem, st>>>(jobs, ml.nj);
  ALPS_CUDA_TRY(cudaGetLastError());
  k_finalize_multi<<<(unsigned)ml.blocks[3], 128, 0, st>>>(jobs, ml.nj);
  ALPS_CUDA_TRY(cudaGetLastError());
  return ALPS_OK;
}

// ===========================================================================
// det D batch without any device allocation.
//
// Some callers cannot let this library allocate device memory while they
// run: a host application whose own caching allocator owns the device heap
// and must see every byte, a real-time loop that cannot afford the implicit
// device-wide synchronisation of cudaMalloc/cudaFree, or a plugin host that
// forbids plugins from creating allocations behind its back.  For them,
// alps_disp_batch_noalloc runs the same kernels as
// alps_disp_batch_device with all of their scratch (partial sums,
// resonant-order slots, resonant results, error flag) carved from the
// file-scope device array below instead of context buffers.
//
// The array is ALPS_NOALLOC_SCRATCH_BYTES (16 MiB) and lives on every device
// that loads this library until the process exits.  Its device address is
// looked up once per device with cudaGetSymbolAddress, by the first call on
// that device (with that device current); make that first call before any
// stream capture.  Every call shares the one array: two calls whose kernels
// overlap on the GPU (different streams, or different host threads) race on
// it and must be ordered by the caller.  The error flag is cleared at the
// start of every call; every other word a call reads it writes first.  The
// flag word's device address is recorded in the context, so
// alps_batch_status reports the call's device errors (read it before the
// next call on the device clears the word).
// ===========================================================================
#define ALPS_NOALLOC_SCRATCH_BYTES (16u << 20)
#define ALPS_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_scratch[ALPS_NOALLOC_SCRATCH_BYTES];

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_addr[ALPS_NOALLOC_MAX_DEVICES] = {nullptr};

// 256-byte aligned carve-out of n bytes from the scratch array
inline size_t carve(size_t& off, size_t bytes) {
  size_t at = (off + 255) & ~(size_t)255;
  off = at + bytes;
  return at;
}
}  // namespace

extern "C" int alps_disp_batch_noalloc(alps_ctx* c, int n, const alps_complex* d_om, alps_complex* d_D,
                                       void* stream, size_t* scratch_bytes) {
  if (!c || n < 0 || !c->kset) return ALPS_E_INVALID;
  if (n == 0) return ALPS_OK;
  if (!d_om || !d_D) return ALPS_E_INVALID;
  int dev = -1;
  ALPS_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= ALPS_NOALLOC_MAX_DEVICES) return ALPS_E_INVALID;
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        alps_set_last_cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
        return ALPS_E_CUDA;
      }
      g_noalloc_addr[dev] = p;
    }
    base = g_noalloc_addr[dev];
  }
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  const int S_ = c->sys.nspec;
  DispArgs a;
  int maxn = 0;
  build_disp_args(c, &a, &maxn);
  const BatchGeom bg = batch_geom(c, n, S_, maxn, a.rcap);
  const DispShape sh = bg.sh;
  const int js = bg.js, tiles = bg.tiles;
  // scratch layout: flags | count | slot_nn | part | items | relativistic orders | NHDS
  size_t off = 0;
  size_t o_flags = carve(off, sizeof(int));
  size_t o_count = carve(off, (size_t)n * S_ * sizeof(int));
  size_t nslots = bg.nslots;
  size_t o_slots = carve(off, nslots * sizeof(int));
  size_t o_part = carve(off, (size_t)n * S_ * sh.nchunk * 6 * sizeof(double2));
  size_t o_items = carve(off, nslots * 6 * sizeof(double2));
  size_t o_rel = carve(off, (size_t)n * S_ * a.relcap * 2 * REL_RB * 6 * sizeof(double2));
  size_t o_bm = carve(off, (size_t)n * S_ * (a.has_bm ? 24 : 0) * sizeof(double2));
  size_t o_args = carve(off, sizeof(DispArgs));
  size_t o_job = carve(off, sizeof(DispJob));
  if (scratch_bytes) *scratch_bytes = off;
  if (off > ALPS_NOALLOC_SCRATCH_BYTES) return ALPS_E_INVALID;  // batch too large for the static scratch
  unsigned char* b = static_cast<unsigned char*>(base);
  int* flags = reinterpret_cast<int*>(b + o_flags);
  int* count = reinterpret_cast<int*>(b + o_count);
  int* slots = reinterpret_cast<int*>(b + o_slots);
  double2* part = reinterpret_cast<double2*>(b + o_part);
  double2* items = reinterpret_cast<double2*>(b + o_items);
  double2* relb = reinterpret_cast<double2*>(b + o_rel);
  double2* bmb = reinterpret_cast<double2*>(b + o_bm);
  const double2* om = reinterpret_cast<const double2*>(d_om);
  double2* D = reinterpret_cast<double2*>(d_D);
  ALPS_CUDA_TRY(cudaMemsetAsync(flags, 0, sizeof(int), st));
  DispJob job = lone_job(sh, n, js, tiles, S_, om, D, part, count, slots, items, flags);
  job.rel = a.relcap ? relb : nullptr;
  job.bm = a.has_bm ? bmb : nullptr;
  DispArgs* da = reinterpret_cast<DispArgs*>(b + o_args);
  DispJob* dj = reinterpret_cast<DispJob*>(b + o_job);
  k_stage<<<1, 128, 0, st>>>(a, job, da, dj);
  ALPS_CUDA_TRY(cudaGetLastError());
  k_classify_multi<<<(unsigned)cls_blocks(n, S_), 128, 0, st>>>(dj, 1);
  ALPS_CUDA_TRY(cudaGetLastError());
  k_pole_sums_multi<false><<<(unsigned)((long)tiles * S_ * sh.nchunk), 128, 0, st>>>(dj, 1);
  ALPS_CUDA_TRY(cudaGetLastError());
  const size_t smem = res_smem(c);
  int rcode0 = res_smem_optin(smem);
  if (rcode0) return rcode0;
  long blocks = ((long)nslots + RES_WARPS * sh.ipw - 1) / (RES_WARPS * sh.ipw);
  k_resonant_multi<<<(unsigned)blocks, RES_WARPS * 32, smem, st>>>(dj, 1);
  ALPS_CUDA_TRY(cudaGetLastError());
  if (a.relcap) {
    int rcode = launch_rel_orders(a.sys, a.sp, a.relcap, n, om, relb, flags, st);
    if (rcode) return rcode;
  }
  if (a.has_bm) {
    int rcode = launch_nhds(a.sys, a.sp, n, om, bmb, st);
    if (rcode) return rcode;
  }
  k_finalize_multi<<<(unsigned)fin_blocks(sh, n), 128, 0, st>>>(dj, 1);
  ALPS_CUDA_TRY(cudaGetLastError());
  c->async_flags = flags;  // alps_batch_status reads the word before the next call clears it
  return ALPS_OK;
}

// ---------------------------------------------------------------------------
// The autotuner: times the candidate launch shapes of a batch of n omegas
// on this context (at its k and precision path) and keeps the fastest for
// the batch's bucket.  Candidates: j slices per omega 1, 2, 4, 8, 16, 32 x
// pole-sum blocks per SM 2, 4, 8 x resonant warps per SM 6, 12, 24, each
// the best of two timed launches after a warm-up on the context's stream.
// A shape changes only the summation order of the pole sums (slices and
// order chunks), never which terms are summed.
// ---------------------------------------------------------------------------
extern "C" int alps_autotune(alps_ctx* c, int n, const alps_complex* d_om_in, alps_tune_result* out) {
  if (!c || !c->kset || n <= 0 || !out) return ALPS_E_INVALID;
  std::memset(out, 0, sizeof(*out));
  double2* d_D = nullptr;
  double2* d_omb = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = ALPS_OK;
  auto fail = [&](int code) {
    rc = code;
    return code;
  };
  const double2* d_om = reinterpret_cast<const double2*>(d_om_in);
  if (cudaMalloc(&d_D, (size_t)n * sizeof(double2)) != cudaSuccess) return ALPS_E_OOM;
  if (!d_om) {
    // a lattice over Re omega in [0.05, 2.5], Im omega in [-0.4, 0.05]
    const int nr = std::max(1, (int)std::ceil(std::sqrt((double)n)));
    std::vector<double2> h(n);
    for (int i = 0; i < n; ++i) {
      const int ir = i % nr, ii = i / nr;
      h[i] = make_double2(0.05 + 2.45 * (ir + 0.5) / nr, -0.4 + 0.45 * (ii + 0.5) / std::max(1, (n + nr - 1) / nr));
    }
    if (cudaMalloc(&d_omb, (size_t)n * sizeof(double2)) != cudaSuccess) {
      cudaFree(d_D);
      return ALPS_E_OOM;
    }
    if (cudaMemcpy(d_omb, h.data(), (size_t)n * sizeof(double2), cudaMemcpyHostToDevice) != cudaSuccess)
      fail(ALPS_E_CUDA);
    d_om = d_omb;
  }
  if (!rc && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) fail(ALPS_E_CUDA);
  DispArgs a;
  int maxn = 0;
  build_disp_args(c, &a, &maxn);
  // best of two timed launches of one shape (nullptr: the default rule)
  auto time_shape = [&](const TuneShape* sh, float* ms) -> int {
    t_tune_force = sh;
    int st = launch_disp_batch(c, n, d_om, d_D, nullptr, c->stream);
    float best = 3.0e38f;
    for (int r = 0; r < 2 && !st; ++r) {
      if (cudaEventRecord(e0, c->stream) != cudaSuccess) st = ALPS_E_CUDA;
      if (!st) st = launch_disp_batch(c, n, d_om, d_D, nullptr, c->stream);
      if (!st && cudaEventRecord(e1, c->stream) != cudaSuccess) st = ALPS_E_CUDA;
      if (!st && cudaEventSynchronize(e1) != cudaSuccess) st = ALPS_E_CUDA;
      float t = 0.0f;
      if (!st && cudaEventElapsedTime(&t, e0, e1) != cudaSuccess) st = ALPS_E_CUDA;
      if (!st) best = std::min(best, t);
    }
    t_tune_force = nullptr;
    *ms = best;
    return st;
  };
  TuneShape best{};
  float t_def = 0.0f, t_best = 3.0e38f;
  if (!rc) rc = time_shape(nullptr, &t_def);
  if (!rc) {
    t_best = t_def;
    const int jsv[6] = {1, 2, 4, 8, 16, 32}, bpv[3] = {2, 4, 8}, wpv[3] = {6, 12, 24};
    for (int x = 0; x < 6 && !rc; ++x)
      for (int y = 0; y < 3 && !rc; ++y)
        for (int z = 0; z < 3 && !rc; ++z) {
          TuneShape cand;
          cand.js = jsv[x];
          cand.blocks_per_sm = bpv[y];
          cand.warps_per_sm = wpv[z];
          float t = 0.0f;
          rc = time_shape(&cand, &t);
          out->candidates++;
          // a candidate replaces the default only when it is 3 % faster
          if (!rc && t < t_best && t < 0.97f * t_def) {
            t_best = t;
            best = cand;
          }
        }
  }
  if (!rc) {
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      g_tune[tune_key(c, n, maxn)] = best;
    }
    g_tune_epoch++;
    const BatchGeom bg = batch_geom(c, n, c->sys.nspec, maxn, a.rcap);
    out->js = bg.js;
    out->blocks_per_sm = best.blocks_per_sm ? best.blocks_per_sm : 4;
    out->warps_per_sm = best.warps_per_sm ? best.warps_per_sm : 12;
    out->tuned = best.js != 0;
    out->ms_default = t_def;
    out->ms_best = t_best;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(d_D);
  if (d_omb) cudaFree(d_omb);
  return rc;
}

extern "C" int alps_tune_clear(void) {
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.clear();
  }
  g_tune_epoch++;
  return ALPS_OK;
}
