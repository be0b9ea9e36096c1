// root_machine.cuh -- the reference's three root finders as plain-data state
// machines that run unchanged on the host and on the device.
//
// A root asks for up to two det D evaluations at a time (want[0..nwant-1]);
// the caller evaluates them (on the device, batched with every other root)
// and feeds the determinants back with root_feed, which advances the
// reference's control flow to the next evaluation it needs.  nwant = 0
// means finished: om is the root, Dfin its det, iter the iterations.
//
//   method 2  secant_osc  src/ALPS_fns.f90:1919-2101
//   method 0  secant      src/ALPS_fns.f90:1815-1917
//   method 1  rtsec       src/ALPS_fns.f90:2105-2195
//
// The reference stops on |D| < D_threshold (absolute; rtsec: |dx| < D_tol).
// With om_rtol > 0 a root also stops once its update is at most
// om_rtol |om| (the update is applied first): the polish criterion for det
// D whose scale keeps |D| from reaching an absolute threshold.  converged
// records whether either rule stopped the root (0: numiter ran out and the
// best-|D| iterate is returned, as in the reference).
//
// Complex arithmetic is spelled out (Smith's division, hypot for the
// modulus, the reference's single-precision constants 0.1 and 1.E-3), so a
// root follows the same iterates wherever the machine runs.
#pragma once

#include <cuda_runtime.h>

#include "alps_internal.cuh"

struct RootParams {
  int numiter;
  double D_threshold, D_prec, D_tol;
  double om_rtol;  // 0: the reference's stopping rules only
};

struct RootState {
  int method, state, iter, osc, nwant, converged;
  double damping;
  double2 om, D, minom, minD, prevom, prev2om, prev3om, prev4om, prevD, jump, delta, Dfin;
  double2 x1, x2, fl, f, xl, dx;  // rtsec (rts is om)
  double2 want[2];
};

namespace rootm {

__host__ __device__ inline double2 rc(double r) { return make_double2(r, 0.0); }
__host__ __device__ inline double cab(double2 a) { return hypot(a.x, a.y); }
// complex / real, component-wise
__host__ __device__ inline double2 cdivr(double2 a, double s) { return make_double2(a.x / s, a.y / s); }

__host__ __device__ inline bool osc_close(double2 a, double2 b) {
  const double thr = (double)1.E-3f;
  return (fabs(a.x - b.x) < fabs(a.x) * thr) && (fabs(a.y - b.y) < fabs(a.y) * thr);
}

__host__ __device__ inline void ask1(RootState& s, double2 a) {
  s.want[0] = a;
  s.nwant = 1;
}
__host__ __device__ inline void ask2(RootState& s, double2 a, double2 b) {
  s.want[0] = a;
  s.want[1] = b;
  s.nwant = 2;
}
__host__ __device__ inline void finish(RootState& s, int conv) {
  s.nwant = 0;
  s.converged = conv;
  s.state = 99;
}

// secant_osc (src/ALPS_fns.f90:1919-2101)
__host__ __device__ inline void step_osc(RootState& s, const RootParams& p, const double2* got) {
  for (;;) {
    switch (s.state) {
      case 0:
        s.delta = make_double2(1.0e-6, 1.0e-8);
        s.state = 1;
        ask1(s, s.om);
        return;
      case 1:
        s.D = got[0];
        s.minom = s.om;
        s.minD = s.D;
        s.prevom = cscale(s.om, 1.0 - p.D_prec);
        s.prev2om = s.prev3om = s.prev4om = s.om;
        s.state = 2;
        ask1(s, s.prevom);
        return;
      case 2:
        s.prevD = got[0];
        if (cab(s.prevD) < cab(s.minD)) {
          s.minom = s.prevom;
          s.minD = s.prevD;
        }
        s.iter = 0;
        s.state = 3;
        break;
      case 3:  // loop head
        if (!(s.iter <= p.numiter - 1)) {
          s.state = 9;
          break;
        }
        s.iter++;
        s.state = 4;
        ask1(s, s.om);
        return;
      case 4:
        s.D = got[0];
        if (cab(csub(s.D, s.prevD)) < 1.0e-80) {
          s.prevom = cadd(s.prevom, rc(1.0e-8));
          s.state = 5;
          ask1(s, s.prevom);
          return;
        }
        s.state = 6;
        break;
      case 5:
        s.prevD = got[0];
        s.state = 6;
        break;
      case 6:
        if (cab(s.D) < p.D_threshold) {
          s.jump = rc(0.0);
          s.Dfin = s.D;
          if (s.iter >= p.numiter) {  // the reference's after-loop rule
            s.om = s.minom;
            s.Dfin = s.minD;
          }
          finish(s, 1);
          return;
        }
        if (s.iter > 4) {
          if (osc_close(s.om, s.prevom) || osc_close(s.om, s.prev2om) || osc_close(s.om, s.prev3om) ||
              osc_close(s.om, s.prev4om)) {
            s.osc++;
            s.damping = fmin(0.5, s.damping * 0.75);
          }
        }
        if (s.osc > 1) {
          s.state = 7;
          ask2(s, cmul(s.om, cadd(rc(1.0), s.delta)), cmul(s.om, csub(rc(1.0), s.delta)));
          return;
        }
        s.jump = cdiv(cmul(cscale(s.D, s.damping), csub(s.om, s.prevom)), csub(s.D, s.prevD));
        s.state = 8;
        break;
      case 7: {
        const double2 Dprime = cdiv(csub(got[0], got[1]), cmul(cscale(s.om, 2.0), s.delta));
        s.jump = cdiv(s.D, cadd(Dprime, cscale(s.D, (double)0.1f)));
        s.state = 8;
        break;
      }
      case 8: {
        const double aom = cab(s.om);
        if (cab(s.jump) > (double)0.1f * aom) s.jump = cscale(cdivr(s.jump, cab(s.jump)), (double)0.1f * aom);
        if (cab(s.D) > cab(s.prevD)) s.jump = cscale(s.jump, (double)0.5f);
        s.prev4om = s.prev3om;
        s.prev3om = s.prev2om;
        s.prev2om = s.prevom;
        s.prevom = s.om;
        s.prevD = s.D;
        if (cab(s.D) < cab(s.minD)) {
          s.minom = s.om;
          s.minD = s.D;
        }
        s.om = csub(s.om, s.jump);
        if (p.om_rtol > 0.0 && cab(s.jump) <= p.om_rtol * aom) {
          s.Dfin = s.D;
          finish(s, 1);
          return;
        }
        s.state = 3;
        break;
      }
      case 9:  // numiter exhausted: the best iterate
        s.om = s.minom;
        s.Dfin = s.minD;
        finish(s, 0);
        return;
      default:
        s.nwant = 0;
        return;
    }
  }
}

// secant (src/ALPS_fns.f90:1815-1917)
__host__ __device__ inline void step_plain(RootState& s, const RootParams& p, const double2* got) {
  for (;;) {
    switch (s.state) {
      case 0:
        s.prevom = cscale(s.om, 1.0 - p.D_prec);
        s.state = 1;
        ask2(s, s.prevom, s.om);
        return;
      case 1:
        s.prevD = got[0];
        s.minD = got[1];
        s.minom = s.om;
        if (cab(s.prevD) < cab(s.minD)) {
          s.minom = s.prevom;
          s.minD = s.prevD;
        }
        s.iter = 0;
        s.state = 2;
        break;
      case 2:
        if (!(s.iter <= p.numiter - 1)) {
          s.om = s.minom;
          s.Dfin = s.minD;
          finish(s, 0);
          return;
        }
        s.iter++;
        s.state = 3;
        ask1(s, s.om);
        return;
      case 3:
        s.D = got[0];
        if (cab(csub(s.D, s.prevD)) < 1.0e-80) {
          s.prevom = cadd(s.prevom, rc(1.0e-8));
          s.state = 4;
          ask1(s, s.prevom);
          return;
        }
        s.state = 5;
        break;
      case 4:
        s.prevD = got[0];
        s.state = 5;
        break;
      case 5: {
        const bool conv = cab(s.D) < p.D_threshold;
        const double aom = cab(s.om);
        s.jump = conv ? rc(0.0) : cdiv(cmul(s.D, csub(s.om, s.prevom)), csub(s.D, s.prevD));
        s.prevom = s.om;
        s.om = csub(s.om, s.jump);
        s.prevD = s.D;
        if (cab(s.D) < cab(s.minD)) {
          s.minom = s.om;
          s.minD = s.D;
        }
        if (conv) {
          s.Dfin = s.D;
          if (s.iter >= p.numiter) {
            s.om = s.minom;
            s.Dfin = s.minD;
          }
          finish(s, 1);
          return;
        }
        if (p.om_rtol > 0.0 && cab(s.jump) <= p.om_rtol * aom) {
          s.Dfin = s.D;
          finish(s, 1);
          return;
        }
        s.state = 2;
        break;
      }
      default:
        s.nwant = 0;
        return;
    }
  }
}

// rtsec (src/ALPS_fns.f90:2105-2195); rts is kept in om
__host__ __device__ inline void step_rtsec(RootState& s, const RootParams& p, const double2* got) {
  for (;;) {
    switch (s.state) {
      case 0:
        s.x1 = cscale(s.om, 1.0);
        s.x2 = cscale(s.om, 1.0 + p.D_prec);
        s.state = 1;
        ask2(s, s.x1, s.x2);
        return;
      case 1:
        s.fl = got[0];
        s.f = got[1];
        if (cab(s.fl) < cab(s.f)) {
          s.om = s.x1;
          s.xl = s.x2;
          const double2 t = s.fl;
          s.fl = s.f;
          s.f = t;
        } else {
          s.xl = s.x1;
          s.om = s.x2;
        }
        s.iter = 0;
        s.state = 2;
        break;
      case 2:
        s.iter++;
        if (s.iter > p.numiter - 1) {
          s.Dfin = s.f;
          finish(s, 0);
          return;
        }
        if (cab(csub(s.f, s.fl)) > 1.0e-40)
          s.dx = cdiv(cmul(csub(s.xl, s.om), s.f), csub(s.f, s.fl));
        else
          s.dx = cdivr(csub(s.x2, s.x1), 25.0);
        s.xl = s.om;
        s.fl = s.f;
        s.om = cadd(s.om, cdivr(s.dx, 2.0));
        s.state = 3;
        ask1(s, s.om);
        return;
      case 3:
        s.f = got[0];
        if ((cab(s.dx) < p.D_tol) || (cab(s.f) == 0.0) || (p.om_rtol > 0.0 && cab(s.dx) <= p.om_rtol * cab(s.om))) {
          s.Dfin = s.f;
          finish(s, 1);
          return;
        }
        s.state = 2;
        break;
      default:
        s.nwant = 0;
        return;
    }
  }
}

}  // namespace rootm

// Starts a root at om: sets the first evaluations it needs.
__host__ __device__ inline void root_start(RootState& s, const RootParams& p, int method, double2 om) {
  s.method = method;
  s.state = 0;
  s.iter = 0;
  s.osc = 0;
  s.nwant = 0;
  s.converged = 0;
  s.damping = 1.0;
  s.om = om;
  s.Dfin = make_double2(0.0, 0.0);
  if (method == 2) rootm::step_osc(s, p, nullptr);
  else if (method == 0) rootm::step_plain(s, p, nullptr);
  else rootm::step_rtsec(s, p, nullptr);
}

// Feeds the determinants of want[0..nwant-1] and advances to the next request.
__host__ __device__ inline void root_feed(RootState& s, const RootParams& p, const double2* got) {
  if (s.nwant == 0) return;
  if (s.method == 2) rootm::step_osc(s, p, got);
  else if (s.method == 0) rootm::step_plain(s, p, got);
  else rootm::step_rtsec(s, p, got);
}

__host__ __device__ inline RootParams root_params(const alps_system& sy, double om_rtol) {
  RootParams p;
  p.numiter = sy.numiter;
  p.D_threshold = sy.D_threshold;
  p.D_prec = sy.D_prec;
  p.D_tol = sy.D_tol;
  p.om_rtol = om_rtol;
  return p;
}
