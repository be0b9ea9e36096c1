// root_finders.h -- the reference's root finders as host state machines.
//
// Each root runs the reference's control flow and yields the frequencies it
// needs next; the caller evaluates them on the device (all pending requests
// of all roots in one batch) and feeds the determinants back.  Used by
// alps_secant and by the request server.
#ifndef ALPS_ROOT_FINDERS_H
#define ALPS_ROOT_FINDERS_H

#include <cmath>
#include <complex>
#include <vector>

#include "../../include/alps_gb300.h"

// ---------------------------------------------------------------------------
// Root finders.  Each root runs the reference's control flow as a state
// machine that yields the frequencies it needs; all pending requests of all
// roots go to the device in one batch per round.
// ---------------------------------------------------------------------------
namespace {
typedef std::complex<double> cplx;

struct Req {
  std::vector<cplx> om;
  std::vector<cplx> D;
};

// secant_osc (src/ALPS_fns.f90:1919-2101)
struct SecantOsc {
  const alps_system* sy;
  int state = 0;
  cplx om, D, minom, minD, prevom, prev2om, prev3om, prev4om, prevD, jump, delta;
  int iter = 0, osc = 0;
  double damping = 1.0;
  bool done = false;
  cplx Dfin;
  const double lambda = (double)0.1f, osc_thr = (double)1.E-3f;
  bool close(cplx a, cplx b) const {
    return (std::fabs(a.real() - b.real()) < std::fabs(a.real()) * osc_thr) &&
           (std::fabs(a.imag() - b.imag()) < std::fabs(a.imag()) * osc_thr);
  }
  // returns frequencies to evaluate (empty when finished)
  std::vector<cplx> step(const std::vector<cplx>& got) {
    for (;;) {
      switch (state) {
        case 0:
          delta = cplx(1.0e-6, 1.0e-8);
          state = 1;
          return {om};
        case 1:
          D = got[0];
          minom = om;
          minD = D;
          prevom = om * (1.0 - sy->D_prec);
          prev2om = prev3om = prev4om = om;
          state = 2;
          return {prevom};
        case 2:
          prevD = got[0];
          if (std::abs(prevD) < std::abs(minD)) { minom = prevom; minD = prevD; }
          iter = 0;
          state = 3;
          break;
        case 3:  // loop head
          if (!(iter <= sy->numiter - 1)) { state = 9; break; }
          iter++;
          state = 4;
          return {om};
        case 4:
          D = got[0];
          if (std::abs(D - prevD) < 1.0e-80) {
            prevom = prevom + 1.0e-8;
            state = 5;
            return {prevom};
          }
          state = 6;
          break;
        case 5:
          prevD = got[0];
          state = 6;
          break;
        case 6:
          if (std::abs(D) < sy->D_threshold) {
            jump = 0.0;
            Dfin = D;
            if (iter >= sy->numiter) {  // after-loop rule of the reference
              om = minom;
              Dfin = minD;
            }
            done = true;
            state = 10;
            return {};
          }
          if (iter > 4) {
            if (close(om, prevom) || close(om, prev2om) || close(om, prev3om) || close(om, prev4om)) {
              osc++;
              damping = std::min(0.5, damping * 0.75);
            }
          }
          if (osc > 1) {
            state = 7;
            return {om * (1.0 + delta), om * (1.0 - delta)};
          }
          jump = damping * D * (om - prevom) / (D - prevD);
          state = 8;
          break;
        case 7: {
          cplx Dprime = (got[0] - got[1]) / (2.0 * om * delta);
          jump = D / (Dprime + lambda * D);
          state = 8;
          break;
        }
        case 8:
          if (std::abs(jump) > (double)0.1f * std::abs(om)) jump = ((double)0.1f * std::abs(om)) * (jump / std::abs(jump));
          if (std::abs(D) > std::abs(prevD)) jump = (double)0.5f * jump;
          prev4om = prev3om;
          prev3om = prev2om;
          prev2om = prevom;
          prevom = om;
          prevD = D;
          if (std::abs(D) < std::abs(minD)) { minom = om; minD = D; }
          om = om - jump;
          state = 3;
          break;
        case 9:  // numiter exhausted
          om = minom;
          Dfin = minD;
          done = true;
          state = 10;
          return {};
        default:
          return {};
      }
    }
  }
};

// secant (src/ALPS_fns.f90:1815-1917)
struct SecantPlain {
  const alps_system* sy;
  int state = 0;
  cplx om, prevom, Dprev, minD, minom, D, jump;
  int iter = 0;
  bool done = false;
  cplx Dfin;
  std::vector<cplx> step(const std::vector<cplx>& got) {
    for (;;) {
      switch (state) {
        case 0:
          prevom = om * (1.0 - sy->D_prec);
          state = 1;
          return {prevom, om};
        case 1:
          Dprev = got[0];
          minD = got[1];
          minom = om;
          if (std::abs(Dprev) < std::abs(minD)) { minom = prevom; minD = Dprev; }
          iter = 0;
          state = 2;
          break;
        case 2:
          if (!(iter <= sy->numiter - 1)) {
            om = minom;
            Dfin = minD;
            done = true;
            state = 9;
            return {};
          }
          iter++;
          state = 3;
          return {om};
        case 3:
          D = got[0];
          if (std::abs(D - Dprev) < 1.0e-80) {
            prevom = prevom + 1.0e-8;
            state = 4;
            return {prevom};
          }
          state = 5;
          break;
        case 4:
          Dprev = got[0];
          state = 5;
          break;
        case 5: {
          bool conv = std::abs(D) < sy->D_threshold;
          jump = conv ? cplx(0.0) : D * (om - prevom) / (D - Dprev);
          prevom = om;
          om = om - jump;
          Dprev = D;
          if (std::abs(D) < std::abs(minD)) { minom = om; minD = D; }
          if (conv) {
            Dfin = D;
            if (iter >= sy->numiter) {
              om = minom;
              Dfin = minD;
            }
            done = true;
            state = 9;
            return {};
          }
          state = 2;
          break;
        }
        default:
          return {};
      }
    }
  }
};

// rtsec (src/ALPS_fns.f90:2105-2195)
struct Rtsec {
  const alps_system* sy;
  int state = 0;
  cplx xin, x1, x2, fl, f, rts, xl, dx;
  int j = 0;
  bool done = false;
  cplx om, Dfin;
  std::vector<cplx> step(const std::vector<cplx>& got) {
    for (;;) {
      switch (state) {
        case 0:
          x1 = xin * 1.0;
          x2 = xin * (1.0 + sy->D_prec);
          state = 1;
          return {x1, x2};
        case 1:
          fl = got[0];
          f = got[1];
          if (std::abs(fl) < std::abs(f)) {
            rts = x1;
            xl = x2;
            std::swap(fl, f);
          } else {
            xl = x1;
            rts = x2;
          }
          j = 0;
          state = 2;
          break;
        case 2:
          j++;
          if (j > sy->numiter - 1) {
            om = rts;
            Dfin = f;
            done = true;
            state = 9;
            return {};
          }
          if (std::abs(f - fl) > 1.0e-40) dx = (xl - rts) * f / (f - fl);
          else dx = (x2 - x1) / 25.0;
          xl = rts;
          fl = f;
          rts = rts + dx / 2.0;
          state = 3;
          return {rts};
        case 3:
          f = got[0];
          if ((std::abs(dx) < sy->D_tol) || (std::abs(f) == 0.0)) {
            om = rts;
            Dfin = f;
            done = true;
            state = 9;
            return {};
          }
          state = 2;
          break;
        default:
          return {};
      }
    }
  }
};

}  // namespace

// One root under any of the three methods (0 secant, 1 rtsec, 2 secant_osc).
namespace {
struct RootMachine {
  int method = 2;
  SecantOsc so;
  SecantPlain sp;
  Rtsec rt;
  std::vector<cplx> start(const alps_system* sy, int m, cplx o) {
    method = m;
    if (m == 2) { so.sy = sy; so.om = o; return so.step({}); }
    if (m == 0) { sp.sy = sy; sp.om = o; return sp.step({}); }
    rt.sy = sy;
    rt.xin = o;
    return rt.step({});
  }
  std::vector<cplx> step(const std::vector<cplx>& got) {
    if (method == 2) return so.step(got);
    if (method == 0) return sp.step(got);
    return rt.step(got);
  }
  cplx root() const { return method == 2 ? so.om : (method == 0 ? sp.om : rt.om); }
  cplx dfinal() const { return method == 2 ? so.Dfin : (method == 0 ? sp.Dfin : rt.Dfin); }
  int iters() const { return method == 2 ? so.iter : (method == 0 ? sp.iter : rt.j); }
};
}  // namespace

namespace {
// One step of a k scan (the select case of om_scan / om_double_scan):
// sets the components the scan type moves, from the start point (kp0, kz0)
// or, for types 1 and 2, from its angle th0 and magnitude k0.
void scan_k(const alps_scan_def& sc, int it, double kp0, double kz0, double th0, double k0, double& kperp,
            double& kpar) {
  switch (sc.type_s) {
    case 0:
      if (sc.log_scan) {
        kperp = std::pow(10.0, std::log10(kp0) + sc.diff * it);
        kpar = std::pow(10.0, std::log10(kz0) + sc.diff2 * it);
      } else {
        kperp = kp0 + sc.diff * it;
        kpar = kz0 + sc.diff2 * it;
      }
      break;
    case 1: {
      double th = sc.log_scan ? std::pow(10.0, std::log10(th0) + sc.diff * it) : th0 + sc.diff * it;
      kperp = k0 * std::sin(th);
      kpar = k0 * std::cos(th);
      break;
    }
    case 2: {
      double kt = sc.log_scan ? std::pow(10.0, std::log10(k0) + sc.diff * it) : (k0) + sc.diff * it;
      kperp = kt * std::sin(th0);
      kpar = kt * std::cos(th0);
      break;
    }
    case 3:
      kperp = sc.log_scan ? std::pow(10.0, std::log10(kp0) + sc.diff * it) : kp0 + sc.diff * it;
      break;
    case 4:
      kpar = sc.log_scan ? std::pow(10.0, std::log10(kz0) + sc.diff * it) : kz0 + sc.diff * it;
      break;
  }
}

}  // namespace

#endif
