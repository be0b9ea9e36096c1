// root_finders.h -- host drivers' view of the root finders, and the k steps
// of the scans.
//
// Each root runs the reference's control flow (root_machine.cuh) and yields
// the frequencies it needs next; the caller evaluates them on the device (all
// pending requests of all roots in one batch) and feeds the determinants
// back.  Used by alps_secant and by the request server.
#ifndef ALPS_ROOT_FINDERS_H
#define ALPS_ROOT_FINDERS_H

#include <cmath>
#include <complex>
#include <vector>

#include "../../include/alps_gb300.h"
#include "root_machine.cuh"

// One root under any of the three methods (0 secant, 1 rtsec, 2
// secant_osc): the plain-data machine of root_machine.cuh behind a
// vector interface for the host drivers.
namespace {
typedef std::complex<double> cplx;

struct RootMachine {
  RootState st;
  RootParams pr;
  std::vector<cplx> wanted() const {
    std::vector<cplx> w;
    for (int q = 0; q < st.nwant; ++q) w.push_back(cplx(st.want[q].x, st.want[q].y));
    return w;
  }
  std::vector<cplx> start(const alps_system* sy, int m, cplx o, double om_rtol = 0.0) {
    pr = root_params(*sy, om_rtol);
    root_start(st, pr, m, make_double2(o.real(), o.imag()));
    return wanted();
  }
  std::vector<cplx> step(const std::vector<cplx>& got) {
    double2 g[2];
    for (int q = 0; q < st.nwant && q < 2; ++q) g[q] = make_double2(got[q].real(), got[q].imag());
    root_feed(st, pr, g);
    return wanted();
  }
  cplx root() const { return cplx(st.om.x, st.om.y); }
  cplx dfinal() const { return cplx(st.Dfin.x, st.Dfin.y); }
  int iters() const { return st.iter; }
  bool converged() const { return st.converged != 0; }
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
