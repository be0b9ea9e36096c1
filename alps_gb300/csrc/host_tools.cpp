// host_tools.cpp -- host-only entry points: the f0 table generator and the
// map minimum finder.  Neither evaluates det D.
#include <algorithm>
#include <cmath>

#include "../../include/alps_gb300.h"

extern "C" {

// generate_distribution (distribution/generate_distribution.f90:176-300):
// grid dpperp = pperp_max/nperp, dppar = 2 ppar_max/npar,
// ppar = ipar*dppar - ppar_max + p_drift, f0 = norm * shape.
int alps_generate_f0(const alps_dist_params* dp, int nperp, int npar, double* pperp, double* ppar, double* f0,
                     double* ideal) {
  if (!dp || !pperp || !ppar || !f0 || nperp < 1 || npar < 1) return ALPS_E_INVALID;
  const double pi = std::atan(1.0) * 4.0;
  const double ms = dp->ms, tau = dp->tau, alph = dp->alph, pd = dp->p_drift, kap = dp->kappa;
  const double beta = dp->beta, maxP = dp->maxP;
  double norm = 1.0, pperp_max = dp->maxPperp, ppar_max = dp->maxPpar, a = 0.0;
  double fit[5] = {0, 0, 0, 0, 0}, perpcorr = 0.0;
  if (dp->kind == 1) {  // bi-Maxwellian
    norm = std::pow(pi, -1.5) / (std::pow(ms * beta * tau, 1.5) * alph);
    if (dp->autoscale) {
      pperp_max = maxP * std::sqrt(ms * tau * alph);
      ppar_max = maxP * std::sqrt(ms * tau);
    }
    fit[0] = norm;
    fit[1] = 1.0 / (beta * ms * tau);
    fit[2] = pd;
    perpcorr = 1.0 / (tau * beta * ms * alph);
  } else if (dp->kind == 2) {  // bi-kappa
    a = std::sqrt((2.0 * kap - 3.0) / (2.0 * kap));
    norm = 1.0 / (std::pow(ms * beta * tau * pi * kap, 1.5) * alph);
    norm = norm * std::tgamma(kap + 1.0) / (std::tgamma(kap - 0.5) * a * a * a);
    if (dp->autoscale) {
      double sc = std::sqrt((kap - 1.5) / (dp->kappa1 - 1.5));
      pperp_max = maxP * std::sqrt(ms * tau * alph) * sc;
      ppar_max = maxP * std::sqrt(ms * tau) * sc;
    }
    fit[0] = norm;
    fit[1] = 1.0 / (beta * ms * kap * a * a * tau);
    fit[2] = pd;
    fit[3] = -1.0 - kap;
    fit[4] = 1.0;
    perpcorr = 1.0 / (tau * beta * ms * kap * a * a * alph);
  } else if (dp->kind == 4) {  // bi-Moyal, renormalised numerically below
    if (dp->autoscale) {
      pperp_max = maxP * std::sqrt(ms * tau * alph);
      ppar_max = maxP * std::sqrt(ms * tau);
    }
    fit[0] = 1.0;
    fit[1] = 1.0 / (beta * ms * tau);
    fit[2] = pd;
    fit[3] = 1.0;
    perpcorr = 1.0 / (tau * beta * ms * alph);
  } else {
    return ALPS_E_UNSUPPORTED;
  }
  const double dpperp = pperp_max / (double)(float)nperp;
  const double dppar = 2.0 * ppar_max / (double)(float)npar;
  auto shape = [&](double p1, double p2) {
    double d = p2 - pd;
    if (dp->kind == 1) return std::exp(-((d * d) / (beta * ms * tau) + (p1 * p1) / (tau * beta * ms * alph)));
    if (dp->kind == 2)
      return std::pow(1.0 + (d * d / (beta * ms * kap * a * a * tau)) + (p1 * p1) / (tau * beta * ms * kap * a * a * alph),
                      -1.0 - kap);
    double q = (d * d) / (beta * ms * tau) + (p1 * p1) / (tau * beta * ms * alph);
    return std::exp(0.5 * (q - std::exp(q)));
  };
  double integral = 0.0;
  for (int i = 0; i <= nperp; ++i) {
    double p1 = (double)(float)i * dpperp;
    for (int j = 0; j <= npar; ++j) {
      double p2 = (double)(float)j * dppar - ppar_max + pd;
      double f = shape(p1, p2) * norm;
      integral = integral + dpperp * dppar * 2.0 * pi * p1 * f;
      size_t k = (size_t)i * (npar + 1) + j;
      pperp[k] = p1;
      ppar[k] = p2;
      f0[k] = f;
    }
  }
  if (dp->kind == 4) {
    norm = 1.0 / integral;
    fit[0] = norm;
    for (size_t k = 0; k < (size_t)(nperp + 1) * (npar + 1); ++k) f0[k] = norm * shape(pperp[k], ppar[k]);
  }
  if (ideal) {
    for (int k = 0; k < 5; ++k) ideal[k] = fit[k];
    ideal[5] = perpcorr;
  }
  return ALPS_OK;
}

// find_minima (src/ALPS_fns.f90:3860-3966): strict minima against the
// horizontal neighbours (ir) and vertical neighbours (ii), edges compared on
// their one inner side; visited ii = ni..1 (outer), ir = 1..nr (inner).
int alps_find_minima(const double* val, int nr, int ni, int numroots, int* iroots, int* nfound) {
  if (!val || !nfound || nr < 2 || ni < 2 || numroots < 0 || (numroots > 0 && !iroots)) return ALPS_E_INVALID;
  auto V = [&](int ir, int ii) { return val[(size_t)ir * ni + ii]; };
  int n = 0;
  for (int ii = ni - 1; ii >= 0; --ii)
    for (int ir = 0; ir < nr; ++ir) {
      double v = V(ir, ii);
      bool h = (ir == 0) ? v < V(ir + 1, ii) : (ir == nr - 1) ? v < V(ir - 1, ii)
                                                              : (v < V(ir - 1, ii) && v < V(ir + 1, ii));
      if (!h) continue;
      bool vt = (ii == 0) ? v < V(ir, ii + 1) : (ii == ni - 1) ? v < V(ir, ii - 1)
                                                               : (v < V(ir, ii - 1) && v < V(ir, ii + 1));
      if (!vt) continue;
      if (n < numroots) {
        iroots[2 * n] = ir;
        iroots[2 * n + 1] = ii;
      }
      n++;
    }
  *nfound = std::min(n, numroots);
  return ALPS_OK;
}

}  // extern "C"
