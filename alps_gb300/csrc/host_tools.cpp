// host_tools.cpp -- host-only entry points: the f0 table generator and the
// map minimum finder.  Neither evaluates det D.
#include <algorithm>
#include <cmath>

#include "../../include/alps_gb300.h"

namespace {
// Modified Bessel functions of generate_distribution
// (distribution/generate_distribution.f90:708-868): Numerical-Recipes
// polynomial approximations, used by the Juettner normalisation.
double g_bessi0(double x) {
  if (std::fabs(x) < 3.75) {
    double y = (x / 3.75) * (x / 3.75);
    return 1.0 + y * (3.5156229 + y * (3.0899424 + y * (1.2067429 + y * (0.2659732 + y * (0.360768e-1 + y * 0.45813e-2)))));
  }
  double ax = std::fabs(x), y = 3.75 / ax, bx = std::exp(ax) / std::sqrt(ax);
  return (0.39894228 + y * (0.1328592e-1 + y * (0.225319e-2 + y * (-0.157565e-2 + y * (0.916281e-2 +
          y * (-0.2057706e-1 + y * (0.2635537e-1 + y * (-0.1647633e-1 + y * 0.392377e-2)))))))) * bx;
}
double g_bessi1(double x) {
  if (std::fabs(x) < 3.75) {
    double y = (x / 3.75) * (x / 3.75);
    return x * (0.5 + y * (0.87890594 + y * (0.51498869 + y * (0.15084934 + y * (0.2658733e-1 + y * (0.301532e-2 + y * 0.32411e-3))))));
  }
  double ax = std::fabs(x), y = 3.75 / ax, bx = std::exp(ax) / std::sqrt(ax);
  return (0.39894228 + y * (-0.3988024e-1 + y * (-0.362018e-2 + y * (0.163801e-2 + y * (-0.1031555e-1 +
          y * (0.2282967e-1 + y * (-0.2895312e-1 + y * (0.1787654e-1 + y * -0.420059e-2)))))))) * bx;
}
double g_bessk0(double x) {
  if (x == 0.0) return 1.0e30;
  if (x <= 2.0) {
    double y = x * x / 4.0, ax = -std::log(x / 2.0) * g_bessi0(x);
    return ax + (-0.57721566 + y * (0.42278420 + y * (0.23069756 + y * (0.3488590e-1 + y * (0.262698e-2 + y * (0.10750e-3 + y * 0.74e-5))))));
  }
  double y = (2.0 / x), ax = std::exp(-x) / std::sqrt(x);
  return ax * (1.25331414 + y * (-0.7832358e-1 + y * (0.2189568e-1 + y * (-0.1062446e-1 + y * (0.587872e-2 + y * (-0.251540e-2 + y * 0.53208e-3))))));
}
double g_bessk1(double x) {
  if (x == 0.0) return 1.0e32;
  if (x <= 2.0) {
    double y = x * x / 4.0, ax = std::log(x / 2.0) * g_bessi1(x);
    return ax + (1.0 / x) * (1.0 + y * (0.15443144 + y * (-0.67278579 + y * (-0.18156897 + y * (-0.1919402e-1 + y * (-0.110404e-2 + y * -0.4686e-4))))));
  }
  double y = (2.0 / x), ax = std::exp(-x) / std::sqrt(x);
  return ax * (1.25331414 + y * (0.23498619 + y * (-0.3655620e-1 + y * (0.1504268e-1 + y * (-0.780353e-2 + y * (0.325614e-2 + y * -0.68245e-3))))));
}
double g_bessk(int n, double x) {
  if (n == 0) return g_bessk0(x);
  if (n == 1) return g_bessk1(x);
  if (x == 0.0) return 1.0e30;
  double tox = 2.0 / x, bk = g_bessk1(x), bkm = g_bessk0(x), bkp;
  for (int j = 1; j <= n - 1; ++j) {
    bkp = bkm + (double)j * tox * bk;
    bkm = bk;
    bk = bkp;
  }
  return bk;
}
}  // namespace

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
  } else if (dp->kind == 3) {  // Juettner
    const double vA = dp->vA;
    norm = vA / (2.0 * pi * std::sqrt(alph) * (ms * ms) * beta * tau);
    norm = norm / g_bessk(2, 2.0 * ms / (vA * vA * alph * beta * tau));
    if (dp->autoscale) {
      pperp_max = std::sqrt(maxP * maxP * tau + (tau - ms * ms) / (vA * vA)) * std::sqrt(alph);
      ppar_max = std::sqrt(maxP * maxP * tau + (tau - ms * ms) / (vA * vA));
    }
    fit[0] = norm;
    fit[1] = vA * vA * alph / (ms * ms);
    fit[2] = pd;
    perpcorr = (2.0 * ms / (vA * vA * beta * tau * alph));
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
  } else if (dp->kind == 0) {  // distribution_analyt: no normalisation, no autoscale
    if (dp->species != 1 && dp->species != 2) return ALPS_E_UNSUPPORTED;
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
    if (dp->kind == 3) {
      const double vA = dp->vA;
      return std::exp(-(2.0 * ms / (vA * vA * beta * tau * alph)) *
                      std::sqrt(1.0 + p1 * p1 * vA * vA / (ms * ms) + d * d * vA * vA * alph / (ms * ms)));
    }
    if (dp->kind == 0) {
      // the reference's example (distribution/distribution_analyt.f90:59-79):
      // a Maxwellian with beta = 1 and m = 1 (species 1) or 1/1836 (species 2)
      const double m0 = (dp->species == 1) ? 1.0 : 1.0 / 1836.0, b0 = 1.0;
      return (std::pow(pi, -1.5) / std::pow(m0 * b0, 1.5)) * std::exp(-(p2 * p2 / (b0 * m0) + (p1 * p1) / (b0 * m0)));
    }
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
