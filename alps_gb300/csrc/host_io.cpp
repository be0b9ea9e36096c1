// host_io.cpp -- the reference's input and output formats and its main
// program, as host code over the library's own entry points:
//   alps_read_input  init_param + scan_read (src/ALPS_io.f90:46-552)
//   alps_read_f0     read_f0 (src/ALPS_io.f90:643-692)
//   alps_run_input   program alps (src/ALPS.f90:19-147): map_search /
//                    refine_guess / om_scan (src/ALPS_fns.f90:2198-2600,
//                    3595-3856) with their output files.
// Every det D evaluation goes through alps_disp / alps_secant / alps_map.
#include <sys/stat.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/alps_gb300.h"
#include "root_finders.h"

namespace {

typedef std::complex<double> cplx;

std::string lower(std::string s) {
  for (auto& ch : s) ch = (char)std::tolower((unsigned char)ch);
  return s;
}

std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// One namelist group: key -> raw value text (lower-case keys).
typedef std::map<std::string, std::string> Group;

// Splits the file into groups "&name ... /"; comments start with '!'
// outside quotes.
std::map<std::string, Group> parse_namelists(const std::string& text) {
  std::map<std::string, Group> out;
  std::istringstream in(text);
  std::string line, cur;
  bool inside = false;
  std::string pending;  // "key=value" pieces across the group
  auto flush_pairs = [&](Group& g, const std::string& body) {
    // split on commas/newlines that are outside quotes, then key=value
    std::vector<std::string> items;
    std::string item;
    char q = 0;
    for (char ch : body) {
      if (q) {
        item += ch;
        if (ch == q) q = 0;
      } else if (ch == '\'' || ch == '"') {
        q = ch;
        item += ch;
      } else if (ch == ',' || ch == '\n') {
        items.push_back(item);
        item.clear();
      } else {
        item += ch;
      }
    }
    items.push_back(item);
    std::string lastkey;
    for (auto& it : items) {
      std::string t = trim(it);
      if (t.empty()) continue;
      size_t eq = t.find('=');
      if (eq == std::string::npos) {
        if (!lastkey.empty()) g[lastkey] += " " + t;
        continue;
      }
      std::string k = lower(trim(t.substr(0, eq)));
      g[k] = trim(t.substr(eq + 1));
      lastkey = k;
    }
  };
  while (std::getline(in, line)) {
    // strip comments outside quotes
    std::string l;
    char q = 0;
    for (char ch : line) {
      if (q) {
        l += ch;
        if (ch == q) q = 0;
      } else if (ch == '\'' || ch == '"') {
        q = ch;
        l += ch;
      } else if (ch == '!') {
        break;
      } else {
        l += ch;
      }
    }
    std::string t = trim(l);
    if (!inside) {
      if (!t.empty() && t[0] == '&') {
        size_t e = t.find_first_of(" \t", 1);
        cur = lower(t.substr(1, e == std::string::npos ? std::string::npos : e - 1));
        inside = true;
        pending = (e == std::string::npos) ? "" : t.substr(e) + "\n";
      }
      continue;
    }
    if (!t.empty() && (t[0] == '/' || t == "&end")) {
      flush_pairs(out[cur], pending);
      inside = false;
      continue;
    }
    // a value line may also end with '/'
    if (!t.empty() && t.back() == '/' && t.find('\'') == std::string::npos) {
      pending += t.substr(0, t.size() - 1) + "\n";
      flush_pairs(out[cur], pending);
      inside = false;
      continue;
    }
    pending += t + "\n";
  }
  return out;
}

double to_double(const std::string& v) {
  std::string t = v;
  for (auto& ch : t)
    if (ch == 'd' || ch == 'D') ch = 'E';
  return std::strtod(t.c_str(), nullptr);
}

int to_logical(const std::string& v) {
  std::string t = lower(trim(v));
  if (!t.empty() && t[0] == '.') t = t.substr(1);
  return (!t.empty() && t[0] == 't') ? 1 : 0;
}

std::string to_string_val(const std::string& v) {
  std::string t = trim(v);
  if (t.size() >= 2 && (t[0] == '\'' || t[0] == '"')) return t.substr(1, t.find(t[0], 1) - 1);
  return t;
}

struct Reader {
  const Group* g;
  // a key given without a value (a Fortran null value) keeps the default
  bool has(const char* k) const { return g && g->count(k) && !trim(g->at(k)).empty(); }
  void d(const char* k, double& x) const {
    if (has(k)) x = to_double(g->at(k));
  }
  void i(const char* k, int& x) const {
    if (has(k)) x = (int)std::lround(to_double(g->at(k)));
  }
  void l(const char* k, int& x) const {
    if (has(k)) x = to_logical(g->at(k));
  }
  void s(const char* k, char* out, size_t n) const {
    if (has(k)) {
      std::string v = to_string_val(g->at(k));
      std::snprintf(out, n, "%s", v.c_str());
    }
  }
};

// Fortran ESw.dEe output (e.g. es14.4e3 -> "   1.0000E-002")
std::string fmt_es(double x, int w, int d, int e) {
  char buf[64];
  std::string s;
  if (std::isnan(x)) {
    s = "NaN";
  } else if (std::isinf(x)) {
    s = x < 0 ? "-Infinity" : "Infinity";
  } else {
    if (x == 0.0) x = 0.0;  // exact zeros print unsigned, as in the reference's files
    std::snprintf(buf, sizeof(buf), "%.*E", d, x);
    std::string t(buf);
    size_t ep = t.find('E');
    std::string mant = t.substr(0, ep);
    int ex = std::atoi(t.c_str() + ep + 1);
    if (x == 0.0) ex = 0;
    char eb[16];
    std::snprintf(eb, sizeof(eb), "E%c%0*d", ex < 0 ? '-' : '+', e, std::abs(ex));
    s = mant + eb;
  }
  if ((int)s.size() < w) s = std::string(w - s.size(), ' ') + s;
  return s;
}

// one output row: es14.4e3 fields (om_scan's eigen/heat formats,
// src/ALPS_fns.f90:2261-2268)
void write_row(FILE* f, const std::vector<double>& v) {
  for (double x : v) std::fputs(fmt_es(x, 14, 4, 3).c_str(), f);
  std::fputc('\n', f);
}

// columns of the .eigen_, .heat_ and .heat_mech_ rows after (kperp, kpar, om)
void eigen_columns(const alps_eigen& e, int nspec, std::vector<double>& eig, std::vector<double>& heat,
                   std::vector<double>& mech) {
  eig.clear();
  heat.clear();
  mech.clear();
  for (int i = 0; i < 3; ++i) {
    eig.push_back(e.electric[i].re);
    eig.push_back(e.electric[i].im);
  }
  for (int i = 0; i < 3; ++i) {
    eig.push_back(e.magnetic[i].re);
    eig.push_back(e.magnetic[i].im);
  }
  for (int s = 0; s < nspec; ++s)
    for (int j = 0; j < 3; ++j) {
      eig.push_back(e.vmean[s][j].re);
      eig.push_back(e.vmean[s][j].im);
    }
  for (int s = 0; s < nspec; ++s) {
    eig.push_back(e.ds[s].re);
    eig.push_back(e.ds[s].im);
  }
  for (int s = 0; s < nspec; ++s) heat.push_back(e.Ps[s]);
  heat.push_back(e.ewave);
  for (int s = 0; s < nspec; ++s)
    for (int q = 0; q < 4; ++q) mech.push_back(e.Ps_split[s][q]);
}

bool file_exists(const std::string& p) {
  struct stat st;
  return stat(p.c_str(), &st) == 0;
}

void ensure_dir(const std::string& p) { mkdir(p.c_str(), 0755); }



int append_line(const std::string& path, const std::vector<double>* row) {
  FILE* f = std::fopen(path.c_str(), "a");
  if (!f) return ALPS_E_IO;
  if (row) write_row(f, *row);
  else std::fputc('\n', f);
  std::fclose(f);
  return ALPS_OK;
}

// om_double_scan (src/ALPS_fns.f90:2904-3591), scan_option 2: scan 2 runs
// from every output point of scan 1.  Outer steps start from the roots of
// the previous outer step (omlast), inner steps from the previous inner
// step; files are <run>.scan_<id1><id2>.root_<n> (and .eigen_/.heat_/
// .heat_mech_ when scan 1 asks for them) with a blank line after every
// inner scan, as in the reference.
int double_scan(alps_ctx* ctx, const alps_input& in, const std::string& soldir, const std::string& run, int nroots,
                std::vector<alps_complex>& wroots, double kperp, double kpar) {
  const alps_system& s = in.sys;
  const alps_scan_def& s1 = in.scan[0];
  const alps_scan_def& s2 = in.scan[1];
  const char* ids1[5] = {"k1_k2_", "theta_", "kcstq_", "kperp_", "kpara_"};
  const char* ids2[5] = {"k1_k2", "theta", "kcstq", "kperp", "kpara"};
  const std::string tag = std::string(ids1[s1.type_s]) + ids2[s2.type_s];
  auto name = [&](const char* kind, int r) {
    return soldir + "/" + run + "." + kind + "_" + tag + ".root_" + std::to_string(r + 1);
  };
  const bool want_eig = s1.eigen || s1.heating;
  int st;
  for (int r = 0; r < nroots; ++r) {
    const char* kinds[4] = {"scan", "eigen", "heat", "heat_mech"};
    for (int q = 0; q < 4; ++q) {
      if (q == 1 && !s1.eigen) continue;
      if (q >= 2 && !s1.heating) continue;
      FILE* f = std::fopen(name(kinds[q], r).c_str(), "w");
      if (!f) return ALPS_E_IO;
      std::fclose(f);
    }
  }
  // (the reference also evaluates calc_eigen at the start point here but
  // writes nothing from it)
  const int nt = s1.n_out * s1.n_res, nt2 = s2.n_out * s2.n_res;
  const double kperp_last = kperp, kpar_last = kpar;
  const double theta_0 = std::atan(kperp_last / kpar_last);
  const double k_0 = std::sqrt(kperp_last * kperp_last + kpar_last * kpar_last);
  std::vector<alps_complex> omlast(wroots.begin(), wroots.begin() + nroots);
  std::vector<char> jump(nroots, 1);
  // the roots still followed
  auto active = [&](std::vector<int>& idx, std::vector<alps_complex>& sub) {
    idx.clear();
    sub.clear();
    for (int r = 0; r < nroots; ++r)
      if (jump[r]) idx.push_back(r);
  };
  for (int it = 0; it <= nt; ++it) {
    scan_k(s1, it, kperp_last, kpar_last, theta_0, k_0, kperp, kpar);
    if ((st = alps_set_k(ctx, kperp, kpar))) return st;
    bool alljump = false;
    for (int r = 0; r < nroots; ++r) alljump = alljump || jump[r];
    if (!alljump) return ALPS_E_ROOTS_DIVERGED;
    std::vector<int> idx;
    std::vector<alps_complex> sub;
    active(idx, sub);
    for (int r : idx) sub.push_back(omlast[r]);
    if ((st = alps_secant(ctx, s.secant_method, (int)sub.size(), sub.data(), nullptr, nullptr))) return st;
    for (size_t q = 0; q < idx.size(); ++q) {
      int r = idx[q];
      wroots[r] = omlast[r] = sub[q];
      double re = sub[q].re;
      if (std::fabs(re) >= 1.79769313486231571e308 || re != re) jump[r] = 0;
      for (int imm = 0; imm < r; ++imm)
        if (std::hypot(wroots[r].re - wroots[imm].re, wroots[r].im - wroots[imm].im) < s.D_gap) {
          wroots[r] = alps_complex{0.0, 0.0};
          jump[r] = 0;
        }
    }
    if (it % s1.n_res == 0) {
      double kperpi = kperp, kpari = kpar, theta_i = 0.0, k_i = 0.0;
      for (int it2 = 0; it2 <= nt2; ++it2) {
        if (it2 == 0) {
          kperpi = kperp;
          kpari = kpar;
          theta_i = std::atan(kperpi / kpari);
          k_i = std::sqrt(kperpi * kperpi + kpari * kpari);
          for (int r = 0; r < nroots; ++r) wroots[r] = omlast[r];
        }
        scan_k(s2, it2, kperpi, kpari, theta_i, k_i, kperp, kpar);
        if ((st = alps_set_k(ctx, kperp, kpar))) return st;
        active(idx, sub);
        for (int r : idx) sub.push_back(wroots[r]);
        if ((st = alps_secant(ctx, s.secant_method, (int)sub.size(), sub.data(), nullptr, nullptr))) return st;
        std::vector<alps_complex> Dr(sub.size());
        if (!sub.empty() && (st = alps_disp_batch(ctx, (int)sub.size(), sub.data(), Dr.data()))) return st;
        const bool out = (it % s1.n_res == 0) && (it2 % s2.n_res == 0);
        std::vector<alps_eigen> eg;
        if (out && want_eig && !sub.empty()) {
          eg.resize(sub.size());
          if ((st = alps_calc_eigen(ctx, (int)sub.size(), sub.data(), s1.eigen, s1.heating, eg.data()))) return st;
        }
        for (size_t q = 0; q < idx.size(); ++q) {
          int r = idx[q];
          wroots[r] = sub[q];
          double re = sub[q].re;
          if (std::fabs(re) >= 1.79769313486231571e308 || re != re) jump[r] = 0;
          if (std::hypot(Dr[q].re, Dr[q].im) > 1.0e100) jump[r] = 0;
          for (int imm = 0; imm < r; ++imm)
            if (std::hypot(wroots[r].re - wroots[imm].re, wroots[r].im - wroots[imm].im) < s.D_gap) {
              wroots[r] = alps_complex{0.0, 0.0};
              jump[r] = 0;
            }
          if (!out) continue;
          std::vector<double> head = {kperp, kpar, wroots[r].re, wroots[r].im};
          if ((st = append_line(name("scan", r), &head))) return st;
          if (want_eig) {
            std::vector<double> ev, hv, mv;
            eigen_columns(eg[q], s.nspec, ev, hv, mv);
            const char* kinds[3] = {"eigen", "heat", "heat_mech"};
            const std::vector<double>* cols[3] = {&ev, &hv, &mv};
            for (int c = 0; c < 3; ++c) {
              if ((c == 0 && !s1.eigen) || (c > 0 && !s1.heating)) continue;
              std::vector<double> row = head;
              row.insert(row.end(), cols[c]->begin(), cols[c]->end());
              if ((st = append_line(name(kinds[c], r), &row))) return st;
            }
          }
        }
      }
      for (int r = 0; r < nroots; ++r) {
        if ((st = append_line(name("scan", r), nullptr))) return st;
        if (s1.eigen && (st = append_line(name("eigen", r), nullptr))) return st;
        if (s1.heating && (st = append_line(name("heat", r), nullptr))) return st;
        if (s1.heating && (st = append_line(name("heat_mech", r), nullptr))) return st;
      }
    }
    // back to the start of scan 2's parameter (itt = 0 with the original k)
    scan_k(s2, 0, kperp_last, kpar_last, theta_0, k_0, kperp, kpar);
    if (s2.type_s == 2) {  // the reset of type 2 reuses the type-0 formulas
      alps_scan_def t0 = s2;
      t0.type_s = 0;
      scan_k(t0, 0, kperp_last, kpar_last, theta_0, k_0, kperp, kpar);
    }
  }
  return ALPS_OK;
}

}  // namespace

extern "C" {

int alps_read_input(const char* path, alps_input* in) {
  if (!path || !in) return ALPS_E_INVALID;
  std::ifstream f(path);
  if (!f) return ALPS_E_IO;
  std::stringstream ss;
  ss << f.rdbuf();
  auto nl = parse_namelists(ss.str());
  std::memset(in, 0, sizeof(*in));
  alps_system_defaults(&in->sys);
  in->ngamma = 100;
  in->npparbar = 200;
  in->writeOut = 1;
  in->determine_minima = 1;
  in->scan_option = 1;
  in->n_scan = 0;
  // runname = file name without folder and ".in"
  std::string p(path);
  size_t sl = p.find_last_of('/');
  std::string base = sl == std::string::npos ? p : p.substr(sl + 1);
  if (base.size() > 3 && base.substr(base.size() - 3) == ".in") base = base.substr(0, base.size() - 3);
  std::snprintf(in->runname, sizeof(in->runname), "%s", base.c_str());
  if (!nl.count("system")) return ALPS_E_NAMELIST;
  Reader r{&nl["system"]};
  alps_system& s = in->sys;
  r.d("kperp", s.kperp);
  r.d("kpar", s.kpar);
  r.i("nspec", s.nspec);
  r.i("nroots", in->nroots);
  r.l("use_map", in->use_map);
  r.l("writeout", in->writeOut);
  r.i("nperp", s.nperp);
  r.i("npar", s.npar);
  r.i("ngamma", in->ngamma);
  r.i("npparbar", in->npparbar);
  s.ngamma = in->ngamma;
  s.npparbar = in->npparbar;
  r.d("va", s.vA);
  r.s("arrayname", in->arrayName, sizeof(in->arrayName));
  r.d("bessel_zero", s.Bessel_zero);
  r.i("secant_method", s.secant_method);
  r.i("numiter", s.numiter);
  r.l("kperp_norm", s.kperp_norm);
  r.d("d_threshold", s.D_threshold);
  r.d("d_prec", s.D_prec);
  r.d("d_gap", s.D_gap);
  r.d("d_tol", s.D_tol);
  r.i("positions_principal", s.positions_principal);
  r.d("tlim", s.Tlim);
  r.i("maxsteps_fit", s.maxsteps_fit);
  r.d("lambda_initial_fit", s.lambda_initial_fit);
  r.d("lambdafac_fit", s.lambdafac_fit);
  r.d("epsilon_fit", s.epsilon_fit);
  r.l("determine_minima", in->determine_minima);
  r.i("n_resonance_interval", s.n_resonance_interval);
  r.i("scan_option", in->scan_option);
  r.i("n_scan", in->n_scan);
  if (s.nspec < 1 || s.nspec > ALPS_MAX_INPUT_SPECIES) return ALPS_E_INVALID;
  if (in->nroots > ALPS_MAX_ROOTS || in->n_scan > ALPS_MAX_SCANS || in->n_scan < 0) return ALPS_E_INVALID;
  char key[64];
  if (in->use_map) {
    if (!nl.count("maps_1")) return ALPS_E_NAMELIST;
    Reader m{&nl["maps_1"]};
    in->map.nr = 128;
    in->map.ni = 128;
    m.l("loggridw", in->map.loggridw);
    m.l("loggridg", in->map.loggridg);
    m.d("omi", in->map.omi);
    m.d("omf", in->map.omf);
    m.d("gami", in->map.gami);
    m.d("gamf", in->map.gamf);
    m.i("ni", in->map.ni);
    m.i("nr", in->map.nr);
  } else {
    for (int k = 1; k <= in->nroots; ++k) {
      std::snprintf(key, sizeof(key), "guess_%d", k);
      if (!nl.count(key)) return ALPS_E_NAMELIST;
      Reader g{&nl[key]};
      double om = 0, gam = 0;
      g.d("g_om", om);
      g.d("g_gam", gam);
      in->guess[k - 1] = alps_complex{om, gam};
    }
  }
  for (int is = 1; is <= s.nspec; ++is) {
    alps_species& sp = in->species[is - 1];
    alps_species_defaults(&sp);
    sp.ns = sp.qs = sp.ms = 0.0;
    std::snprintf(key, sizeof(key), "spec_%d", is);
    if (!nl.count(key)) return ALPS_E_NAMELIST;
    Reader g{&nl[key]};
    double acm = 1.0;
    g.d("nn", sp.ns);
    g.d("qq", sp.qs);
    g.d("mm", sp.ms);
    g.d("ac_method", acm);
    sp.ac_method = (int)acm;
    g.i("ff", sp.n_fits);
    g.l("relat", sp.relat);
    g.l("log_fit", sp.log_fit);
    g.l("use_bm", sp.use_bM);
    if (sp.use_bM) {
      std::snprintf(key, sizeof(key), "bm_spec_%d", is);
      if (!nl.count(key)) return ALPS_E_NAMELIST;
      Reader b{&nl[key]};
      b.i("bm_nmaxs", sp.bM_nmaxs);
      b.d("bm_bessel_zeros", sp.bM_Bessel_zeros);
      b.d("bm_betas", sp.bM_betas);
      b.d("bm_alphas", sp.bM_alphas);
      b.d("bm_pdrifts", sp.bM_pdrifts);
    } else if (sp.ac_method == 1) {
      if (sp.n_fits < 1 || sp.n_fits > ALPS_MAX_FITS) return ALPS_E_INVALID;
      for (int f = 1; f <= sp.n_fits; ++f) {
        std::snprintf(key, sizeof(key), "ffit_%d_%d", is, f);
        if (!nl.count(key)) return ALPS_E_NAMELIST;
        Reader b{&nl[key]};
        int t = 0;
        b.i("fit_type_in", t);
        sp.fit_type[f - 1] = t;
        const char* names[5] = {"fit_1", "fit_2", "fit_3", "fit_4", "fit_5"};
        for (int k = 0; k < 5; ++k) b.d(names[k], sp.fit_init[f - 1][k]);
        b.d("perpcorr", sp.perp_correction[f - 1]);
      }
    } else if (sp.ac_method == 2) {
      std::snprintf(key, sizeof(key), "poly_spec_%d", is);
      if (!nl.count(key)) return ALPS_E_NAMELIST;
      Reader b{&nl[key]};
      b.i("kind", sp.poly_kind);
      b.i("order", sp.poly_order);
      b.d("log_max", sp.poly_log_max);
    }
  }
  // scans with the step sizes of scan_read (chained through kperp_last)
  double kperp_last = s.kperp, kpar_last = s.kpar;
  const double pi4 = 4.0 * std::atan(1.0);
  for (int k = 1; k <= in->n_scan; ++k) {
    std::snprintf(key, sizeof(key), "scan_input_%d", k);
    if (!nl.count(key)) return ALPS_E_NAMELIST;
    Reader b{&nl[key]};
    alps_scan_def& sc = in->scan[k - 1];
    b.i("scan_type", sc.type_s);
    b.d("swi", sc.swi);
    b.d("swf", sc.swf);
    b.l("swlog", sc.log_scan);
    b.i("ns", sc.n_out);
    b.i("nres", sc.n_res);
    b.l("heating", sc.heating);
    b.l("eigen", sc.eigen);
    double nsr = 1.0 * sc.n_out * sc.n_res;
    double theta_0 = std::atan(kperp_last / kpar_last);
    double k_0 = std::sqrt(kperp_last * kperp_last + kpar_last * kpar_last);
    switch (sc.type_s) {
      case 0:
        sc.diff = sc.log_scan ? (std::log10(sc.swi) - std::log10(kperp_last)) / nsr : (sc.swi - kperp_last) / nsr;
        sc.diff2 = sc.log_scan ? (std::log10(sc.swf) - std::log10(kpar_last)) / nsr : (sc.swf - kpar_last) / nsr;
        kperp_last = sc.swi;
        kpar_last = sc.swf;
        break;
      case 1: {
        double tf = sc.swf * pi4 / (double)180.0f;
        sc.diff = sc.log_scan ? (std::log10(tf) - std::log10(theta_0)) / nsr : (tf - theta_0) / nsr;
        kpar_last = k_0 * std::cos(sc.swf * pi4 / 180.0);
        kperp_last = k_0 * std::sin(sc.swf * pi4 / 180.0);
        break;
      }
      case 2:
        sc.diff = sc.log_scan ? (std::log10(sc.swf) - std::log10(k_0)) / nsr : (sc.swf - k_0) / nsr;
        kpar_last = k_0 * std::cos(theta_0);
        kperp_last = k_0 * std::sin(theta_0);
        break;
      case 3:
        sc.diff = sc.log_scan ? (std::log10(sc.swf) - std::log10(kperp_last)) / nsr : (sc.swf - kperp_last) / nsr;
        kperp_last = sc.swf;
        break;
      case 4:
        sc.diff = sc.log_scan ? (std::log10(sc.swf) - std::log10(kpar_last)) / nsr : (sc.swf - kpar_last) / nsr;
        kpar_last = sc.swf;
        break;
      default:
        return ALPS_E_INVALID;
    }
  }
  return ALPS_OK;
}

int alps_read_f0(const char* path, int nperp, int npar, double* pperp, double* ppar, double* f0) {
  if (!path || !pperp || !ppar || !f0) return ALPS_E_INVALID;
  std::ifstream f(path);
  if (!f) return ALPS_E_IO;
  size_t n = (size_t)(nperp + 1) * (npar + 1);
  std::string tok;
  for (size_t k = 0; k < n; ++k) {
    double v[3];
    for (int q = 0; q < 3; ++q) {
      if (!(f >> tok)) return ALPS_E_IO;
      v[q] = to_double(tok);
    }
    pperp[k] = v[0];
    ppar[k] = v[1];
    f0[k] = v[2];
  }
  return ALPS_OK;
}

int alps_run_input(const char* input_path, const char* workdir) {
  if (!input_path || !workdir) return ALPS_E_INVALID;
  alps_input in;
  int st = alps_read_input(input_path, &in);
  if (st) return st;
  if (in.n_scan > 0 && in.scan_option != 1 && in.scan_option != 2) return ALPS_E_SCAN_OPTION;
  if (in.n_scan > 0 && in.scan_option == 2 && in.n_scan != 2) return ALPS_E_NSCAN;
  const alps_system& s = in.sys;
  std::string wd(workdir);
  std::string soldir = wd + "/solution";
  ensure_dir(soldir);
  alps_ctx* ctx = nullptr;
  if ((st = alps_create(&s, &ctx))) return st;
  struct Guard {
    alps_ctx* c;
    ~Guard() { alps_destroy(c); }
  } guard{ctx};
  int N = s.nperp, M = s.npar;
  size_t nn = (size_t)(N + 1) * (M + 1);
  std::vector<double> pperp(nn), ppar(nn), f0(nn);
  for (int is = 1; is <= s.nspec; ++is) {
    if (in.species[is - 1].use_bM) {  // closed-form species read no table (src/ALPS_io.f90:672-675)
      if ((st = alps_set_species(ctx, is - 1, &in.species[is - 1], nullptr, nullptr, nullptr))) return st;
      continue;
    }
    char fn[1024];
    std::snprintf(fn, sizeof(fn), "%s/distribution/%s.%d.array", workdir, in.arrayName, is);
    if ((st = alps_read_f0(fn, N, M, pperp.data(), ppar.data(), f0.data()))) return st;
    if ((st = alps_set_species(ctx, is - 1, &in.species[is - 1], pperp.data(), ppar.data(), f0.data()))) return st;
  }
  if ((st = alps_prepare(ctx))) return st;
  double kperp = s.kperp, kpar = s.kpar;
  if ((st = alps_set_k(ctx, kperp, kpar))) return st;
  std::vector<alps_complex> wroots(ALPS_MAX_ROOTS, alps_complex{0, 0});
  int nroots = in.nroots;
  std::string run = in.runname;
  if (in.use_map) {
    // map_search (src/ALPS_fns.f90:3595-3788)
    const alps_map_params& mp = in.map;
    int n = mp.nr * mp.ni;
    std::vector<alps_complex> om(n), cal(n);
    std::vector<double> val(n);
    if ((st = alps_map(ctx, &mp, om.data(), cal.data(), val.data()))) return st;
    FILE* fm = std::fopen((soldir + "/" + run + ".map").c_str(), "w");
    if (!fm) return ALPS_E_IO;
    for (int ir = 0; ir < mp.nr; ++ir) {
      for (int ii = 0; ii < mp.ni; ++ii) {
        int k = ir * mp.ni + ii;
        std::fprintf(fm, "%s%s%s%s%s\n", fmt_es(om[k].re, 16, 6, 3).c_str(), fmt_es(om[k].im, 16, 6, 3).c_str(),
                     fmt_es(val[k], 16, 6, 3).c_str(), fmt_es(cal[k].re, 16, 6, 3).c_str(),
                     fmt_es(cal[k].im, 16, 6, 3).c_str());
      }
      std::fprintf(fm, "\n");
    }
    std::fclose(fm);
    if (in.determine_minima && mp.nr > 1 && mp.ni > 1) {
      std::vector<int> iroots(2 * ALPS_MAX_ROOTS);
      int nfound = 0;
      if ((st = alps_find_minima(val.data(), mp.nr, mp.ni, ALPS_MAX_ROOTS, iroots.data(), &nfound))) return st;
      for (int iw = 0; iw < nfound; ++iw) wroots[iw] = om[iroots[2 * iw] * mp.ni + iroots[2 * iw + 1]];
      nroots = std::min(nroots, nfound);
    }
  } else {
    for (int k = 0; k < nroots; ++k) wroots[k] = in.guess[k];
  }
  // refine_guess (src/ALPS_fns.f90:3793-3856)
  {
    if ((st = alps_secant(ctx, s.secant_method, nroots, wroots.data(), nullptr, nullptr))) return st;
    FILE* fr = std::fopen((soldir + "/" + run + ".roots").c_str(), "w");
    if (!fr) return ALPS_E_IO;
    for (int iw = 0; iw < nroots; ++iw) {
      alps_complex D;
      if ((st = alps_disp(ctx, wroots[iw], &D, nullptr, nullptr, nullptr))) {
        std::fclose(fr);
        return st;
      }
      double a = std::hypot(D.re, D.im);
      if (a != 0.0)
        std::fprintf(fr, "%4d%s%s%s%s%s\n", iw + 1, fmt_es(wroots[iw].re, 14, 4, 3).c_str(),
                     fmt_es(wroots[iw].im, 14, 4, 3).c_str(), fmt_es(std::log10(a), 14, 4, 3).c_str(),
                     fmt_es(D.re, 14, 4, 3).c_str(), fmt_es(D.im, 14, 4, 3).c_str());
    }
    std::fclose(fr);
  }
  if (in.n_scan > 0 && in.scan_option == 2)
    return double_scan(ctx, in, soldir, run, nroots, wroots, kperp, kpar);
  // om_scan (src/ALPS_fns.f90:2198-2600), scan_option 1: scans in sequence
  const char* ids[5] = {"k1_k2_", "theta_", "kcstq_", "kperp_", "kpara_"};
  for (int ik = 1; ik <= in.n_scan; ++ik) {
    const alps_scan_def& sc = in.scan[ik - 1];
    std::vector<std::string> names(nroots);
    for (int r = 0; r < nroots; ++r) {
      names[r] = soldir + "/" + run + ".scan_" + ids[sc.type_s] + std::to_string(ik) + ".root_" + std::to_string(r + 1);
      FILE* fo = std::fopen(names[r].c_str(), "w");
      if (!fo) return ALPS_E_IO;
      std::fprintf(fo, "%s%s%s%s\n", fmt_es(kperp, 14, 4, 3).c_str(), fmt_es(kpar, 14, 4, 3).c_str(),
                   fmt_es(wroots[r].re, 14, 4, 3).c_str(), fmt_es(wroots[r].im, 14, 4, 3).c_str());
      std::fclose(fo);
    }
    // eigenfunctions and heating rates (calc_eigen) on every output row
    const bool want_eig = sc.eigen || sc.heating;
    auto eig_name = [&](const char* kind, int r) {
      return soldir + "/" + run + "." + kind + "_" + ids[sc.type_s] + std::to_string(ik) + ".root_" +
             std::to_string(r + 1);
    };
    auto write_eigen = [&](int r, const alps_eigen& e, const char* mode) -> int {
      std::vector<double> head = {kperp, kpar, wroots[r].re, wroots[r].im}, ev, hv, mv;
      eigen_columns(e, s.nspec, ev, hv, mv);
      const char* kinds[3] = {"eigen", "heat", "heat_mech"};
      const std::vector<double>* cols[3] = {&ev, &hv, &mv};
      for (int q = 0; q < 3; ++q) {
        if (q == 0 && !sc.eigen) continue;
        if (q > 0 && !sc.heating) continue;
        FILE* f = std::fopen(eig_name(kinds[q], r).c_str(), mode);
        if (!f) return ALPS_E_IO;
        std::vector<double> row = head;
        row.insert(row.end(), cols[q]->begin(), cols[q]->end());
        write_row(f, row);
        std::fclose(f);
      }
      return ALPS_OK;
    };
    if (want_eig) {
      std::vector<alps_eigen> eg(nroots);
      if ((st = alps_calc_eigen(ctx, nroots, wroots.data(), sc.eigen, sc.heating, eg.data()))) return st;
      for (int r = 0; r < nroots; ++r)
        if ((st = write_eigen(r, eg[r], "w"))) return st;
    }
    int nt = sc.n_out * sc.n_res;
    double kperp_last = kperp, kpar_last = kpar;
    double theta_0 = std::atan(kperp_last / kpar_last);
    double k_0 = std::sqrt(kperp_last * kperp_last + kpar_last * kpar_last);
    std::vector<char> jump(nroots, 1);
    for (int it = 1; it <= nt; ++it) {
      switch (sc.type_s) {
        case 0:
          if (sc.log_scan) {
            kperp = std::pow(10.0, std::log10(kperp_last) + sc.diff * it);
            kpar = std::pow(10.0, std::log10(kpar_last) + sc.diff2 * it);
          } else {
            kperp = kperp_last + sc.diff * it;
            kpar = kpar_last + sc.diff2 * it;
          }
          break;
        case 1: {
          double th = sc.log_scan ? std::pow(10.0, std::log10(theta_0) + sc.diff * it) : theta_0 + sc.diff * it;
          kperp = k_0 * std::sin(th);
          kpar = k_0 * std::cos(th);
          break;
        }
        case 2: {
          double kt = sc.log_scan ? std::pow(10.0, std::log10(k_0) + sc.diff * it) : (k_0) + sc.diff * it;
          kperp = kt * std::sin(theta_0);
          kpar = kt * std::cos(theta_0);
          break;
        }
        case 3:
          kperp = sc.log_scan ? std::pow(10.0, std::log10(kperp_last) + sc.diff * it) : kperp_last + sc.diff * it;
          break;
        case 4:
          kpar = sc.log_scan ? std::pow(10.0, std::log10(kpar_last) + sc.diff * it) : kpar_last + sc.diff * it;
          break;
      }
      if ((st = alps_set_k(ctx, kperp, kpar))) return st;
      bool alljump = false;
      for (int r = 0; r < nroots; ++r) alljump = alljump || jump[r];
      if (!alljump) return ALPS_E_ROOTS_DIVERGED;
      std::vector<int> idx;
      std::vector<alps_complex> sub;
      for (int r = 0; r < nroots; ++r)
        if (jump[r]) {
          idx.push_back(r);
          sub.push_back(wroots[r]);
        }
      if ((st = alps_secant(ctx, s.secant_method, (int)sub.size(), sub.data(), nullptr, nullptr))) return st;
      std::vector<alps_eigen> eg;
      if (want_eig && it % sc.n_res == 0) {
        eg.resize(sub.size());
        if ((st = alps_calc_eigen(ctx, (int)sub.size(), sub.data(), sc.eigen, sc.heating, eg.data()))) return st;
      }
      for (size_t q = 0; q < idx.size(); ++q) {
        int r = idx[q];
        wroots[r] = sub[q];
        double re = wroots[r].re;
        if (std::fabs(re) >= 1.79769313486231571e308 || re != re) jump[r] = 0;
        for (int imm = 0; imm < r; ++imm)
          if (std::hypot(wroots[r].re - wroots[imm].re, wroots[r].im - wroots[imm].im) < s.D_gap) {
            wroots[r] = alps_complex{0.0, 0.0};
            jump[r] = 0;
          }
        if (it % sc.n_res == 0) {
          FILE* fo = std::fopen(names[r].c_str(), "a");
          if (!fo) return ALPS_E_IO;
          std::fprintf(fo, "%s%s%s%s\n", fmt_es(kperp, 14, 4, 3).c_str(), fmt_es(kpar, 14, 4, 3).c_str(),
                       fmt_es(wroots[r].re, 14, 4, 3).c_str(), fmt_es(wroots[r].im, 14, 4, 3).c_str());
          std::fclose(fo);
          if (!eg.empty() && (st = write_eigen(r, eg[q], "a"))) return st;
        }
      }
    }
  }
  return ALPS_OK;
}


// interpolation/interpolation.f90 (program interpolate): namelist, coarse
// table, spline on the device, .array output
int alps_run_interpolation(const char* input_path, const char* workdir) {
  if (!input_path) return ALPS_E_INVALID;
  std::ifstream fin(input_path);
  if (!fin) return ALPS_E_IO;
  std::stringstream ss;
  ss << fin.rdbuf();
  auto nl = parse_namelists(ss.str());
  Reader r{nl.count("system") ? &nl.at("system") : nullptr};
  // defaults of read_in_params (interpolation.f90:259-273)
  char filename[512] = "";
  double smoothing = 1.0, threshold = 0.0, mult_pperp = 1.0, mult_ppar = 1.0, mult_f = 1.0;
  double pperp_max_set = -9999.0, ppar_max_set = -9999.0, pperp_min_set = -9999.0, ppar_min_set = -9999.0;
  int nperp = 50, npar = 100, mode = 1, out_to_file = 0, do_normalize = 0;
  r.s("filename", filename, sizeof filename);
  r.d("smoothing", smoothing);
  r.i("nperp", nperp);
  r.i("npar", npar);
  r.d("ppar_min_set", ppar_min_set);
  r.d("ppar_max_set", ppar_max_set);
  r.d("pperp_min_set", pperp_min_set);
  r.d("pperp_max_set", pperp_max_set);
  r.i("mode", mode);
  r.d("threshold", threshold);
  r.l("out_to_file", out_to_file);
  r.l("do_normalize", do_normalize);
  r.d("mult_pperp", mult_pperp);
  r.d("mult_ppar", mult_ppar);
  r.d("mult_f", mult_f);
  std::string in(input_path), dir;
  size_t slash = in.rfind('/');
  if (slash != std::string::npos) dir = in.substr(0, slash + 1);
  std::string cpath = filename;
  if (!cpath.empty() && cpath[0] != '/') cpath = dir + cpath;
  std::ifstream fc(cpath);
  if (!fc) return ALPS_E_IO;
  // samples with f above the threshold (mode 1: pperp ppar f; 2: ppar pperp f)
  std::vector<double> gp, gl, gf;
  double a, b, c;
  while (fc >> a >> b >> c) {
    if (!(c > threshold)) continue;
    gp.push_back(mode == 2 ? b : a);
    gl.push_back(mode == 2 ? a : b);
    gf.push_back(c);
  }
  if (gf.empty()) return ALPS_E_INVALID;  // "No data points in selection."
  double pperp_max = -999999.0, pperp_min = 999999.0, ppar_max = -999999.0, ppar_min = 999999.0;
  for (size_t k = 0; k < gf.size(); ++k) {
    pperp_max = std::max(pperp_max, gp[k]);
    pperp_min = std::min(pperp_min, gp[k]);
    ppar_max = std::max(ppar_max, gl[k]);
    ppar_min = std::min(ppar_min, gl[k]);
  }
  pperp_max *= mult_pperp;
  pperp_min *= mult_pperp;
  ppar_max *= mult_ppar;
  ppar_min *= mult_ppar;
  if (pperp_max_set != -9999.0) pperp_max = pperp_max_set;
  if (ppar_max_set != -9999.0) ppar_max = ppar_max_set;
  if (pperp_min_set != -9999.0) pperp_min = pperp_min_set;
  if (ppar_min_set != -9999.0) ppar_min = ppar_min_set;
  for (size_t k = 0; k < gf.size(); ++k) {
    gp[k] *= mult_pperp;
    gl[k] *= mult_ppar;
  }
  alps_interp_params ip;
  ip.nperp = nperp;
  ip.npar = npar;
  ip.smoothing = smoothing;
  ip.pperp_min = pperp_min;
  ip.pperp_max = pperp_max;
  ip.ppar_min = ppar_min;
  ip.ppar_max = ppar_max;
  ip.do_normalize = do_normalize;
  ip.mult_f = mult_f;
  const size_t nf = (size_t)(nperp + 1) * (npar + 1);
  std::vector<double> op(nf), ol(nf), of(nf);
  int st = alps_interpolate(gp.data(), gl.data(), gf.data(), (int)gf.size(), &ip, op.data(), ol.data(), of.data());
  if (st) return st;
  FILE* out = stdout;
  if (out_to_file) {
    std::string base = in.substr(slash == std::string::npos ? 0 : slash + 1);
    if (base.size() > 3 && base.compare(base.size() - 3, 3, ".in") == 0) base = base.substr(0, base.size() - 3);
    std::string wd = workdir ? workdir : ".";
    out = std::fopen((wd + "/" + base + ".array").c_str(), "w");
    if (!out) return ALPS_E_IO;
  }
  for (size_t t = 0; t < nf; ++t) std::fprintf(out, "%25.16E %25.16E %25.16E\n", op[t], ol[t], of[t]);
  if (out_to_file) std::fclose(out);
  return ALPS_OK;
}

}  // extern "C"
