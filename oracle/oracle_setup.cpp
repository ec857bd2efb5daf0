// CPU oracle, setup half: potential-file reader, basis enumeration,
// Clebsch-Gordan couplings and the cubic-Hermite radial lookup tables.
//
// TEST INFRASTRUCTURE ONLY (the parity checker; see oracle.h). Each routine
// restates the reference routine cited beside it.
#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>
#include <vector>

#include "oracle.h"

namespace {

const double kPi = 3.14159265358979323846264338327950288419;

// ---------------------------------------------------------------------------
// Fortran list-directed input (the reference reads every record with read(1,*)).
// Each read starts on a fresh line, takes as many lines as it needs and drops
// the rest of its last line.
class ListReader {
 public:
  explicit ListReader(std::istream& in) : in_(in) {}
  // returns false at end of file before all n items were read (iostat = -1)
  bool read(int n, std::vector<std::string>& out) {
    out.clear();
    std::string line;
    while ((int)out.size() < n) {
      if (!std::getline(in_, line)) return false;
      split(line, out);
    }
    if ((int)out.size() > n) out.resize(n);
    return true;
  }
  bool skip() {
    std::string line;
    return (bool)std::getline(in_, line);
  }

 private:
  static void split(const std::string& line, std::vector<std::string>& out) {
    size_t i = 0, n = line.size();
    while (i < n) {
      while (i < n && (std::isspace((unsigned char)line[i]) || line[i] == ',')) ++i;
      if (i >= n) break;
      if (line[i] == '/') return;  // slash terminates a list-directed record
      if (line[i] == '\'' || line[i] == '"') {
        char q = line[i++];
        size_t j = line.find(q, i);
        if (j == std::string::npos) j = n;
        out.push_back(line.substr(i, j - i));
        i = j + 1;
        continue;
      }
      size_t j = i;
      while (j < n && !std::isspace((unsigned char)line[j]) && line[j] != ',') ++j;
      out.push_back(line.substr(i, j - i));
      i = j;
    }
  }
  std::istream& in_;
};

bool to_int(const std::string& t, int& v) {
  char* end = nullptr;
  long x = std::strtol(t.c_str(), &end, 10);
  if (end == t.c_str() || *end != '\0') return false;
  v = (int)x;
  return true;
}

bool to_double(std::string t, double& v) {
  for (auto& ch : t)
    if (ch == 'd' || ch == 'D') ch = 'E';
  char* end = nullptr;
  v = std::strtod(t.c_str(), &end);
  return !(end == t.c_str() || *end != '\0');
}

bool to_logical(const std::string& t, bool& v) {
  size_t i = 0;
  if (i < t.size() && t[i] == '.') ++i;
  if (i >= t.size()) return false;
  char c = (char)std::toupper((unsigned char)t[i]);
  if (c == 'T') { v = true; return true; }
  if (c == 'F') { v = false; return true; }
  return false;
}

// ---------------------------------------------------------------------------
// src/radial.F90:6-33
void calcCheb(int n, double x, std::vector<double>& cheb1, std::vector<double>& dcheb1) {
  std::vector<double> cheb2(n + 1);
  cheb1.assign(n + 1, 0.0);
  dcheb1.assign(n + 1, 0.0);
  double tx = 2.0 * x;
  cheb1[0] = 1.0;
  dcheb1[0] = 0.0;
  cheb2[0] = 1.0;
  if (n > 0) {
    cheb1[1] = x;
    cheb2[1] = tx;
    for (int m = 1; m <= n - 1; ++m) {
      cheb1[m + 1] = tx * cheb1[m] - cheb1[m - 1];
      cheb2[m + 1] = tx * cheb2[m] - cheb2[m - 1];
    }
    for (int m = 1; m <= n; ++m) dcheb1[m] = (double)m * cheb2[m - 1];
  }
}

// src/radial.F90:430-606; gr/dgr are 1-based (index 0 unused)
bool radbase(int radtype, double radpara, int nradbase, double cutoff, double dcutoff, double r,
             std::vector<double>& gr, std::vector<double>& dgr) {
  gr.assign(nradbase + 1, 0.0);
  dgr.assign(nradbase + 1, 0.0);
  if (r >= cutoff) return true;
  std::vector<double> cheb, dcheb;
  double x, dx, x0, y1, dy1, y2, env, denv, y0;
  switch (radtype) {
    case 3: {
      x0 = r / cutoff;
      y1 = std::exp(-radpara * x0);
      dy1 = -radpara * y1 / cutoff;
      y2 = std::exp(-radpara);
      x = 1.0 - 2.0 * (y1 - y2) / (1.0 - y2);
      dx = -2.0 * dy1 / (1.0 - y2);
      int ncheb = nradbase - 1;
      calcCheb(ncheb, x, cheb, dcheb);
      gr[1] = cheb[0];
      dgr[1] = dcheb[0] * dx;
      for (int n = 2; n <= nradbase; ++n) {
        gr[n] = 0.5 - 0.5 * cheb[n - 1];
        dgr[n] = -0.5 * dcheb[n - 1] * dx;
      }
      env = 0.5 * (1.0 + std::cos(kPi * x0));
      denv = -0.5 * std::sin(kPi * x0) * kPi / cutoff;
      for (int n = 1; n <= nradbase; ++n) {
        dgr[n] = gr[n] * denv + dgr[n] * env;
        gr[n] = gr[n] * env;
      }
      break;
    }
    case 4: {
      x0 = r / cutoff;
      y1 = std::exp(-radpara * x0);
      dy1 = -radpara * y1 / cutoff;
      y2 = std::exp(-radpara);
      x = 1.0 - 2.0 * (y1 - y2) / (1.0 - y2);
      dx = -2.0 * dy1 / (1.0 - y2);
      int ncheb = nradbase - 1;
      calcCheb(ncheb, x, cheb, dcheb);
      gr[1] = cheb[0];
      dgr[1] = dcheb[0] * dx;
      for (int n = 2; n <= nradbase; ++n) {
        gr[n] = 0.5 - 0.5 * cheb[n - 1];
        dgr[n] = -0.5 * dcheb[n - 1] * dx;
      }
      break;
    }
    case 5: {
      x0 = r / cutoff;
      y0 = (1.0 - x0);
      dy1 = std::pow(y0, radpara - 1.0);
      y1 = 1.0 - dy1 * y0;
      dy1 = radpara / cutoff * dy1;
      x = 2.0 * y1 - 1.0;
      dx = 2.0 * dy1;
      int ncheb = nradbase;
      calcCheb(ncheb, x, cheb, dcheb);
      for (int n = 1; n <= nradbase; ++n) {
        gr[n] = 0.5 - 0.5 * cheb[n];
        dgr[n] = -0.5 * dcheb[n] * dx;
      }
      break;
    }
    case 6: {
      x0 = r / cutoff;
      y0 = (1.0 - x0);
      dy1 = std::pow(y0, radpara - 1.0);
      y1 = 1.0 - dy1 * y0;
      dy1 = radpara / cutoff * dy1;
      x = 2.0 * y1 - 1.0;
      dx = 2.0 * dy1;
      int ncheb = nradbase - 1;
      calcCheb(ncheb, x, cheb, dcheb);
      gr[1] = cheb[0];
      dgr[1] = dcheb[0] * dx;
      for (int n = 1; n <= nradbase - 1; ++n) {
        gr[n + 1] = 0.5 - 0.5 * cheb[n];
        dgr[n + 1] = -0.5 * dcheb[n] * dx;
      }
      env = 0.5 * (1.0 + std::cos(kPi * x0));
      denv = -0.5 * std::sin(kPi * x0) * kPi / cutoff;
      for (int n = 1; n <= nradbase; ++n) {
        dgr[n] = gr[n] * denv + dgr[n] * env;
        gr[n] = gr[n] * env;
      }
      break;
    }
    case 7: {
      x0 = r / cutoff;
      x = 1.0 - 2.0 * x0 * x0;
      dx = -(4.0 / cutoff) * x0;
      int ncheb = nradbase;
      calcCheb(ncheb, x, cheb, dcheb);
      for (int n = 1; n <= nradbase; ++n) {
        gr[n] = cheb[n];
        dgr[n] = dcheb[n] * dx;
      }
      break;
    }
    case 8: {
      x0 = r / cutoff;
      x = 1.0 - 2.0 * x0;
      dx = -2.0 / cutoff;
      int ncheb = nradbase;
      calcCheb(ncheb, x, cheb, dcheb);
      for (int n = 1; n <= nradbase; ++n) {
        gr[n] = cheb[n] - 1.0;
        dgr[n] = dcheb[n] * dx;
      }
      break;
    }
    default:
      return false;  // types 0-2 stop with "Not working." in the reference
  }
  dx = cutoff - dcutoff;
  if (r > dx) {
    double fcut = 0.5 * (1.0 + std::cos(kPi * (r - dx) / dcutoff));
    double dfcut = -0.5 * std::sin(kPi * (r - dx) / dcutoff) * kPi / dcutoff;
    for (int n = 1; n <= nradbase; ++n) {
      dgr[n] = gr[n] * dfcut + dgr[n] * fcut;
      gr[n] = gr[n] * fcut;
    }
  }
  return true;
}

// src/radial.F90:610-626 for one element pair; fr/dfr(nr, l) with nr 1-based
void radfunc(int nradbase, int nradial, int lmax, FArr<double>& crad, const std::vector<double>& gr,
             const std::vector<double>& dgr, FArr<double>& fr, FArr<double>& dfr) {
  for (int l = 0; l <= lmax; ++l)
    for (int nr = 1; nr <= nradial; ++nr) {
      double s = 0.0, ds = 0.0;
      for (int n = 1; n <= nradbase; ++n) {
        s += crad(n, nr, l) * gr[n];
        ds += crad(n, nr, l) * dgr[n];
      }
      fr(nr, l) = s;
      dfr(nr, l) = ds;
    }
}

// src/radial.F90:630-668 (pre and lambda are local copies, made positive)
void radcore(double r, double pre, double lambda, double cutoff, double& cr, double& dcr) {
  if (r < cutoff) {
    pre = std::fabs(pre);
    lambda = std::fabs(lambda);
    double r2 = r * r;
    double lr2 = lambda * r2;
    if (lr2 < 50.0) {
      double y = std::exp(-lr2);
      cr = pre * y / r;
      dcr = -pre * y * (2.0 * lr2 + 1.0) / r2;
      double x0 = r / cutoff;
      double env = 0.5 * (1.0 + std::cos(kPi * x0));
      double denv = -0.5 * std::sin(kPi * x0) * kPi / cutoff;
      dcr = cr * denv + dcr * env;
      cr = cr * env;
    } else {
      cr = 0.0;
      dcr = 0.0;
    }
  } else {
    cr = 0.0;
    dcr = 0.0;
  }
}

// cubic-Hermite coefficients on [n, n+1] in bin units (src/radial.F90:244-254)
inline void hermite(double f0, double f0d1, double f1, double f1d1, double* c) {
  c[0] = f0;
  c[1] = f0d1;
  c[2] = 3.0 * (f1 - f0) - f1d1 - 2.0 * f0d1;
  c[3] = -2.0 * (f1 - f0) + f1d1 + f0d1;
}

// src/radial.F90:164-305 (single element; the scoreRnl smoothness scores do not
// feed the energy and are not restated)
bool setup_lut_atomic(OracleState& s) {
  const int nlut = s.nlut;
  const int nb = s.nradbase_atomic, nrad = s.nradial3_atomic, lm = s.l3max_atomic;
  s.rscalelookup_atomic = (double)nlut / s.cutoff;
  s.invrscalelookup_atomic = 1.0 / s.rscalelookup_atomic;
  s.lutfrs_atomic.init({{0, 3}, {1, nrad}, {0, lm}, {1, nlut}});
  s.lutgrs_atomic.init({{0, 3}, {1, nb}, {1, nlut}});
  s.luthcrs_atomic.init({{0, 3}, {1, nlut}});
  std::vector<double> f1g(nb + 1, 0.0), f1gd1(nb + 1, 0.0);
  FArr<double> f1f({{1, nrad}, {0, lm}}), f1fd1({{1, nrad}, {0, lm}});
  FArr<double> fr({{1, nrad}, {0, lm}}), dfr({{1, nrad}, {0, lm}});
  double f1cr = 0.0, f1crd1 = 0.0;
  std::vector<double> gr, dgr;
  double c[4];
  for (int n = nlut; n >= 1; --n) {
    double x = s.invrscalelookup_atomic * (double)n;
    double lam = s.lambda[0], cu = s.cut[0], dc = s.dcut[0];
    if (!radbase(s.radtype_atomic, lam, nb, cu, dc, x, gr, dgr)) return false;
    radfunc(nb, nrad, lm, s.crad_atomic, gr, dgr, fr, dfr);
    double pc = s.corepara(1), lc = s.corepara(2), cr, dcr;
    radcore(x, pc, lc, cu, cr, dcr);
    for (int nr = 1; nr <= nb; ++nr) {
      hermite(gr[nr], dgr[nr] * s.invrscalelookup_atomic, f1g[nr], f1gd1[nr], c);
      for (int q = 0; q < 4; ++q) s.lutgrs_atomic(q, nr, n) = c[q];
      f1g[nr] = c[0];
      f1gd1[nr] = c[1];
    }
    for (int l = 0; l <= lm; ++l)
      for (int nr = 1; nr <= nrad; ++nr) {
        hermite(fr(nr, l), dfr(nr, l) * s.invrscalelookup_atomic, f1f(nr, l), f1fd1(nr, l), c);
        for (int q = 0; q < 4; ++q) s.lutfrs_atomic(q, nr, l, n) = c[q];
        f1f(nr, l) = c[0];
        f1fd1(nr, l) = c[1];
      }
    hermite(cr, dcr * s.invrscalelookup_atomic, f1cr, f1crd1, c);
    for (int q = 0; q < 4; ++q) s.luthcrs_atomic(q, n) = c[q];
    f1cr = c[0];
    f1crd1 = c[1];
  }
  return true;
}

// src/radial.F90:309-426
bool setup_lut_magnetic(OracleState& s) {
  const int nlut = s.nlut;
  const int nb = s.nradbase_magnetic, nrad = s.nradial2_magnetic, lm = s.l2max_magnetic;
  s.rscalelookup_magnetic = (double)nlut / s.cutoff_magnetic;
  s.invrscalelookup_magnetic = 1.0 / s.rscalelookup_magnetic;
  s.lutfrs_magnetic.init({{0, 3}, {1, nrad}, {0, lm}, {1, nlut}});
  s.lutgrs_magnetic.init({{0, 3}, {1, nb}, {1, nlut}});
  std::vector<double> f1g(nb + 1, 0.0), f1gd1(nb + 1, 0.0);
  FArr<double> f1f({{1, nrad}, {0, lm}}), f1fd1({{1, nrad}, {0, lm}});
  FArr<double> fr({{1, nrad}, {0, lm}}), dfr({{1, nrad}, {0, lm}});
  std::vector<double> gr, dgr;
  double c[4];
  for (int n = nlut; n >= 1; --n) {
    double x = s.invrscalelookup_magnetic * (double)n;
    double lam = s.lambda[1], cu = s.cut[1], dc = s.dcut[1];
    if (!radbase(s.radtype_magnetic, lam, nb, cu, dc, x, gr, dgr)) return false;
    radfunc(nb, nrad, lm, s.crad_magnetic, gr, dgr, fr, dfr);
    for (int nr = 1; nr <= nb; ++nr) {
      hermite(gr[nr], dgr[nr] * s.invrscalelookup_magnetic, f1g[nr], f1gd1[nr], c);
      for (int q = 0; q < 4; ++q) s.lutgrs_magnetic(q, nr, n) = c[q];
      f1g[nr] = c[0];
      f1gd1[nr] = c[1];
    }
    for (int l = 0; l <= lm; ++l)
      for (int nr = 1; nr <= nrad; ++nr) {
        hermite(fr(nr, l), dfr(nr, l) * s.invrscalelookup_magnetic, f1f(nr, l), f1fd1(nr, l), c);
        for (int q = 0; q < 4; ++q) s.lutfrs_magnetic(q, nr, l, n) = c[q];
        f1f(nr, l) = c[0];
        f1fd1(nr, l) = c[1];
      }
  }
  return true;
}

// src/util.F90:4149-4252 (Racah formula with FP64 factorials)
void setupcg(OracleState& s) {
  const int lmax = s.lmax;
  s.cgcoeff.init({{0, 2 * lmax}, {0, 2 * lmax}, {0, 4 * lmax}, {-2 * lmax, 2 * lmax},
                  {-2 * lmax, 2 * lmax}, {-4 * lmax, 4 * lmax}});
  auto& fac = s.fac;
  for (int J = 0; J <= 4 * lmax; ++J)
    for (int j1 = 0; j1 <= 2 * lmax; ++j1)
      for (int j2 = 0; j2 <= 2 * lmax; ++j2) {
        if (!((j1 + j2 >= J) && (std::abs(j1 - j2) <= J))) continue;
        for (int m1 = -j1; m1 <= j1; ++m1)
          for (int m2 = -j2; m2 <= j2; ++m2) {
            int M = m1 + m2;
            if (std::abs(M) > J) continue;
            double prefac = ((double)(2 * J + 1) * fac(j1 + j2 - J) * fac(j1 - j2 + J) *
                             fac(-j1 + j2 + J) / fac(j1 + j2 + J + 1)) *
                            (fac(J + M) * fac(J - M) * fac(j1 + m1) * fac(j1 - m1) * fac(j2 + m2) *
                             fac(j2 - m2));
            prefac = std::sqrt(prefac);
            double xsum = 0.0;
            for (int k = 0; k <= 4 * lmax; ++k) {
              int a = j1 + j2 - J - k, b = j1 - m1 - k, c = j2 + m2 - k, d = J - j2 + m1 + k,
                  e = J - j1 - m2 + k;
              if (a >= 0 && b >= 0 && c >= 0 && d >= 0 && e >= 0) {
                xsum += (double)((k % 2 == 0) ? 1 : -1) /
                        (fac(k) * fac(a) * fac(b) * fac(c) * fac(d) * fac(e));
              }
            }
            s.cgcoeff(j1, j2, J, m1, m2, M) = prefac * xsum;
          }
      }
}

// rank-2/3/4 selection rules of bcreate (src/util.F90:4673-4946) for one element.
// veck orders by element, then l, then n (src/util.F90:4738).
int veck(const OracleState& s, int nele, int l, int nr) {
  const int nelements = 1;
  return ((nelements + 1 - nele) * (s.lmax + 1) + l) * (s.nradial + 1) + nr;
}

bool triangle_even(int a, int b, int c) {
  return (a + b >= c) && (std::abs(a - b) <= c) && ((a + b + c) % 2 == 0);
}

// bcreate rank 4 (src/util.F90:4790-4857): allowed intermediate couplings
void rank4_lints(const OracleState& s, const int* vecn, const int* vecnr, const int* vecl,
                 std::vector<int>& lints, bool& isbasis) {
  int nc[4];
  for (int i = 0; i < 4; ++i) nc[i] = veck(s, vecn[i], vecl[i], vecnr[i]);
  int l1 = vecl[0], l2 = vecl[1], l3 = vecl[2], l4 = vecl[3];
  int lintmax = 2 * std::max(std::max(l1, l2), std::max(l3, l4));
  lints.clear();
  for (int lint = 0; lint <= lintmax; ++lint) {
    bool ok = true;
    if (lint > l1 + l2 || lint > l3 + l4) ok = false;
    if (lint < std::abs(l1 - l2) || lint < std::abs(l3 - l4)) ok = false;
    if (nc[0] == nc[1] && lint % 2 != 0) ok = false;
    if (nc[2] == nc[3] && lint % 2 != 0) ok = false;
    if (ok) lints.push_back(lint);
  }
  isbasis = !lints.empty();
  if ((l1 + l2 + l3 + l4) % 2 != 0) isbasis = false;
}

// src/util.F90:1613-2814 restricted to one element and ranks 1-4
bool setuptables(OracleState& s, std::string& err) {
  // angular bounds (src/util.F90:1677-1698)
  s.lmaxsq_atomic = (s.l3max_atomic + 1) * (s.l3max_atomic + 1);
  s.lmaxhalf_atomic = (s.l3max_atomic + 1) * (s.l3max_atomic + 2) / 2;
  s.lmaxsq_magnetic = (s.l2max_magnetic + 1) * (s.l2max_magnetic + 1);
  s.lmaxhalf_magnetic = (s.l2max_magnetic + 1) * (s.l2max_magnetic + 2) / 2;

  // factorials (src/util.F90:1703-1714)
  s.fac.init({{0, 8 * s.lmax + 1}});
  double xfac = 1.0;
  s.fac(0) = xfac;
  for (int l = 0; l <= 8 * s.lmax; ++l) {
    xfac = (double)(l + 1) * xfac;
    s.fac(l + 1) = xfac;
  }

  // shindex: m >= 0 first, then m < 0 (src/util.F90:1717-1776)
  auto make_sh = [](int lm, FArr<int>& idx, FArr<int>& back) {
    idx.init({{0, lm}, {-lm, lm}});
    back.init({{1, (lm + 1) * (lm + 1)}});
    int k = 1;
    idx(0, 0) = k;
    back(k) = 0;
    if (lm >= 1) {
      for (int l = 1; l <= lm; ++l)
        for (int m = 0; m <= l; ++m) {
          ++k;
          idx(l, m) = k;
          back(k) = l;
        }
      for (int l = 1; l <= lm; ++l)
        for (int m = -l; m <= -1; ++m) {
          ++k;
          idx(l, m) = k;
          back(k) = l;
        }
    }
  };
  make_sh(s.l3max_atomic, s.shindex_atomic, s.shback_atomic);
  make_sh(s.l2max_magnetic, s.shindex_magnetic, s.shback_magnetic);

  setupcg(s);

  // 1-body (src/util.F90:1812-1827)
  s.nvar1 = s.nradbase_magnetic;
  s.b1occ.init({{1, std::max(1, s.nvar1)}});
  s.b1index.init({{1, std::max(1, s.nvar1)}});
  for (int nr = 1; nr <= s.nradbase_magnetic; ++nr) {
    s.b1occ(nr) = 1;
    s.b1index(nr) = nr;
  }

  // 2-body (src/util.F90:1838-1959)
  s.nvar2l = s.l2max_magnetic + 1;
  s.b2lindex.init({{1, s.nvar2l}});
  for (int l = 0; l <= s.l2max_magnetic; ++l) s.b2lindex(l + 1) = l;
  {
    std::vector<std::array<int, 4>> rows;
    for (int nr1 = 1; nr1 <= s.nradial2_magnetic; ++nr1)
      for (int nr2 = 1; nr2 <= s.nradial2_magnetic; ++nr2)
        for (int nr3 = 1; nr3 <= s.nradbase_atomic; ++nr3)
          for (int k = 1; k <= s.nvar2l; ++k) {
            int l = s.b2lindex(k);
            // bcreate rank 2: isbasis (l1 >= l2) always true here, isordered on veck
            if (veck(s, 1, l, nr1) >= veck(s, 1, l, nr2)) rows.push_back({nr1, nr2, nr3, l});
          }
    s.nvar2 = (int)rows.size();
    int nv = std::max(1, s.nvar2);
    s.b2occ.init({{1, nv}});
    s.b2index.init({{1, 4}, {1, nv}});
    s.b2map.init({{1, nv}});
    for (int n = 1; n <= s.nvar2; ++n) {
      s.b2occ(n) = 1;
      for (int q = 0; q < 4; ++q) s.b2index(q + 1, n) = rows[n - 1][q];
      s.b2map(n) = s.b2index(4, n) + 1;
    }
    s.madd2.init({{1, s.nvar2l}});
    int maddmax = 0;
    for (int k = 1; k <= s.nvar2l; ++k) {
      s.madd2(k) = 2 * s.b2lindex(k) + 1;
      maddmax = std::max(maddmax, s.madd2(k));
    }
    s.b2lm.init({{1, s.nvar2l}, {1, maddmax}});
    for (int k = 1; k <= s.nvar2l; ++k) {
      int l1 = s.b2lindex(k), m = 0;
      for (int m1 = -l1; m1 <= l1; ++m1) s.b2lm(k, ++m) = m1;
    }
  }

  // 3-body angular lists (src/util.F90:2004-2050)
  s.nvar3l_atomic = s.l3max_atomic + 1;
  s.b3lindex_atomic.init({{1, s.nvar3l_atomic}});
  for (int l1 = 0; l1 <= s.l3max_atomic; ++l1) s.b3lindex_atomic(l1 + 1) = l1;
  {
    std::vector<std::array<int, 3>> rows;
    for (int l2 = 0; l2 <= s.l3max_magnetic; ++l2)
      for (int l3 = 0; l3 <= s.l3max_magnetic; ++l3)
        for (int l4 = 0; l4 <= s.l3max_magnetic; ++l4)
          if (triangle_even(l2, l3, l4)) rows.push_back({l2, l3, l4});
    s.nvar3l_magnetic = (int)rows.size();
    s.b3lindex_magnetic.init({{1, 3}, {1, std::max(1, s.nvar3l_magnetic)}});
    for (int k = 1; k <= s.nvar3l_magnetic; ++k)
      for (int q = 0; q < 3; ++q) s.b3lindex_magnetic(q + 1, k) = rows[k - 1][q];
  }

  // 3-body clusters (src/util.F90:2055-2230)
  {
    std::vector<std::array<int, 9>> rows;
    const int na = s.nradial3_atomic, nm = s.nradial3_magnetic;
    const int kmax_atomic = na * (s.l3max_atomic + 1);
    const int kmax_magnetic = nm * (s.l3max_magnetic + 1);
    const int nele1 = 1, nele2 = 1;
    for (int nr1 = 1; nr1 <= na; ++nr1)
      for (int nr2 = 1; nr2 <= na; ++nr2)
        for (int nr3 = 1; nr3 <= nm; ++nr3)
          for (int nr4 = 1; nr4 <= nm; ++nr4)
            for (int nr5 = 1; nr5 <= nm; ++nr5)
              for (int l1 = 0; l1 <= s.l3max_atomic; ++l1)
                for (int l2 = 0; l2 <= s.l3max_magnetic; ++l2)
                  for (int l3 = 0; l3 <= s.l3max_magnetic; ++l3)
                    for (int l4 = 0; l4 <= s.l3max_magnetic; ++l4) {
                      int ka1 = na * l1 + nr1, ka2 = na * l1 + nr2;
                      int km1 = nm * l3 + nr4, km2 = nm * l4 + nr5;
                      long nc1 = (long)((kmax_magnetic + 1) * kmax_atomic + kmax_magnetic) * nele1 +
                                 (long)(kmax_magnetic + 1) * ka1 + km1;
                      long nc2 = (long)((kmax_magnetic + 1) * kmax_atomic + kmax_magnetic) * nele2 +
                                 (long)(kmax_magnetic + 1) * ka2 + km2;
                      if (nc1 < nc2) continue;
                      // bcreate atomic rank 2 (isordered on veck) and magnetic rank 3 (isbasis)
                      bool ord_a = veck(s, 1, l1, nr1) >= veck(s, 1, l1, nr2);
                      bool basis_m = triangle_even(l2, l3, l4);
                      if (ord_a && basis_m) rows.push_back({nr1, nr2, nr3, nr4, nr5, l1, l2, l3, l4});
                    }
    s.nvar3 = (int)rows.size();
    int nv = std::max(1, s.nvar3);
    s.b3occ.init({{1, 2}, {1, nv}});
    s.b3index.init({{1, 9}, {1, nv}});
    s.b3map_atomic.init({{1, nv}});
    s.b3map_magnetic.init({{1, nv}});
    for (int n = 1; n <= s.nvar3; ++n) {
      s.b3occ(1, n) = 1;
      s.b3occ(2, n) = 1;
      for (int q = 0; q < 9; ++q) s.b3index(q + 1, n) = rows[n - 1][q];
      for (int k = 1; k <= s.nvar3l_atomic; ++k)
        if (s.b3lindex_atomic(k) == s.b3index(6, n)) s.b3map_atomic(n) = k;
      for (int k = 1; k <= s.nvar3l_magnetic; ++k)
        if (s.b3lindex_magnetic(1, k) == s.b3index(7, n) &&
            s.b3lindex_magnetic(2, k) == s.b3index(8, n) &&
            s.b3lindex_magnetic(3, k) == s.b3index(9, n))
          s.b3map_magnetic(n) = k;
    }
    // m lists (src/util.F90:2264-2336)
    s.madd3_atomic.init({{1, s.nvar3l_atomic}});
    int maxa = 0;
    for (int k = 1; k <= s.nvar3l_atomic; ++k) {
      s.madd3_atomic(k) = 2 * s.b3lindex_atomic(k) + 1;
      maxa = std::max(maxa, s.madd3_atomic(k));
    }
    s.madd3_magnetic.init({{1, std::max(1, s.nvar3l_magnetic)}});
    int maxm = 1;
    for (int k = 1; k <= s.nvar3l_magnetic; ++k) {
      int l2 = s.b3lindex_magnetic(1, k), l3 = s.b3lindex_magnetic(2, k), l4 = s.b3lindex_magnetic(3, k);
      int cnt = 0;
      for (int m2 = -l2; m2 <= l2; ++m2)
        for (int m3 = -l3; m3 <= l3; ++m3)
          if (std::abs(m2 + m3) <= l4) ++cnt;
      s.madd3_magnetic(k) = cnt;
      maxm = std::max(maxm, cnt);
    }
    s.b3lm_atomic.init({{1, s.nvar3l_atomic}, {1, maxa}});
    for (int k = 1; k <= s.nvar3l_atomic; ++k) {
      int l1 = s.b3lindex_atomic(k), m = 0;
      for (int m1 = -l1; m1 <= l1; ++m1) s.b3lm_atomic(k, ++m) = m1;
    }
    s.b3lm_magnetic.init({{1, std::max(1, s.nvar3l_magnetic)}, {1, maxm}, {1, 3}});
    for (int k = 1; k <= s.nvar3l_magnetic; ++k) {
      int l2 = s.b3lindex_magnetic(1, k), l3 = s.b3lindex_magnetic(2, k), l4 = s.b3lindex_magnetic(3, k);
      int m = 0;
      for (int m2 = -l2; m2 <= l2; ++m2)
        for (int m3 = -l3; m3 <= l3; ++m3) {
          int m4 = -(m2 + m3);
          if (std::abs(m4) <= l4) {
            ++m;
            s.b3lm_magnetic(k, m, 1) = m2;
            s.b3lm_magnetic(k, m, 2) = m3;
            s.b3lm_magnetic(k, m, 3) = m4;
          }
        }
    }
  }

  // 4-body angular list for the atomic part (src/util.F90:2341-2371)
  {
    std::vector<std::array<int, 3>> rows;
    for (int l1 = 0; l1 <= s.l4max_atomic; ++l1)
      for (int l2 = 0; l2 <= s.l4max_atomic; ++l2)
        for (int l3 = 0; l3 <= s.l4max_atomic; ++l3)
          if (triangle_even(l1, l2, l3)) rows.push_back({l1, l2, l3});
    s.nvar4l_atomic = (int)rows.size();
    s.b4lindex_atomic.init({{1, 3}, {1, std::max(1, s.nvar4l_atomic)}});
    for (int k = 1; k <= s.nvar4l_atomic; ++k)
      for (int q = 0; q < 3; ++q) s.b4lindex_atomic(q + 1, k) = rows[k - 1][q];
  }

  // 4-body clusters (src/util.F90:2374-2582)
  {
    std::vector<std::array<int, 15>> rows;
    std::vector<int> nint;
    const int na = s.nradial4_atomic, nm = s.nradial4_magnetic;
    const int la = s.l4max_atomic, lmg = s.l4max_magnetic;
    const int kmax_atomic = na * (la + 1);
    const int kmax_magnetic = nm * (lmg + 1);
    const long base = (long)((kmax_magnetic + 1) * kmax_atomic + kmax_magnetic);
    std::vector<int> lints;
    for (int nr1 = 1; nr1 <= na; ++nr1)
      for (int nr2 = 1; nr2 <= na; ++nr2)
        for (int nr3 = 1; nr3 <= na; ++nr3)
          for (int nr4 = 1; nr4 <= nm; ++nr4)
            for (int nr5 = 1; nr5 <= nm; ++nr5)
              for (int nr6 = 1; nr6 <= nm; ++nr6)
                for (int nr7 = 1; nr7 <= nm; ++nr7)
                  for (int l1 = 0; l1 <= la; ++l1)
                    for (int l2 = 0; l2 <= la; ++l2)
                      for (int l3 = 0; l3 <= la; ++l3)
                        for (int l4 = 0; l4 <= lmg; ++l4)
                          for (int l5 = 0; l5 <= lmg; ++l5)
                            for (int l6 = 0; l6 <= lmg; ++l6)
                              for (int l7 = 0; l7 <= lmg; ++l7) {
                                int ka1 = na * l1 + nr1, ka2 = na * l2 + nr2, ka3 = na * l3 + nr3;
                                int km1 = nm * l5 + nr5, km2 = nm * l6 + nr6, km3 = nm * l7 + nr7;
                                long nc1 = base + (long)(kmax_magnetic + 1) * ka1 + km1;
                                long nc2 = base + (long)(kmax_magnetic + 1) * ka2 + km2;
                                long nc3 = base + (long)(kmax_magnetic + 1) * ka3 + km3;
                                if (!(nc1 >= nc2 && nc2 >= nc3)) continue;
                                // atomic rank 3 (src/util.F90:4766-4787)
                                bool basis_a = triangle_even(l1, l2, l3);
                                int v1 = veck(s, 1, l1, nr1), v2 = veck(s, 1, l2, nr2),
                                    v3 = veck(s, 1, l3, nr3);
                                bool ord_a = (v1 >= v2) && (v2 >= v3);
                                int vn[4] = {1, 1, 1, 1};
                                int vnr[4] = {nr4, nr5, nr6, nr7};
                                int vl[4] = {l4, l5, l6, l7};
                                bool basis_m;
                                rank4_lints(s, vn, vnr, vl, lints, basis_m);
                                if (ord_a && basis_a && basis_m) {
                                  for (size_t q = 0; q < lints.size(); ++q) {
                                    rows.push_back({nr1, nr2, nr3, nr4, nr5, nr6, nr7, l1, l2, l3, l4,
                                                    l5, l6, l7, lints[q]});
                                    nint.push_back(q == 0 ? (int)lints.size() : 0);
                                  }
                                }
                              }
    s.nvar4 = (int)rows.size();
    int nv = std::max(1, s.nvar4);
    s.b4occ.init({{1, 3}, {1, nv}});
    s.b4index.init({{1, 15}, {1, nv}});
    s.b4nint.init({{1, nv}});
    s.b4map_atomic.init({{1, nv}});
    s.b4map_magnetic.init({{1, nv}});
    for (int n = 1; n <= s.nvar4; ++n) {
      for (int q = 1; q <= 3; ++q) s.b4occ(q, n) = 1;
      for (int q = 0; q < 15; ++q) s.b4index(q + 1, n) = rows[n - 1][q];
      s.b4nint(n) = nint[n - 1];
      for (int k = 1; k <= s.nvar4l_atomic; ++k)
        if (s.b4lindex_atomic(1, k) == s.b4index(8, n) && s.b4lindex_atomic(2, k) == s.b4index(9, n) &&
            s.b4lindex_atomic(3, k) == s.b4index(10, n))
          s.b4map_atomic(n) = k;
    }
    // group clusters by (l0',l1',l2',l3',L01') in order of first appearance
    // (src/util.F90:2615-2702)
    std::vector<std::array<int, 5>> groups;
    for (int n = 1; n <= s.nvar4; ++n) {
      std::array<int, 5> key{s.b4index(11, n), s.b4index(12, n), s.b4index(13, n), s.b4index(14, n),
                             s.b4index(15, n)};
      int found = 0;
      for (size_t g = 0; g < groups.size(); ++g)
        if (groups[g] == key) found = (int)g + 1;
      if (!found) {
        groups.push_back(key);
        found = (int)groups.size();
      }
      s.b4map_magnetic(n) = found;
    }
    s.nvar4l_magnetic = (int)groups.size();
    s.b4lindex_magnetic.init({{1, 5}, {1, std::max(1, s.nvar4l_magnetic)}});
    for (int k = 1; k <= s.nvar4l_magnetic; ++k)
      for (int q = 0; q < 5; ++q) s.b4lindex_magnetic(q + 1, k) = groups[k - 1][q];

    // m lists (src/util.F90:2705-2814)
    s.madd4_atomic.init({{1, std::max(1, s.nvar4l_atomic)}});
    int maxa = 1;
    for (int k = 1; k <= s.nvar4l_atomic; ++k) {
      int l1 = s.b4lindex_atomic(1, k), l2 = s.b4lindex_atomic(2, k), l3 = s.b4lindex_atomic(3, k);
      int cnt = 0;
      for (int m1 = -l1; m1 <= l1; ++m1)
        for (int m2 = -l2; m2 <= l2; ++m2)
          if (std::abs(m1 + m2) <= l3) ++cnt;
      s.madd4_atomic(k) = cnt;
      maxa = std::max(maxa, cnt);
    }
    s.madd4_magnetic.init({{1, std::max(1, s.nvar4l_magnetic)}});
    int maxm = 1;
    auto count4m = [&](int k, bool fill) {
      int l4 = s.b4lindex_magnetic(1, k), l5 = s.b4lindex_magnetic(2, k), l6 = s.b4lindex_magnetic(3, k),
          l7 = s.b4lindex_magnetic(4, k), L = s.b4lindex_magnetic(5, k);
      int n = 0;
      for (int M = -L; M <= L; ++M)
        for (int m4 = -l4; m4 <= l4; ++m4)
          for (int m5 = -l5; m5 <= l5; ++m5)
            for (int m6 = -l6; m6 <= l6; ++m6)
              for (int m7 = -l7; m7 <= l7; ++m7)
                if ((M - (m4 + m5) == 0) && (M + (m6 + m7) == 0)) {
                  ++n;
                  if (fill) {
                    s.b4lm_magnetic(k, n, 1) = m4;
                    s.b4lm_magnetic(k, n, 2) = m5;
                    s.b4lm_magnetic(k, n, 3) = m6;
                    s.b4lm_magnetic(k, n, 4) = m7;
                  }
                }
      return n;
    };
    for (int k = 1; k <= s.nvar4l_magnetic; ++k) {
      s.madd4_magnetic(k) = count4m(k, false);
      maxm = std::max(maxm, s.madd4_magnetic(k));
    }
    s.b4lm_atomic.init({{1, std::max(1, s.nvar4l_atomic)}, {1, maxa}, {1, 3}});
    for (int k = 1; k <= s.nvar4l_atomic; ++k) {
      int l1 = s.b4lindex_atomic(1, k), l2 = s.b4lindex_atomic(2, k), l3 = s.b4lindex_atomic(3, k);
      int n = 0;
      for (int m1 = -l1; m1 <= l1; ++m1)
        for (int m2 = -l2; m2 <= l2; ++m2) {
          int m3 = -(m1 + m2);
          if (std::abs(m3) <= l3) {
            ++n;
            s.b4lm_atomic(k, n, 1) = m1;
            s.b4lm_atomic(k, n, 2) = m2;
            s.b4lm_atomic(k, n, 3) = m3;
          }
        }
    }
    s.b4lm_magnetic.init({{1, std::max(1, s.nvar4l_magnetic)}, {1, maxm}, {1, 4}});
    for (int k = 1; k <= s.nvar4l_magnetic; ++k) count4m(k, true);
  }

  // generalized couplings (src/util.F90:4256-4388)
  const int lm = s.lmax;
  auto& cg = s.cgcoeff;
  s.cg01_magnetic.init({{1, s.nvar2l}, {-lm, lm}});
  for (int k = 1; k <= s.nvar2l; ++k) {
    int l0 = s.b2lindex(k);
    for (int n = 1; n <= s.madd2(k); ++n) {
      int m0 = s.b2lm(k, n);
      s.cg01_magnetic(k, m0) += cg(l0, l0, 0, m0, -m0, 0);
    }
  }
  s.cg02_atomic.init({{1, s.nvar3l_atomic}, {-lm, lm}});
  for (int k = 1; k <= s.nvar3l_atomic; ++k) {
    int l1 = s.b3lindex_atomic(k);
    for (int n = 1; n <= s.madd3_atomic(k); ++n) {
      int m1 = s.b3lm_atomic(k, n);
      s.cg02_atomic(k, m1) += cg(l1, l1, 0, m1, -m1, 0);
    }
  }
  s.cg02_magnetic.init({{1, std::max(1, s.nvar3l_magnetic)}, {-lm, lm}, {-lm, lm}, {-lm, lm}});
  for (int k = 1; k <= s.nvar3l_magnetic; ++k) {
    int l0 = s.b3lindex_magnetic(1, k), l1 = s.b3lindex_magnetic(2, k), l2 = s.b3lindex_magnetic(3, k);
    for (int n = 1; n <= s.madd3_magnetic(k); ++n) {
      int m0 = s.b3lm_magnetic(k, n, 1), m1 = s.b3lm_magnetic(k, n, 2), m2 = s.b3lm_magnetic(k, n, 3);
      s.cg02_magnetic(k, m0, m1, m2) += cg(l0, l1, l2, m0, m1, -m2) * cg(l2, l2, 0, m2, -m2, 0);
    }
  }
  s.cg03_atomic.init({{1, std::max(1, s.nvar4l_atomic)}, {-lm, lm}, {-lm, lm}, {-lm, lm}});
  for (int k = 1; k <= s.nvar4l_atomic; ++k) {
    int l1 = s.b4lindex_atomic(1, k), l2 = s.b4lindex_atomic(2, k), l3 = s.b4lindex_atomic(3, k);
    for (int n = 1; n <= s.madd4_atomic(k); ++n) {
      int m1 = s.b4lm_atomic(k, n, 1), m2 = s.b4lm_atomic(k, n, 2), m3 = s.b4lm_atomic(k, n, 3);
      s.cg03_atomic(k, m1, m2, m3) += cg(l1, l2, l3, m1, m2, -m3) * cg(l3, l3, 0, m3, -m3, 0);
    }
  }
  s.cg03_magnetic.init(
      {{1, std::max(1, s.nvar4l_magnetic)}, {-lm, lm}, {-lm, lm}, {-lm, lm}, {-lm, lm}});
  for (int k = 1; k <= s.nvar4l_magnetic; ++k) {
    int l0 = s.b4lindex_magnetic(1, k), l1 = s.b4lindex_magnetic(2, k), l2 = s.b4lindex_magnetic(3, k),
        l3 = s.b4lindex_magnetic(4, k), L = s.b4lindex_magnetic(5, k);
    for (int n = 1; n <= s.madd4_magnetic(k); ++n) {
      int m0 = s.b4lm_magnetic(k, n, 1), m1 = s.b4lm_magnetic(k, n, 2), m2 = s.b4lm_magnetic(k, n, 3),
          m3 = s.b4lm_magnetic(k, n, 4);
      int M = m0 + m1;
      s.cg03_magnetic(k, m0, m1, m2, m3) +=
          cg(l0, l1, L, m0, m1, M) * cg(l2, l3, L, m2, m3, -M) * cg(L, L, 0, M, -M, 0);
    }
  }

  // Y_lm recurrence constants (src/spherical.F90:5-51), indexed by shindex
  auto make_ab = [&](int lmax, FArr<int>& sh, FArr<double>& a, FArr<double>& b) {
    int half = (lmax + 1) * (lmax + 2) / 2;
    a.init({{1, half}});
    b.init({{1, half}});
    for (int l = 1; l <= lmax; ++l) {
      double lsq = l * l, ld = 2 * l, l1 = 4 * lsq - 1, l2 = lsq - ld + 1;
      for (int m = 0; m <= l - 2; ++m) {
        double msq = m * m;
        a(sh(l, m)) = std::sqrt(l1 / (lsq - msq));
        b(sh(l, m)) = -std::sqrt((l2 - msq) / (4 * l2 - 1));
      }
    }
  };
  make_ab(s.l3max_atomic, s.shindex_atomic, s.alm_atomic, s.blm_atomic);
  make_ab(s.l2max_magnetic, s.shindex_magnetic, s.alm_magnetic, s.blm_magnetic);
  int lmx = std::max(s.l3max_atomic, s.l2max_magnetic);
  s.cl.init({{1, lmx + 1}});
  s.dl.init({{1, lmx + 1}});
  for (int l = 1; l <= lmx; ++l) {
    s.cl(l) = -std::sqrt((double)(1.0 + 0.5 / (double)l));
    s.dl(l) = std::sqrt((double)(2.0 * (l - 1) + 3.0));
  }
  (void)err;
  return true;
}

// bcreate rank 5 (src/util.F90:4944-5022): allowed intermediate couplings
// (L12, L34) of ((1 2)L12 (3 4)L34)l5, in loop order
void rank5_lints(const OracleState& s, const int* vecnr, const int* vecl, std::vector<std::array<int, 3>>& lints,
                 bool& isbasis) {
  int nc[5];
  for (int i = 0; i < 5; ++i) nc[i] = veck(s, 1, vecl[i], vecnr[i]);
  const int l1 = vecl[0], l2 = vecl[1], l3 = vecl[2], l4 = vecl[3], l5 = vecl[4];
  const int lintmax = 2 * *std::max_element(vecl, vecl + 5);
  lints.clear();
  for (int a = 0; a <= lintmax; ++a)
    for (int b = 0; b <= lintmax; ++b) {
      bool ok = true;
      if (a > l1 + l2 || b > l3 + l4) ok = false;
      if (a < std::abs(l1 - l2) || b < std::abs(l3 - l4)) ok = false;
      if (l5 > a + b || l5 < std::abs(a - b)) ok = false;
      if (nc[0] == nc[1] && a % 2 != 0) ok = false;
      if (nc[2] == nc[3] && b % 2 != 0) ok = false;
      if (nc[0] == nc[2] && nc[1] == nc[3] && a == b && l5 % 2 != 0) ok = false;
      if (ok) lints.push_back({a, b, 0});
    }
  isbasis = !lints.empty();
  if ((l1 + l2 + l3 + l4 + l5) % 2 != 0) isbasis = false;
}

// bcreate rank 6 (src/util.F90:5131-5220): couplings (L12, L34, L56) of
// (((1 2)L12 (3 4)L34)L56 (5 6)L56)0, in loop order
void rank6_lints(const OracleState& s, const int* vecnr, const int* vecl, std::vector<std::array<int, 3>>& lints,
                 bool& isbasis) {
  int nc[6];
  for (int i = 0; i < 6; ++i) nc[i] = veck(s, 1, vecl[i], vecnr[i]);
  const int l1 = vecl[0], l2 = vecl[1], l3 = vecl[2], l4 = vecl[3], l5 = vecl[4], l6 = vecl[5];
  const int lintmax = 2 * *std::max_element(vecl, vecl + 6);
  lints.clear();
  for (int a = 0; a <= lintmax; ++a)
    for (int b = 0; b <= lintmax; ++b)
      for (int c = 0; c <= lintmax; ++c) {
        bool ok = true;
        if (a > l1 + l2 || b > l3 + l4 || c > l5 + l6) ok = false;
        if (a < std::abs(l1 - l2) || b < std::abs(l3 - l4) || c < std::abs(l5 - l6)) ok = false;
        if (c > a + b || c < std::abs(a - b)) ok = false;
        if (nc[0] == nc[1] && a % 2 != 0) ok = false;
        if (nc[2] == nc[3] && b % 2 != 0) ok = false;
        if (nc[4] == nc[5] && c % 2 != 0) ok = false;
        if (nc[0] == nc[2] && nc[1] == nc[3] && a == b && c % 2 != 0) ok = false;
        if (ok) lints.push_back({a, b, c});
      }
  isbasis = !lints.empty();
  if ((l1 + l2 + l3 + l4 + l5 + l6) % 2 != 0) isbasis = false;
}

// Every tuple of a nested loop over `n` digits with ranges [lo[q], hi[q]],
// the last digit fastest (the reference's loop nests).
template <class Fn>
void nested(int n, const int* lo, const int* hi, Fn&& fn) {
  std::vector<int> v(lo, lo + n);
  for (int q = 0; q < n; ++q)
    if (lo[q] > hi[q]) return;
  while (true) {
    fn(v.data());
    int q = n - 1;
    while (q >= 0 && v[q] == hi[q]) {
      v[q] = lo[q];
      --q;
    }
    if (q < 0) return;
    ++v[q];
  }
}

// The reordering of the internal couplings after the enumeration
// (src/util.F90:3079-3094, :3705-3740): within each group of clusters that
// share everything but their couplings, the entries after the group's first
// exchange the coupling columns [c0, c0 + w) so that smaller sums come first.
void reorder_lints(std::vector<std::vector<int>>& rows, const std::vector<int>& nint, int c0, int w) {
  for (size_t n = 0; n < rows.size(); ++n)
    for (int m = 1; m <= nint[n] - 2; ++m)
      for (int k = m + 1; k <= nint[n] - 1; ++k) {
        int s1 = 0, s2 = 0;
        for (int q = 0; q < w; ++q) {
          s1 += rows[n + m][c0 + q];
          s2 += rows[n + k][c0 + q];
        }
        if (s1 > s2)
          for (int q = 0; q < w; ++q) std::swap(rows[n + m][c0 + q], rows[n + k][c0 + q]);
      }
}

// 5- and 6-body clusters (src/util.F90:2817-3760) for one element, with the
// m-terms and couplings of each (src/util.F90:3100-3420, :3760-4140,
// :4389-4546). Returns false (with err) where the reference stops.
bool setuptables56(OracleState& s, std::string& err) {
  auto& cg = s.cgcoeff;
  std::vector<std::array<int, 3>> la, lm;
  bool ba = false, bm = false;
  // ---- 5-body
  {
    std::vector<std::vector<int>> rows;
    std::vector<int> nint;
    const int na = s.nradial5_atomic, nm = s.nradial5_magnetic, lam = s.l5max_atomic, lmm = s.l5max_magnetic;
    const long kma = (long)na * (lam + 1), kmm = (long)nm * (lmm + 1), base = (kmm + 1) * kma + kmm;
    const int lo[18] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int hi[18] = {na, na, na, na, nm, nm, nm, nm, nm, lam, lam, lam, lam, lmm, lmm, lmm, lmm, lmm};
    bool bad_order = false;
    if (na > 0 && nm > 0)
      nested(18, lo, hi, [&](const int* v) {
        // v: n1..n4, n0'..n4', l1..l4, l0'..l4'
        long nc[4];
        long ka[4];
        for (int q = 0; q < 4; ++q) {
          ka[q] = (long)na * v[9 + q] + v[q];
          const long km = (long)nm * v[14 + q] + v[5 + q];
          nc[q] = base + (kmm + 1) * ka[q] + km;
        }
        if (nc[0] < nc[1] || nc[1] < nc[2] || nc[2] < nc[3]) return;
        if (ka[0] < ka[1] || ka[1] < ka[2] || ka[2] < ka[3]) bad_order = true;
        // atomic rank 4, magnetic rank 5 (bcreate)
        std::vector<int> lints;
        bool basis_a;
        const int vn[4] = {1, 1, 1, 1};
        rank4_lints(s, vn, v, v + 9, lints, basis_a);
        rank5_lints(s, v + 4, v + 13, lm, bm);
        if (!(basis_a && bm)) return;
        const int numa = (int)lints.size(), numm = (int)lm.size(), num = std::max(numa, numm);
        for (int k = 0; k < num; ++k) {
          std::vector<int> r(21, 0);
          if (k < numa) {
            for (int q = 0; q < 4; ++q) {
              r[q] = v[q];
              r[9 + q] = v[9 + q];
            }
            r[18] = lints[k];
          }
          if (k < numm) {
            for (int q = 0; q < 5; ++q) {
              r[4 + q] = v[4 + q];
              r[13 + q] = v[13 + q];
            }
            r[19] = lm[k][0];
            r[20] = lm[k][1];
          }
          rows.push_back(r);
          nint.push_back(k == 0 ? num : 0);
        }
      });
    if (bad_order) {
      err = "the atomic basis is not ordered lexicographically (5-body)";
      return false;
    }
    reorder_lints(rows, nint, 19, 2);
    s.nvar5 = (int)rows.size();
    s.b5index.init({{1, 21}, {1, std::max(1, s.nvar5)}});
    s.b5mt_atomic.assign(s.nvar5, {});
    s.b5mt_magnetic.assign(s.nvar5, {});
    for (int n = 0; n < s.nvar5; ++n) {
      const auto& r = rows[n];
      for (int q = 0; q < 21; ++q) s.b5index(q + 1, n + 1) = r[q];
      if (r[0] > 0) {  // atomic m-terms: (m1..m4) with M12 = m1 + m2 = -(m3 + m4)
        const int l1 = r[9], l2 = r[10], l3 = r[11], l4 = r[12], L = r[18];
        for (int M = -L; M <= L; ++M)
          for (int m1 = -l1; m1 <= l1; ++m1)
            for (int m2 = -l2; m2 <= l2; ++m2)
              for (int m3 = -l3; m3 <= l3; ++m3)
                for (int m4 = -l4; m4 <= l4; ++m4) {
                  if (M != m1 + m2 || M != -(m3 + m4)) continue;
                  const double c = cg(l1, l2, L, m1, m2, M) * cg(l3, l4, L, m3, m4, -M) * cg(L, L, 0, M, -M, 0);
                  s.b5mt_atomic[n].push_back({{m1, m2, m3, m4, 0, 0}, c});
                }
      }
      if (r[4] > 0) {  // magnetic m-terms: (m0'..m4') with -m4' = M01' + M23'
        const int l0 = r[13], l1 = r[14], l2 = r[15], l3 = r[16], l4 = r[17], A = r[19], B = r[20];
        for (int Ma = -A; Ma <= A; ++Ma)
          for (int Mb = -B; Mb <= B; ++Mb)
            for (int m0 = -l0; m0 <= l0; ++m0)
              for (int m1 = -l1; m1 <= l1; ++m1)
                for (int m2 = -l2; m2 <= l2; ++m2)
                  for (int m3 = -l3; m3 <= l3; ++m3)
                    for (int m4 = -l4; m4 <= l4; ++m4) {
                      if (Ma != m0 + m1 || Mb != m2 + m3 || -m4 != Ma + Mb) continue;
                      const double c = cg(l0, l1, A, m0, m1, Ma) * cg(l2, l3, B, m2, m3, Mb) *
                                       cg(A, B, l4, Ma, Mb, -m4) * cg(l4, l4, 0, -m4, m4, 0);
                      s.b5mt_magnetic[n].push_back({{m0, m1, m2, m3, m4, 0}, c});
                    }
      }
    }
  }
  // ---- 6-body (the ordering key takes the 5-body dims, src/util.F90:3490-3491)
  {
    std::vector<std::vector<int>> rows;
    std::vector<int> nint;
    const int na = s.nradial6_atomic, nm = s.nradial6_magnetic, lam = s.l6max_atomic, lmm = s.l6max_magnetic;
    const long kma = (long)s.nradial5_atomic * (s.l5max_atomic + 1);
    const long kmm = (long)s.nradial5_magnetic * (s.l5max_magnetic + 1), base = (kmm + 1) * kma + kmm;
    const int lo[22] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int hi[22] = {na, na, na, na, na, nm, nm, nm, nm, nm, nm, lam, lam, lam, lam, lam, lmm, lmm, lmm, lmm, lmm, lmm};
    bool bad_order = false;
    if (na > 0 && nm > 0) {
      if (2 * lam > s.l3max_atomic || 2 * lmm > s.l2max_magnetic) {
        err = "6-body couplings not worked for lmax > 6 (src/util.F90:3430-3434)";
        return false;
      }
      nested(22, lo, hi, [&](const int* v) {
        // v: n1..n5, n0'..n5', l1..l5, l0'..l5'
        long nc[5], ka[5];
        for (int q = 0; q < 5; ++q) {
          ka[q] = (long)na * v[11 + q] + v[q];
          const long km = (long)nm * v[17 + q] + v[6 + q];
          nc[q] = base + (kmm + 1) * ka[q] + km;
        }
        if (nc[0] < nc[1] || nc[1] < nc[2] || nc[2] < nc[3] || nc[3] < nc[4]) return;
        if (ka[0] < ka[1] || ka[1] < ka[2] || ka[2] < ka[3] || ka[3] < ka[4]) bad_order = true;
        rank5_lints(s, v, v + 11, la, ba);
        rank6_lints(s, v + 5, v + 16, lm, bm);
        if (!(ba && bm)) return;
        const int numa = (int)la.size(), numm = (int)lm.size(), num = std::max(numa, numm);
        for (int k = 0; k < num; ++k) {
          std::vector<int> r(27, 0);
          if (k < numa) {
            for (int q = 0; q < 5; ++q) {
              r[q] = v[q];
              r[11 + q] = v[11 + q];
            }
            r[22] = la[k][0];
            r[23] = la[k][1];
          }
          if (k < numm) {
            for (int q = 0; q < 6; ++q) {
              r[5 + q] = v[5 + q];
              r[16 + q] = v[16 + q];
            }
            r[24] = lm[k][0];
            r[25] = lm[k][1];
            r[26] = lm[k][2];
          }
          rows.push_back(r);
          nint.push_back(k == 0 ? num : 0);
        }
      });
    }
    if (bad_order) {
      err = "the atomic basis is not ordered lexicographically (6-body, src/util.F90:3512-3517)";
      return false;
    }
    reorder_lints(rows, nint, 22, 2);
    reorder_lints(rows, nint, 24, 3);
    s.nvar6 = (int)rows.size();
    s.b6index.init({{1, 27}, {1, std::max(1, s.nvar6)}});
    s.b6mt_atomic.assign(s.nvar6, {});
    s.b6mt_magnetic.assign(s.nvar6, {});
    for (int n = 0; n < s.nvar6; ++n) {
      const auto& r = rows[n];
      for (int q = 0; q < 27; ++q) s.b6index(q + 1, n + 1) = r[q];
      if (r[0] > 0) {  // atomic: M12 = m1 + m2, M34 = m3 + m4, -m5 = M12 + M34
        const int l1 = r[11], l2 = r[12], l3 = r[13], l4 = r[14], l5 = r[15], A = r[22], B = r[23];
        for (int Ma = -A; Ma <= A; ++Ma)
          for (int Mb = -B; Mb <= B; ++Mb)
            for (int m1 = -l1; m1 <= l1; ++m1)
              for (int m2 = -l2; m2 <= l2; ++m2)
                for (int m3 = -l3; m3 <= l3; ++m3)
                  for (int m4 = -l4; m4 <= l4; ++m4)
                    for (int m5 = -l5; m5 <= l5; ++m5) {
                      if (Ma != m1 + m2 || Mb != m3 + m4 || -m5 != Ma + Mb) continue;
                      const double c = cg(l1, l2, A, m1, m2, Ma) * cg(l3, l4, B, m3, m4, Mb) *
                                       cg(A, B, l5, Ma, Mb, -m5) * cg(l5, l5, 0, -m5, m5, 0);
                      s.b6mt_atomic[n].push_back({{m1, m2, m3, m4, m5, 0}, c});
                    }
      }
      if (r[5] > 0) {  // magnetic: M01', M23', M45' with M01' + M23' = -M45'
        const int l0 = r[16], l1 = r[17], l2 = r[18], l3 = r[19], l4 = r[20], l5 = r[21];
        const int A = r[24], B = r[25], Cc = r[26];
        for (int Ma = -A; Ma <= A; ++Ma)
          for (int Mb = -B; Mb <= B; ++Mb)
            for (int Mc = -Cc; Mc <= Cc; ++Mc)
              for (int m0 = -l0; m0 <= l0; ++m0)
                for (int m1 = -l1; m1 <= l1; ++m1)
                  for (int m2 = -l2; m2 <= l2; ++m2)
                    for (int m3 = -l3; m3 <= l3; ++m3)
                      for (int m4 = -l4; m4 <= l4; ++m4)
                        for (int m5 = -l5; m5 <= l5; ++m5) {
                          if (Ma != m0 + m1 || Mb != m2 + m3 || Mc != m4 + m5 || Ma + Mb != -Mc) continue;
                          const double c = cg(l0, l1, A, m0, m1, Ma) * cg(l2, l3, B, m2, m3, Mb) *
                                           cg(l4, l5, Cc, m4, m5, Mc) * cg(A, B, Cc, Ma, Mb, -Mc) *
                                           cg(Cc, Cc, 0, -Mc, Mc, 0);
                          s.b6mt_magnetic[n].push_back({{m0, m1, m2, m3, m4, m5}, c});
                        }
      }
    }
  }
  (void)ba;
  return true;
}

}  // namespace

// Reads the potential file (src/util.F90:459-1108, read branch only) and builds
// all tables (src/util.F90:6-455).
int oracle_setup(OracleState& s, const char* path, const char* element, double rcut,
                 double rcut_magnetic, double smear, int xcnumber, std::string& err) {
  s = OracleState();
  s.element = element;
  s.cutoff = rcut;
  s.cutoff_magnetic = rcut_magnetic;
  s.smearing = smear;
  if (xcnumber == 1) s.xc = "pbe";
  else if (xcnumber == 2) s.xc = "lda";
  else {
    err = "unknown XC functional";
    return ORACLE_ERR_ARGS;
  }
  std::ifstream f(path);
  if (!f) {
    err = std::string("file not found: ") + path;
    return ORACLE_ERR_FILE;
  }
  ListReader rd(f);
  std::vector<std::string> t;
  auto bad = [&](const char* what) {
    err = std::string("malformed potential file: ") + what;
    return ORACLE_ERR_FORMAT;
  };
  if (!rd.skip()) return bad("empty");
  if (!rd.read(7, t)) return bad("created line");
  if (!rd.read(2, t)) return bad("Elements line");
  if (t[1] != s.element) {
    err = "inconsistent element information";
    return ORACLE_ERR_FORMAT;
  }
  if (!rd.read(2, t)) return bad("XC line");
  if (t[1] != s.xc) {
    err = "inconsistent XC functional";
    return ORACLE_ERR_FORMAT;
  }
  double smr;
  if (!rd.read(2, t) || !to_double(t[1], smr)) return bad("gauss-smearing line");
  if (std::fabs(s.smearing - smr) > 1e-6) {
    err = "inconsistent gauss-smearing";
    return ORACLE_ERR_FORMAT;
  }
  if (!rd.read(3, t) || !to_double(t[1], s.lambda[0]) || !to_double(t[2], s.lambda[1]))
    return bad("lambda line");
  if (!rd.read(10, t)) return bad("rcut line");
  if (!to_double(t[4], s.cut[0]) || !to_double(t[5], s.cut[1]) || !to_double(t[6], s.dcut[0]) ||
      !to_double(t[7], s.dcut[1]) || !to_double(t[8], s.ecut) || !to_double(t[9], s.decut))
    return bad("rcut values");
  int* dims[5][4] = {
      {&s.nradbase_atomic, &s.nradbase_magnetic, &s.nradial2_magnetic, &s.l2max_magnetic},
      {&s.nradial3_atomic, &s.nradial3_magnetic, &s.l3max_atomic, &s.l3max_magnetic},
      {&s.nradial4_atomic, &s.nradial4_magnetic, &s.l4max_atomic, &s.l4max_magnetic},
      {&s.nradial5_atomic, &s.nradial5_magnetic, &s.l5max_atomic, &s.l5max_magnetic},
      {&s.nradial6_atomic, &s.nradial6_magnetic, &s.l6max_atomic, &s.l6max_magnetic}};
  for (int r = 0; r < 5; ++r) {
    if (!rd.read(6, t)) return bad("basis dims");
    for (int q = 0; q < 4; ++q)
      if (!to_int(t[2 + q], *dims[r][q])) return bad("basis dims value");
  }
  if (!rd.read(2, t) || !to_int(t[1], s.ndensity)) return bad("ndensity");
  if (!rd.read(5, t) || !to_int(t[1], s.npot) || !to_int(t[2], s.nfemb) ||
      !to_int(t[3], s.radtype_atomic) || !to_int(t[4], s.radtype_magnetic))
    return bad("npot line");

  // derived sizes and the limit checks of src/util.F90:223-272
  s.nradbase = std::max(s.nradbase_atomic, s.nradbase_magnetic);
  s.nradial = std::max(s.nradial3_atomic, s.nradial2_magnetic);
  s.lmax = std::max(s.l3max_atomic, s.l2max_magnetic);
  if (s.l3max_atomic < s.l4max_atomic || s.l3max_atomic < s.l5max_atomic || s.l3max_atomic < s.l6max_atomic ||
      s.l2max_magnetic < s.l3max_magnetic || s.l2max_magnetic < s.l4max_magnetic ||
      s.l2max_magnetic < s.l5max_magnetic || s.l2max_magnetic < s.l6max_magnetic ||
      s.nradial3_atomic < s.nradial4_atomic || s.nradial3_atomic < s.nradial5_atomic ||
      s.nradial3_atomic < s.nradial6_atomic || s.nradial2_magnetic < s.nradial5_magnetic ||
      s.nradial2_magnetic < s.nradial6_magnetic ||
      s.nradial2_magnetic < s.nradial3_magnetic || s.nradial2_magnetic < s.nradial4_magnetic ||
      s.nradial3_atomic > s.nradbase_atomic || s.nradial2_magnetic > s.nradbase_magnetic ||
      s.nradial > s.nradbase) {
    err = "basis dimension limits violated";
    return ORACLE_ERR_FORMAT;
  }
  // 5/6-body factors live in the 3-body A basis (n' <= nradial3_magnetic,
  // l' <= l3max_magnetic here); the reference evaluates a rank only when the
  // ranks below it are present (src/b_basis.F90:217-218, :312-313)
  if (s.nradial5_magnetic > s.nradial3_magnetic || s.nradial6_magnetic > s.nradial3_magnetic ||
      s.l5max_magnetic > s.l3max_magnetic || s.l6max_magnetic > s.l3max_magnetic) {
    err = "5/6-body magnetic dims beyond the 3-body ones";
    return ORACLE_ERR_UNSUPPORTED;
  }
  if (((s.nradial5_atomic || s.nradial5_magnetic) && !(s.nradial4_atomic || s.nradial4_magnetic)) ||
      ((s.nradial6_atomic || s.nradial6_magnetic) && !(s.nradial5_atomic || s.nradial5_magnetic))) {
    err = "a rank of clusters without the rank below it";
    return ORACLE_ERR_UNSUPPORTED;
  }
  if (s.ndensity < 1 || s.ndensity > 2) {
    err = "ndensity must be 1 or 2";
    return ORACLE_ERR_UNSUPPORTED;
  }
  if (s.nfemb < 0 || s.nfemb > 2) {
    err = "embedding type without gradient";
    return ORACLE_ERR_UNSUPPORTED;
  }
  if (!setuptables(s, err)) return ORACLE_ERR_FORMAT;
  if (!setuptables56(s, err)) return ORACLE_ERR_FORMAT;

  // defaults (src/util.F90:281-350)
  s.crad_atomic.init({{1, s.nradbase_atomic}, {1, std::max(1, s.nradial3_atomic)}, {0, s.l3max_atomic}});
  for (int m = 1; m <= s.nradial3_atomic; ++m)
    for (int l = 0; l <= s.l3max_atomic; ++l) s.crad_atomic(m, m, l) = 1.0;
  s.crad_magnetic.init(
      {{1, s.nradbase_magnetic}, {1, std::max(1, s.nradial2_magnetic)}, {0, s.l2max_magnetic}});
  for (int m = 1; m <= s.nradial2_magnetic; ++m)
    for (int l = 0; l <= s.l2max_magnetic; ++l) s.crad_magnetic(m, m, l) = 1.0;
  s.corepara.init({{1, 2}});
  s.corepara.fill(3.0);
  s.p1.init({{1, 2}, {1, s.ndensity}});
  s.p1.fill(1.0);
  s.c0.init({{1, std::max(1, s.nvar1)}, {1, s.ndensity}});
  s.c2.init({{1, std::max(1, s.nvar2)}, {1, s.ndensity}});
  s.c3.init({{1, std::max(1, s.nvar3)}, {1, s.ndensity}});
  s.c4.init({{1, std::max(1, s.nvar4)}, {1, s.ndensity}});
  s.c5.init({{1, std::max(1, s.nvar5)}, {1, s.ndensity}});
  s.c6.init({{1, std::max(1, s.nvar6)}, {1, s.ndensity}});

  // parameter records (src/util.F90:669-1106)
  while (true) {
    if (!rd.read(3, t)) break;
    std::string paratype = t[0];
    int norder, nd;
    if (!to_int(t[1], norder) || !to_int(t[2], nd)) return bad("record header");
    if (paratype == "clu") {
      if (norder == 1) {
        if (!rd.read(4, t)) break;
        int nr;
        double x;
        if (!to_int(t[1], nr) || !to_double(t[2], x)) return bad("clu 1");
        if (t[0] == s.element && nd <= s.ndensity)
          for (int n = 1; n <= s.nvar1; ++n)
            if (nr == s.b1index(n)) s.c0(n, nd) = x;
      } else if (norder == 2) {
        if (!rd.read(8, t)) break;
        int v[4];
        double x;
        for (int q = 0; q < 4; ++q)
          if (!to_int(t[2 + q], v[q])) return bad("clu 2");
        if (!to_double(t[6], x)) return bad("clu 2 value");
        if (t[0] != s.element || t[1] != s.element) {
          err = "incorrect elements for interaction of order 2";
          return ORACLE_ERR_FORMAT;
        }
        if (nd <= s.ndensity)
          for (int n = 1; n <= s.nvar2; ++n) {
            bool match = true;
            for (int q = 0; q < 4; ++q)
              if (v[q] != s.b2index(q + 1, n)) match = false;
            if (match) s.c2(n, nd) = x;
          }
      } else if (norder == 3) {
        if (!rd.read(14, t)) break;
        int v[9];
        double x;
        for (int q = 0; q < 9; ++q)
          if (!to_int(t[3 + q], v[q])) return bad("clu 3");
        if (!to_double(t[12], x)) return bad("clu 3 value");
        for (int q = 0; q < 3; ++q)
          if (t[q] != s.element) {
            err = "incorrect elements for interaction of order 3";
            return ORACLE_ERR_FORMAT;
          }
        if (nd <= s.ndensity)
          for (int n = 1; n <= s.nvar3; ++n) {
            bool match = true;
            for (int q = 0; q < 9 && match; ++q)
              if (v[q] != s.b3index(q + 1, n)) match = false;
            if (match) s.c3(n, nd) = x;
          }
      } else if (norder == 4) {
        if (!rd.read(21, t)) break;
        int v[15];
        double x;
        for (int q = 0; q < 15; ++q)
          if (!to_int(t[4 + q], v[q])) return bad("clu 4");
        if (!to_double(t[19], x)) return bad("clu 4 value");
        for (int q = 0; q < 4; ++q)
          if (t[q] != s.element) {
            err = "incorrect elements for interaction of order 4";
            return ORACLE_ERR_FORMAT;
          }
        if (nd <= s.ndensity)
          for (int n = 1; n <= s.nvar4; ++n) {
            bool match = true;
            for (int q = 0; q < 15 && match; ++q)
              if (v[q] != s.b4index(q + 1, n)) match = false;
            if (match) s.c4(n, nd) = x;
          }
      } else if (norder == 5 || norder == 6) {
        // 5-body: 5 elements, 21 indices (src/util.F90:826-889); 6-body: 6
        // elements, 27 indices (src/util.F90:894-955)
        const int w = norder == 5 ? 21 : 27;
        if (!rd.read(norder + w + 2, t)) break;
        std::vector<int> v(w);
        double x;
        for (int q = 0; q < w; ++q)
          if (!to_int(t[norder + q], v[q])) return bad("clu 5/6");
        if (!to_double(t[norder + w], x)) return bad("clu 5/6 value");
        for (int q = 0; q < norder; ++q)
          if (t[q] != s.element) {
            err = "incorrect elements for interaction of order 5/6";
            return ORACLE_ERR_FORMAT;
          }
        const int nv = norder == 5 ? s.nvar5 : s.nvar6;
        const FArr<int>& idx = norder == 5 ? s.b5index : s.b6index;
        if (nd <= s.ndensity)
          for (int n = 1; n <= nv; ++n) {
            bool match = true;
            for (int q = 0; q < w && match; ++q)
              if (v[q] != idx(q + 1, n)) match = false;
            if (match) (norder == 5 ? s.c5 : s.c6)(n, nd) = x;
          }
      }
    } else if (paratype == "par") {
      if (norder < 1 || norder > 2) return bad("par order");
      if (!rd.read(3, t)) break;
      double x;
      if (!to_double(t[1], x)) return bad("par value");
      if (t[0] == s.element && nd <= s.ndensity) s.p1(norder, nd) = x;
    } else if (paratype == "rad_atomic") {
      if (!rd.read(7, t)) break;
      int nr1, nr2, l1;
      double x;
      if (!to_int(t[2], nr1) || !to_int(t[3], nr2) || !to_int(t[4], l1) || !to_double(t[5], x))
        return bad("rad_atomic");
      if (t[0] != s.element || t[1] != s.element) {
        err = "error when reading radial parameters";
        return ORACLE_ERR_FORMAT;
      }
      if (nr1 >= 1 && nr1 <= s.nradbase_atomic && nr2 >= 1 && nr2 <= s.nradial3_atomic && l1 >= 0 &&
          l1 <= s.l3max_atomic)
        s.crad_atomic(nr1, nr2, l1) = x;
    } else if (paratype == "rad_magnetic") {
      if (!rd.read(7, t)) break;
      int nr0, nr1, l0;
      double x;
      if (!to_int(t[2], nr0) || !to_int(t[3], nr1) || !to_int(t[4], l0) || !to_double(t[5], x))
        return bad("rad_magnetic");
      if (t[0] != s.element || t[1] != s.element) {
        err = "error when reading radial parameters";
        return ORACLE_ERR_FORMAT;
      }
      if (nr0 >= 1 && nr0 <= s.nradbase_magnetic && nr1 >= 1 && nr1 <= s.nradial2_magnetic &&
          l0 >= 0 && l0 <= s.l2max_magnetic)
        s.crad_magnetic(nr0, nr1, l0) = x;
    } else if (paratype == "core") {
      if (norder < 1 || norder > 2) return bad("core order");
      if (!rd.read(4, t)) break;
      double x;
      if (!to_double(t[2], x)) return bad("core value");
      if (t[0] != s.element || t[1] != s.element) {
        err = "error when reading radial parameters";
        return ORACLE_ERR_FORMAT;
      }
      s.corepara(norder) = x;
    }
  }

  // cutoff consistency (src/util.F90:421-444)
  if (s.cut[0] > s.cutoff || s.cut[1] > s.cutoff_magnetic) {
    err = "global cutoff too short";
    return ORACLE_ERR_FORMAT;
  }
  s.nlut = 10000;  // src/radial.F90:43
  if (!setup_lut_atomic(s) || !setup_lut_magnetic(s)) {
    err = "unsupported radial basis type";
    return ORACLE_ERR_UNSUPPORTED;
  }
  s.initialized = true;
  return ORACLE_OK;
}
