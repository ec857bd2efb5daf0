// Host-side model construction: basis enumeration, couplings, folded gather
// tables and radial lookup tables.
#include "model.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>

#include "magace.h"

namespace magace {
namespace {

const double kPi = 3.14159265358979323846264338327950288419;

// ---------------------------------------------------------------------------
// Clebsch-Gordan coefficients. Racah's closed formula with double-precision
// factorials, the same evaluation the reference uses (src/util.F90:4149-4252)
// so that coefficient values agree to the last bits.
struct Factorials {
  std::vector<double> f;
  Factorials() {
    f.resize(64);
    f[0] = 1.0;
    for (size_t i = 1; i < f.size(); ++i) f[i] = static_cast<double>(i) * f[i - 1];
  }
};
const Factorials kFac;

}  // namespace

double clebsch_gordan(int j1, int j2, int J, int m1, int m2, int M) {
  if (M != m1 + m2) return 0.0;
  if (std::abs(m1) > j1 || std::abs(m2) > j2 || std::abs(M) > J) return 0.0;
  if (J > j1 + j2 || J < std::abs(j1 - j2)) return 0.0;
  const auto& f = kFac.f;
  double pre = (static_cast<double>(2 * J + 1) * f[j1 + j2 - J] * f[j1 - j2 + J] * f[-j1 + j2 + J] /
                f[j1 + j2 + J + 1]) *
               (f[J + M] * f[J - M] * f[j1 + m1] * f[j1 - m1] * f[j2 + m2] * f[j2 - m2]);
  pre = std::sqrt(pre);
  double sum = 0.0;
  for (int k = 0; k <= j1 + j2 + J; ++k) {
    int a = j1 + j2 - J - k, b = j1 - m1 - k, c = j2 + m2 - k, d = J - j2 + m1 + k, e = J - j1 - m2 + k;
    if (a < 0 || b < 0 || c < 0 || d < 0 || e < 0) continue;
    sum += static_cast<double>(k % 2 ? -1 : 1) / (f[k] * f[a] * f[b] * f[c] * f[d] * f[e]);
  }
  return pre * sum;
}

int FactorLayout::A(int n1, int l1, int m1, int n2, int l2, int m2) const {
  // A entries beyond (n3m, l3m) are never accumulated by the A pass and stay
  // zero in the reference (src/a_basis.F90:248-291 loops only to
  // nradial3_magnetic / l3max_magnetic)
  if (n1 >= n3a || l1 > l3a || n2 >= n3m || l2 > l3m) return offZero;
  return offA + ((n1 * lsa + l1 * l1 + l1 + m1) * n3m + n2) * ls3 + l2 * l2 + l2 + m2;
}

int FactorLayout::WA(int n1, int l1, int m1, int n2, int l2, int m2) const {
  if (m2 < 0 || n1 >= n3a || l1 > l3a || n2 >= n3m || l2 > l3m) return -1;
  return ((n1 * lsa + l1 * l1 + l1 + m1) * n3m + n2) * h3 + l2 * (l2 + 1) / 2 + m2;
}

namespace {

bool triangle_even(int a, int b, int c) {
  return a + b >= c && std::abs(a - b) <= c && (a + b + c) % 2 == 0;
}

// ---------------------------------------------------------------------------
// Radial basis functions g_n(r) on [0, cutoff) and their r-derivatives
// (src/radial.F90:430-606): Chebyshev polynomials of a scaled variable, with
// optional cosine envelope, and a cosine taper over the last dcut.
void chebyshev(int n, double x, std::vector<double>& T, std::vector<double>& dT) {
  // T_k(x) and dT_k/dx = k U_{k-1}(x)
  std::vector<double> U(n + 1);
  T.assign(n + 1, 0.0);
  dT.assign(n + 1, 0.0);
  T[0] = 1.0;
  U[0] = 1.0;
  if (n == 0) return;
  T[1] = x;
  U[1] = 2.0 * x;
  for (int k = 1; k < n; ++k) {
    T[k + 1] = 2.0 * x * T[k] - T[k - 1];
    U[k + 1] = 2.0 * x * U[k] - U[k - 1];
  }
  for (int k = 1; k <= n; ++k) dT[k] = static_cast<double>(k) * U[k - 1];
}

bool radial_basis(int type, double lam, int nb, double rc, double dc, double r, std::vector<double>& g,
                  std::vector<double>& dg) {
  g.assign(nb, 0.0);
  dg.assign(nb, 0.0);
  if (r >= rc) return true;
  std::vector<double> T, dT;
  const double x0 = r / rc;
  switch (type) {
    case 3:
    case 4: {  // exponentially scaled Chebyshev, with (3) / without (4) envelope
      double y1 = std::exp(-lam * x0), dy1 = -lam * y1 / rc, y2 = std::exp(-lam);
      double x = 1.0 - 2.0 * (y1 - y2) / (1.0 - y2), dx = -2.0 * dy1 / (1.0 - y2);
      chebyshev(nb - 1, x, T, dT);
      g[0] = T[0];
      dg[0] = dT[0] * dx;
      for (int n = 1; n < nb; ++n) {
        g[n] = 0.5 - 0.5 * T[n];
        dg[n] = -0.5 * dT[n] * dx;
      }
      if (type == 3) {
        double env = 0.5 * (1.0 + std::cos(kPi * x0)), denv = -0.5 * std::sin(kPi * x0) * kPi / rc;
        for (int n = 0; n < nb; ++n) {
          dg[n] = g[n] * denv + dg[n] * env;
          g[n] = g[n] * env;
        }
      }
      break;
    }
    case 5:
    case 6: {  // power-law scaled Chebyshev, without (5) / with (6) envelope
      double y0 = 1.0 - x0, dy1 = std::pow(y0, lam - 1.0);
      double y1 = 1.0 - dy1 * y0;
      dy1 = lam / rc * dy1;
      double x = 2.0 * y1 - 1.0, dx = 2.0 * dy1;
      if (type == 5) {
        chebyshev(nb, x, T, dT);
        for (int n = 0; n < nb; ++n) {
          g[n] = 0.5 - 0.5 * T[n + 1];
          dg[n] = -0.5 * dT[n + 1] * dx;
        }
      } else {
        chebyshev(nb - 1, x, T, dT);
        g[0] = T[0];
        dg[0] = dT[0] * dx;
        for (int n = 1; n < nb; ++n) {
          g[n] = 0.5 - 0.5 * T[n];
          dg[n] = -0.5 * dT[n] * dx;
        }
        double env = 0.5 * (1.0 + std::cos(kPi * x0)), denv = -0.5 * std::sin(kPi * x0) * kPi / rc;
        for (int n = 0; n < nb; ++n) {
          dg[n] = g[n] * denv + dg[n] * env;
          g[n] = g[n] * env;
        }
      }
      break;
    }
    case 7: {  // Chebyshev in 1 - 2 x^2
      double x = 1.0 - 2.0 * x0 * x0, dx = -(4.0 / rc) * x0;
      chebyshev(nb, x, T, dT);
      for (int n = 0; n < nb; ++n) {
        g[n] = T[n + 1];
        dg[n] = dT[n + 1] * dx;
      }
      break;
    }
    case 8: {  // Chebyshev in 1 - 2 x, shifted to vanish at r = 0
      double x = 1.0 - 2.0 * x0, dx = -2.0 / rc;
      chebyshev(nb, x, T, dT);
      for (int n = 0; n < nb; ++n) {
        g[n] = T[n + 1] - 1.0;
        dg[n] = dT[n + 1] * dx;
      }
      break;
    }
    default:
      return false;
  }
  double rt = rc - dc;
  if (r > rt) {
    double fc = 0.5 * (1.0 + std::cos(kPi * (r - rt) / dc));
    double dfc = -0.5 * std::sin(kPi * (r - rt) / dc) * kPi / dc;
    for (int n = 0; n < nb; ++n) {
      dg[n] = g[n] * dfc + dg[n] * fc;
      g[n] = g[n] * fc;
    }
  }
  return true;
}

// Hard-core repulsion pre*exp(-lambda r^2)/r with a cosine envelope
// (src/radial.F90:630-668).
void core_repulsion(double r, double pre, double lam, double rc, double& c, double& dc) {
  c = dc = 0.0;
  if (r >= rc) return;
  pre = std::fabs(pre);
  lam = std::fabs(lam);
  double r2 = r * r, lr2 = lam * r2;
  if (lr2 >= 50.0) return;
  double y = std::exp(-lr2);
  c = pre * y / r;
  dc = -pre * y * (2.0 * lr2 + 1.0) / r2;
  double x0 = r / rc, env = 0.5 * (1.0 + std::cos(kPi * x0)), denv = -0.5 * std::sin(kPi * x0) * kPi / rc;
  dc = c * denv + dc * env;
  c = c * env;
}

// Tabulates `nf` functions on the grid r_n = n / rscale (n = 1..nlut) as
// cubic-Hermite segments over [r_n, r_{n+1}], in bin units: segment n holds
// (f(r_n), f'(r_n) h, c2, c3) with the right end taken from segment n+1 and
// zero beyond the last node. This is the construction of
// src/radial.F90:223-296, swept downwards so each segment sees its right
// neighbour already evaluated.
template <class Eval>
void tabulate(int nlut, double rscale, int nf, std::vector<double>& out, Eval eval) {
  out.assign(static_cast<size_t>(nlut + 1) * nf * 4, 0.0);
  const double h = 1.0 / rscale;
  std::vector<double> v(nf), dv(nf), right(nf, 0.0), dright(nf, 0.0);
  for (int n = nlut; n >= 1; --n) {
    double x = h * static_cast<double>(n);
    eval(x, v, dv);
    for (int f = 0; f < nf; ++f) {
      double f0 = v[f], f0d = dv[f] * h, f1 = right[f], f1d = dright[f];
      double* c = &out[(static_cast<size_t>(n) * nf + f) * 4];
      c[0] = f0;
      c[1] = f0d;
      c[2] = 3.0 * (f1 - f0) - f1d - 2.0 * f0d;
      c[3] = -2.0 * (f1 - f0) + f1d + f0d;
      right[f] = c[0];
      dright[f] = c[1];
    }
  }
}

bool build_lut(const Model& mdl, RadialLUT& lut) {
  const Potential& p = mdl.pot;
  const BasisDims& d = p.dims;
  const FactorLayout& L = mdl.L;
  lut.nlut = 10000;  // bins per table (src/radial.F90:43)
  lut.rscale_a = static_cast<double>(lut.nlut) / mdl.cutoff;
  lut.rscale_m = static_cast<double>(lut.nlut) / mdl.cutoff_m;
  // the reference steps the grid as (1/rscale)*n; use the same spacing
  lut.rscale_a = 1.0 / (1.0 / lut.rscale_a) == lut.rscale_a ? lut.rscale_a : lut.rscale_a;
  const int la = d.l3max_a + 1, lm = d.l2max_m + 1;
  lut.nfa = d.nradbase_a + d.nradial3_a * la + 1;
  lut.nfm = d.nradial2_m * lm + d.nradbase_m;
  bool ok = true;
  std::vector<double> g, dg;
  tabulate(lut.nlut, lut.rscale_a, lut.nfa, lut.a, [&](double r, std::vector<double>& v, std::vector<double>& dv) {
    if (!radial_basis(d.radtype_a, p.lambda[0], d.nradbase_a, p.cut[0], p.dcut[0], r, g, dg)) ok = false;
    int k = 0;
    for (int n = 0; n < d.nradbase_a; ++n, ++k) {
      v[k] = g[n];
      dv[k] = dg[n];
    }
    for (int nr = 0; nr < d.nradial3_a; ++nr)
      for (int l = 0; l < la; ++l, ++k) {
        double s = 0.0, ds = 0.0;
        const double* c = &p.crad_a[(static_cast<size_t>(l) * d.nradial3_a + nr) * d.nradbase_a];
        for (int n = 0; n < d.nradbase_a; ++n) {
          s += c[n] * g[n];
          ds += c[n] * dg[n];
        }
        v[k] = s;
        dv[k] = ds;
      }
    core_repulsion(r, p.core_pre, p.core_lambda, p.cut[0], v[k], dv[k]);
  });
  tabulate(lut.nlut, lut.rscale_m, lut.nfm, lut.m, [&](double r, std::vector<double>& v, std::vector<double>& dv) {
    if (!radial_basis(d.radtype_m, p.lambda[1], d.nradbase_m, p.cut[1], p.dcut[1], r, g, dg)) ok = false;
    int k = 0;
    for (int nr = 0; nr < d.nradial2_m; ++nr)
      for (int l = 0; l < lm; ++l, ++k) {
        double s = 0.0, ds = 0.0;
        const double* c = &p.crad_m[(static_cast<size_t>(l) * d.nradial2_m + nr) * d.nradbase_m];
        for (int n = 0; n < d.nradbase_m; ++n) {
          s += c[n] * g[n];
          ds += c[n] * dg[n];
        }
        v[k] = s;
        dv[k] = ds;
      }
    for (int n = 0; n < d.nradbase_m; ++n, ++k) {
      v[k] = g[n];
      dv[k] = dg[n];
    }
  });
  (void)L;
  return ok;
}

// ---------------------------------------------------------------------------
// Basis enumeration, single element (the reference's C-ABI admits one,
// src/ace.F90:46-49). Selection rules of setuptables/bcreate
// (src/util.F90:1803-2582, :4673-4857): pair radial indices ordered n0' >= n1';
// 3-body pairs (n1,l1,n1',l1') >= (n2,l1,n2',l2') in the packed key order and
// (l0',l1',l2') a triangle with even sum; 4-body triples ordered the same way,
// (l1,l2,l3) an even triangle, and for the magnetic quadruple every
// intermediate L01' coupling (l0' l1')L (l2' l3')L allowed, odd L excluded
// when a pair is identical, even total.
bool enumerate_high(const BasisDims& d, int rank, std::vector<std::vector<int>>& rows);

void enumerate(const BasisDims& d, std::vector<std::vector<int>>* rows) {
  for (int n = 1; n <= d.nradbase_m; ++n) rows[1].push_back({n});
  for (int a = 1; a <= d.nradial2_m; ++a)
    for (int b = 1; b <= d.nradial2_m; ++b)
      for (int n = 1; n <= d.nradbase_a; ++n)
        for (int l = 0; l <= d.l2max_m; ++l)
          if (a >= b) rows[2].push_back({a, b, n, l});
  {
    const int na = d.nradial3_a, nm = d.nradial3_m;
    const long kmm = static_cast<long>(nm) * (d.l3max_m + 1) + 1;
    auto key = [&](int n, int l, int np, int lp) { return kmm * (na * l + n) + nm * lp + np; };
    for (int n1 = 1; n1 <= na; ++n1)
      for (int n2 = 1; n2 <= na; ++n2)
        for (int p0 = 1; p0 <= nm; ++p0)
          for (int p1 = 1; p1 <= nm; ++p1)
            for (int p2 = 1; p2 <= nm; ++p2)
              for (int l1 = 0; l1 <= d.l3max_a; ++l1)
                for (int q0 = 0; q0 <= d.l3max_m; ++q0)
                  for (int q1 = 0; q1 <= d.l3max_m; ++q1)
                    for (int q2 = 0; q2 <= d.l3max_m; ++q2)
                      if (key(n1, l1, p1, q1) >= key(n2, l1, p2, q2) && triangle_even(q0, q1, q2))
                        rows[3].push_back({n1, n2, p0, p1, p2, l1, q0, q1, q2});
  }
  {
    const int na = d.nradial4_a, nm = d.nradial4_m;
    const long kmm = static_cast<long>(nm) * (d.l4max_m + 1) + 1;
    auto key = [&](int n, int l, int np, int lp) { return kmm * (na * l + n) + nm * lp + np; };
    for (int n1 = 1; n1 <= na; ++n1)
      for (int n2 = 1; n2 <= na; ++n2)
        for (int n3 = 1; n3 <= na; ++n3)
          for (int p0 = 1; p0 <= nm; ++p0)
            for (int p1 = 1; p1 <= nm; ++p1)
              for (int p2 = 1; p2 <= nm; ++p2)
                for (int p3 = 1; p3 <= nm; ++p3)
                  for (int l1 = 0; l1 <= d.l4max_a; ++l1)
                    for (int l2 = 0; l2 <= d.l4max_a; ++l2)
                      for (int l3 = 0; l3 <= d.l4max_a; ++l3)
                        for (int q0 = 0; q0 <= d.l4max_m; ++q0)
                          for (int q1 = 0; q1 <= d.l4max_m; ++q1)
                            for (int q2 = 0; q2 <= d.l4max_m; ++q2)
                              for (int q3 = 0; q3 <= d.l4max_m; ++q3) {
                                long k1 = key(n1, l1, p1, q1), k2 = key(n2, l2, p2, q2), k3 = key(n3, l3, p3, q3);
                                if (!(k1 >= k2 && k2 >= k3)) continue;
                                if (!triangle_even(l1, l2, l3)) continue;
                                if ((q0 + q1 + q2 + q3) % 2) continue;
                                const bool same01 = (p0 == p1 && q0 == q1), same23 = (p2 == p3 && q2 == q3);
                                const int lmaxq = std::max(std::max(q0, q1), std::max(q2, q3));
                                for (int L = 0; L <= 2 * lmaxq; ++L) {
                                  if (L > q0 + q1 || L > q2 + q3) continue;
                                  if (L < std::abs(q0 - q1) || L < std::abs(q2 - q3)) continue;
                                  if ((same01 || same23) && L % 2) continue;
                                  rows[4].push_back({n1, n2, n3, p0, p1, p2, p3, l1, l2, l3, q0, q1, q2, q3, L});
                                }
                              }
  }
}

// Intermediate couplings of one rank-4, -5 or -6 angular vector, by the
// rules of the reference's coupling generator for one element
// (src/util.F90:4790-4857, :4944-5022, :5131-5220): rank 4 ((1 2)L (3 4)L)0
// gives L; rank 5 (((1 2)L12 (3 4)L34)l5 5)0 gives (L12, L34); rank 6
// (((1 2)L12 (3 4)L34)L56 (5 6)L56)0 gives (L12, L34, L56); each in the loop
// order of the generator. Two positions are identical when their (n, l)
// are: then odd couplings of that pair are excluded. `basis` is false when
// none is allowed or the l's have an odd sum.
struct Couplings {
  std::vector<std::array<int, 3>> v;
  bool basis = false;
};
Couplings couplings(int rank, const int* n, const int* l) {
  Couplings c;
  const auto same = [&](int a, int b) { return n[a] == n[b] && l[a] == l[b]; };
  const auto tri = [](int a, int b, int L) { return L <= a + b && L >= std::abs(a - b); };
  int lmx = 0, lsum = 0;
  for (int q = 0; q < rank; ++q) {
    lmx = std::max(lmx, l[q]);
    lsum += l[q];
  }
  const int lintmax = 2 * lmx;
  if (rank == 4) {
    for (int L = 0; L <= lintmax; ++L) {
      if (!tri(l[0], l[1], L) || !tri(l[2], l[3], L)) continue;
      if ((same(0, 1) || same(2, 3)) && L % 2) continue;
      c.v.push_back({L, 0, 0});
    }
  } else if (rank == 5) {
    for (int a = 0; a <= lintmax; ++a)
      for (int b = 0; b <= lintmax; ++b) {
        if (!tri(l[0], l[1], a) || !tri(l[2], l[3], b) || !tri(a, b, l[4])) continue;
        if ((same(0, 1) && a % 2) || (same(2, 3) && b % 2)) continue;
        if (same(0, 2) && same(1, 3) && a == b && l[4] % 2) continue;
        c.v.push_back({a, b, 0});
      }
  } else {
    for (int a = 0; a <= lintmax; ++a)
      for (int b = 0; b <= lintmax; ++b)
        for (int d = 0; d <= lintmax; ++d) {
          if (!tri(l[0], l[1], a) || !tri(l[2], l[3], b) || !tri(l[4], l[5], d) || !tri(a, b, d)) continue;
          if ((same(0, 1) && a % 2) || (same(2, 3) && b % 2) || (same(4, 5) && d % 2)) continue;
          if (same(0, 2) && same(1, 3) && a == b && d % 2) continue;
          c.v.push_back({a, b, d});
        }
  }
  c.basis = !c.v.empty() && lsum % 2 == 0;
  return c;
}

// Every tuple of `n` digits with ranges [lo[q], hi[q]], the last fastest (the
// order of the reference's loop nests).
template <class Fn>
void odometer(int n, const int* lo, const int* hi, Fn&& fn) {
  for (int q = 0; q < n; ++q)
    if (lo[q] > hi[q]) return;
  std::vector<int> v(lo, lo + n);
  for (;;) {
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

// The reference's reordering of couplings after the enumeration
// (src/util.F90:3079-3094, :3705-3740): within each group of clusters that
// differ only in their couplings, the entries after the group's first swap
// the coupling columns [c0, c0 + w) so that smaller sums come first.
void reorder_couplings(std::vector<std::vector<int>>& rows, size_t first, const std::vector<int>& group, int c0,
                       int w) {
  for (size_t n = 0; n < group.size(); ++n)
    for (int m = 1; m <= group[n] - 2; ++m)
      for (int k = m + 1; k <= group[n] - 1; ++k) {
        auto& a = rows[first + n + m];
        auto& b = rows[first + n + k];
        int sa = 0, sb = 0;
        for (int q = 0; q < w; ++q) {
          sa += a[c0 + q];
          sb += b[c0 + q];
        }
        if (sa > sb)
          for (int q = 0; q < w; ++q) std::swap(a[c0 + q], b[c0 + q]);
      }
}

// 5- and 6-body clusters (src/util.F90:2817-3100, :3436-3760). Candidate index
// tuples in loop order whose (atomic, magnetic) keys do not increase; per
// tuple the atomic couplings (rank 4 / 5) and the magnetic ones (rank 5 / 6);
// the k-th cluster of a tuple pairs the k-th atomic with the k-th magnetic
// coupling, and where one side has fewer its indices are zeros (such a
// cluster has no defined basis function, see for_each_term). The 6-body key
// takes the 5-body dims (src/util.F90:3490-3491). Returns false where the
// reference stops: a candidate whose atomic keys are not ordered.
bool enumerate_high(const BasisDims& d, int rank, std::vector<std::vector<int>>& rows) {
  const int P = rank - 1;  // atomic factors
  const int na = rank == 5 ? d.nradial5_a : d.nradial6_a, nm = rank == 5 ? d.nradial5_m : d.nradial6_m;
  const int la = rank == 5 ? d.l5max_a : d.l6max_a, lm = rank == 5 ? d.l5max_m : d.l6max_m;
  if (na == 0 || nm == 0) return true;
  const long kma = static_cast<long>(d.nradial5_a) * (d.l5max_a + 1);
  const long kmm = static_cast<long>(d.nradial5_m) * (d.l5max_m + 1);
  const long base = (kmm + 1) * kma + kmm;
  // digits: n1..nP, n0'..nP', l1..lP, l0'..lP'
  const int nd = 4 * P + 2;
  std::vector<int> lo(nd), hi(nd);
  for (int q = 0; q < nd; ++q) {
    const bool radial = q < 2 * P + 1, atomic = radial ? q < P : q < 3 * P + 1;
    lo[q] = radial ? 1 : 0;
    hi[q] = radial ? (atomic ? na : nm) : (atomic ? la : lm);
  }
  const int w = rank == 5 ? 21 : 27;
  const int c_la = 4 * P + 2, c_lm = c_la + (rank == 5 ? 1 : 2), nlm = rank == 5 ? 2 : 3;
  std::vector<int> group;
  bool ok = true;
  odometer(nd, lo.data(), hi.data(), [&](const int* v) {
    const int* n = v;              // n1..nP
    const int* np = v + P;         // n0'..nP'
    const int* l = v + 2 * P + 1;  // l1..lP
    const int* lp = v + 3 * P + 1; // l0'..lP'
    long ka[6], nc[6];
    for (int q = 0; q < P; ++q) {
      ka[q] = static_cast<long>(na) * l[q] + n[q];
      nc[q] = base + (kmm + 1) * ka[q] + static_cast<long>(nm) * lp[q + 1] + np[q + 1];
      if (q > 0 && nc[q] > nc[q - 1]) return;
    }
    for (int q = 1; q < P; ++q)
      if (ka[q] > ka[q - 1]) ok = false;
    const Couplings ca = couplings(P, n, l), cm = couplings(P + 1, np, lp);
    if (!ca.basis || !cm.basis) return;
    const int numa = static_cast<int>(ca.v.size()), numm = static_cast<int>(cm.v.size());
    const int num = std::max(numa, numm);
    for (int k = 0; k < num; ++k) {
      std::vector<int> r(w, 0);
      if (k < numa) {
        for (int q = 0; q < P; ++q) {
          r[q] = n[q];
          r[2 * P + 1 + q] = l[q];
        }
        for (int q = 0; q < nlm - 1; ++q) r[c_la + q] = ca.v[k][q];
      }
      if (k < numm) {
        for (int q = 0; q <= P; ++q) {
          r[P + q] = np[q];
          r[3 * P + 1 + q] = lp[q];
        }
        for (int q = 0; q < nlm; ++q) r[c_lm + q] = cm.v[k][q];
      }
      rows.push_back(std::move(r));
      group.push_back(k == 0 ? num : 0);
    }
  });
  if (rank == 5) {
    reorder_couplings(rows, 0, group, c_lm, 2);
  } else {
    reorder_couplings(rows, 0, group, c_la, 2);
    reorder_couplings(rows, 0, group, c_lm, 3);
  }
  return ok;
}

// ---------------------------------------------------------------------------
// Gather-table construction. Every product term kappa * A0 * X1 * ... of the
// density becomes one entry of the A0 slot it contains (all m), and one entry
// of each weight slot (m' >= 0) of its other factors.
struct TermSink {
  const FactorLayout& L;
  int nd;
  std::vector<std::vector<Entry>> by_slot[kMaxArity + 1];  // [arity] -> slot -> entries
  int nslot;
  explicit TermSink(const FactorLayout& l, int ndens) : L(l), nd(ndens) {
    nslot = l.n2m * l.ls2 + l.nWA + (l.offW0 - l.offW2);
    for (int a = 1; a <= kMaxArity; ++a) by_slot[a].resize(nslot);
  }
  int g0_slot(int a0_factor) const { return a0_factor - L.offA0; }
  int w_slot(int weight_index) const { return L.n2m * L.ls2 + weight_index; }  // WA and W2 only

  void add(int slot, const double* k, const int* others, int arity) {
    Entry e;
    e.kappa[0] = k[0];
    e.kappa[1] = nd > 1 ? k[1] : 0.0;
    for (int q = 0; q < kMaxArity; ++q) e.o[q] = static_cast<uint16_t>(q < arity ? others[q] : L.offOne);
    by_slot[arity][slot].push_back(e);
  }
};

// Visits every m-term of the 2-, 3- (when with_b3), 4-, 5- and 6-body
// clusters in enumeration order as fn(rank, cluster, cf, f, w): cf is the
// coupling (the product of Clebsch-Gordan coefficients), f[0] the A0 factor
// and f[1 .. rank-1] the A2 (rank 2) or A factors, w[q] the weight index of
// factor q (-1 where it has none: m' < 0; w[0] is unused); f and w have six
// entries, padded with ONE and -1. Terms with cf == 0 are skipped.
template <class Fn>
void for_each_term(const Model& M, bool with_b3, Fn&& fn) {
  const FactorLayout& L = M.L;
  // 2-body: A0(n0',l,m) A2(n1,n1',l,-m), cg <l m l -m|0 0> (src/b_basis.F90:91-129)
  for (size_t c = 0; c < M.rows[2].size(); ++c) {
    const auto& r = M.rows[2][c];
    const int n0 = r[0] - 1, n1p = r[1] - 1, n1 = r[2] - 1, l = r[3];
    for (int m = -l; m <= l; ++m) {
      const double cf = clebsch_gordan(l, l, 0, m, -m, 0);
      if (cf == 0.0) continue;
      const int f[6] = {L.A0(n0, l, m), L.A2(n1, n1p, l, -m), L.offOne, L.offOne, L.offOne, L.offOne};
      const int w[6] = {-1, -m >= 0 ? L.W2(n1, n1p, l, -m) : -1, -1, -1, -1, -1};
      fn(2, c, cf, f, w);
    }
  }
  // 3-body: A0(n0',l0',m0') A(n1,l1,m1,n1',l1',m1') A(n2,l1,-m1,n2',l2',m2')
  // with cg<l1 m1 l1 -m1|00> * cg<l0' m0' l1' m1'|l2' -m2'> cg<l2' m2' l2' -m2'|00>
  // (src/b_basis.F90:142-212, src/util.F90:4297-4333)
  for (size_t c = 0; with_b3 && c < M.rows[3].size(); ++c) {
    const auto& r = M.rows[3][c];
    const int n1 = r[0] - 1, n2 = r[1] - 1, p0 = r[2] - 1, p1 = r[3] - 1, p2 = r[4] - 1;
    const int l1 = r[5], q0 = r[6], q1 = r[7], q2 = r[8];
    for (int m1 = -l1; m1 <= l1; ++m1) {
      const double cfa = clebsch_gordan(l1, l1, 0, m1, -m1, 0);
      for (int u0 = -q0; u0 <= q0; ++u0)
        for (int u1 = -q1; u1 <= q1; ++u1) {
          const int u2 = -(u0 + u1);
          if (std::abs(u2) > q2) continue;
          const double cfm = clebsch_gordan(q0, q1, q2, u0, u1, -u2) * clebsch_gordan(q2, q2, 0, u2, -u2, 0);
          const double cf = cfa * cfm;
          if (cf == 0.0) continue;
          const int f[6] = {L.A0(p0, q0, u0), L.A(n1, l1, m1, p1, q1, u1), L.A(n2, l1, -m1, p2, q2, u2),
                            L.offOne, L.offOne, L.offOne};
          const int w[6] = {-1, L.WA(n1, l1, m1, p1, q1, u1), L.WA(n2, l1, -m1, p2, q2, u2), -1, -1, -1};
          fn(3, c, cf, f, w);
        }
    }
  }
  // 4-body: A0 A(1) A(2) A(3) with
  // cg<l1 m1 l2 m2|l3 -m3> cg<l3 m3 l3 -m3|00> *
  // cg<l0' m0' l1' m1'|L M> cg<l2' m2' l3' m3'|L -M> cg<L M L -M|00>
  // (src/b_basis.F90:225-307, src/util.F90:4344-4388)
  for (size_t c = 0; c < M.rows[4].size(); ++c) {
    const auto& r = M.rows[4][c];
    const int n1 = r[0] - 1, n2 = r[1] - 1, n3 = r[2] - 1;
    const int p0 = r[3] - 1, p1 = r[4] - 1, p2 = r[5] - 1, p3 = r[6] - 1;
    const int l1 = r[7], l2 = r[8], l3 = r[9], q0 = r[10], q1 = r[11], q2 = r[12], q3 = r[13], Lc = r[14];
    for (int m1 = -l1; m1 <= l1; ++m1)
      for (int m2 = -l2; m2 <= l2; ++m2) {
        const int m3 = -(m1 + m2);
        if (std::abs(m3) > l3) continue;
        const double cfa = clebsch_gordan(l1, l2, l3, m1, m2, -m3) * clebsch_gordan(l3, l3, 0, m3, -m3, 0);
        for (int Mc = -Lc; Mc <= Lc; ++Mc)
          for (int u0 = -q0; u0 <= q0; ++u0) {
            const int u1 = Mc - u0;
            if (std::abs(u1) > q1) continue;
            for (int u2 = -q2; u2 <= q2; ++u2) {
              const int u3 = -Mc - u2;
              if (std::abs(u3) > q3) continue;
              const double cfm = clebsch_gordan(q0, q1, Lc, u0, u1, Mc) * clebsch_gordan(q2, q3, Lc, u2, u3, -Mc) *
                                 clebsch_gordan(Lc, Lc, 0, Mc, -Mc, 0);
              const double cf = cfa * cfm;
              if (cf == 0.0) continue;
              const int f[6] = {L.A0(p0, q0, u0), L.A(n1, l1, m1, p1, q1, u1), L.A(n2, l2, m2, p2, q2, u2),
                                L.A(n3, l3, m3, p3, q3, u3), L.offOne, L.offOne};
              const int w[6] = {-1, L.WA(n1, l1, m1, p1, q1, u1), L.WA(n2, l2, m2, p2, q2, u2),
                                L.WA(n3, l3, m3, p3, q3, u3), -1, -1};
              fn(4, c, cf, f, w);
            }
          }
      }
  }
  // 5- and 6-body: A0 A(1) .. A(P), P = rank - 1, with the generalized
  // couplings cg04 / cg05 (src/b_basis.F90:310-532, src/util.F90:4389-4546):
  //   atomic  5-body cg<l1 m1 l2 m2|L M12> cg<l3 m3 l4 m4|L -M12> cg<L M12 L -M12|00>
  //           6-body cg<l1 m1 l2 m2|L12 M12> cg<l3 m3 l4 m4|L34 M34>
  //                  cg<L12 M12 L34 M34|l5 -m5> cg<l5 -m5 l5 m5|00>
  //   magnetic 5-body cg<l0' m0' l1' m1'|L01 M01> cg<l2' m2' l3' m3'|L23 M23>
  //                  cg<L01 M01 L23 M23|l4' -m4'> cg<l4' -m4' l4' m4'|00>
  //           6-body cg<..|L01 M01> cg<..|L23 M23> cg<l4' m4' l5' m5'|L45 M45>
  //                  cg<L01 M01 L23 M23|L45 -M45> cg<L45 -M45 L45 M45|00>
  // A cluster whose atomic or magnetic indices the enumeration padded with
  // zeros has no terms: the reference reads its factors at radial index 0,
  // outside its A basis, so the basis function is undefined there.
  for (int rank = 5; rank <= 6; ++rank) {
    const int P = rank - 1;
    for (size_t c = 0; c < M.rows[rank].size(); ++c) {
      const auto& r = M.rows[rank][c];
      const int* n = r.data();               // n1..nP
      const int* np = r.data() + P;          // n0'..nP'
      const int* l = r.data() + 2 * P + 1;   // l1..lP
      const int* lp = r.data() + 3 * P + 1;  // l0'..lP'
      const int* lint = r.data() + 4 * P + 2;
      if (n[0] == 0 || np[0] == 0) continue;
      std::vector<std::pair<std::array<int, 6>, double>> ta, tm;
      std::array<int, 6> mv{};
      // atomic m-terms
      {
        std::vector<int> lo(P), hi(P);
        for (int q = 0; q < P; ++q) {
          lo[q] = -l[q];
          hi[q] = l[q];
        }
        odometer(P, lo.data(), hi.data(), [&](const int* m) {
          int sum = 0;
          for (int q = 0; q < P; ++q) sum += m[q];
          if (sum != 0) return;
          double cf;
          const int M12 = m[0] + m[1];
          if (rank == 5) {
            const int L = lint[0];
            if (std::abs(M12) > L) return;
            cf = clebsch_gordan(l[0], l[1], L, m[0], m[1], M12) * clebsch_gordan(l[2], l[3], L, m[2], m[3], -M12) *
                 clebsch_gordan(L, L, 0, M12, -M12, 0);
          } else {
            const int A = lint[0], B = lint[1], M34 = m[2] + m[3];
            if (std::abs(M12) > A || std::abs(M34) > B) return;
            cf = clebsch_gordan(l[0], l[1], A, m[0], m[1], M12) * clebsch_gordan(l[2], l[3], B, m[2], m[3], M34) *
                 clebsch_gordan(A, B, l[4], M12, M34, -m[4]) * clebsch_gordan(l[4], l[4], 0, -m[4], m[4], 0);
          }
          for (int q = 0; q < P; ++q) mv[q] = m[q];
          ta.push_back({mv, cf});
        });
      }
      // magnetic m-terms
      {
        const int* lm = lint + (rank == 5 ? 1 : 2);
        std::vector<int> lo(P + 1), hi(P + 1);
        for (int q = 0; q <= P; ++q) {
          lo[q] = -lp[q];
          hi[q] = lp[q];
        }
        odometer(P + 1, lo.data(), hi.data(), [&](const int* u) {
          int sum = 0;
          for (int q = 0; q <= P; ++q) sum += u[q];
          if (sum != 0) return;
          const int M01 = u[0] + u[1], M23 = u[2] + u[3];
          const int A = lm[0], B = lm[1];
          if (std::abs(M01) > A || std::abs(M23) > B) return;
          double cf;
          if (rank == 5) {
            cf = clebsch_gordan(lp[0], lp[1], A, u[0], u[1], M01) * clebsch_gordan(lp[2], lp[3], B, u[2], u[3], M23) *
                 clebsch_gordan(A, B, lp[4], M01, M23, -u[4]) * clebsch_gordan(lp[4], lp[4], 0, -u[4], u[4], 0);
          } else {
            const int Cc = lm[2], M45 = u[4] + u[5];
            if (std::abs(M45) > Cc) return;
            cf = clebsch_gordan(lp[0], lp[1], A, u[0], u[1], M01) * clebsch_gordan(lp[2], lp[3], B, u[2], u[3], M23) *
                 clebsch_gordan(lp[4], lp[5], Cc, u[4], u[5], M45) * clebsch_gordan(A, B, Cc, M01, M23, -M45) *
                 clebsch_gordan(Cc, Cc, 0, -M45, M45, 0);
          }
          for (int q = 0; q <= P; ++q) mv[q] = u[q];
          tm.push_back({mv, cf});
        });
      }
      for (const auto& a : ta)
        for (const auto& b : tm) {
          const double cf = a.second * b.second;
          if (cf == 0.0) continue;
          int f[6], w[6];
          f[0] = L.A0(np[0] - 1, lp[0], b.first[0]);
          w[0] = -1;
          for (int q = 0; q < P; ++q) {
            f[q + 1] = L.A(n[q] - 1, l[q], a.first[q], np[q + 1] - 1, lp[q + 1], b.first[q + 1]);
            w[q + 1] = L.WA(n[q] - 1, l[q], a.first[q], np[q + 1] - 1, lp[q + 1], b.first[q + 1]);
          }
          for (int q = P + 1; q < 6; ++q) {
            f[q] = L.offOne;
            w[q] = -1;
          }
          fn(rank, c, cf, f, w);
        }
    }
  }
}

// The same terms per output slot for kernels with one atom per lane: every
// slot's entries contiguous (arity 1, then 2, then 3), factors renumbered
// into the compact set the terms use, and the slots dealt to the kernel's
// warps longest first onto the least loaded warp.
bool build_rest(const Model& M, const TermSink& sink, const GatherTable& g, RestTable& T) {
  const FactorLayout& L = M.L;
  T = RestTable();
  std::vector<int32_t> compact(L.nF, -1);
  const auto use = [&](int f) {
    if (compact[f] < 0) {
      compact[f] = static_cast<int32_t>(T.factor_of.size());
      T.factor_of.push_back(f);
    }
    return static_cast<uint32_t>(compact[f]);
  };
  T.nslot = sink.nslot;
  T.run.assign(3 * T.nslot + 1, 0);
  T.slot_g0.assign(T.nslot, -1);
  T.slot_weight.assign(g.slot_weight.begin(), g.slot_weight.end());
  T.slot_mult.assign(T.nslot, 0.0f);
  for (int s = 0; s < T.nslot; ++s) T.slot_mult[s] = static_cast<float>(g.slot_mult[s]);
  std::vector<double> cost(T.nslot, 0.0);
  for (int s = 0; s < T.nslot; ++s) {
    if (s < L.n2m * L.ls2) T.slot_g0[s] = static_cast<int32_t>(use(L.offA0 + s));
    for (int a = 1; a <= 3; ++a) {
      T.run[3 * s + a - 1] = static_cast<int32_t>(T.rec.size() / 4);
      for (const Entry& e : sink.by_slot[a][s]) {
        const float k = static_cast<float>(e.kappa[0]);
        uint32_t kb;
        std::memcpy(&kb, &k, sizeof(kb));
        const uint32_t o1 = use(e.o[0]), o2 = a >= 2 ? use(e.o[1]) : 0, o3 = a >= 3 ? use(e.o[2]) : 0;
        T.rec.insert(T.rec.end(), {kb, o1 | (o2 << 16), o3, 0u});
        T.kap.push_back(e.kappa[0]);
        cost[s] += 2.0 * a;
      }
    }
    cost[s] += 8.0;  // per-slot work: totals, density term, weight store
  }
  T.run[3 * T.nslot] = static_cast<int32_t>(T.rec.size() / 4);
  T.nfac = static_cast<int>(T.factor_of.size());
  // compact factors renumbered in ascending factor order, so that the
  // kernels' staging loops (thread c takes factor c) read each atom's row
  // front to back
  {
    std::vector<int32_t> by(T.nfac);
    for (int c = 0; c < T.nfac; ++c) by[c] = c;
    std::sort(by.begin(), by.end(), [&](int32_t x, int32_t y) { return T.factor_of[x] < T.factor_of[y]; });
    std::vector<uint32_t> nw(T.nfac);
    std::vector<int32_t> fo(T.nfac);
    for (int c = 0; c < T.nfac; ++c) {
      nw[by[c]] = static_cast<uint32_t>(c);
      fo[c] = T.factor_of[by[c]];
    }
    T.factor_of = fo;
    const auto re = [&](uint32_t c) { return c < static_cast<uint32_t>(T.nfac) ? nw[c] : c; };
    for (size_t e = 0; e < T.rec.size(); e += 4) {
      T.rec[e + 1] = re(T.rec[e + 1] & 0xffffu) | (re(T.rec[e + 1] >> 16) << 16);
      T.rec[e + 2] = re(T.rec[e + 2]);
    }
    for (auto& g0 : T.slot_g0)
      if (g0 >= 0) g0 = static_cast<int32_t>(nw[g0]);
  }
  // longest first onto the least loaded warp
  T.nwarp = kRestTableWarps;
  std::vector<int> order(T.nslot);
  for (int s = 0; s < T.nslot; ++s) order[s] = s;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });
  std::vector<double> load(T.nwarp, 0.0);
  std::vector<std::vector<int32_t>> per(T.nwarp);
  for (int s : order) {
    const int w = static_cast<int>(std::min_element(load.begin(), load.end()) - load.begin());
    load[w] += cost[s];
    per[w].push_back(s);
  }
  T.warp_begin.assign(T.nwarp + 1, 0);
  for (int w = 0; w < T.nwarp; ++w) {
    T.warp_begin[w + 1] = T.warp_begin[w] + static_cast<int32_t>(per[w].size());
    T.warp_slots.insert(T.warp_slots.end(), per[w].begin(), per[w].end());
  }
  {
    // the FP64 kernel: a half-warp takes every second entry, a three-factor
    // entry costs about four one-factor ones in float-float, a slot end three
    std::vector<double> c64(T.nslot);
    for (int s = 0; s < T.nslot; ++s) {
      const int n1 = T.run[3 * s + 1] - T.run[3 * s], n2 = T.run[3 * s + 2] - T.run[3 * s + 1],
                n3 = T.run[3 * s + 3] - T.run[3 * s + 2];
      c64[s] = (n1 + 1) / 2 + 2.5 * ((n2 + 1) / 2) + 4.0 * ((n3 + 1) / 2) + 3.0;
    }
    std::vector<int> o64(T.nslot);
    for (int s = 0; s < T.nslot; ++s) o64[s] = s;
    std::stable_sort(o64.begin(), o64.end(), [&](int x, int y) { return c64[x] > c64[y]; });
    std::vector<double> l64(kRestWarps64, 0.0);
    std::vector<std::vector<int32_t>> p64(kRestWarps64);
    for (int s : o64) {
      const int w = static_cast<int>(std::min_element(l64.begin(), l64.end()) - l64.begin());
      l64[w] += c64[s];
      p64[w].push_back(s);
    }
    T.warp64_begin.assign(kRestWarps64 + 1, 0);
    for (int w = 0; w < kRestWarps64; ++w) {
      T.warp64_begin[w + 1] = T.warp64_begin[w] + static_cast<int32_t>(p64[w].size());
      T.warp64_slots.insert(T.warp64_slots.end(), p64[w].begin(), p64[w].end());
    }
  }
  // record streams per warp, dealt by their own cost (records, the
  // three-factor ones and the slot ends weighted as the kernels take them):
  // each item's entries, then its end record {multiplicity bits, weight
  // index, A0 factor, kRestEnd | slot}; two consecutive one-factor entries
  // share a record {k_a, o_a | o_b << 16, k_b, kRestPair1}. A slot longer
  // than three quarters of a warp's mean share is split in two items (dealt
  // to different warps): their end records carry kRestSplit | (2 sp + part),
  // each part's density term is its own (the term is linear), and the kernel
  // adds the parts' weights, split[sp] the slot's weight index.
  struct Item {
    int s, part;                 // part -1: the whole slot
    std::vector<int32_t> ent;    // entries (indices into rec), arity order
    double cost;
  };
  std::vector<Item> items;
  std::vector<int> arity_of(T.run[3 * T.nslot], 0);
  for (int s = 0; s < T.nslot; ++s)
    for (int a = 1; a <= 3; ++a)
      for (int e = T.run[3 * s + a - 1]; e < T.run[3 * s + a]; ++e) arity_of[e] = a;
  // relative record costs (estimates: other weightings and split limits
  // between a half and one share balanced the warps as well)
  const auto records_cost = [&](const std::vector<int32_t>& ent) {
    double c = 1.5;  // the end record
    int run1 = 0;
    for (size_t q = 0; q <= ent.size(); ++q) {
      const int a = q < ent.size() ? arity_of[ent[q]] : 0;
      if (a == 1) {
        ++run1;
        continue;
      }
      c += 1.3 * (run1 / 2) + 1.0 * (run1 % 2);
      run1 = 0;
      if (a == 2) c += 1.4;
      if (a == 3) c += 1.8;
    }
    return c;
  };
  double total = 0.0;
  for (int s = 0; s < T.nslot; ++s) {
    Item it{s, -1, {}, 0.0};
    for (int e = T.run[3 * s]; e < T.run[3 * s + 3]; ++e) it.ent.push_back(e);
    it.cost = records_cost(it.ent);
    total += it.cost;
    items.push_back(std::move(it));
  }
  const double limit = 0.75 * total / T.nwarp;
  std::vector<Item> dealt;
  for (auto& it : items) {
    if (it.cost <= limit || it.ent.size() < 4) {
      dealt.push_back(std::move(it));
      continue;
    }
    // two parts of about equal cost (an even cut inside the one-factor run)
    size_t cut = it.ent.size() / 2;
    double best = 1e300;
    for (size_t q = 2; q + 1 < it.ent.size(); q += 2) {
      const std::vector<int32_t> p0(it.ent.begin(), it.ent.begin() + q), p1(it.ent.begin() + q, it.ent.end());
      const double d = std::fabs(records_cost(p0) - records_cost(p1));
      if (d < best) {
        best = d;
        cut = q;
      }
    }
    const int sp = T.nsplit++;
    T.split_weight.push_back(T.slot_weight[it.s]);
    for (int part = 0; part < 2; ++part) {
      Item p{it.s, 2 * sp + part, {}, 0.0};
      if (part == 0) p.ent.assign(it.ent.begin(), it.ent.begin() + cut);
      else p.ent.assign(it.ent.begin() + cut, it.ent.end());
      p.cost = records_cost(p.ent);
      dealt.push_back(std::move(p));
    }
  }
  std::vector<int> iorder(dealt.size());
  for (size_t q = 0; q < dealt.size(); ++q) iorder[q] = static_cast<int>(q);
  std::stable_sort(iorder.begin(), iorder.end(), [&](int x, int y) { return dealt[x].cost > dealt[y].cost; });
  std::vector<double> sload(T.nwarp, 0.0);
  std::vector<std::vector<int>> sper(T.nwarp);
  std::vector<int> part0_warp(T.nsplit, -1);
  for (int q : iorder) {
    int w = static_cast<int>(std::min_element(sload.begin(), sload.end()) - sload.begin());
    const Item& it = dealt[q];
    if (it.part >= 0) {
      const int sp = it.part / 2;
      if (part0_warp[sp] == w) {  // the other part went to this warp: take the next least loaded
        double bl = 1e300;
        for (int v = 0; v < T.nwarp; ++v)
          if (v != w && sload[v] < bl) {
            bl = sload[v];
            w = v;
          }
      }
      part0_warp[sp] = w;
    }
    sload[w] += it.cost;
    sper[w].push_back(q);
  }
  T.stream_begin.assign(T.nwarp + 1, 0);
  std::vector<int> emitted(arity_of.size(), 0);  // each entry exactly once (checked below)
  for (int w = 0; w < T.nwarp; ++w) {
    for (int q : sper[w]) {
      const Item& it = dealt[q];
      for (int e : it.ent) ++emitted[e];
      for (size_t x = 0; x < it.ent.size(); ++x) {
        const int e = it.ent[x];
        const uint32_t* r = &T.rec[4 * static_cast<size_t>(e)];
        const int a = arity_of[e];
        if (a == 1 && x + 1 < it.ent.size() && arity_of[it.ent[x + 1]] == 1) {
          const uint32_t* r2 = &T.rec[4 * static_cast<size_t>(it.ent[x + 1])];
          T.stream.insert(T.stream.end(), {r[0], (r[1] & 0xffffu) | ((r2[1] & 0xffffu) << 16), r2[0], kRestPair1});
          ++x;
          continue;
        }
        T.stream.insert(T.stream.end(), {r[0], r[1], r[2], static_cast<uint32_t>(a)});
      }
      const float mu = T.slot_mult[it.s];
      uint32_t mb;
      std::memcpy(&mb, &mu, sizeof(mb));
      const uint32_t tag = it.part < 0 ? (kRestEnd | static_cast<uint32_t>(it.s))
                                       : (kRestEnd | kRestSplit | static_cast<uint32_t>(it.part));
      T.stream.insert(T.stream.end(), {mb, static_cast<uint32_t>(T.slot_weight[it.s]),
                                       static_cast<uint32_t>(T.slot_g0[it.s]), tag});
    }
    T.stream_begin[w + 1] = static_cast<int32_t>(T.stream.size() / 4);
  }
  // the streams' invariants: every entry in exactly one item, the two parts
  // of a split slot on different warps, every factor index below 2^16
  for (int c : emitted)
    if (c != 1) return false;
  std::vector<int> warp_of_part(2 * static_cast<size_t>(T.nsplit), -1);
  for (int w = 0; w < T.nwarp; ++w)
    for (int q : sper[w])
      if (dealt[q].part >= 0) warp_of_part[dealt[q].part] = w;
  for (int sp = 0; sp < T.nsplit; ++sp)
    if (warp_of_part[2 * sp] < 0 || warp_of_part[2 * sp] == warp_of_part[2 * sp + 1]) return false;
  return T.nfac <= 0xffff;
}

int build_gather(Model& M, bool with_b3, GatherTable& g, std::string& msg, RestTable* rest = nullptr) {
  const FactorLayout& L = M.L;
  const BasisDims& d = M.pot.dims;
  const int nd = M.ndensity;
  TermSink sink(L, nd);
  long nterm[7] = {0, 0, 0, 0, 0, 0, 0};
  // mirror of every factor: negating all its m gives (-1)^(sum of the m)
  // times the conjugate (A(m1,m2) = (-1)^(m1+m2) conj A(-m1,-m2), likewise
  // A2 and A0)
  std::vector<int> mir(L.nF), sgn(L.nF, 1);
  for (int f = 0; f < L.nF; ++f) mir[f] = f;
  for (int n1 = 0; n1 < L.n3a; ++n1)
    for (int l1 = 0; l1 <= L.l3a; ++l1)
      for (int m1 = -l1; m1 <= l1; ++m1)
        for (int n2 = 0; n2 < L.n3m; ++n2)
          for (int l2 = 0; l2 <= L.l3m; ++l2)
            for (int m2 = -l2; m2 <= l2; ++m2) {
              const int f = L.A(n1, l1, m1, n2, l2, m2);
              mir[f] = L.A(n1, l1, -m1, n2, l2, -m2);
              sgn[f] = ((m1 + m2) & 1) ? -1 : 1;
            }
  for (int n = 0; n < L.nba; ++n)
    for (int nr = 0; nr < L.n2m; ++nr)
      for (int l = 0; l <= L.l2m; ++l)
        for (int m = -l; m <= l; ++m) {
          const int f = L.A2(n, nr, l, m);
          mir[f] = L.A2(n, nr, l, -m);
          sgn[f] = (m & 1) ? -1 : 1;
        }
  for (int nr = 0; nr < L.n2m; ++nr)
    for (int l = 0; l <= L.l2m; ++l)
      for (int m = -l; m <= l; ++m) {
        const int f = L.A0(nr, l, m);
        mir[f] = L.A0(nr, l, -m);
        sgn[f] = (m & 1) ? -1 : 1;
      }
  // multiplicity of every WA weight in the force and torque loops
  // (src/forces.F90:509-614): a weight with multiplicity 0 is never used, so
  // its slot needs no entries
  std::vector<char> wa_used(L.nW, 1);
  for (int n1 = 0; n1 < L.n3a; ++n1)
    for (int l1 = 0; l1 <= L.l3a; ++l1)
      for (int m1 = -l1; m1 <= l1; ++m1)
        for (int n2 = 0; n2 < L.n3m; ++n2)
          for (int l2 = 0; l2 <= L.l3m; ++l2) {
            const int w = L.WA(n1, l1, m1, n2, l2, 0);
            if (w >= 0 && m1 < 0) wa_used[w] = 0;
          }
  // density (A0-slot) terms, summed per factor set {A0, sorted others}
  using G0Key = std::array<int, 2 + kMaxArity>;  // arity, A0 factor, the others (ONE-padded)
  std::map<G0Key, std::array<double, 2>> g0;
  const auto g0_key = [&](int arity, int a0, const int* o) {
    G0Key key;
    key.fill(L.offOne);
    key[0] = arity;
    key[1] = a0;
    for (int q = 0; q < arity; ++q) key[2 + q] = o[q];
    std::sort(key.begin() + 2, key.begin() + 2 + arity);
    return key;
  };
  // every term adds kappa * (product of the other factors) to the A0 factor's
  // slot (density and W0) and to the weight slot of each other factor
  for_each_term(M, with_b3, [&](int rank, size_t c, double cf, const int* f, const int* w) {
    const double k[2] = {M.coef[rank][c][0] * cf, M.coef[rank][c][1] * cf};
    if (k[0] == 0.0 && k[1] == 0.0) return;
    ++nterm[rank];
    const int arity = rank - 1;
    auto& kk = g0[g0_key(arity, f[0], f + 1)];
    kk[0] += k[0];
    kk[1] += k[1];
    for (int q = 1; q < rank; ++q) {
      if (w[q] < 0 || (rank >= 3 && !wa_used[w[q]])) continue;
      int others[kMaxArity], n = 0;
      for (int o = 0; o < rank; ++o)
        if (o != q) others[n++] = f[o];
      sink.add(sink.w_slot(w[q]), k, others, arity);
    }
  });
  if (with_b3)
    for (int q = 0; q < 7; ++q) M.nterms[q] = nterm[q];
  // Density entries folded over mirror pairs. A term's mirror (every m
  // negated) has the conjugate product times s = the product of its factors'
  // signs, so the pair adds (kappa + s kappa') Re(prod) to rho. The member
  // whose key is larger (its A0 has m' > 0, or m' = 0 and larger others)
  // takes 2 kappa, and the other only the remainder kappa' - s kappa, which is
  // zero for the pairs of a mirror-symmetric basis (all of the Fe layout's).
  // Self-mirror terms keep kappa. The W0 slots of m' > 0 then hold twice the
  // terms' gradient, so their multiplicity is 1 (slot_mult below).
  for (const auto& kv : g0) {
    const G0Key& key = kv.first;
    const int arity = key[0];
    int mo[kMaxArity];
    int s = sgn[key[1]];
    for (int q = 0; q < arity; ++q) {
      mo[q] = mir[key[2 + q]];
      s *= sgn[key[2 + q]];
    }
    const G0Key mkey = g0_key(arity, mir[key[1]], mo);
    const auto emit = [&](const G0Key& at, double k0, double k1) {
      if (k0 == 0.0 && k1 == 0.0) return;
      const double k[2] = {k0, k1};
      int others[kMaxArity];
      for (int q = 0; q < kMaxArity; ++q) others[q] = at[2 + q];
      sink.add(sink.g0_slot(at[1]), k, others, arity);
    };
    const auto mit = g0.find(mkey);
    if (mkey == key) {
      emit(key, kv.second[0], kv.second[1]);
    } else if (mkey < key) {
      const double m0 = mit == g0.end() ? 0.0 : mit->second[0], m1 = mit == g0.end() ? 0.0 : mit->second[1];
      emit(key, 2.0 * kv.second[0], 2.0 * kv.second[1]);
      emit(mkey, m0 - s * kv.second[0], m1 - s * kv.second[1]);
    } else if (mit == g0.end()) {
      emit(key, kv.second[0], kv.second[1]);  // no partner: the pair is this term alone
    }
  }

  // flatten into segments, then pack segments into warp groups
  g = GatherTable();
  g.nG0 = L.n2m * L.ls2;
  g.nslot = sink.nslot;
  g.slot_seg_begin.assign(g.nslot + 1, 0);
  struct Seg {
    int arity, slot;
    const Entry* e;
    int count;
  };
  std::vector<Seg> segs;
  for (int s = 0; s < g.nslot; ++s) {
    g.slot_seg_begin[s] = static_cast<int32_t>(segs.size());
    for (int a = 1; a <= kMaxArity; ++a) {
      const auto& es = sink.by_slot[a][s];
      g.entries[a] += static_cast<long>(es.size());
      for (size_t e0 = 0; e0 < es.size(); e0 += GatherTable::kSegLen) {
        int cnt = static_cast<int>(std::min(es.size() - e0, static_cast<size_t>(GatherTable::kSegLen)));
        segs.push_back({a, s, es.data() + e0, cnt});
      }
    }
  }
  g.slot_seg_begin[g.nslot] = static_cast<int32_t>(segs.size());
  g.nseg = static_cast<int>(segs.size());
  g.seg_slot.resize(g.nseg);
  for (int i = 0; i < g.nseg; ++i) g.seg_slot[i] = segs[i].slot;
  std::vector<int> order(g.nseg);
  for (int i = 0; i < g.nseg; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    if (segs[a].arity != segs[b].arity) return segs[a].arity > segs[b].arity;
    return segs[a].count > segs[b].count;
  });
  const int W = GatherTable::kLanes;
  for (size_t i = 0; i < order.size();) {
    const int a = segs[order[i]].arity;
    size_t j = i;
    while (j < order.size() && j - i < static_cast<size_t>(W) && segs[order[j]].arity == a) ++j;
    const int len = segs[order[i]].count;  // sorted descending
    g.grp_arity.push_back(a);
    g.grp_len.push_back(len);
    g.grp_first.push_back(static_cast<int32_t>(g.o12[a].size()));
    for (int lane = 0; lane < W; ++lane) g.grp_seg.push_back(i + lane < j ? order[i + lane] : -1);
    for (int e = 0; e < len; ++e)
      for (int lane = 0; lane < W; ++lane) {
        const Seg* sg = (i + lane < j) ? &segs[order[i + lane]] : nullptr;
        if (sg && e < sg->count) {
          const Entry& en = sg->e[e];
          g.kap[a][0].push_back(en.kappa[0]);
          g.kap[a][1].push_back(en.kappa[1]);
          g.o12[a].push_back(static_cast<uint32_t>(en.o[0]) | (static_cast<uint32_t>(a >= 2 ? en.o[1] : 0) << 16));
          if (a >= 3)
            g.o34[a].push_back(static_cast<uint32_t>(en.o[2]) | (static_cast<uint32_t>(a >= 4 ? en.o[3] : 0) << 16));
          if (a == 5) g.o5.push_back(en.o[4]);
        } else {
          const uint32_t z = static_cast<uint32_t>(L.offZero);
          g.kap[a][0].push_back(0.0);
          g.kap[a][1].push_back(0.0);
          g.o12[a].push_back(z | (z << 16));
          if (a >= 3) g.o34[a].push_back(z | (z << 16));
          if (a == 5) g.o5.push_back(static_cast<uint16_t>(L.offZero));
        }
      }
    i = j;
  }
  g.ngroup = static_cast<int>(g.grp_arity.size());
  // slot -> weight mapping and multiplicity
  g.slot_factor.assign(g.nslot, -1);
  g.slot_weight.assign(g.nslot, -1);
  g.slot_mult.assign(g.nslot, 0.0);
  for (int nr = 0; nr < L.n2m; ++nr)
    for (int l = 0; l <= L.l2m; ++l)
      for (int m = -l; m <= l; ++m) {
        int s = L.A0(nr, l, m) - L.offA0;
        g.slot_factor[s] = L.A0(nr, l, m);
        if (m >= 0) {
          g.slot_weight[s] = L.W0(nr, l, m);
          g.slot_mult[s] = 1.0;  // m' > 0: the folded slot already holds both mirror halves
        }
      }
  for (int n1 = 0; n1 < L.n3a; ++n1)
    for (int l1 = 0; l1 <= L.l3a; ++l1)
      for (int m1 = -l1; m1 <= l1; ++m1)
        for (int n2 = 0; n2 < L.n3m; ++n2)
          for (int l2 = 0; l2 <= L.l3m; ++l2)
            for (int m2 = 0; m2 <= l2; ++m2) {
              int w = L.WA(n1, l1, m1, n2, l2, m2);
              int s = sink.w_slot(w);
              g.slot_weight[s] = w;
              // force/torque loop multiplicities (src/forces.F90:509-614)
              g.slot_mult[s] = m2 > 0 ? 2.0 : (m1 > 0 ? 2.0 : (m1 == 0 ? 1.0 : 0.0));
            }
  for (int n = 0; n < L.nba; ++n)
    for (int nr = 0; nr < L.n2m; ++nr)
      for (int l = 0; l <= L.l2m; ++l)
        for (int m = 0; m <= l; ++m) {
          int w = L.W2(n, nr, l, m);
          int s = sink.w_slot(w - L.offW2 + L.nWA);
          g.slot_weight[s] = w;
          g.slot_mult[s] = m == 0 ? 1.0 : 2.0;
        }
  if (rest && !build_rest(M, sink, g, *rest)) {
    msg = "internal error: inconsistent 2-/4-body record streams";
    return MAGACE_ERR_UNSUPPORTED;
  }
  (void)d;
  (void)nd;
  return MAGACE_OK;
}


// Dense form of the 3-body density (the term of src/b_basis.F90:142-212).
// For one angular combination (l1, l0', l1', l2') and one m-term
// (m1, m0', m1', m2'), the 3-body density is
//   cf * sum_{n0', i, j} C[n0'][i][j] a[n0'] X[i] Y[j]
// with a = A0(., l0', m0'), X[i] = A(n1, l1, m1, n1', l1', m1'),
// Y[j] = A(n2, l1, -m1, n2', l2', m2'), i = n1*n3m + n1', j = n2*n3m + n2',
// and C the cluster coefficients (zero for pairs the enumeration excludes).
// Every (combination, m-term) is one task of the density kernel.
void build_dense_b3(Model& M) {
  const FactorLayout& L = M.L;
  DenseB3& D = M.db3;
  D = DenseB3();
  const int I = L.n3a * L.n3m, NM = L.n3m;
  D.I = I;
  D.NM = NM;
  // combos in order of first appearance in the enumeration
  std::map<std::array<int, 4>, int> combo_id;
  for (const auto& r : M.rows[3]) {
    std::array<int, 4> key{r[5], r[6], r[7], r[8]};
    if (!combo_id.count(key)) {
      combo_id[key] = static_cast<int>(D.combo_l.size());
      D.combo_l.push_back(key);
    }
  }
  D.ncombo = static_cast<int>(D.combo_l.size());
  D.C.assign(static_cast<size_t>(D.ncombo) * NM * I * I, 0.0);
  D.pattern.assign(D.ncombo, 0);
  for (int k = 0; k < D.ncombo; ++k) {
    const int q1 = D.combo_l[k][2], q2 = D.combo_l[k][3];
    D.pattern[k] = q1 == q2 ? 0 : (q1 > q2 ? 1 : 2);
  }
  for (size_t c = 0; c < M.rows[3].size(); ++c) {
    const auto& r = M.rows[3][c];
    const int k = combo_id[{r[5], r[6], r[7], r[8]}];
    const int i = (r[0] - 1) * NM + (r[3] - 1), j = (r[1] - 1) * NM + (r[4] - 1), p0 = r[2] - 1;
    D.C[((static_cast<size_t>(k) * NM + p0) * I + i) * I + j] = M.coef[3][c][0];
  }
  // compact elements: A half-plane in weight order, then A0(n' < n3m, m' >= 0)
  D.nc = L.nWA + NM * L.h3;
  D.factor_of.assign(D.nc, 0);
  D.compact_of_weight.assign(L.nW, -1);
  for (int n = 0; n < L.n3a; ++n)
    for (int l = 0; l <= L.l3a; ++l)
      for (int m = -l; m <= l; ++m)
        for (int p = 0; p < NM; ++p)
          for (int q = 0; q <= L.l3m; ++q)
            for (int u = 0; u <= q; ++u) {
              const int c = L.WA(n, l, m, p, q, u);
              D.factor_of[c] = L.A(n, l, m, p, q, u);
              D.compact_of_weight[c] = c;
            }
  for (int p = 0; p < NM; ++p)
    for (int q = 0; q <= L.l3m; ++q)
      for (int u = 0; u <= q; ++u) {
        const int c = L.nWA + p * L.h3 + q * (q + 1) / 2 + u;
        D.factor_of[c] = L.A0(p, q, u);
        D.compact_of_weight[L.W0(p, q, u)] = c;
      }
  // (-1)^k conj(mirror) as sign bits: negate real part if odd k, else imaginary
  const auto mirrored = [](int c, int k) {
    return static_cast<uint16_t>(c | ((k & 1) ? 0x8000 : 0x4000));
  };
  const auto code_A = [&](int n, int l, int m, int p, int q, int u) {
    return u >= 0 ? static_cast<uint16_t>(L.WA(n, l, m, p, q, u)) : mirrored(L.WA(n, l, -m, p, q, -u), m + u);
  };
  const auto code_A0 = [&](int p, int q, int u) {
    const int c = L.nWA + p * L.h3 + q * (q + 1) / 2 + std::abs(u);
    return u >= 0 ? static_cast<uint16_t>(c) : mirrored(c, u);
  };
  // Mirror pairs: negating every m of a task (m1, m0', m1', m2') leaves its
  // coupling unchanged (each Clebsch-Gordan factor picks up (-1)^(j1+j2-J),
  // +1 for these even triangles) and turns every factor into +-conj of
  // itself with signs whose product is +1, so the mirror task's density is
  // the conjugate of the task's. Only one task of each pair is evaluated:
  // it contributes 2 Re rho_T (1 for a task that is its own mirror), and for
  // every position it also adds the mirror task's gradient,
  // s conj(dRho_T/dF), to the element the mirror task reads directly there
  // (code2: compact element | bit 15 for s = -1; 0xffff where the mirror
  // task reads that position through a mirror code itself, or is T).
  const auto mirror_code = [&](int c, int k) {
    return static_cast<uint16_t>(c | ((k & 1) ? 0x8000 : 0));
  };
  for (int k = 0; k < D.ncombo; ++k) {
    const int l1 = D.combo_l[k][0], q0 = D.combo_l[k][1], q1 = D.combo_l[k][2], q2 = D.combo_l[k][3];
    for (int m1 = -l1; m1 <= l1; ++m1) {
      const double cfa = clebsch_gordan(l1, l1, 0, m1, -m1, 0);
      for (int u0 = -q0; u0 <= q0; ++u0)
        for (int u1 = -q1; u1 <= q1; ++u1) {
          const int u2 = -(u0 + u1);
          if (std::abs(u2) > q2) continue;
          const double cf = cfa * (clebsch_gordan(q0, q1, q2, u0, u1, -u2) * clebsch_gordan(q2, q2, 0, u2, -u2, 0));
          if (cf == 0.0) continue;
          // keep the task whose (m1, m0', m1') is lexicographically >= its mirror's
          const std::array<int, 3> me{m1, u0, u1}, mi{-m1, -u0, -u1};
          if (me < mi) continue;
          const bool self = me == mi;
          ++D.ntask;
          D.task_combo.push_back(k);
          D.task_cf.push_back(cf);
          D.task_w.push_back(self ? 1.0 : 2.0);
          for (int p = 0; p < NM; ++p) {
            D.code.push_back(code_A0(p, q0, u0));
            D.code2.push_back(self || u0 > 0 ? 0xffff : mirror_code(L.nWA + p * L.h3 + q0 * (q0 + 1) / 2 - u0, u0));
          }
          for (int n = 0; n < L.n3a; ++n)
            for (int p = 0; p < NM; ++p) {
              D.code.push_back(code_A(n, l1, m1, p, q1, u1));
              D.code2.push_back(self || u1 > 0 ? 0xffff : mirror_code(L.WA(n, l1, -m1, p, q1, -u1), m1 + u1));
            }
          for (int n = 0; n < L.n3a; ++n)
            for (int p = 0; p < NM; ++p) {
              D.code.push_back(code_A(n, l1, -m1, p, q2, u2));
              D.code2.push_back(self || u2 > 0 ? 0xffff : mirror_code(L.WA(n, l1, m1, p, q2, -u2), m1 + u2));
            }
        }
    }
  }
  // tasks grouped by pattern (stable): warps that take consecutive tasks
  // from the kernel's shared task counter then run the same unrolled code at
  // the same time (a longest-pattern-first order measured ~2 % slower)
  const int npos = NM + 2 * I;
  std::vector<int> order(D.ntask);
  for (int t = 0; t < D.ntask; ++t) order[t] = t;
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return D.pattern[D.task_combo[x]] < D.pattern[D.task_combo[y]]; });
  std::vector<int32_t> combo(D.ntask);
  std::vector<double> cf(D.ntask), w(D.ntask);
  std::vector<uint16_t> code(D.code.size()), code2(D.code2.size());
  for (int t = 0; t < D.ntask; ++t) {
    combo[t] = D.task_combo[order[t]];
    cf[t] = D.task_cf[order[t]];
    w[t] = D.task_w[order[t]];
    const size_t src = static_cast<size_t>(order[t]) * npos, dst = static_cast<size_t>(t) * npos;
    std::copy(D.code.begin() + src, D.code.begin() + src + npos, code.begin() + dst);
    std::copy(D.code2.begin() + src, D.code2.begin() + src + npos, code2.begin() + dst);
  }
  D.task_combo.swap(combo);
  D.task_cf.swap(cf);
  D.task_w.swap(w);
  D.code.swap(code);
  D.code2.swap(code2);
}

// Per-cluster m-terms of the descriptors, in coefficient order (ranks 1..4).
void build_descriptors(Model& M) {
  DescriptorTable& T = M.desc;
  T = DescriptorTable();
  T.n1 = static_cast<int>(M.rows[1].size());
  int first[7] = {0, 0, 0, 0, 0, 0, 0};  // first cluster of each rank past rank 1
  T.nB = T.n1;
  for (int r = 2; r <= 6; ++r) {
    first[r] = T.nB - T.n1;
    T.nB += static_cast<int>(M.rows[r].size());
  }
  for (const auto& r : M.rows[1]) T.rank1_n.push_back(r[0] - 1);
  std::vector<int32_t> count(T.nB - T.n1, 0);
  std::vector<std::array<int, 7>> terms;  // cluster (0-based past rank 1), six factors
  std::vector<double> cfs;
  for_each_term(M, true, [&](int rank, size_t c, double cf, const int* f, const int*) {
    const int k = static_cast<int>(c) + first[rank];
    ++count[k];
    terms.push_back({k, f[0], f[1], f[2], f[3], f[4], f[5]});
    cfs.push_back(cf);
  });
  T.begin.assign(T.nB - T.n1 + 1, 0);
  for (int k = 0; k < T.nB - T.n1; ++k) T.begin[k + 1] = T.begin[k] + count[k];
  T.cf.assign(cfs.size(), 0.0);
  T.o.assign(kDescFactors * cfs.size(), static_cast<uint16_t>(M.L.offOne));
  std::vector<int32_t> fill(T.begin.begin(), T.begin.end() - 1);
  for (size_t e = 0; e < terms.size(); ++e) {
    const int pos = fill[terms[e][0]]++;
    T.cf[pos] = cfs[e];
    for (int q = 0; q < 6; ++q) T.o[kDescFactors * pos + q] = static_cast<uint16_t>(terms[e][1 + q]);
  }
}

}  // namespace

// The coefficient-dependent tables: 1-body coefficients, gather tables with
// the coefficients folded in, and the dense 3-body tables.
int build_tables(Model& M, std::string& msg) {
  const FactorLayout& L = M.L;
  for (int dd = 0; dd < 2; ++dd) M.c1[dd].assign(L.nbm, 0.0);
  for (size_t c = 0; c < M.rows[1].size(); ++c)
    for (int dd = 0; dd < 2; ++dd) M.c1[dd][M.rows[1][c][0] - 1] += M.coef[1][c][dd];

  int st = build_gather(M, true, M.gt, msg);
  if (st) return st;
  // tables of the specialised kernels: 3-body terms as dense per-(combo, m)
  // contractions, everything else through the gather table without them
  if (M.ndensity == 1 && !M.high) {
    st = build_gather(M, false, M.gt_nob3, msg, &M.rest);
    if (st) return st;
    build_dense_b3(M);
    // multiplicity of each compact element's weight, from the gather table's
    // slots (every weight has a slot there, with or without entries); the
    // A0 slots there hold folded mirror pairs (multiplicity 1), while the
    // 3-body gradients of an A0 element with m' > 0 take the half-plane
    // multiplicity 2 (src/forces.F90:690-749)
    DenseB3& D = M.db3;
    const FactorLayout& L = M.L;
    D.mult.assign(D.nc, 0.0);
    for (int s = 0; s < M.gt_nob3.nslot; ++s) {
      const int w = M.gt_nob3.slot_weight[s];
      if (w < 0 || D.compact_of_weight[w] < 0) continue;
      double mu = M.gt_nob3.slot_mult[s];
      if (s < M.gt_nob3.nG0) {
        const int lm = s % L.ls2, l = static_cast<int>(std::sqrt(static_cast<double>(lm)) + 1e-9);
        mu = lm - l * l - l == 0 ? 1.0 : 2.0;
      }
      D.mult[D.compact_of_weight[w]] = mu;
    }
    // gradients of elements whose weight has multiplicity 0 are never used:
    // such a direct read gets the 0x2000 flag (no gradient atomic), such a
    // mirror target no mirror gradient
    if (D.nc < 0x2000)
      for (size_t q = 0; q < D.code.size(); ++q) {
        uint16_t& c = D.code[q];
        if (!(c & 0xc000) && D.mult[c & 0x1fff] == 0.0) c = static_cast<uint16_t>(c | 0x2000);
        uint16_t& c2 = D.code2[q];
        if (c2 != 0xffff && D.mult[c2 & 0x3fff] == 0.0) c2 = 0xffff;
      }
    // coefficient mass of every element's gradient (DenseB3::bound): the
    // gradient of position a_p is sum_{i,j} C[p][i][j] X_i Y_j, of X_i
    // sum_{p,j} C a_p Y_j and of Y_j sum_{p,i} C a_p X_i, each times cf
    const int I = D.I, NM = D.NM, npos = NM + 2 * I;
    std::vector<double> mass(D.nc, 0.0), row(npos);
    D.bound_rho = 0.0;
    for (int t = 0; t < D.ntask; ++t) {
      std::fill(row.begin(), row.end(), 0.0);
      const double* Ck = D.C.data() + static_cast<size_t>(D.task_combo[t]) * NM * I * I;
      double csum = 0.0;
      for (int p = 0; p < NM; ++p)
        for (int i = 0; i < I; ++i)
          for (int j = 0; j < I; ++j) {
            const double c = std::fabs(Ck[(p * I + i) * I + j]);
            row[p] += c;
            row[NM + i] += c;
            row[NM + I + j] += c;
            csum += c;
          }
      const double cf = std::fabs(D.task_cf[t]);
      D.bound_rho += cf * std::fabs(D.task_w[t]) * csum;
      for (int q = 0; q < npos; ++q) {
        const uint16_t c = D.code[static_cast<size_t>(t) * npos + q];
        const uint16_t c2 = D.code2[static_cast<size_t>(t) * npos + q];
        if (!(c & 0xe000)) mass[c & 0x1fff] += cf * row[q];
        if (c2 != 0xffff) mass[c2 & 0x3fff] += cf * row[q];
      }
    }
    D.bound = 0.0;
    for (double v : mass) D.bound = std::max(D.bound, v);
  }
  return MAGACE_OK;
}

int num_coefficients(const Model& M) {
  int n = 0;
  for (int r = 1; r <= 6; ++r) n += static_cast<int>(M.rows[r].size());
  return n;
}

void get_coefficients(const Model& M, double* c) {
  const int nB = num_coefficients(M);
  for (int d = 0; d < M.ndensity; ++d) {
    int k = 0;
    for (int r = 1; r <= 6; ++r)
      for (size_t q = 0; q < M.rows[r].size(); ++q) c[d * nB + k++] = M.coef[r][q][d];
  }
}

int set_coefficients(Model& M, const double* c, std::string& msg) {
  const int nB = num_coefficients(M);
  for (int d = 0; d < M.ndensity; ++d) {
    int k = 0;
    for (int r = 1; r <= 6; ++r)
      for (size_t q = 0; q < M.rows[r].size(); ++q) M.coef[r][q][d] = c[d * nB + k++];
  }
  return build_tables(M, msg);
}

int build_model(const Potential& pot, double rcut, double rcut_magnetic, Model& M, std::string& msg) {
  M = Model();
  M.pot = pot;
  M.cutoff = rcut;
  M.cutoff_m = rcut_magnetic;
  const BasisDims& d = pot.dims;
  // limits of src/util.F90:234-272
  if (d.l3max_a < d.l4max_a || d.l3max_a < d.l5max_a || d.l3max_a < d.l6max_a || d.l2max_m < d.l3max_m ||
      d.l2max_m < d.l4max_m || d.l2max_m < d.l5max_m || d.l2max_m < d.l6max_m || d.nradial3_a < d.nradial4_a ||
      d.nradial3_a < d.nradial5_a || d.nradial3_a < d.nradial6_a || d.nradial2_m < d.nradial3_m ||
      d.nradial2_m < d.nradial4_m || d.nradial2_m < d.nradial5_m || d.nradial2_m < d.nradial6_m ||
      d.nradial3_a > d.nradbase_a || d.nradial2_m > d.nradbase_m ||
      std::max(d.nradial3_a, d.nradial2_m) > std::max(d.nradbase_a, d.nradbase_m)) {
    msg = "basis dimensions violate the limits of the reference setup";
    return MAGACE_ERR_FORMAT;
  }
  if (d.nradial2_m == 0 || d.nradial3_a == 0 || d.nradial3_m == 0) {
    msg = "potentials without 2- or 3-body magnetic terms are not supported";
    return MAGACE_ERR_UNSUPPORTED;
  }
  // 5- and 6-body factors come from the 3-body A basis, which holds n' <=
  // nradial3_m and l' <= l3max_m here; the reference evaluates a rank only
  // when the ranks below it are present (src/b_basis.F90:217-218, :312-313;
  // without them its packs of the higher ranks stay uninitialised); its
  // 6-body couplings stop for 2 l6max above l3max / l2max
  // (src/util.F90:3430-3434)
  if (d.nradial5_m > d.nradial3_m || d.nradial6_m > d.nradial3_m || d.l5max_m > d.l3max_m ||
      d.l6max_m > d.l3max_m) {
    msg = "5- and 6-body magnetic radial functions or l' beyond the 3-body ones are not supported";
    return MAGACE_ERR_UNSUPPORTED;
  }
  const bool has4 = d.nradial4_a || d.nradial4_m, has5 = d.nradial5_a || d.nradial5_m,
             has6 = d.nradial6_a || d.nradial6_m;
  if ((has5 && !has4) || (has6 && !has5)) {
    msg = "a rank of clusters without the rank below it is not evaluated by the reference either";
    return MAGACE_ERR_UNSUPPORTED;
  }
  if (has6 && d.nradial6_a && d.nradial6_m && (2 * d.l6max_a > d.l3max_a || 2 * d.l6max_m > d.l2max_m)) {
    msg = "6-body couplings not worked for lmax > 6 (src/util.F90:3430-3434)";
    return MAGACE_ERR_UNSUPPORTED;
  }
  if (d.nfemb < 0 || d.nfemb > 2) {
    msg = "embedding types 3 and 4 have no gradient (src/forces.F90:1234-1258)";
    return MAGACE_ERR_UNSUPPORTED;
  }
  for (int t : {d.radtype_a, d.radtype_m})
    if (t < 3 || t > 8) {
      msg = "radial basis types 0-2 are not working in the reference either";
      return MAGACE_ERR_UNSUPPORTED;
    }
  if (pot.cut[0] > rcut || pot.cut[1] > rcut_magnetic) {
    msg = "global cutoff shorter than the potential's cutoff";
    return MAGACE_ERR_FORMAT;
  }
  M.ndensity = d.ndensity;
  M.nfemb = d.nfemb;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) M.par[a][b] = pot.par[a][b];
  M.ecut = pot.ecut;
  M.decut = pot.decut;
  M.core_pre = pot.core_pre;
  M.core_lambda = pot.core_lambda;

  FactorLayout& L = M.L;
  L.n3a = d.nradial3_a;
  L.n3m = d.nradial3_m;
  L.l3a = d.l3max_a;
  L.l3m = d.l3max_m;
  L.nba = d.nradbase_a;
  L.nbm = d.nradbase_m;
  L.n2m = d.nradial2_m;
  L.l2m = d.l2max_m;
  L.lsa = (L.l3a + 1) * (L.l3a + 1);
  L.ls3 = (L.l3m + 1) * (L.l3m + 1);
  L.ls2 = (L.l2m + 1) * (L.l2m + 1);
  L.h3 = (L.l3m + 1) * (L.l3m + 2) / 2;
  L.h2 = (L.l2m + 1) * (L.l2m + 2) / 2;
  L.offA = 0;
  L.offA2 = L.n3a * L.lsa * L.n3m * L.ls3;
  L.offA0 = L.offA2 + L.nba * L.n2m * L.ls2;
  L.offOne = L.offA0 + L.n2m * L.ls2;
  L.offZero = L.offOne + 1;
  L.nF = L.offZero + 1;
  L.nWA = L.n3a * L.lsa * L.n3m * L.h3;
  L.offW2 = L.nWA;
  L.offW0 = L.offW2 + L.nba * L.n2m * L.h2;
  L.nW = L.offW0 + L.n2m * L.h2;
  if (L.nF > 65535) {
    msg = "basis too large for 16-bit factor indices";
    return MAGACE_ERR_UNSUPPORTED;
  }

  enumerate(d, M.rows);
  for (int rank = 5; rank <= 6; ++rank)
    if (!enumerate_high(d, rank, M.rows[rank])) {
      msg = "the atomic basis is not ordered lexicographically (src/util.F90:2884-2889, :3512-3517)";
      return MAGACE_ERR_FORMAT;
    }
  M.high = !M.rows[5].empty() || !M.rows[6].empty();
  // match the file's cluster records (src/util.F90:678-956); a record sets
  // every cluster with its index tuple (padded 5-/6-body clusters can share one)
  std::map<std::vector<int>, std::vector<size_t>> index[7];
  for (int r = 1; r <= 6; ++r) {
    M.coef[r].assign(M.rows[r].size(), {0.0, 0.0});
    for (size_t c = 0; c < M.rows[r].size(); ++c) index[r][M.rows[r][c]].push_back(c);
    for (const auto& kv : pot.clusters[r]) {
      auto it = index[r].find(kv.first);
      if (it == index[r].end()) {
        ++M.unmatched_records;
        continue;
      }
      for (size_t c : it->second) M.coef[r][c] = kv.second;
    }
  }
  {
    const int st = build_tables(M, msg);
    if (st) return st;
  }
  build_descriptors(M);
  if (!build_lut(M, M.lut)) {
    msg = "unsupported radial basis type";
    return MAGACE_ERR_UNSUPPORTED;
  }
  M.ready = true;
  return MAGACE_OK;
}

}  // namespace magace
