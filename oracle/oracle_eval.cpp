// CPU oracle, evaluation half: prepA, prepB, forceweights, forcecompute and
// torquecompute restated for chunks of atoms, plus the exported C API.
//
// TEST INFRASTRUCTURE ONLY (the parity checker; see oracle.h). The loops keep
// the reference's order and its per-atom pack arrays (including the stored
// dB/dA packs) so that the timed CPU baseline has the reference's memory
// behaviour; atoms are processed in chunks because the dB/dA packs take
// about 2.4 MB per atom for the Fe.pbe.in layout (src/util.F90:1520).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "oracle.h"

namespace {

const double kPi = 3.14159265358979323846264338327950288419;

OracleState g_state;
std::string g_err;

// flat views of the acelib arguments, with the reference's 1-based indexing
struct Inputs {
  int natom = 0, nei = 0;
  const int *nstart = nullptr, *nstop = nullptr;
  const double *dlist = nullptr, *elist = nullptr, *dlist_momi = nullptr, *elist_momi = nullptr;
  const double *dlist_mom = nullptr, *elist_mom = nullptr;
  double d2l(int ij) const { return dlist[ij - 1]; }
  double e2l(int c, int ij) const { return elist[3 * (ij - 1) + c - 1]; }
  double d2l_mom(int ij) const { return dlist_mom[ij - 1]; }
  double e2l_mom(int c, int ij) const { return elist_mom[3 * (ij - 1) + c - 1]; }
  double d2l_momi(int a) const { return dlist_momi[a - 1]; }
  double e2l_momi(int c, int a) const { return elist_momi[3 * (a - 1) + c - 1]; }
};

// ---------------------------------------------------------------------------
// src/radial.F90:53-107
int lookupRadspline_atomic(const OracleState& s, double r, FArr<double>& fr, FArr<double>& dfr,
                           std::vector<double>& gr, std::vector<double>& dgr, double& cr, double& dcr) {
  const double rs = s.rscalelookup_atomic;
  double x = r * rs;
  double fl = std::floor(x);
  if (!(fl > 0.0)) return ORACLE_ERR_SMALL_R;  // also rejects NaN
  if (fl >= (double)s.nlut) {
    std::fill(gr.begin(), gr.end(), 0.0);
    std::fill(dgr.begin(), dgr.end(), 0.0);
    fr.fill(0.0);
    dfr.fill(0.0);
    cr = 0.0;
    dcr = 0.0;
    return ORACLE_OK;
  }
  int nl = (int)fl;
  double wl = x - (double)nl, wl2 = wl * wl, wl3 = wl2 * wl, w2l1 = 2.0 * wl, w3l2 = 3.0 * wl2;
  for (int nr = 1; nr <= s.nradbase_atomic; ++nr) {
    const double* c = &s.lutgrs_atomic(0, nr, nl);
    gr[nr] = c[0] + c[1] * wl + c[2] * wl2 + c[3] * wl3;
    dgr[nr] = (c[1] + c[2] * w2l1 + c[3] * w3l2) * rs;
  }
  for (int l = 0; l <= s.l3max_atomic; ++l)
    for (int nr = 1; nr <= s.nradial3_atomic; ++nr) {
      const double* c = &s.lutfrs_atomic(0, nr, l, nl);
      fr(nr, l) = c[0] + c[1] * wl + c[2] * wl2 + c[3] * wl3;
      dfr(nr, l) = (c[1] + c[2] * w2l1 + c[3] * w3l2) * rs;
    }
  const double* c = &s.luthcrs_atomic(0, nl);
  cr = c[0] + c[1] * wl + c[2] * wl2 + c[3] * wl3;
  dcr = (c[1] + c[2] * w2l1 + c[3] * w3l2) * rs;
  return ORACLE_OK;
}

// src/radial.F90:111-160. The reference has no upper bound check and reads past
// its table for |m| >= the magnetic cutoff; here that is an error.
int lookupRadspline_magnetic(const OracleState& s, double r, FArr<double>& fr, FArr<double>& dfr,
                             std::vector<double>& gr, std::vector<double>& dgr) {
  const double rs = s.rscalelookup_magnetic;
  double x = r * rs;
  double fl = std::floor(x);
  if (!(fl >= 0.0)) return ORACLE_ERR_MOMENT;
  if (fl >= (double)s.nlut) return ORACLE_ERR_MOMENT;
  int nl = (int)fl;
  if (nl == 0) {
    std::fill(gr.begin(), gr.end(), 1.0);
    std::fill(dgr.begin(), dgr.end(), 0.0);
    fr.fill(1.0);
    dfr.fill(0.0);
    return ORACLE_OK;
  }
  double wl = x - (double)nl, wl2 = wl * wl, wl3 = wl2 * wl, w2l1 = 2.0 * wl, w3l2 = 3.0 * wl2;
  for (int nr = 1; nr <= s.nradbase_magnetic; ++nr) {
    const double* c = &s.lutgrs_magnetic(0, nr, nl);
    gr[nr] = c[0] + c[1] * wl + c[2] * wl2 + c[3] * wl3;
    dgr[nr] = (c[1] + c[2] * w2l1 + c[3] * w3l2) * rs;
  }
  for (int l = 0; l <= s.l2max_magnetic; ++l)
    for (int nr = 1; nr <= s.nradial2_magnetic; ++nr) {
      const double* c = &s.lutfrs_magnetic(0, nr, l, nl);
      fr(nr, l) = c[0] + c[1] * wl + c[2] * wl2 + c[3] * wl3;
      dfr(nr, l) = (c[1] + c[2] * w2l1 + c[3] * w3l2) * rs;
    }
  return ORACLE_OK;
}

// src/spherical.F90:55-282. sh(l,m) is the packed index; Y and dY are 1-based.
void compute_ylm_cart(const OracleState& s, bool atomic, double rx, double ry, double rz, int lmax,
                      FArr<cplx>& shvec, FArr<cplx>& dshvec) {
  const FArr<int>& sh = atomic ? s.shindex_atomic : s.shindex_magnetic;
  const FArr<double>& alm = atomic ? s.alm_atomic : s.alm_magnetic;
  const FArr<double>& blm = atomic ? s.blm_atomic : s.blm_magnetic;
  const int half = (lmax + 1) * (lmax + 2) / 2;
  std::vector<double> plm(half + 1), dplm(half + 1);
  const double Y00 = 1.0, sq3 = 1.73205080756887719318, sq3o2 = 1.22474487139158894067;
  plm[sh(0, 0)] = Y00;
  dplm[sh(0, 0)] = 0.0;
  if (lmax > 0) {
    int k = sh(1, 0);
    plm[k] = Y00 * sq3 * rz;
    dplm[k] = Y00 * sq3;
    k = sh(1, 1);
    plm[k] = -sq3o2 * Y00;
    dplm[k] = 0.0;
    for (int l = 2; l <= lmax; ++l) {
      for (int m = 0; m <= l - 2; ++m) {
        int kk = sh(l, m), k1 = sh(l - 1, m), k2 = sh(l - 2, m);
        plm[kk] = alm(kk) * (rz * plm[k1] + blm(kk) * plm[k2]);
        dplm[kk] = alm(kk) * (plm[k1] + rz * dplm[k1] + blm(kk) * dplm[k2]);
      }
      int kk = sh(l - 1, l - 1), k1 = sh(l, l - 1), k2 = sh(l, l);
      double t = s.dl(l) * plm[kk];
      plm[k1] = t * rz;
      dplm[k1] = t;
      plm[k2] = s.cl(l) * plm[kk];
      dplm[k2] = 0.0;
    }
  }
  const cplx phase(rx, ry);
  // m = 0
  for (int l = 0; l <= lmax; ++l) {
    int k = sh(l, 0);
    shvec(k) = cplx(plm[k], 0.0);
    double dyz = dplm[k];
    double rdy = dyz * rz;
    dshvec(1, k) = cplx(-rdy * rx, 0.0);
    dshvec(2, k) = cplx(-rdy * ry, 0.0);
    dshvec(3, k) = cplx(dyz - rdy * rz, 0.0);
  }
  // m = 1
  for (int l = 1; l <= lmax; ++l) {
    int k = sh(l, 1);
    shvec(k) = phase * plm[k];
    cplx dyx(plm[k], 0.0);
    cplx dyy(0.0, plm[k]);
    cplx dyz(phase.real() * dplm[k], phase.imag() * dplm[k]);
    cplx rdy(rx * dyx.real() + rz * dyz.real(), ry * dyy.imag() + rz * dyz.imag());
    dshvec(1, k) = cplx(dyx.real() - rdy.real() * rx, -(rdy.imag() * rx));
    dshvec(2, k) = cplx(-rdy.real() * ry, dyy.imag() - rdy.imag() * ry);
    dshvec(3, k) = cplx(dyz.real() - rdy.real() * rz, dyz.imag() - rdy.imag() * rz);
  }
  // m > 1
  cplx phasem = phase;
  for (int m = 2; m <= lmax; ++m) {
    cplx mphasem1(phasem.real() * (double)m, phasem.imag() * (double)m);
    phasem = phasem * phase;
    for (int l = m; l <= lmax; ++l) {
      int k = sh(l, m);
      shvec(k) = cplx(phasem.real() * plm[k], phasem.imag() * plm[k]);
      cplx dyx = mphasem1 * plm[k];
      cplx dyy(-dyx.imag(), dyx.real());
      cplx dyz = phasem * dplm[k];
      cplx rdy(rx * dyx.real() + ry * dyy.real() + rz * dyz.real(),
               rx * dyx.imag() + ry * dyy.imag() + rz * dyz.imag());
      dshvec(1, k) = cplx(dyx.real() - rdy.real() * rx, dyx.imag() - rdy.imag() * rx);
      dshvec(2, k) = cplx(dyy.real() - rdy.real() * ry, dyy.imag() - rdy.imag() * ry);
      dshvec(3, k) = cplx(dyz.real() - rdy.real() * rz, dyz.imag() - rdy.imag() * rz);
    }
  }
  // m < 0 by conjugation
  for (int l = 1; l <= lmax; ++l)
    for (int m = 1; m <= l; ++m) {
      cplx ph((m % 2 == 0) ? 1.0 : -1.0, 0.0);
      int k = sh(l, -m), k1 = sh(l, m);
      shvec(k) = std::conj(shvec(k1)) * ph;
      for (int c = 1; c <= 3; ++c) dshvec(c, k) = std::conj(dshvec(c, k1)) * ph;
    }
}

inline double sgn(int m) { return (m % 2 == 0) ? 1.0 : -1.0; }

// src/forces.F90:1134-1266 (nfemb 0-2; types 3 and 4 have no gradient)
void Fexp(double rho, double wpre, double mexp, int nfemb, double& F, double& dF) {
  const double w = 10.0, eps = 1e-10;
  double g, dg, omg, a, da, dy, y1, dy1, y2, dy2, srho;
  switch (nfemb) {
    case 0:
      F = rho;
      dF = 1.0;
      break;
    case 1:
      if (std::fabs(rho) > eps) {
        y1 = w * rho * rho;
        g = (y1 > 30.0) ? 0.0 : std::exp(-y1);
        omg = 1.0 - g;
        a = std::fabs(rho);
        y1 = std::pow(omg * a, mexp);
        y2 = mexp * g * a;
        F = wpre * std::copysign(1.0, rho) * (y1 + y2);
        dg = -2.0 * w * rho * g;
        da = std::copysign(1.0, rho);
        dy = (std::fabs(y1) < eps) ? 0.0 : mexp * y1 / (omg * a);
        dy1 = dy * (-dg * a + omg * da);
        dy2 = mexp * (dg * a + g * da);
        dF = wpre * std::copysign(1.0, rho) * (dy1 + dy2);
      } else {
        F = wpre * mexp * rho;
        dF = wpre * mexp;
      }
      break;
    case 2:
      srho = 1.0 + rho;
      if (std::fabs(srho) > eps) {
        y1 = w * srho * srho;
        g = (y1 > 30.0) ? 0.0 : std::exp(-y1);
        omg = 1.0 - g;
        a = std::fabs(srho);
        y1 = std::pow(omg * a, mexp);
        y2 = mexp * g * a;
        F = wpre * (std::copysign(1.0, srho) * (y1 + y2) - 1.0);
        dg = -2.0 * w * srho * g;
        da = std::copysign(1.0, srho);
        dy = (std::fabs(y1) < eps) ? 0.0 : mexp * y1 / (omg * a);
        dy1 = dy * (-dg * a + omg * da);
        dy2 = mexp * (dg * a + g * da);
        dF = wpre * std::copysign(1.0, srho) * (dy1 + dy2);
      } else {
        F = wpre * mexp * (srho - 1.0);
        dF = wpre * mexp;
      }
      break;
    default:
      F = 0.0;
      dF = 0.0;
  }
}

// src/forces.F90:1270-1289
void innercutoff(double e, double ecutin, double decutin, double& fcut, double& dfcut) {
  double elow = ecutin - decutin;
  if (e >= ecutin) {
    fcut = 0.0;
    dfcut = 0.0;
  } else if (e <= elow) {
    fcut = 1.0;
    dfcut = 0.0;
  } else {
    fcut = 0.5 * (1.0 + std::cos(kPi * (e - elow) / decutin));
    dfcut = -0.5 * std::sin(kPi * (e - elow) / decutin) * kPi / decutin;
  }
}

// ---------------------------------------------------------------------------
// Per-chunk workspace: the modprepA / global / modforces packs of
// src/modules.F90 for `na` atoms and `nb` bonds, indexed locally.
struct Chunk {
  int na = 0;               // atoms in the current chunk
  int cap_a = 0, cap_b = 0; // allocated capacity
  std::vector<int> atom;    // local atom -> global atom (1-based)
  std::vector<int> lbase;   // local atom -> first local bond (1-based)
  FArr<double> fr2pack_atomic, gradfr2pack_atomic, fr2hcpack, gradfr2hcpack;
  FArr<double> frpack_atomic, gradfrpack_atomic, frpack_magnetic, gradfrpack_magnetic;
  FArr<cplx> shpack_atomic, gradshpack_atomic, shpack_magnetic, gradshpack_magnetic;
  FArr<double> grpack_magnetic_0, gradgrpack_magnetic_0, frpack_magnetic_0, gradfrpack_magnetic_0;
  FArr<cplx> shpack_magnetic_0, gradshpack_magnetic_0;
  FArr<cplx> abasepack, abase2pack, abase2pack_magnetic;
  FArr<double> abase2hcpack;
  FArr<double> b1pack, b2pack, b2hcpack, b3pack, b4pack, b5pack, b6pack;
  FArr<cplx> db2pack, db2pack_0, db3pack, db3pack_0, db4pack, db4pack_0, db5pack, db5pack_0, db6pack, db6pack_0;
  FArr<double> wf1;
  FArr<cplx> wf2, wf, wf_0;
  std::vector<double> eicalc, edfcut, rho_out, dEdrho_out;

  void alloc(const OracleState& s, int natoms, int nbonds) {
    if (natoms <= cap_a && nbonds <= cap_b && abasepack.allocated()) return;
    cap_a = std::max(natoms, cap_a);
    cap_b = std::max(nbonds, std::max(cap_b, 1));
    const int A = cap_a, B = cap_b;
    const int nba = s.nradbase_atomic, nbm = s.nradbase_magnetic;
    const int n3a = s.nradial3_atomic, n3m = s.nradial3_magnetic, n2m = s.nradial2_magnetic;
    const int l3a = s.l3max_atomic, l3m = s.l3max_magnetic, l2m = s.l2max_magnetic;
    const int l4a = s.l4max_atomic, l4m = s.l4max_magnetic;
    const int lsa = s.lmaxsq_atomic, lsm = s.lmaxsq_magnetic;
    fr2pack_atomic.init({{1, nba}, {1, B}});
    gradfr2pack_atomic.init({{1, nba}, {1, B}});
    fr2hcpack.init({{1, B}});
    gradfr2hcpack.init({{1, B}});
    frpack_atomic.init({{1, n3a}, {0, l3a}, {1, B}});
    gradfrpack_atomic.init({{1, n3a}, {0, l3a}, {1, B}});
    frpack_magnetic.init({{1, n2m}, {0, l2m}, {1, B}});
    gradfrpack_magnetic.init({{1, n2m}, {0, l2m}, {1, B}});
    shpack_atomic.init({{1, lsa}, {1, B}});
    gradshpack_atomic.init({{1, 3}, {1, lsa}, {1, B}});
    shpack_magnetic.init({{1, lsm}, {1, B}});
    gradshpack_magnetic.init({{1, 3}, {1, lsm}, {1, B}});
    grpack_magnetic_0.init({{1, nbm}, {1, A}});
    gradgrpack_magnetic_0.init({{1, nbm}, {1, A}});
    frpack_magnetic_0.init({{1, n2m}, {0, l2m}, {1, A}});
    gradfrpack_magnetic_0.init({{1, n2m}, {0, l2m}, {1, A}});
    shpack_magnetic_0.init({{1, lsm}, {1, A}});
    gradshpack_magnetic_0.init({{1, 3}, {1, lsm}, {1, A}});
    abasepack.init({{1, std::max(1, n3a)}, {1, lsa}, {1, std::max(1, n3m)}, {1, lsm}, {1, A}});
    abase2pack.init({{1, nba}, {1, n2m}, {1, lsm}, {1, A}});
    abase2pack_magnetic.init({{1, n2m}, {1, lsm}, {1, A}});
    abase2hcpack.init({{1, A}});
    b1pack.init({{1, std::max(1, s.nvar1)}, {1, A}});
    b2pack.init({{1, std::max(1, s.nvar2)}, {1, A}});
    b2hcpack.init({{1, A}});
    b3pack.init({{1, std::max(1, s.nvar3)}, {1, A}});
    b4pack.init({{1, std::max(1, s.nvar4)}, {1, A}});
    db2pack.init({{-l2m, l2m}, {1, std::max(1, s.nvar2)}, {1, A}});
    db2pack_0.init({{-l2m, l2m}, {1, std::max(1, s.nvar2)}, {1, A}});
    db3pack.init({{1, 2}, {-l3a, l3a}, {-l3m, l3m}, {1, std::max(1, s.nvar3)}, {1, A}});
    db3pack_0.init({{-l3m, l3m}, {1, std::max(1, s.nvar3)}, {1, A}});
    db4pack.init({{1, 3}, {-l4a, l4a}, {-l4m, l4m}, {1, std::max(1, s.nvar4)}, {1, A}});
    db4pack_0.init({{-l4m, l4m}, {1, std::max(1, s.nvar4)}, {1, A}});
    const int l5a = s.l5max_atomic, l5m = s.l5max_magnetic, l6a = s.l6max_atomic, l6m = s.l6max_magnetic;
    b5pack.init({{1, std::max(1, s.nvar5)}, {1, A}});
    b6pack.init({{1, std::max(1, s.nvar6)}, {1, A}});
    db5pack.init({{1, 4}, {-l5a, l5a}, {-l5m, l5m}, {1, std::max(1, s.nvar5)}, {1, A}});
    db5pack_0.init({{-l5m, l5m}, {1, std::max(1, s.nvar5)}, {1, A}});
    db6pack.init({{1, 5}, {-l6a, l6a}, {-l6m, l6m}, {1, std::max(1, s.nvar6)}, {1, A}});
    db6pack_0.init({{-l6m, l6m}, {1, std::max(1, s.nvar6)}, {1, A}});
    wf1.init({{1, nbm}, {1, A}});
    wf2.init({{1, nba}, {0, l2m}, {0, l2m}, {1, n2m}, {1, A}});
    wf.init({{-l3a, l3a}, {0, l3a}, {1, std::max(1, n3a)}, {0, l3m}, {0, l3m}, {1, std::max(1, n3m)}, {1, A}});
    wf_0.init({{0, l2m}, {0, l2m}, {1, n2m}, {1, A}});
    eicalc.assign(A + 1, 0.0);
    edfcut.assign(A + 1, 0.0);
    rho_out.assign(2 * (A + 1), 0.0);
    dEdrho_out.assign(2 * (A + 1), 0.0);
  }
};

// src/a_basis.F90:5-361 for the chunk's atoms
int prepA(const OracleState& s, const Inputs& in, Chunk& ch) {
  const int nba = s.nradbase_atomic, nbm = s.nradbase_magnetic;
  const int n3a = s.nradial3_atomic, n3m = s.nradial3_magnetic, n2m = s.nradial2_magnetic;
  const int l3a = s.l3max_atomic, l3m = s.l3max_magnetic, l2m = s.l2max_magnetic;
  const int lsa = s.lmaxsq_atomic, lsm = s.lmaxsq_magnetic;
  const auto& sha = s.shindex_atomic;
  const auto& shm = s.shindex_magnetic;
  const auto& sba = s.shback_atomic;
  const auto& sbm = s.shback_magnetic;
  FArr<cplx> shvec_atomic({{1, lsa}}), dshvec_atomic({{1, 3}, {1, lsa}});
  FArr<cplx> shvec_magnetic({{1, lsm}}), dshvec_magnetic({{1, 3}, {1, lsm}});
  FArr<cplx> shvec_magnetic_i({{1, lsm}}), dshvec_magnetic_i({{1, 3}, {1, lsm}});
  FArr<cplx> abase({{1, std::max(1, n3a)}, {1, lsa}, {1, std::max(1, n3m)}, {1, lsm}});
  FArr<cplx> abase2_magnetic({{1, n2m}, {1, lsm}});
  FArr<cplx> abase2({{1, nba}, {1, n2m}, {1, lsm}});
  FArr<double> fr_atomic({{1, n3a}, {0, l3a}}), dfr_atomic({{1, n3a}, {0, l3a}});
  FArr<double> fr_magnetic({{1, n2m}, {0, l2m}}), dfr_magnetic({{1, n2m}, {0, l2m}});
  FArr<double> fr_magnetic_i({{1, n2m}, {0, l2m}}), dfr_magnetic_i({{1, n2m}, {0, l2m}});
  std::vector<double> gr_atomic(nba + 1), dgr_atomic(nba + 1);
  std::vector<double> gr_magnetic(nbm + 1), dgr_magnetic(nbm + 1);
  std::vector<double> gr_magnetic_i(nbm + 1), dgr_magnetic_i(nbm + 1);
  double cr = 0, dcr = 0;

  for (int la = 1; la <= ch.na; ++la) {
    const int atomi = ch.atom[la];
    abase.fill(cplx(0, 0));
    abase2.fill(cplx(0, 0));
    abase2_magnetic.fill(cplx(0, 0));
    double abase2hc = 0.0;
    const int ijstart = in.nstart[atomi - 1], ijstop = in.nstop[atomi - 1];

    double mi = in.d2l_momi(atomi);
    int st = lookupRadspline_magnetic(s, mi, fr_magnetic_i, dfr_magnetic_i, gr_magnetic_i, dgr_magnetic_i);
    if (st) return st;
    compute_ylm_cart(s, false, in.e2l_momi(1, atomi), in.e2l_momi(2, atomi), in.e2l_momi(3, atomi), l2m,
                     shvec_magnetic_i, dshvec_magnetic_i);
    for (int nr = 1; nr <= n2m; ++nr)
      for (int nsh = 1; nsh <= s.lmaxhalf_magnetic; ++nsh)
        abase2_magnetic(nr, nsh) = fr_magnetic_i(nr, sbm(nsh)) * shvec_magnetic_i(nsh);
    for (int nr = 1; nr <= n2m; ++nr)
      for (int l = 1; l <= l2m; ++l)
        for (int m = 1; m <= l; ++m)
          abase2_magnetic(nr, shm(l, -m)) = sgn(m) * std::conj(abase2_magnetic(nr, shm(l, m)));
    for (int nr = 1; nr <= nbm; ++nr) {
      ch.grpack_magnetic_0(nr, la) = gr_magnetic_i[nr];
      ch.gradgrpack_magnetic_0(nr, la) = dgr_magnetic_i[nr];
    }
    for (int l = 0; l <= l2m; ++l)
      for (int nr = 1; nr <= n2m; ++nr) {
        ch.frpack_magnetic_0(nr, l, la) = fr_magnetic_i(nr, l);
        ch.gradfrpack_magnetic_0(nr, l, la) = dfr_magnetic_i(nr, l);
      }
    for (int k = 1; k <= s.lmaxhalf_magnetic; ++k) {
      ch.shpack_magnetic_0(k, la) = shvec_magnetic_i(k);
      for (int c = 1; c <= 3; ++c) ch.gradshpack_magnetic_0(c, k, la) = dshvec_magnetic_i(c, k);
    }
    for (int l = 1; l <= l2m; ++l)
      for (int m = 1; m <= l; ++m) {
        int k = shm(l, -m), k1 = shm(l, m);
        ch.shpack_magnetic_0(k, la) = sgn(m) * std::conj(shvec_magnetic_i(k1));
        for (int c = 1; c <= 3; ++c)
          ch.gradshpack_magnetic_0(c, k, la) = sgn(m) * std::conj(dshvec_magnetic_i(c, k1));
      }

    for (int ij = ijstart; ij <= ijstop; ++ij) {
      const int lb = ch.lbase[la] + (ij - ijstart);
      double x = in.d2l(ij);
      double mag_mom = in.d2l_mom(ij);
      if (nba > 0) {
        st = lookupRadspline_atomic(s, x, fr_atomic, dfr_atomic, gr_atomic, dgr_atomic, cr, dcr);
        if (st) return st;
      }
      st = lookupRadspline_magnetic(s, mag_mom, fr_magnetic, dfr_magnetic, gr_magnetic, dgr_magnetic);
      if (st) return st;
      compute_ylm_cart(s, true, in.e2l(1, ij), in.e2l(2, ij), in.e2l(3, ij), l3a, shvec_atomic,
                       dshvec_atomic);
      compute_ylm_cart(s, false, in.e2l_mom(1, ij), in.e2l_mom(2, ij), in.e2l_mom(3, ij), l2m,
                       shvec_magnetic, dshvec_magnetic);
      // A2 (src/a_basis.F90:193-201)
      for (int nr = 1; nr <= n2m; ++nr)
        for (int l = 0; l <= l2m; ++l)
          for (int m = 0; m <= l; ++m) {
            int k = shm(l, m);
            for (int n = 1; n <= nba; ++n)
              abase2(n, nr, k) += (gr_atomic[n] * fr_magnetic(nr, sbm(k))) * shvec_magnetic(k);
          }
      abase2hc += cr;
      // per-bond caches (src/a_basis.F90:204-240)
      for (int n = 1; n <= nba; ++n) {
        ch.fr2pack_atomic(n, lb) = gr_atomic[n];
        ch.gradfr2pack_atomic(n, lb) = dgr_atomic[n];
      }
      ch.fr2hcpack(lb) = cr;
      ch.gradfr2hcpack(lb) = dcr;
      for (int l = 0; l <= l3a; ++l)
        for (int nr = 1; nr <= n3a; ++nr) {
          ch.frpack_atomic(nr, l, lb) = fr_atomic(nr, l);
          ch.gradfrpack_atomic(nr, l, lb) = dfr_atomic(nr, l);
        }
      for (int l = 0; l <= l2m; ++l)
        for (int nr = 1; nr <= n2m; ++nr) {
          ch.frpack_magnetic(nr, l, lb) = fr_magnetic(nr, l);
          ch.gradfrpack_magnetic(nr, l, lb) = dfr_magnetic(nr, l);
        }
      for (int k = 1; k <= s.lmaxhalf_atomic; ++k) {
        ch.shpack_atomic(k, lb) = shvec_atomic(k);
        for (int c = 1; c <= 3; ++c) ch.gradshpack_atomic(c, k, lb) = dshvec_atomic(c, k);
      }
      for (int k = 1; k <= s.lmaxhalf_magnetic; ++k) {
        ch.shpack_magnetic(k, lb) = shvec_magnetic(k);
        for (int c = 1; c <= 3; ++c) ch.gradshpack_magnetic(c, k, lb) = dshvec_magnetic(c, k);
      }
      for (int l = 1; l <= l2m; ++l)
        for (int m = 1; m <= l; ++m) {
          int k = shm(l, -m), k1 = shm(l, m);
          ch.shpack_magnetic(k, lb) = sgn(m) * std::conj(shvec_magnetic(k1));
          for (int c = 1; c <= 3; ++c)
            ch.gradshpack_magnetic(c, k, lb) = sgn(m) * std::conj(dshvec_magnetic(c, k1));
        }
      for (int l = 1; l <= l3a; ++l)
        for (int m = 1; m <= l; ++m) {
          int k = sha(l, -m), k1 = sha(l, m);
          ch.shpack_atomic(k, lb) = sgn(m) * std::conj(shvec_atomic(k1));
          for (int c = 1; c <= 3; ++c)
            ch.gradshpack_atomic(c, k, lb) = sgn(m) * std::conj(dshvec_atomic(c, k1));
        }
      // A (src/a_basis.F90:248-291)
      for (int nr1 = 1; nr1 <= n3a; ++nr1)
        for (int nr2 = 1; nr2 <= n3m; ++nr2)
          for (int l1 = 0; l1 <= l3a; ++l1)
            for (int l2 = 0; l2 <= l3m; ++l2)
              for (int m2 = -l2; m2 <= l2; ++m2) {
                int k1 = sha(l1, 0), k2 = shm(l2, m2);
                cplx x1 = (fr_atomic(nr1, sba(k1)) * fr_magnetic(nr2, sbm(k2))) * shvec_magnetic(k2);
                cplx y1 = shvec_atomic(k1);
                abase(nr1, k1, nr2, k2) += x1 * y1;
              }
      for (int nr1 = 1; nr1 <= n3a; ++nr1)
        for (int nr2 = 1; nr2 <= n3m; ++nr2)
          for (int l1 = 1; l1 <= l3a; ++l1)
            for (int l2 = 0; l2 <= l3m; ++l2)
              for (int m1 = 1; m1 <= l1; ++m1)
                for (int m2 = 0; m2 <= l2; ++m2) {
                  int k1 = sha(l1, m1), k2 = shm(l2, m2), k3 = sha(l1, -m1);
                  double xs = sgn(m1);
                  cplx x1 = (fr_atomic(nr1, sba(k1)) * fr_magnetic(nr2, sbm(k2))) * shvec_magnetic(k2);
                  cplx y1 = shvec_atomic(k1);
                  abase(nr1, k1, nr2, k2) += x1 * y1;
                  abase(nr1, k3, nr2, k2) += (x1 * std::conj(y1)) * xs;
                }
    }
    // missing halves (src/a_basis.F90:303-344)
    for (int nr1 = 1; nr1 <= n3a; ++nr1)
      for (int nr2 = 1; nr2 <= n3m; ++nr2)
        for (int l1 = 1; l1 <= l3a; ++l1)
          for (int l2 = 1; l2 <= l3m; ++l2)
            for (int m1 = 1; m1 <= l1; ++m1)
              for (int m2 = -l2; m2 <= -1; ++m2) {
                int k1 = sha(l1, m1), k2 = sha(l1, -m1), k3 = shm(l2, m2), k4 = shm(l2, -m2);
                double xs = sgn(m1 + m2);
                abase(nr1, k1, nr2, k3) = xs * std::conj(abase(nr1, k2, nr2, k4));
                abase(nr1, k2, nr2, k3) = xs * std::conj(abase(nr1, k1, nr2, k4));
              }
    for (int nr = 1; nr <= n2m; ++nr)
      for (int l = 1; l <= l2m; ++l)
        for (int m = 1; m <= l; ++m) {
          int k = shm(l, -m), k1 = shm(l, m);
          for (int n = 1; n <= nba; ++n) abase2(n, nr, k) = sgn(m) * std::conj(abase2(n, nr, k1));
        }
    // copy to the packs
    for (int k2 = 1; k2 <= lsm; ++k2)
      for (int nr2 = 1; nr2 <= n3m; ++nr2)
        for (int k1 = 1; k1 <= lsa; ++k1)
          for (int nr1 = 1; nr1 <= n3a; ++nr1) ch.abasepack(nr1, k1, nr2, k2, la) = abase(nr1, k1, nr2, k2);
    for (int k = 1; k <= lsm; ++k)
      for (int nr = 1; nr <= n2m; ++nr) {
        for (int n = 1; n <= nba; ++n) ch.abase2pack(n, nr, k, la) = abase2(n, nr, k);
        ch.abase2pack_magnetic(nr, k, la) = abase2_magnetic(nr, k);
      }
    ch.abase2hcpack(la) = abase2hc;
  }
  return ORACLE_OK;
}

// src/b_basis.F90:6-307 for the chunk's atoms (ranks 1-4)
void prepB(const OracleState& s, Chunk& ch) {
  const auto& sha = s.shindex_atomic;
  const auto& shm = s.shindex_magnetic;
  const int l2m = s.l2max_magnetic, l3a = s.l3max_atomic, l3m = s.l3max_magnetic;
  const int l4a = s.l4max_atomic, l4m = s.l4max_magnetic;
  for (int la = 1; la <= ch.na; ++la)
    for (int nclu = 1; nclu <= s.nvar1; ++nclu) {
      int nr = s.b1index(nclu);
      ch.b1pack(nclu, la) = ch.grpack_magnetic_0(nr, la) - 1.0;
    }
  if (s.nradial2_magnetic == 0) return;

  // 2-body
  FArr<cplx> db2({{-l2m, l2m}, {1, std::max(1, s.nvar2)}}), db2_0({{-l2m, l2m}, {1, std::max(1, s.nvar2)}});
  for (int la = 1; la <= ch.na; ++la) {
    db2.fill(cplx(0, 0));
    db2_0.fill(cplx(0, 0));
    for (int nclu = 1; nclu <= s.nvar2; ++nclu) {
      int nr1 = s.b2index(1, nclu), nr2 = s.b2index(2, nclu), nr3 = s.b2index(3, nclu);
      int l = s.b2index(4, nclu), k = s.b2map(nclu);
      cplx xiy(0, 0);
      for (int m = 1; m <= s.madd2(k); ++m) {
        int m1 = s.b2lm(k, m), m2 = -m1;
        int k1 = shm(l, m1), k2 = shm(l, m2);
        cplx ap0 = ch.abase2pack_magnetic(nr1, k1, la);
        cplx ap1 = ch.abase2pack(nr3, nr2, k2, la);
        double cf = s.cg01_magnetic(k, m1);
        xiy += (cf * ap0) * ap1;
        db2(m2, nclu) += cf * ap0;
        db2_0(m1, nclu) += cf * ap1;
      }
      ch.b2pack(nclu, la) = xiy.real();
    }
    for (int nclu = 1; nclu <= s.nvar2; ++nclu)
      for (int m = -l2m; m <= l2m; ++m) {
        ch.db2pack(m, nclu, la) = db2(m, nclu);
        ch.db2pack_0(m, nclu, la) = db2_0(m, nclu);
      }
    ch.b2hcpack(la) = ch.abase2hcpack(la);
  }

  // 3-body (src/b_basis.F90:142-212)
  if (s.nradial3_atomic == 0 && s.nradial3_magnetic == 0) return;
  for (int la = 1; la <= ch.na; ++la) {
    for (int nclu = 1; nclu <= s.nvar3; ++nclu) {
      for (int m4 = -l3m; m4 <= l3m; ++m4)
        for (int m1 = -l3a; m1 <= l3a; ++m1) {
          ch.db3pack(1, m1, m4, nclu, la) = cplx(0, 0);
          ch.db3pack(2, m1, m4, nclu, la) = cplx(0, 0);
        }
      for (int m = -l3m; m <= l3m; ++m) ch.db3pack_0(m, nclu, la) = cplx(0, 0);
    }
    for (int nclu = 1; nclu <= s.nvar3; ++nclu) {
      int nr1 = s.b3index(1, nclu), nr2 = s.b3index(2, nclu), nr3 = s.b3index(3, nclu);
      int nr4 = s.b3index(4, nclu), nr5 = s.b3index(5, nclu);
      int l1 = s.b3index(6, nclu), l2 = s.b3index(7, nclu), l3 = s.b3index(8, nclu), l4 = s.b3index(9, nclu);
      int ka = s.b3map_atomic(nclu), km = s.b3map_magnetic(nclu);
      cplx xiy(0, 0);
      for (int ma = 1; ma <= s.madd3_atomic(ka); ++ma) {
        int m1 = s.b3lm_atomic(ka, ma), m2 = -m1;
        int k1 = sha(l1, m1), k2 = sha(l1, m2);
        double cf_atomic = s.cg02_atomic(ka, m1);
        for (int mm = 1; mm <= s.madd3_magnetic(km); ++mm) {
          int m3 = s.b3lm_magnetic(km, mm, 1), m4 = s.b3lm_magnetic(km, mm, 2), m5 = s.b3lm_magnetic(km, mm, 3);
          int k3 = shm(l2, m3), k4 = shm(l3, m4), k5 = shm(l4, m5);
          cplx ap0 = ch.abase2pack_magnetic(nr3, k3, la);
          cplx ap1 = ch.abasepack(nr1, k1, nr4, k4, la);
          cplx ap2 = ch.abasepack(nr2, k2, nr5, k5, la);
          double cf = cf_atomic * s.cg02_magnetic(km, m3, m4, m5);
          xiy += ((cf * ap0) * ap1) * ap2;
          ch.db3pack(1, m1, m4, nclu, la) += (cf * ap0) * ap2;
          ch.db3pack(2, m2, m5, nclu, la) += (cf * ap0) * ap1;
          ch.db3pack_0(m3, nclu, la) += (cf * ap1) * ap2;
        }
      }
      ch.b3pack(nclu, la) = xiy.real();
    }
  }

  // 4-body (src/b_basis.F90:217-307)
  if (s.nradial4_atomic == 0 && s.nradial4_magnetic == 0) return;
  for (int la = 1; la <= ch.na; ++la) {
    for (int nclu = 1; nclu <= s.nvar4; ++nclu) {
      for (int q = 1; q <= 3; ++q)
        for (int mm = -l4m; mm <= l4m; ++mm)
          for (int ma = -l4a; ma <= l4a; ++ma) ch.db4pack(q, ma, mm, nclu, la) = cplx(0, 0);
      for (int m = -l4m; m <= l4m; ++m) ch.db4pack_0(m, nclu, la) = cplx(0, 0);
    }
    for (int nclu = 1; nclu <= s.nvar4; ++nclu) {
      int nr1 = s.b4index(1, nclu), nr2 = s.b4index(2, nclu), nr3 = s.b4index(3, nclu);
      int nr4 = s.b4index(4, nclu), nr5 = s.b4index(5, nclu), nr6 = s.b4index(6, nclu), nr7 = s.b4index(7, nclu);
      int l1 = s.b4index(8, nclu), l2 = s.b4index(9, nclu), l3 = s.b4index(10, nclu);
      int l4 = s.b4index(11, nclu), l5 = s.b4index(12, nclu), l6 = s.b4index(13, nclu), l7 = s.b4index(14, nclu);
      int ka = s.b4map_atomic(nclu), km = s.b4map_magnetic(nclu);
      cplx xiy(0, 0);
      for (int ma = 1; ma <= s.madd4_atomic(ka); ++ma) {
        int m1 = s.b4lm_atomic(ka, ma, 1), m2 = s.b4lm_atomic(ka, ma, 2), m3 = s.b4lm_atomic(ka, ma, 3);
        int k1 = sha(l1, m1), k2 = sha(l2, m2), k3 = sha(l3, m3);
        double cf_atomic = s.cg03_atomic(ka, m1, m2, m3);
        for (int mm = 1; mm <= s.madd4_magnetic(km); ++mm) {
          int m4 = s.b4lm_magnetic(km, mm, 1), m5 = s.b4lm_magnetic(km, mm, 2);
          int m6 = s.b4lm_magnetic(km, mm, 3), m7 = s.b4lm_magnetic(km, mm, 4);
          int k4 = shm(l4, m4), k5 = shm(l5, m5), k6 = shm(l6, m6), k7 = shm(l7, m7);
          cplx ap0 = ch.abase2pack_magnetic(nr4, k4, la);
          cplx ap1 = ch.abasepack(nr1, k1, nr5, k5, la);
          cplx ap2 = ch.abasepack(nr2, k2, nr6, k6, la);
          cplx ap3 = ch.abasepack(nr3, k3, nr7, k7, la);
          double cf = cf_atomic * s.cg03_magnetic(km, m4, m5, m6, m7);
          cplx xb3 = (ap0 * ap2) * ap3;
          cplx xb4 = cf * ap1;
          xiy += xb4 * xb3;
          ch.db4pack(1, m1, m5, nclu, la) += cf * xb3;
          ch.db4pack(2, m2, m6, nclu, la) += (ap0 * xb4) * ap3;
          ch.db4pack(3, m3, m7, nclu, la) += (ap0 * xb4) * ap2;
          ch.db4pack_0(m4, nclu, la) += (xb4 * ap2) * ap3;
        }
      }
      ch.b4pack(nclu, la) = xiy.real();
    }
  }

  // 5-body (src/b_basis.F90:310-409). A cluster whose atomic or magnetic half
  // the enumeration padded with zeros has no m-terms here: the reference
  // reads its factors at radial index 0, outside abasepack.
  if (s.nradial5_atomic == 0 && s.nradial5_magnetic == 0) return;
  {
    const int l5a = s.l5max_atomic, l5m = s.l5max_magnetic;
    for (int la = 1; la <= ch.na; ++la) {
      for (int nclu = 1; nclu <= s.nvar5; ++nclu) {
        for (int q = 1; q <= 4; ++q)
          for (int mm = -l5m; mm <= l5m; ++mm)
            for (int ma = -l5a; ma <= l5a; ++ma) ch.db5pack(q, ma, mm, nclu, la) = cplx(0, 0);
        for (int m = -l5m; m <= l5m; ++m) ch.db5pack_0(m, nclu, la) = cplx(0, 0);
      }
      for (int nclu = 1; nclu <= s.nvar5; ++nclu) {
        int nr[10], l[10];
        for (int q = 0; q < 9; ++q) {
          nr[q] = s.b5index(q + 1, nclu);
          l[q] = s.b5index(q + 10, nclu);
        }
        // nr/l: [0..3] n1..n4 / l1..l4, [4] n0' / l0', [5..8] n1'..n4' / l1'..l4'
        cplx xiy(0, 0);
        for (const auto& ta : s.b5mt_atomic[nclu - 1]) {
          const int m1 = ta.m[0], m2 = ta.m[1], m3 = ta.m[2], m4 = ta.m[3];
          const int k1 = sha(l[0], m1), k2 = sha(l[1], m2), k3 = sha(l[2], m3), k4 = sha(l[3], m4);
          for (const auto& tm : s.b5mt_magnetic[nclu - 1]) {
            const int m5 = tm.m[0], m6 = tm.m[1], m7 = tm.m[2], m8 = tm.m[3], m9 = tm.m[4];
            const cplx ap0 = ch.abase2pack_magnetic(nr[4], shm(l[4], m5), la);
            const cplx ap1 = ch.abasepack(nr[0], k1, nr[5], shm(l[5], m6), la);
            const cplx ap2 = ch.abasepack(nr[1], k2, nr[6], shm(l[6], m7), la);
            const cplx ap3 = ch.abasepack(nr[2], k3, nr[7], shm(l[7], m8), la);
            const cplx ap4 = ch.abasepack(nr[3], k4, nr[8], shm(l[8], m9), la);
            const double cf = ta.cf * tm.cf;
            const cplx xb1 = ap0 * cf * ap1 * ap2;
            const cplx xb2 = ap3 * ap4;
            xiy += xb1 * xb2;
            ch.db5pack(1, m1, m6, nclu, la) += ap0 * cf * ap2 * xb2;
            ch.db5pack(2, m2, m7, nclu, la) += ap0 * cf * ap1 * xb2;
            ch.db5pack(3, m3, m8, nclu, la) += xb1 * ap4;
            ch.db5pack(4, m4, m9, nclu, la) += xb1 * ap3;
            ch.db5pack_0(m5, nclu, la) += cf * ap1 * ap2 * xb2;
          }
        }
        ch.b5pack(nclu, la) = xiy.real();
      }
    }
  }

  // 6-body (src/b_basis.F90:412-532)
  if (s.nradial6_atomic == 0 && s.nradial6_magnetic == 0) return;
  {
    const int l6a = s.l6max_atomic, l6m = s.l6max_magnetic;
    for (int la = 1; la <= ch.na; ++la) {
      for (int nclu = 1; nclu <= s.nvar6; ++nclu) {
        for (int q = 1; q <= 5; ++q)
          for (int mm = -l6m; mm <= l6m; ++mm)
            for (int ma = -l6a; ma <= l6a; ++ma) ch.db6pack(q, ma, mm, nclu, la) = cplx(0, 0);
        for (int m = -l6m; m <= l6m; ++m) ch.db6pack_0(m, nclu, la) = cplx(0, 0);
      }
      for (int nclu = 1; nclu <= s.nvar6; ++nclu) {
        int nr[11], l[11];
        for (int q = 0; q < 11; ++q) {
          nr[q] = s.b6index(q + 1, nclu);
          l[q] = s.b6index(q + 12, nclu);
        }
        // nr/l: [0..4] n1..n5 / l1..l5, [5] n0' / l0', [6..10] n1'..n5' / l1'..l5'
        cplx xiy(0, 0);
        for (const auto& ta : s.b6mt_atomic[nclu - 1]) {
          const int m1 = ta.m[0], m2 = ta.m[1], m3 = ta.m[2], m4 = ta.m[3], m5 = ta.m[4];
          const int k1 = sha(l[0], m1), k2 = sha(l[1], m2), k3 = sha(l[2], m3), k4 = sha(l[3], m4),
                    k5 = sha(l[4], m5);
          for (const auto& tm : s.b6mt_magnetic[nclu - 1]) {
            const int m6 = tm.m[0], m7 = tm.m[1], m8 = tm.m[2], m9 = tm.m[3], m10 = tm.m[4], m11 = tm.m[5];
            const cplx ap0 = ch.abase2pack_magnetic(nr[5], shm(l[5], m6), la);
            const cplx ap1 = ch.abasepack(nr[0], k1, nr[6], shm(l[6], m7), la);
            const cplx ap2 = ch.abasepack(nr[1], k2, nr[7], shm(l[7], m8), la);
            const cplx ap3 = ch.abasepack(nr[2], k3, nr[8], shm(l[8], m9), la);
            const cplx ap4 = ch.abasepack(nr[3], k4, nr[9], shm(l[9], m10), la);
            const cplx ap5 = ch.abasepack(nr[4], k5, nr[10], shm(l[10], m11), la);
            const double cf = ta.cf * tm.cf;
            const cplx xb1 = ap0 * cf * ap1 * ap2;
            const cplx xb2 = ap3 * ap4 * ap5;
            xiy += xb1 * xb2;
            ch.db6pack(1, m1, m7, nclu, la) += ap0 * cf * ap2 * xb2;
            ch.db6pack(2, m2, m8, nclu, la) += ap0 * cf * ap1 * xb2;
            ch.db6pack(3, m3, m9, nclu, la) += xb1 * ap4 * ap5;
            ch.db6pack(4, m4, m10, nclu, la) += xb1 * ap3 * ap5;
            ch.db6pack(5, m5, m11, nclu, la) += xb1 * ap3 * ap4;
            ch.db6pack_0(m6, nclu, la) += cf * ap1 * ap2 * xb2;
          }
        }
        ch.b6pack(nclu, la) = xiy.real();
      }
    }
  }
}

// src/forces.F90:5-362 with calcenergyatom (:1093-1130) and expansionvariables (:976-1048)
void forceweights(const OracleState& s, Chunk& ch) {
  const int nd = s.ndensity;
  const int l2m = s.l2max_magnetic, l3a = s.l3max_atomic, l3m = s.l3max_magnetic;
  const int l4a = s.l4max_atomic, l4m = s.l4max_magnetic;
  (void)l4a;
  (void)l4m;
  for (int la = 1; la <= ch.na; ++la) {
    // expansionvariables
    double rho[2] = {0, 0};
    for (int d = 1; d <= nd; ++d) {
      double x = 0;
      for (int n = 1; n <= s.nvar1; ++n) x += s.c0(n, d) * ch.b1pack(n, la);
      rho[d - 1] = x;
    }
    if (s.nradial2_magnetic > 0)
      for (int d = 1; d <= nd; ++d) {
        double x = 0;
        for (int n = 1; n <= s.nvar2; ++n) x += s.c2(n, d) * ch.b2pack(n, la);
        rho[d - 1] += x;
      }
    if (s.nradial3_atomic > 0 || s.nradial3_magnetic > 0)
      for (int d = 1; d <= nd; ++d) {
        double x = 0;
        for (int n = 1; n <= s.nvar3; ++n) x += s.c3(n, d) * ch.b3pack(n, la);
        rho[d - 1] += x;
      }
    if (s.nradial4_atomic > 0 || s.nradial4_magnetic > 0)
      for (int d = 1; d <= nd; ++d) {
        double x = 0;
        for (int n = 1; n <= s.nvar4; ++n) x += s.c4(n, d) * ch.b4pack(n, la);
        rho[d - 1] += x;
      }
    // src/forces.F90:1030-1046
    if (s.nradial5_atomic > 0 || s.nradial5_magnetic > 0)
      for (int d = 1; d <= nd; ++d) {
        double x = 0;
        for (int n = 1; n <= s.nvar5; ++n) x += s.c5(n, d) * ch.b5pack(n, la);
        rho[d - 1] += x;
      }
    if (s.nradial6_atomic > 0 || s.nradial6_magnetic > 0)
      for (int d = 1; d <= nd; ++d) {
        double x = 0;
        for (int n = 1; n <= s.nvar6; ++n) x += s.c6(n, d) * ch.b6pack(n, la);
        rho[d - 1] += x;
      }
    // embedding
    double energyi = 0, dEdrho[2] = {0, 0};
    for (int d = 1; d <= nd; ++d) {
      double F, dF;
      Fexp(rho[d - 1], s.p1(1, d), s.p1(2, d), s.nfemb, F, dF);
      energyi = (d == 1) ? F : energyi + F;
      dEdrho[d - 1] = dF;
    }
    double edfi = 0.0;
    if (s.nradial2_magnetic > 0) {
      double e = ch.b2hcpack(la), fcut, dfcut;
      innercutoff(e, s.ecut, s.decut, fcut, dfcut);
      edfi = dfcut * energyi + 1.0;
      for (int d = 0; d < nd; ++d) dEdrho[d] = fcut * dEdrho[d];
      energyi = fcut * energyi + e;
    }
    ch.edfcut[la] = edfi;
    ch.eicalc[la] = energyi;
    for (int d = 0; d < nd; ++d) {
      ch.rho_out[2 * la + d] = rho[d];
      ch.dEdrho_out[2 * la + d] = dEdrho[d];
    }
    auto ceff = [&](const FArr<double>& c, int n) {
      double x = 0;
      for (int d = 1; d <= nd; ++d) x += dEdrho[d - 1] * c(n, d);
      return x;
    };
    // 1-body
    for (int nr = 1; nr <= s.nradbase_magnetic; ++nr) ch.wf1(nr, la) = 0.0;
    for (int n = 1; n <= s.nvar1; ++n) ch.wf1(s.b1index(n), la) += ceff(s.c0, n);
    for (int nr = 1; nr <= s.nradial2_magnetic; ++nr)
      for (int l = 0; l <= l2m; ++l)
        for (int m = 0; m <= l2m; ++m) {
          ch.wf_0(m, l, nr, la) = cplx(0, 0);
          for (int n = 1; n <= s.nradbase_atomic; ++n) ch.wf2(n, m, l, nr, la) = cplx(0, 0);
        }
    for (int nr2 = 1; nr2 <= std::max(1, s.nradial3_magnetic); ++nr2)
      for (int l2 = 0; l2 <= l3m; ++l2)
        for (int m2 = 0; m2 <= l3m; ++m2)
          for (int nr1 = 1; nr1 <= std::max(1, s.nradial3_atomic); ++nr1)
            for (int l1 = 0; l1 <= l3a; ++l1)
              for (int m1 = -l3a; m1 <= l3a; ++m1) ch.wf(m1, l1, nr1, m2, l2, nr2, la) = cplx(0, 0);
    // 2-body
    for (int n = 1; n <= s.nvar2; ++n) {
      int nr1 = s.b2index(1, n), nr2 = s.b2index(2, n), nr3 = s.b2index(3, n), l = s.b2index(4, n);
      double c = ceff(s.c2, n);
      for (int m = 0; m <= l; ++m) ch.wf2(nr3, m, l, nr2, la) += c * ch.db2pack(m, n, la);
      for (int m = 0; m <= l; ++m) ch.wf_0(m, l, nr1, la) += c * ch.db2pack_0(m, n, la);
    }
    // 3-body
    for (int n = 1; n <= s.nvar3; ++n) {
      int nr1 = s.b3index(1, n), nr2 = s.b3index(2, n), nr3 = s.b3index(3, n), nr4 = s.b3index(4, n),
          nr5 = s.b3index(5, n);
      int l1 = s.b3index(6, n), l2 = s.b3index(7, n), l4 = s.b3index(8, n), l5 = s.b3index(9, n);
      double c = ceff(s.c3, n);
      for (int m1 = -l1; m1 <= l1; ++m1)
        for (int m4 = 0; m4 <= l4; ++m4) ch.wf(m1, l1, nr1, m4, l4, nr4, la) += c * ch.db3pack(1, m1, m4, n, la);
      for (int m1 = -l1; m1 <= l1; ++m1)
        for (int m5 = 0; m5 <= l5; ++m5) ch.wf(m1, l1, nr2, m5, l5, nr5, la) += c * ch.db3pack(2, m1, m5, n, la);
      for (int m2 = 0; m2 <= l2; ++m2) ch.wf_0(m2, l2, nr3, la) += c * ch.db3pack_0(m2, n, la);
    }
    // 4-body
    for (int n = 1; n <= s.nvar4; ++n) {
      int nr1 = s.b4index(1, n), nr2 = s.b4index(2, n), nr3 = s.b4index(3, n), nr4 = s.b4index(4, n);
      int nr5 = s.b4index(5, n), nr6 = s.b4index(6, n), nr7 = s.b4index(7, n);
      int l1 = s.b4index(8, n), l2 = s.b4index(9, n), l3 = s.b4index(10, n), l4 = s.b4index(11, n);
      int l5 = s.b4index(12, n), l6 = s.b4index(13, n), l7 = s.b4index(14, n);
      double c = ceff(s.c4, n);
      for (int m1 = -l1; m1 <= l1; ++m1)
        for (int m5 = 0; m5 <= l5; ++m5) ch.wf(m1, l1, nr1, m5, l5, nr5, la) += c * ch.db4pack(1, m1, m5, n, la);
      for (int m2 = -l2; m2 <= l2; ++m2)
        for (int m6 = 0; m6 <= l6; ++m6) ch.wf(m2, l2, nr2, m6, l6, nr6, la) += c * ch.db4pack(2, m2, m6, n, la);
      for (int m3 = -l3; m3 <= l3; ++m3)
        for (int m7 = 0; m7 <= l7; ++m7) ch.wf(m3, l3, nr3, m7, l7, nr7, la) += c * ch.db4pack(3, m3, m7, n, la);
      for (int m4 = 0; m4 <= l4; ++m4) ch.wf_0(m4, l4, nr4, la) += c * ch.db4pack_0(m4, n, la);
    }
    // 5-body (src/forces.F90:234-277); padded clusters have no gradient
    for (int n = 1; n <= s.nvar5; ++n) {
      if (s.b5mt_atomic[n - 1].empty() || s.b5mt_magnetic[n - 1].empty()) continue;
      const double c = ceff(s.c5, n);
      for (int q = 1; q <= 4; ++q) {
        const int nr = s.b5index(q, n), nrp = s.b5index(5 + q, n), l = s.b5index(9 + q, n), lp = s.b5index(14 + q, n);
        for (int m = -l; m <= l; ++m)
          for (int mp = 0; mp <= lp; ++mp) ch.wf(m, l, nr, mp, lp, nrp, la) += c * ch.db5pack(q, m, mp, n, la);
      }
      const int nr0 = s.b5index(5, n), l0 = s.b5index(14, n);
      for (int m = 0; m <= l0; ++m) ch.wf_0(m, l0, nr0, la) += c * ch.db5pack_0(m, n, la);
    }
    // 6-body (src/forces.F90:280-331)
    for (int n = 1; n <= s.nvar6; ++n) {
      if (s.b6mt_atomic[n - 1].empty() || s.b6mt_magnetic[n - 1].empty()) continue;
      const double c = ceff(s.c6, n);
      for (int q = 1; q <= 5; ++q) {
        const int nr = s.b6index(q, n), nrp = s.b6index(6 + q, n), l = s.b6index(11 + q, n),
                  lp = s.b6index(17 + q, n);
        for (int m = -l; m <= l; ++m)
          for (int mp = 0; mp <= lp; ++mp) ch.wf(m, l, nr, mp, lp, nrp, la) += c * ch.db6pack(q, m, mp, n, la);
      }
      const int nr0 = s.b6index(6, n), l0 = s.b6index(17, n);
      for (int m = 0; m <= l0; ++m) ch.wf_0(m, l0, nr0, la) += c * ch.db6pack_0(m, n, la);
    }
  }
}

inline void acc(double* F, double rew, double imw, const cplx* v, double scale) {
  for (int c = 0; c < 3; ++c) F[c] = F[c] + scale * (rew * v[c].real() - imw * v[c].imag());
}
inline void acc1(double* F, double rew, double imw, const cplx* v) {
  for (int c = 0; c < 3; ++c) F[c] = F[c] + rew * v[c].real() - imw * v[c].imag();
}

// src/forces.F90:366-634 and :638-972 for the chunk's atoms
void forces_and_torques(const OracleState& s, const Inputs& in, Chunk& ch, double* flist, double* tlist,
                        double* tlist0, const std::vector<long>& outoff) {
  const auto& sha = s.shindex_atomic;
  const auto& shm = s.shindex_magnetic;
  const int nba = s.nradbase_atomic, nbm = s.nradbase_magnetic;
  const int n3a = s.nradial3_atomic, n3m = s.nradial3_magnetic, n2m = s.nradial2_magnetic;
  const int l3a = s.l3max_atomic, l3m = s.l3max_magnetic, l2m = s.l2max_magnetic;
  for (int la = 1; la <= ch.na; ++la) {
    const int atomk = ch.atom[la];
    const int ijstart = in.nstart[atomk - 1], ijstop = in.nstop[atomk - 1];
    const double edf = ch.edfcut[la];
    long k3 = outoff[atomk - 1];
    // forcecompute
    for (int ij = ijstart; ij <= ijstop; ++ij, k3 += 3) {
      const int lb = ch.lbase[la] + (ij - ijstart);
      double Fk[3] = {0, 0, 0};
      double ebond[3] = {in.e2l(1, ij), in.e2l(2, ij), in.e2l(3, ij)};
      double x = in.d2l(ij);
      double invr = 1.0 / x;
      cplx xiyvec[3];
      for (int nr1 = 1; nr1 <= nba; ++nr1)
        for (int nr2 = 1; nr2 <= n2m; ++nr2)
          for (int l = 0; l <= l2m; ++l) {
            double v2[3];
            for (int c = 0; c < 3; ++c) v2[c] = ch.gradfr2pack_atomic(nr1, lb) * ebond[c];
            for (int m = 0; m <= l; ++m) {
              cplx wei = ch.wf2(nr1, m, l, nr2, la);
              int k = shm(l, m);
              cplx t = ch.frpack_magnetic(nr2, l, lb) * ch.shpack_magnetic(k, lb);
              for (int c = 0; c < 3; ++c) xiyvec[c] = t * v2[c];
              if (m == 0) acc1(Fk, wei.real(), wei.imag(), xiyvec);
              else acc(Fk, wei.real(), wei.imag(), xiyvec, 2.0);
            }
          }
      for (int c = 0; c < 3; ++c) Fk[c] = Fk[c] + edf * ch.gradfr2hcpack(lb) * ebond[c];
      for (int nr1 = 1; nr1 <= n3a; ++nr1)
        for (int nr2 = 1; nr2 <= n3m; ++nr2)
          for (int l1 = 0; l1 <= l3a; ++l1)
            for (int l2 = 0; l2 <= l3m; ++l2) {
              double x2 = invr * ch.frpack_atomic(nr1, l1, lb);
              double v2[3];
              for (int c = 0; c < 3; ++c) v2[c] = ch.gradfrpack_atomic(nr1, l1, lb) * ebond[c];
              auto term = [&](int m1, int m2, double scale) {
                cplx wei = ch.wf(m1, l1, nr1, m2, l2, nr2, la);
                int k = sha(l1, m1), k1 = shm(l2, m2);
                cplx pre = ch.shpack_magnetic(k1, lb) * ch.frpack_magnetic(nr2, l2, lb);
                for (int c = 0; c < 3; ++c)
                  xiyvec[c] = pre * (v2[c] * ch.shpack_atomic(k, lb) + x2 * ch.gradshpack_atomic(c + 1, k, lb));
                if (scale == 1.0) acc1(Fk, wei.real(), wei.imag(), xiyvec);
                else acc(Fk, wei.real(), wei.imag(), xiyvec, scale);
              };
              term(0, 0, 1.0);
              for (int m1 = 1; m1 <= l1; ++m1)
                for (int m2 = 1; m2 <= l2; ++m2) {
                  term(m1, m2, 2.0);
                  term(-m1, m2, 2.0);
                }
              for (int m1 = 1; m1 <= l1; ++m1) term(m1, 0, 2.0);
              for (int m2 = 1; m2 <= l2; ++m2) term(0, m2, 2.0);
            }
      for (int c = 0; c < 3; ++c) flist[k3 + c] = Fk[c];
    }

    // torquecompute
    double mom = in.d2l_momi(atomk);
    double emom[3] = {in.e2l_momi(1, atomk), in.e2l_momi(2, atomk), in.e2l_momi(3, atomk)};
    double invr_m = 1.0 / mom;
    double Tk0[3] = {0, 0, 0};
    for (int nr = 1; nr <= nbm; ++nr)
      for (int c = 0; c < 3; ++c) Tk0[c] = Tk0[c] + ch.wf1(nr, la) * ch.gradgrpack_magnetic_0(nr, la) * emom[c];
    cplx xiyvec[3];
    for (int nr = 1; nr <= n2m; ++nr)
      for (int l = 0; l <= l2m; ++l) {
        double v2[3];
        for (int c = 0; c < 3; ++c) v2[c] = ch.gradfrpack_magnetic_0(nr, l, la) * emom[c];
        double x2 = invr_m * ch.frpack_magnetic_0(nr, l, la);
        for (int m = 0; m <= l; ++m) {
          cplx wei = ch.wf_0(m, l, nr, la);
          int k = shm(l, m);
          for (int c = 0; c < 3; ++c)
            xiyvec[c] = ch.shpack_magnetic_0(k, la) * v2[c] + ch.gradshpack_magnetic_0(c + 1, k, la) * x2;
          if (m == 0) acc1(Tk0, wei.real(), wei.imag(), xiyvec);
          else acc(Tk0, wei.real(), wei.imag(), xiyvec, 2.0);
        }
      }
    k3 = outoff[atomk - 1];
    for (int ij = ijstart; ij <= ijstop; ++ij, k3 += 3) {
      const int lb = ch.lbase[la] + (ij - ijstart);
      double Tk[3] = {0, 0, 0};
      double em[3] = {in.e2l_mom(1, ij), in.e2l_mom(2, ij), in.e2l_mom(3, ij)};
      double mm = in.d2l_mom(ij);
      double invm = 1.0 / mm;
      for (int nr1 = 1; nr1 <= nba; ++nr1)
        for (int nr2 = 1; nr2 <= n2m; ++nr2)
          for (int l = 0; l <= l2m; ++l) {
            double x2 = invm * ch.frpack_magnetic(nr2, l, lb);
            double v2[3];
            for (int c = 0; c < 3; ++c) v2[c] = ch.gradfrpack_magnetic(nr2, l, lb) * em[c];
            for (int m = 0; m <= l; ++m) {
              cplx wei = ch.wf2(nr1, m, l, nr2, la);
              int k1 = shm(l, m);
              for (int c = 0; c < 3; ++c)
                xiyvec[c] = ch.fr2pack_atomic(nr1, lb) *
                            (v2[c] * ch.shpack_magnetic(k1, lb) + x2 * ch.gradshpack_magnetic(c + 1, k1, lb));
              if (m == 0) acc1(Tk, wei.real(), wei.imag(), xiyvec);
              else acc(Tk, wei.real(), wei.imag(), xiyvec, 2.0);
            }
          }
      for (int nr1 = 1; nr1 <= n3a; ++nr1)
        for (int nr2 = 1; nr2 <= n3m; ++nr2)
          for (int l1 = 0; l1 <= l3a; ++l1)
            for (int l2 = 0; l2 <= l3m; ++l2) {
              double x2 = invm * ch.frpack_magnetic(nr2, l2, lb);
              double v2[3];
              for (int c = 0; c < 3; ++c) v2[c] = ch.gradfrpack_magnetic(nr2, l2, lb) * em[c];
              auto term = [&](int m1, int m2, double scale) {
                cplx wei = ch.wf(m1, l1, nr1, m2, l2, nr2, la);
                int k = sha(l1, m1), k1 = shm(l2, m2);
                cplx pre = ch.shpack_atomic(k, lb) * ch.frpack_atomic(nr1, l1, lb);
                for (int c = 0; c < 3; ++c)
                  xiyvec[c] =
                      pre * (v2[c] * ch.shpack_magnetic(k1, lb) + x2 * ch.gradshpack_magnetic(c + 1, k1, lb));
                if (scale == 1.0) acc1(Tk, wei.real(), wei.imag(), xiyvec);
                else acc(Tk, wei.real(), wei.imag(), xiyvec, scale);
              };
              term(0, 0, 1.0);
              for (int m1 = 1; m1 <= l1; ++m1)
                for (int m2 = 1; m2 <= l2; ++m2) {
                  term(m1, m2, 2.0);
                  term(-m1, m2, 2.0);
                }
              for (int m1 = 1; m1 <= l1; ++m1) term(m1, 0, 2.0);
              for (int m2 = 1; m2 <= l2; ++m2) term(0, m2, 2.0);
            }
      for (int c = 0; c < 3; ++c) tlist[k3 + c] = Tk[c];
    }
    for (int c = 0; c < 3; ++c) tlist0[3 * (atomk - 1) + c] = Tk0[c];
  }
}

struct Args {
  Inputs in;
  double *eout, *flist, *tlist, *tlist0;
  std::vector<long> outoff;
};

// processes global atoms [a0, a1] (1-based, inclusive) in chunks
int run_range(const OracleState& s, const Args& a, int a0, int a1, int chunk) {
  Chunk ch;
  for (int c0 = a0; c0 <= a1; c0 += chunk) {
    int c1 = std::min(a1, c0 + chunk - 1);
    int na = c1 - c0 + 1, nb = 0;
    for (int i = c0; i <= c1; ++i) nb += std::max(0, a.in.nstop[i - 1] - a.in.nstart[i - 1] + 1);
    ch.alloc(s, na, nb);
    ch.atom.assign(na + 1, 0);
    ch.lbase.assign(na + 1, 1);
    int run = 1;
    for (int la = 1; la <= na; ++la) {
      ch.atom[la] = c0 + la - 1;
      ch.lbase[la] = run;
      run += std::max(0, a.in.nstop[c0 + la - 2] - a.in.nstart[c0 + la - 2] + 1);
    }
    ch.na = na;
    int st = prepA(s, a.in, ch);
    if (st) return st;
    prepB(s, ch);
    forceweights(s, ch);
    forces_and_torques(s, a.in, ch, a.flist, a.tlist, a.tlist0, a.outoff);
    for (int la = 1; la <= na; ++la) a.eout[c0 + la - 2] = ch.eicalc[la];
  }
  return ORACLE_OK;
}

int validate(int natom, int nei, const int* occ, const int* occlist, const int* nstart, const int* nstop) {
  for (int i = 0; i < natom; ++i) {
    if (occ && occ[i] != 1) return ORACLE_ERR_ARGS;
    if (nstop[i] >= nstart[i] && (nstart[i] < 1 || nstop[i] > nei)) return ORACLE_ERR_ARGS;
  }
  if (occlist)
    for (int j = 0; j < nei; ++j)
      if (occlist[j] != 1) return ORACLE_ERR_ARGS;
  return ORACLE_OK;
}

}  // namespace

extern "C" {

const char* oracle_last_error() { return g_err.c_str(); }

// Init, as acelibini (src/ace.F90:10-75) but with an explicit file path.
int oracle_init(const char* path, const char* element, double rcut, double rcut_magnetic, double smear,
                int xcnumber) {
  g_err.clear();
  return oracle_setup(g_state, path, element, rcut, rcut_magnetic, smear, xcnumber, g_err);
}

// Sizes of the enumerated basis: out[0..3] = nvar1..nvar4, out[4] = number of
// 3-body m terms, out[5] = 4-body m terms, out[6] = 2-body m terms,
// out[7..8] = nvar5, nvar6.
int oracle_basis_sizes(int* out) {
  const OracleState& s = g_state;
  if (!s.initialized) return ORACLE_ERR_NOT_INIT;
  out[0] = s.nvar1;
  out[1] = s.nvar2;
  out[2] = s.nvar3;
  out[3] = s.nvar4;
  long t3 = 0, t4 = 0, t2 = 0;
  for (int n = 1; n <= s.nvar3; ++n)
    t3 += (long)s.madd3_atomic(s.b3map_atomic(n)) * s.madd3_magnetic(s.b3map_magnetic(n));
  for (int n = 1; n <= s.nvar4; ++n)
    t4 += (long)s.madd4_atomic(s.b4map_atomic(n)) * s.madd4_magnetic(s.b4map_magnetic(n));
  for (int n = 1; n <= s.nvar2; ++n) t2 += s.madd2(s.b2map(n));
  out[4] = (int)t3;
  out[5] = (int)t4;
  out[6] = (int)t2;
  out[7] = s.nvar5;
  out[8] = s.nvar6;
  return ORACLE_OK;
}

// Cluster index rows: rank 2 -> 4 ints per cluster (b2index), rank 3 -> 9
// (b3index), rank 4 -> 15 (b4index), rank 1 -> 1 (b1index).
int oracle_basis_rows(int rank, int* out) {
  const OracleState& s = g_state;
  if (!s.initialized) return ORACLE_ERR_NOT_INIT;
  if (rank == 1)
    for (int n = 1; n <= s.nvar1; ++n) out[n - 1] = s.b1index(n);
  else if (rank == 2)
    for (int n = 1; n <= s.nvar2; ++n)
      for (int q = 0; q < 4; ++q) out[4 * (n - 1) + q] = s.b2index(q + 1, n);
  else if (rank == 3)
    for (int n = 1; n <= s.nvar3; ++n)
      for (int q = 0; q < 9; ++q) out[9 * (n - 1) + q] = s.b3index(q + 1, n);
  else if (rank == 4)
    for (int n = 1; n <= s.nvar4; ++n)
      for (int q = 0; q < 15; ++q) out[15 * (n - 1) + q] = s.b4index(q + 1, n);
  else if (rank == 5)
    for (int n = 1; n <= s.nvar5; ++n)
      for (int q = 0; q < 21; ++q) out[21 * (n - 1) + q] = s.b5index(q + 1, n);
  else if (rank == 6)
    for (int n = 1; n <= s.nvar6; ++n)
      for (int q = 0; q < 27; ++q) out[27 * (n - 1) + q] = s.b6index(q + 1, n);
  else
    return ORACLE_ERR_ARGS;
  return ORACLE_OK;
}

// Same argument list and output layout as acelib (src/ace.F90:79-321), plus
// a thread count and the chunk size (atoms per pack allocation).
int oracle_acelib(int natom, int nall, int nei, const int* nlist, const int* occ, const int* occlist,
                  const int* nstart, const int* nstop, double* eout, const double* dlist, const double* elist,
                  double* flist, const double* dlist_momi, const double* elist_momi, const double* dlist_mom,
                  const double* elist_mom, double* tlist, double* tlist0, int nthreads, int chunk) {
  (void)nall;
  (void)nlist;
  if (!g_state.initialized) return ORACLE_ERR_NOT_INIT;
  int st = validate(natom, nei, occ, occlist, nstart, nstop);
  if (st) return st;
  Args a;
  a.in.natom = natom;
  a.in.nei = nei;
  a.in.nstart = nstart;
  a.in.nstop = nstop;
  a.in.dlist = dlist;
  a.in.elist = elist;
  a.in.dlist_momi = dlist_momi;
  a.in.elist_momi = elist_momi;
  a.in.dlist_mom = dlist_mom;
  a.in.elist_mom = elist_mom;
  a.eout = eout;
  a.flist = flist;
  a.tlist = tlist;
  a.tlist0 = tlist0;
  // output packing of src/ace.F90:291-318: atoms in order, each atom's bonds in order
  a.outoff.assign(natom + 1, 0);
  for (int i = 0; i < natom; ++i) a.outoff[i + 1] = a.outoff[i] + 3L * std::max(0, nstop[i] - nstart[i] + 1);
  if (chunk < 1) chunk = 64;
  if (nthreads < 1) nthreads = 1;
  nthreads = std::min(nthreads, std::max(1, natom));
  std::vector<int> status(nthreads, 0);
  std::vector<std::thread> pool;
  for (int t = 0; t < nthreads; ++t) {
    int a0 = 1 + (int)((long)natom * t / nthreads);
    int a1 = (int)((long)natom * (t + 1) / nthreads);
    if (a1 < a0) continue;
    if (nthreads == 1) status[t] = run_range(g_state, a, a0, a1, chunk);
    else pool.emplace_back([&, t, a0, a1] { status[t] = run_range(g_state, a, a0, a1, chunk); });
  }
  for (auto& th : pool) th.join();
  for (int t = 0; t < nthreads; ++t)
    if (status[t]) {
      g_err = status[t] == ORACLE_ERR_SMALL_R ? "very small distance" : "moment magnitude out of range";
      return status[t];
    }
  return ORACLE_OK;
}

// Intermediates for one atom (1-based `atom`), computed exactly as in
// oracle_acelib. Layouts (all column-major, Fortran order, complex = 2 doubles):
//   A   [nradial3_a][lmaxsq_a][nradial3_m][lmaxsq_m]   (abasepack)
//   A2  [nradbase_a][nradial2_m][lmaxsq_m]             (abase2pack)
//   A0  [nradial2_m][lmaxsq_m]                         (abase2pack_magnetic)
//   wf  [-l3a:l3a][0:l3a][nradial3_a][0:l3m][0:l3m][nradial3_m]
//   wf2 [nradbase_a][0:l2m][0:l2m][nradial2_m]
//   wf0 [0:l2m][0:l2m][nradial2_m]
//   wf1 [nradbase_m]
//   scal = {energy, rho1, rho2, dEdrho1, dEdrho2, core sum, edf}
int oracle_atom_state(int natom, int nei, const int* nstart, const int* nstop, const double* dlist,
                      const double* elist, const double* dlist_momi, const double* elist_momi,
                      const double* dlist_mom, const double* elist_mom, int atom, double* A, double* A2,
                      double* A0, double* wf, double* wf2, double* wf0, double* wf1, double* scal) {
  const OracleState& s = g_state;
  if (!s.initialized) return ORACLE_ERR_NOT_INIT;
  if (atom < 1 || atom > natom) return ORACLE_ERR_ARGS;
  Inputs in;
  in.natom = natom;
  in.nei = nei;
  in.nstart = nstart;
  in.nstop = nstop;
  in.dlist = dlist;
  in.elist = elist;
  in.dlist_momi = dlist_momi;
  in.elist_momi = elist_momi;
  in.dlist_mom = dlist_mom;
  in.elist_mom = elist_mom;
  Chunk ch;
  int nb = std::max(0, nstop[atom - 1] - nstart[atom - 1] + 1);
  ch.alloc(s, 1, nb);
  ch.atom.assign(2, atom);
  ch.lbase.assign(2, 1);
  ch.na = 1;
  int st = prepA(s, in, ch);
  if (st) return st;
  prepB(s, ch);
  forceweights(s, ch);
  auto copyc = [](FArr<cplx>& src, size_t count, double* dst) {
    const cplx* p = src.data();
    for (size_t i = 0; i < count; ++i) {
      dst[2 * i] = p[i].real();
      dst[2 * i + 1] = p[i].imag();
    }
  };
  size_t nA = (size_t)s.nradial3_atomic * s.lmaxsq_atomic * s.nradial3_magnetic * s.lmaxsq_magnetic;
  size_t nA2 = (size_t)s.nradbase_atomic * s.nradial2_magnetic * s.lmaxsq_magnetic;
  size_t nA0 = (size_t)s.nradial2_magnetic * s.lmaxsq_magnetic;
  size_t nwf = (size_t)(2 * s.l3max_atomic + 1) * (s.l3max_atomic + 1) * s.nradial3_atomic *
               (s.l3max_magnetic + 1) * (s.l3max_magnetic + 1) * s.nradial3_magnetic;
  size_t nwf2 = (size_t)s.nradbase_atomic * (s.l2max_magnetic + 1) * (s.l2max_magnetic + 1) * s.nradial2_magnetic;
  size_t nwf0 = (size_t)(s.l2max_magnetic + 1) * (s.l2max_magnetic + 1) * s.nradial2_magnetic;
  if (A) copyc(ch.abasepack, nA, A);
  if (A2) copyc(ch.abase2pack, nA2, A2);
  if (A0) copyc(ch.abase2pack_magnetic, nA0, A0);
  if (wf) copyc(ch.wf, nwf, wf);
  if (wf2) copyc(ch.wf2, nwf2, wf2);
  if (wf0) copyc(ch.wf_0, nwf0, wf0);
  if (wf1)
    for (int nr = 1; nr <= s.nradbase_magnetic; ++nr) wf1[nr - 1] = ch.wf1(nr, 1);
  if (scal) {
    scal[0] = ch.eicalc[1];
    scal[1] = ch.rho_out[2];
    scal[2] = ch.rho_out[3];
    scal[3] = ch.dEdrho_out[2];
    scal[4] = ch.dEdrho_out[3];
    scal[5] = ch.abase2hcpack(1);
    scal[6] = ch.edfcut[1];
  }
  return ORACLE_OK;
}

// Descriptors B[natom][nvar1 + ... + nvar6] (the prepB packs,
// src/b_basis.F90:6-536, in cluster order) and dE/drho [natom][2] (from the
// embedding step of forceweights, src/forces.F90:976-1289). Not part of the
// reference's interface: test support for the differentiation harness.
int oracle_descriptors(int natom, int nei, const int* nstart, const int* nstop, const double* dlist,
                       const double* elist, const double* dlist_momi, const double* elist_momi,
                       const double* dlist_mom, const double* elist_mom, double* B, double* dedrho) {
  const OracleState& s = g_state;
  if (!s.initialized) return ORACLE_ERR_NOT_INIT;
  int st = validate(natom, nei, nullptr, nullptr, nstart, nstop);
  if (st) return st;
  Inputs in;
  in.natom = natom;
  in.nei = nei;
  in.nstart = nstart;
  in.nstop = nstop;
  in.dlist = dlist;
  in.elist = elist;
  in.dlist_momi = dlist_momi;
  in.elist_momi = elist_momi;
  in.dlist_mom = dlist_mom;
  in.elist_mom = elist_mom;
  const int nB = s.nvar1 + s.nvar2 + s.nvar3 + s.nvar4 + s.nvar5 + s.nvar6;
  const int chunk = 32;
  Chunk ch;
  for (int c0 = 1; c0 <= natom; c0 += chunk) {
    const int c1 = std::min(natom, c0 + chunk - 1);
    const int na = c1 - c0 + 1;
    int nb = 0;
    for (int i = c0; i <= c1; ++i) nb += std::max(0, nstop[i - 1] - nstart[i - 1] + 1);
    ch.alloc(s, na, nb);
    ch.atom.assign(na + 1, 0);
    ch.lbase.assign(na + 1, 1);
    int run = 1;
    for (int la = 1; la <= na; ++la) {
      ch.atom[la] = c0 + la - 1;
      ch.lbase[la] = run;
      run += std::max(0, nstop[c0 + la - 2] - nstart[c0 + la - 2] + 1);
    }
    ch.na = na;
    st = prepA(s, in, ch);
    if (st) return st;
    prepB(s, ch);
    forceweights(s, ch);
    for (int la = 1; la <= na; ++la) {
      double* b = B + static_cast<size_t>(c0 + la - 2) * nB;
      int k = 0;
      for (int c = 1; c <= s.nvar1; ++c) b[k++] = ch.b1pack(c, la);
      for (int c = 1; c <= s.nvar2; ++c) b[k++] = ch.b2pack(c, la);
      for (int c = 1; c <= s.nvar3; ++c) b[k++] = ch.b3pack(c, la);
      for (int c = 1; c <= s.nvar4; ++c) b[k++] = ch.b4pack(c, la);
      for (int c = 1; c <= s.nvar5; ++c) b[k++] = ch.b5pack(c, la);
      for (int c = 1; c <= s.nvar6; ++c) b[k++] = ch.b6pack(c, la);
      if (dedrho) {
        dedrho[2 * (c0 + la - 2)] = ch.dEdrho_out[2 * la];
        dedrho[2 * (c0 + la - 2) + 1] = ch.dEdrho_out[2 * la + 1];
      }
    }
  }
  return ORACLE_OK;
}

}  // extern "C"
