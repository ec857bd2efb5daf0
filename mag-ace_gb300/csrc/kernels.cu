// Hot-path kernels for sm_103a.
//
//   k_abasis   one CTA per atom: per-bond radial lookups and spherical
//              harmonics, then the bond sums A, A2 (m' >= 0 half, completed by
//              conjugate symmetry), the on-site A0 and the 1-body density.
//              (reference: src/a_basis.F90:5-361, src/radial.F90:53-160,
//              src/spherical.F90:55-282)
//   k_density  one CTA per atom: density rho = sum kappa * prod(factors) and
//              the weights dE/dA as a deterministic gather over the folded
//              term tables, the embedding F(rho) and the inner cutoff.
//              (reference: src/b_basis.F90:6-307, src/forces.F90:5-362,
//              :976-1289)
//   k_forces   one CTA per atom, one thread per bond: recomputes the bond's
//              features with derivatives and contracts them with the weights
//              into dE_i/d(x_i - x_j) and dE_i/dm_j; thread 0 adds dE_i/dm_i.
//              (reference: src/forces.F90:366-972)
//
// The kernels are templated on the arithmetic type R of features, factors
// and weights (double: the drop-in FP64 path; float: the split path, whose
// per-atom density, energy and output sums stay in double).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <map>
#include <utility>

#include "device_model.hpp"
#include "kernels.hpp"

namespace magace {

__constant__ double c_alm[kMaxHalf];
__constant__ double c_blm[kMaxHalf];
__constant__ double c_cl[kMaxL + 1];
__constant__ double c_dl[kMaxL + 1];

template <class R>
struct C {
  R x, y;
};
template <class R>
__device__ __forceinline__ C<R> cmul(C<R> a, C<R> b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <class R>
__device__ __forceinline__ C<R> cscale(C<R> a, R s) {
  return {a.x * s, a.y * s};
}
template <class R>
__device__ __forceinline__ C<R> cconj(C<R> a) {
  return {a.x, -a.y};
}
template <class R>
__device__ __forceinline__ R re_mul(C<R> a, C<R> b) {
  return a.x * b.x - a.y * b.y;
}

// acc += a b (complex) and acc += Re(a b) as chains of fused multiply-adds:
// two FMA instructions per real part instead of a multiply, an FMA and an
// add (the form a * b - c * d + acc contracts to), which matters most on the
// FP64 pipe
template <class R>
__device__ __forceinline__ void cmac(C<R>& acc, C<R> a, C<R> b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
template <class R>
__device__ __forceinline__ R re_mac(R acc, C<R> a, C<R> b) {
  return fma(-a.y, b.y, fma(a.x, b.x, acc));
}

__device__ __forceinline__ int ph(int l, int m) { return l * (l + 1) / 2 + m; }
__device__ __forceinline__ double parity(int m) { return (m & 1) ? -1.0 : 1.0; }

__device__ __forceinline__ void raise_error(int* err, int code) {
  if (err) atomicCAS(err, 0, code);
}

// The atom at position `it` of the work queue: the neighbour-count-sorted
// order when the evaluation has one, else atom `it`.
__device__ __forceinline__ int queue_atom(const DeviceModel& m, int it) { return m.order ? __ldg(m.order + it) : it; }

// Model constants in the working precision (the split path reads FP32
// copies made on the host instead of converting on the FP64 pipe).
template <class R>
__device__ __forceinline__ R rscale_a(const DeviceModel& m);
template <>
__device__ __forceinline__ double rscale_a<double>(const DeviceModel& m) {
  return m.rscale_a;
}
template <>
__device__ __forceinline__ float rscale_a<float>(const DeviceModel& m) {
  return m.rscale_a_f;
}
template <class R>
__device__ __forceinline__ R rscale_m(const DeviceModel& m);
template <>
__device__ __forceinline__ double rscale_m<double>(const DeviceModel& m) {
  return m.rscale_m;
}
template <>
__device__ __forceinline__ float rscale_m<float>(const DeviceModel& m) {
  return m.rscale_m_f;
}
template <class R>
__device__ __forceinline__ R c1_of(const DeviceModel& m, int k);
template <>
__device__ __forceinline__ double c1_of<double>(const DeviceModel& m, int k) {
  return m.c1[k];
}
template <>
__device__ __forceinline__ float c1_of<float>(const DeviceModel& m, int k) {
  return __ldg(m.c1f + k);
}

// Double <-> float conversions on the integer pipes. A hardware conversion
// issues on the FP64 pipe, which GB300 runs at 1/64 of the FP32 rate; the
// split path converts every input and output, so it uses these instead.
// d2f rounds half away from zero (|error| <= 1/2 float ulp), flushes values
// below the float normal range to signed zero, maps overflow to infinity and
// keeps NaN; f2d is exact for normal floats and flushes float subnormals.
__device__ __forceinline__ float d2f(double x) {
  const unsigned long long b0 = static_cast<unsigned long long>(__double_as_longlong(x));
  const int e0 = static_cast<int>((b0 >> 52) & 0x7ffu);
  const unsigned long long b = b0 + (1ull << 28);  // half a float ulp
  const unsigned hi = static_cast<unsigned>(b >> 32), lo = static_cast<unsigned>(b);
  const unsigned sign = hi & 0x80000000u;
  const int fe = static_cast<int>((hi >> 20) & 0x7ffu) - 1023 + 127;
  const unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);
  unsigned f = sign | (static_cast<unsigned>(fe) << 23) | mant;
  if (fe <= 0) f = sign;
  if (fe >= 255) f = sign | 0x7f800000u;
  if (e0 == 0x7ff) f = (b0 << 12) ? 0x7fc00000u : (sign | 0x7f800000u);
  return __uint_as_float(f);
}
__device__ __forceinline__ double f2d(float x) {
  const unsigned f = __float_as_uint(x);
  const unsigned long long sign = static_cast<unsigned long long>(f & 0x80000000u) << 32;
  const unsigned e = (f >> 23) & 0xffu;
  const unsigned long long mant = static_cast<unsigned long long>(f & 0x7fffffu) << 29;
  unsigned long long d = sign | (static_cast<unsigned long long>(e + 1023 - 127) << 52) | mant;
  if (e == 0) d = sign;
  if (e == 0xff) d = sign | (0x7ffull << 52) | mant;
  return __longlong_as_double(static_cast<long long>(d));
}
template <class R>
__device__ __forceinline__ R to_r(double x);
template <>
__device__ __forceinline__ double to_r<double>(double x) {
  return x;
}
template <>
__device__ __forceinline__ float to_r<float>(double x) {
  return d2f(x);
}
__device__ __forceinline__ double to_d(double x) { return x; }
__device__ __forceinline__ double to_d(float x) { return f2d(x); }
__device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
__device__ __forceinline__ float rcp(float x) { return __frcp_rn(x); }

// Spherical harmonics Y_lm (m >= 0 half, packed by ph) of a unit vector and,
// optionally, their tangential gradients dY = grad Y - (r . grad Y) r, in the
// normalisation and recurrence of src/spherical.F90:55-260 (Y_00 = 1,
// Condon-Shortley phase through cl).
template <class R, bool GRAD>
__device__ __forceinline__ void ylm_half(int L, R rx, R ry, R rz, C<R>* Y, C<R> (*dY)[3]) {
  R plm[kMaxHalf], dplm[kMaxHalf];
  const R sq3 = R(1.73205080756887719318), sq3o2 = R(1.22474487139158894067);
  plm[0] = R(1);
  dplm[0] = R(0);
  if (L > 0) {
    plm[ph(1, 0)] = sq3 * rz;
    dplm[ph(1, 0)] = sq3;
    plm[ph(1, 1)] = -sq3o2;
    dplm[ph(1, 1)] = R(0);
    for (int l = 2; l <= L; ++l) {
      for (int m = 0; m <= l - 2; ++m) {
        const int k = ph(l, m), k1 = ph(l - 1, m), k2 = ph(l - 2, m);
        const R a = R(c_alm[k]), b = R(c_blm[k]);
        plm[k] = a * (rz * plm[k1] + b * plm[k2]);
        dplm[k] = a * (plm[k1] + rz * dplm[k1] + b * dplm[k2]);
      }
      const int k = ph(l - 1, l - 1);
      const R t = R(c_dl[l]) * plm[k];
      plm[ph(l, l - 1)] = t * rz;
      dplm[ph(l, l - 1)] = t;
      plm[ph(l, l)] = R(c_cl[l]) * plm[k];
      dplm[ph(l, l)] = R(0);
    }
  }
  for (int l = 0; l <= L; ++l) {  // m = 0
    const int k = ph(l, 0);
    Y[k] = {plm[k], R(0)};
    if (GRAD) {
      const R dyz = dplm[k], rdy = dyz * rz;
      dY[k][0] = {-rdy * rx, R(0)};
      dY[k][1] = {-rdy * ry, R(0)};
      dY[k][2] = {dyz - rdy * rz, R(0)};
    }
  }
  for (int l = 1; l <= L; ++l) {  // m = 1
    const int k = ph(l, 1);
    Y[k] = {rx * plm[k], ry * plm[k]};
    if (GRAD) {
      const C<R> dyz = {rx * dplm[k], ry * dplm[k]};
      const C<R> rdy = {rx * plm[k] + rz * dyz.x, ry * plm[k] + rz * dyz.y};
      dY[k][0] = {plm[k] - rdy.x * rx, -(rdy.y * rx)};
      dY[k][1] = {-rdy.x * ry, plm[k] - rdy.y * ry};
      dY[k][2] = {dyz.x - rdy.x * rz, dyz.y - rdy.y * rz};
    }
  }
  C<R> phasem = {rx, ry};
  const C<R> phase = {rx, ry};
  for (int m = 2; m <= L; ++m) {  // m > 1
    const C<R> mph = {phasem.x * R(m), phasem.y * R(m)};
    phasem = cmul(phasem, phase);
    for (int l = m; l <= L; ++l) {
      const int k = ph(l, m);
      Y[k] = {phasem.x * plm[k], phasem.y * plm[k]};
      if (GRAD) {
        const C<R> dyx = cscale(mph, plm[k]);
        const C<R> dyy = {-dyx.y, dyx.x};
        const C<R> dyz = cscale(phasem, dplm[k]);
        const C<R> rdy = {rx * dyx.x + ry * dyy.x + rz * dyz.x, rx * dyx.y + ry * dyy.y + rz * dyz.y};
        dY[k][0] = {dyx.x - rdy.x * rx, dyx.y - rdy.y * rx};
        dY[k][1] = {dyy.x - rdy.x * ry, dyy.y - rdy.y * ry};
        dY[k][2] = {dyz.x - rdy.x * rz, dyz.y - rdy.y * rz};
      }
    }
  }
}

// full-range Y_lm (packed l*l+l+m) from the half
template <class R>
__device__ __forceinline__ C<R> y_full(const C<R>* Yh, int l, int m) {
  if (m >= 0) return Yh[ph(l, m)];
  const C<R> y = Yh[ph(l, -m)];
  const R s = R(parity(m));
  return {y.x * s, -y.y * s};
}

// Cubic-Hermite lookup of `count` consecutive functions starting at `f0` of a
// table with `nf` functions per bin (src/radial.F90:85-105). FP64 tables for
// the drop-in path, FP32 copies for the split path.
template <bool GRAD>
__device__ __forceinline__ void lut_eval(const double* __restrict__ lut, int nf, int f0, int count, int nl,
                                         double wl, double rscale, double* v, double* dv) {
  const double wl2 = wl * wl, wl3 = wl2 * wl, w2 = 2.0 * wl, w3 = 3.0 * wl2;
  const double2* c2 = reinterpret_cast<const double2*>(lut) + 2 * (static_cast<size_t>(nl) * nf + f0);
  for (int f = 0; f < count; ++f) {
    const double2 a = __ldg(c2 + 2 * f), b = __ldg(c2 + 2 * f + 1);
    v[f] = a.x + a.y * wl + b.x * wl2 + b.y * wl3;
    if (GRAD) dv[f] = (a.y + b.x * w2 + b.y * w3) * rscale;
  }
}
template <bool GRAD>
__device__ __forceinline__ void lut_eval(const float* __restrict__ lut, int nf, int f0, int count, int nl,
                                         float wl, float rscale, float* v, float* dv) {
  const float wl2 = wl * wl, wl3 = wl2 * wl, w2 = 2.0f * wl, w3 = 3.0f * wl2;
  const float4* c4 = reinterpret_cast<const float4*>(lut) + static_cast<size_t>(nl) * nf + f0;
  for (int f = 0; f < count; ++f) {
    const float4 c = __ldg(c4 + f);
    v[f] = c.x + c.y * wl + c.z * wl2 + c.w * wl3;
    if (GRAD) dv[f] = (c.y + c.z * w2 + c.w * w3) * rscale;
  }
}
template <class R>
__device__ __forceinline__ const R* pick(const double* d, const float* f);
template <>
__device__ __forceinline__ const double* pick<double>(const double* d, const float*) {
  return d;
}
template <>
__device__ __forceinline__ const float* pick<float>(const double*, const float* f) {
  return f;
}

// bins of the atomic table: returns false (features zero) beyond the cutoff
__device__ __forceinline__ int atomic_bin(const DeviceModel& m, double r, double& wl, int* err) {
  const double x = r * m.rscale_a;
  if (!(x >= 1.0)) {
    raise_error(err, kDevSmallR);
    return -1;
  }
  if (x >= static_cast<double>(m.nlut)) return 0;  // zero features (src/radial.F90:77-83)
  const int nl = static_cast<int>(floor(x));
  wl = x - static_cast<double>(nl);
  return nl;
}

// the same in the working precision of the split path (the bin position
// carries ~1e-7 relative error, far inside the interpolant's own)
template <class R>
__device__ __forceinline__ int atomic_bin_r(const DeviceModel& m, R r, R& wl, int* err) {
  const R x = r * rscale_a<R>(m);
  if (!(x >= R(1))) {
    raise_error(err, kDevSmallR);
    return -1;
  }
  if (x >= R(m.nlut)) return 0;
  const int nl = static_cast<int>(floor(x));
  wl = x - R(nl);
  return nl;
}
template <class R>
__device__ __forceinline__ int magnetic_bin_r(const DeviceModel& m, R mag, R& wl, int* err) {
  const R x = mag * rscale_m<R>(m);
  if (!(x >= R(0)) || x >= R(m.nlut)) {
    raise_error(err, kDevMoment);
    return -1;
  }
  const int nl = static_cast<int>(floor(x));
  wl = x - R(nl);
  return nl;
}

// bins of the magnetic table: 0 means |m| inside the first bin, where every
// function is 1 and every derivative 0 (src/radial.F90:135-139)
__device__ __forceinline__ int magnetic_bin(const DeviceModel& m, double mag, double& wl, int* err) {
  const double x = mag * m.rscale_m;
  if (!(x >= 0.0) || x >= static_cast<double>(m.nlut)) {
    raise_error(err, kDevMoment);
    return -1;
  }
  const int nl = static_cast<int>(floor(x));
  wl = x - static_cast<double>(nl);
  return nl;
}

// ===========================================================================
// k_abasis
// Shared memory: acc[nWA + nba*n2m*h2] (complex R), then per tile of TB bonds
// (SoA, [feature][TB]): g[nba], RY[n3a*lsa] (complex), Q[n2m*h2] (complex),
// core[1].
template <class R>
__global__ void __launch_bounds__(kAbasisThreads)
    k_abasis(DeviceModel m, int natom, const int* __restrict__ off, const double* __restrict__ rr,
             const double* __restrict__ ee, const double* __restrict__ magj, const double* __restrict__ mhj,
             const double* __restrict__ magi, const double* __restrict__ mhi, C<R>* __restrict__ F,
             double* __restrict__ rho1, double* __restrict__ core_out, int* err) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int TB = kAbasisTile;
  const int nA2h = m.nba * m.n2m * m.h2;
  const int nacc = m.nWA + nA2h;
  C<R>* acc = reinterpret_cast<C<R>*>(smem);
  C<R>* sRY = acc + nacc;                      // [n3a*lsa][TB]
  C<R>* sQ = sRY + m.n3a * m.lsa * TB;         // [n2m*h2][TB]
  R* sg = reinterpret_cast<R*>(sQ + m.n2m * m.h2 * TB);  // [nba][TB]
  double* score = reinterpret_cast<double*>(sg + m.nba * TB);  // [TB]
  __shared__ double s_core;

  for (int it = blockIdx.x; it < natom; it += gridDim.x) {
    const int atom = queue_atom(m, it);
    for (int s = threadIdx.x; s < nacc; s += blockDim.x) acc[s] = {R(0), R(0)};
    if (threadIdx.x == 0) s_core = 0.0;
    const int b0 = off[atom], b1 = off[atom + 1];
    __syncthreads();
    for (int t0 = b0; t0 < b1; t0 += TB) {
      const int nb = min(TB, b1 - t0);
      if (threadIdx.x < nb) {
        const int b = threadIdx.x, j = t0 + b;
        const double r = rr[j];
        R g[kMaxFeat], Rv[kMaxFeat], Mv[kMaxFeat], cv[1], dummy[1];
        double wl = 0.0;
        const int nla = atomic_bin(m, r, wl, err);
        if (nla > 0) {
          lut_eval<false>(pick<R>(m.lut_a, m.lut_a32), m.nfa, 0, m.nba, nla, R(wl), rscale_a<R>(m), g, dummy);
          lut_eval<false>(pick<R>(m.lut_a, m.lut_a32), m.nfa, m.nba, m.n3a * (m.l3a + 1), nla, R(wl), rscale_a<R>(m), Rv, dummy);
          lut_eval<false>(pick<R>(m.lut_a, m.lut_a32), m.nfa, m.nba + m.n3a * (m.l3a + 1), 1, nla, R(wl), rscale_a<R>(m), cv, dummy);
        } else {
          for (int q = 0; q < m.nba; ++q) g[q] = R(0);
          for (int q = 0; q < m.n3a * (m.l3a + 1); ++q) Rv[q] = R(0);
          cv[0] = R(0);
        }
        double wm = 0.0;
        const int nlm = magnetic_bin(m, magj[j], wm, err);
        const int nM = m.n2m * (m.l2m + 1);
        if (nlm > 0) {
          lut_eval<false>(pick<R>(m.lut_m, m.lut_m32), m.nfm, 0, nM, nlm, R(wm), rscale_m<R>(m), Mv, dummy);
        } else {
          for (int q = 0; q < nM; ++q) Mv[q] = R(nlm == 0 ? 1 : 0);
        }
        C<R> Ya[kMaxHalf], Ym[kMaxHalf];
        ylm_half<R, false>(m.l3a, R(ee[3 * j]), R(ee[3 * j + 1]), R(ee[3 * j + 2]), Ya, nullptr);
        ylm_half<R, false>(m.l2m, R(mhj[3 * j]), R(mhj[3 * j + 1]), R(mhj[3 * j + 2]), Ym, nullptr);
        for (int n1 = 0; n1 < m.n3a; ++n1)
          for (int l1 = 0; l1 <= m.l3a; ++l1)
            for (int m1 = -l1; m1 <= l1; ++m1)
              sRY[(n1 * m.lsa + l1 * l1 + l1 + m1) * TB + b] = cscale(y_full(Ya, l1, m1), Rv[n1 * (m.l3a + 1) + l1]);
        for (int nr = 0; nr < m.n2m; ++nr)
          for (int l = 0; l <= m.l2m; ++l)
            for (int mm = 0; mm <= l; ++mm)
              sQ[(nr * m.h2 + ph(l, mm)) * TB + b] = cscale(Ym[ph(l, mm)], Mv[nr * (m.l2m + 1) + l]);
        for (int n = 0; n < m.nba; ++n) sg[n * TB + b] = g[n];
        score[b] = static_cast<double>(cv[0]);
      }
      __syncthreads();
      for (int s = threadIdx.x; s < nacc; s += blockDim.x) {
        C<R> a = acc[s];
        if (s < m.nWA) {
          // s = ((n1*lsa + lma)*n3m + n2)*h3 + h
          const int h = s % m.h3;
          const int q = s / m.h3;
          const int n2 = q % m.n3m;
          const int ia = q / m.n3m;  // n1*lsa + lma
          const C<R>* ry = sRY + ia * TB;
          const C<R>* qq = sQ + (n2 * m.h2 + h) * TB;
          for (int b = 0; b < nb; ++b) {
            const C<R> u = ry[b], v = qq[b];
            a.x += u.x * v.x - u.y * v.y;
            a.y += u.x * v.y + u.y * v.x;
          }
        } else {
          // A2 half: (s - nWA) = (n*n2m + nr)*h2 + h
          const int t = s - m.nWA;
          const int h = t % m.h2;
          const int q = t / m.h2;
          const int nr = q % m.n2m;
          const int n = q / m.n2m;
          const R* gg = sg + n * TB;
          const C<R>* qq = sQ + (nr * m.h2 + h) * TB;
          for (int b = 0; b < nb; ++b) {
            a.x += gg[b] * qq[b].x;
            a.y += gg[b] * qq[b].y;
          }
        }
        acc[s] = a;
      }
      if (threadIdx.x == 0)
        for (int b = 0; b < nb; ++b) s_core += score[b];
      __syncthreads();
    }
    // complete A and A2 by A(m1,m2) = (-1)^(m1+m2) conj A(-m1,-m2) and write F
    C<R>* Fa = F + static_cast<size_t>(atom) * m.nF;
    const int nA = m.offA2 - m.offA;
    for (int s = threadIdx.x; s < nA; s += blockDim.x) {
      const int lmm = s % m.ls3;
      const int q = s / m.ls3;
      const int n2 = q % m.n3m;
      const int ia = q / m.n3m;
      const int n1 = ia / m.lsa, lma = ia % m.lsa;
      int l2 = 0;
      while ((l2 + 1) * (l2 + 1) <= lmm) ++l2;
      const int m2 = lmm - l2 * l2 - l2;
      int l1 = 0;
      while ((l1 + 1) * (l1 + 1) <= lma) ++l1;
      const int m1 = lma - l1 * l1 - l1;
      C<R> v;
      if (m2 >= 0) {
        v = acc[((n1 * m.lsa + lma) * m.n3m + n2) * m.h3 + ph(l2, m2)];
      } else {
        const int lmb = l1 * l1 + l1 - m1;
        const C<R> w = acc[((n1 * m.lsa + lmb) * m.n3m + n2) * m.h3 + ph(l2, -m2)];
        const R sgn = R(parity(m1 + m2));
        v = {w.x * sgn, -w.y * sgn};
      }
      Fa[m.offA + s] = v;
    }
    const int nA2 = m.offA0 - m.offA2;
    for (int s = threadIdx.x; s < nA2; s += blockDim.x) {
      const int lm = s % m.ls2;
      const int q = s / m.ls2;  // n*n2m + nr
      int l = 0;
      while ((l + 1) * (l + 1) <= lm) ++l;
      const int mm = lm - l * l - l;
      const C<R> w = acc[m.nWA + q * m.h2 + ph(l, mm < 0 ? -mm : mm)];
      C<R> v = w;
      if (mm < 0) {
        const R sgn = R(parity(mm));
        v = {w.x * sgn, -w.y * sgn};
      }
      Fa[m.offA2 + s] = v;
    }
    if (threadIdx.x == 0) {
      // on-site A0, the 1-body density and the constants
      double wl = 0.0;
      const int nl = magnetic_bin(m, magi[atom], wl, err);
      R Mv[32], gm[32], dummy[1];
      const int nM = m.n2m * (m.l2m + 1);
      if (nl > 0) {
        lut_eval<false>(pick<R>(m.lut_m, m.lut_m32), m.nfm, 0, nM, nl, R(wl), rscale_m<R>(m), Mv, dummy);
        lut_eval<false>(pick<R>(m.lut_m, m.lut_m32), m.nfm, nM, m.nbm, nl, R(wl), rscale_m<R>(m), gm, dummy);
      } else {
        for (int q = 0; q < nM; ++q) Mv[q] = R(nl == 0 ? 1 : 0);
        for (int q = 0; q < m.nbm; ++q) gm[q] = R(nl == 0 ? 1 : 0);
      }
      C<R> Yi[kMaxHalf];
      ylm_half<R, false>(m.l2m, R(mhi[3 * atom]), R(mhi[3 * atom + 1]), R(mhi[3 * atom + 2]), Yi, nullptr);
      for (int nr = 0; nr < m.n2m; ++nr)
        for (int l = 0; l <= m.l2m; ++l)
          for (int mm = -l; mm <= l; ++mm)
            Fa[m.offA0 + nr * m.ls2 + l * l + l + mm] = cscale(y_full(Yi, l, mm), Mv[nr * (m.l2m + 1) + l]);
      Fa[m.offOne] = {R(1), R(0)};
      Fa[m.offZero] = {R(0), R(0)};
      for (int d = 0; d < m.nd; ++d) {
        double s = 0.0;
        for (int n = 0; n < m.nbm; ++n) s += m.c1[d * m.nbm + n] * (static_cast<double>(gm[n]) - 1.0);
        rho1[static_cast<size_t>(atom) * 2 + d] = s;
      }
      core_out[atom] = s_core;
    }
    __syncthreads();
  }
}

// ===========================================================================
// Embedding F(rho) and derivative (src/forces.F90:1134-1266, nfemb 0-2)
__device__ void embed(int nfemb, double rho, double wpre, double mexp, double& F, double& dF) {
  const double w = 10.0, eps = 1e-10;
  if (nfemb == 0) {
    F = rho;
    dF = 1.0;
    return;
  }
  const double s = (nfemb == 2) ? 1.0 + rho : rho;
  if (fabs(s) > eps) {
    double y1 = w * s * s;
    const double g = (y1 > 30.0) ? 0.0 : exp(-y1);
    const double omg = 1.0 - g, a = fabs(s), sg = copysign(1.0, s);
    y1 = pow(omg * a, mexp);
    const double y2 = mexp * g * a;
    F = (nfemb == 2) ? wpre * (sg * (y1 + y2) - 1.0) : wpre * sg * (y1 + y2);
    const double dg = -2.0 * w * s * g, da = sg;
    const double dy = (fabs(y1) < eps) ? 0.0 : mexp * y1 / (omg * a);
    const double dy1 = dy * (-dg * a + omg * da), dy2 = mexp * (dg * a + g * da);
    dF = wpre * sg * (dy1 + dy2);
  } else {
    F = (nfemb == 2) ? wpre * mexp * (s - 1.0) : wpre * mexp * rho;
    dF = wpre * mexp;
  }
}

// ===========================================================================
// k_density
// One CTA per atom. Warps walk the warp groups of the gather table (lane l of
// group g owns segment grp_seg[g*32+l]); each lane accumulates its segment's
// entries kappa * prod F[o] into a partial sum. Slot totals then add a slot's
// partials in segment order (compensated in FP32 for the split path), the
// density is rho = rho1 + sum over A0 slots of Re(A0 * total) in FP64, and the
// weights are dE/drho * multiplicity * total.
// Shared memory: Fs[nF] (complex R), part[nseg][ND] (complex R),
// tot[nslot][ND] (complex R, hi) and, for FP32, the low words.
template <class R>
__device__ __forceinline__ const R* kap_ptr(const GatherView& m, int a);
template <>
__device__ __forceinline__ const double* kap_ptr<double>(const GatherView& m, int a) {
  return m.kap[a];
}
template <>
__device__ __forceinline__ const float* kap_ptr<float>(const GatherView& m, int a) {
  return m.kapf[a];
}

// running sum with an error term: exact for double, two-float for float
template <class R>
struct CSum {
  R hi = R(0), lo = R(0);
  __device__ __forceinline__ void add(R b) {
    const R s = hi + b;
    const R bb = s - hi;
    lo += (hi - (s - bb)) + (b - bb);
    hi = s;
  }
  __device__ __forceinline__ double value() const { return static_cast<double>(hi) + static_cast<double>(lo); }
};

template <class R, int ND>
__global__ void __launch_bounds__(kDensityThreads)
    k_density(DeviceModel m, int natom, const C<R>* __restrict__ F, const double* __restrict__ rho1,
              const double* __restrict__ core, C<R>* __restrict__ W, double* __restrict__ energy,
              double* __restrict__ edf_out, double* __restrict__ dedrho_out, int* err) {
  extern __shared__ __align__(16) unsigned char smem[];
  const GatherView& G = m.g;
  C<R>* Fs = reinterpret_cast<C<R>*>(smem);
  C<R>* part = Fs + ((m.nF + 1) & ~1);
  C<R>* tot = part + ((G.nseg * ND + 1) & ~1);
  __shared__ double s_red[kDensityThreads / 32][ND];
  __shared__ double s_dE[ND];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;

  for (int it = blockIdx.x; it < natom; it += gridDim.x) {
    const int atom = queue_atom(m, it);
    const C<R>* Fa = F + static_cast<size_t>(atom) * m.nF;
    for (int s = threadIdx.x; s < m.nF; s += blockDim.x) Fs[s] = Fa[s];
    __syncthreads();
    for (int g = warp; g < G.ngroup; g += nwarp) {
      const int a = G.grp_arity[g], len = G.grp_len[g], base = G.grp_first[g] + lane;
      const int seg = G.grp_seg[g * 32 + lane];
      const R* kp = kap_ptr<R>(G, a) + base;
      const uint32_t* op = G.o12[a] + base;
      const int ks = G.kstride[a];
      C<R> acc[ND];
      for (int d = 0; d < ND; ++d) acc[d] = {R(0), R(0)};
      if (a == 2) {
#pragma unroll 4
        for (int e = 0; e < len; ++e) {
          const uint32_t o = __ldg(op + e * 32);
          const C<R> p = cmul(Fs[o & 0xffffu], Fs[o >> 16]);
          for (int d = 0; d < ND; ++d) {
            const R k = __ldg(kp + d * ks + e * 32);
            acc[d].x += k * p.x;
            acc[d].y += k * p.y;
          }
        }
      } else if (a == 1) {
        for (int e = 0; e < len; ++e) {
          const uint32_t o = __ldg(op + e * 32);
          const C<R> p = Fs[o & 0xffffu];
          for (int d = 0; d < ND; ++d) {
            const R k = __ldg(kp + d * ks + e * 32);
            acc[d].x += k * p.x;
            acc[d].y += k * p.y;
          }
        }
      } else {
        // arity 3 to 5 (the 4-, 5- and 6-body terms)
        const uint32_t* o34p = G.o34[a] + base;
        const uint16_t* o5p = G.o5 + base;
        for (int e = 0; e < len; ++e) {
          const uint32_t o = __ldg(op + e * 32), q = __ldg(o34p + e * 32);
          C<R> p = cmul(cmul(Fs[o & 0xffffu], Fs[o >> 16]), Fs[q & 0xffffu]);
          if (a >= 4) p = cmul(p, Fs[q >> 16]);
          if (a == 5) p = cmul(p, Fs[__ldg(o5p + e * 32)]);
          for (int d = 0; d < ND; ++d) {
            const R k = __ldg(kp + d * ks + e * 32);
            acc[d].x += k * p.x;
            acc[d].y += k * p.y;
          }
        }
      }
      if (seg >= 0)
        for (int d = 0; d < ND; ++d) part[seg * ND + d] = acc[d];
    }
    __syncthreads();
    double rloc[ND];
    for (int d = 0; d < ND; ++d) rloc[d] = 0.0;
    for (int s = threadIdx.x; s < G.nslot; s += blockDim.x) {
      const int q0 = G.slot_seg[s], q1 = G.slot_seg[s + 1];
      for (int d = 0; d < ND; ++d) {
        CSum<R> tx, ty;
        for (int q = q0; q < q1; ++q) {
          tx.add(part[q * ND + d].x);
          ty.add(part[q * ND + d].y);
        }
        tot[s * ND + d] = {tx.hi + tx.lo, ty.hi + ty.lo};
        if (s < G.nG0) {
          const C<R> f = Fs[G.slot_factor[s]];
          rloc[d] += static_cast<double>(f.x) * tx.value() - static_cast<double>(f.y) * ty.value();
        }
      }
    }
    // deterministic block reduction of rho
    for (int d = 0; d < ND; ++d) {
      double v = rloc[d];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) s_red[warp][d] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double energyi = 0.0, dE[ND];
      for (int d = 0; d < ND; ++d) {
        double rho = rho1[static_cast<size_t>(atom) * 2 + d];
        for (int w = 0; w < kDensityThreads / 32; ++w) rho += s_red[w][d];
        if (!isfinite(rho)) raise_error(err, kDevNaN);
        double Fd, dFd;
        embed(m.nfemb, rho, m.par[0][d], m.par[1][d], Fd, dFd);
        energyi = (d == 0) ? Fd : energyi + Fd;
        dE[d] = dFd;
      }
      // inner cutoff on the hard-core energy (src/forces.F90:1112-1128, :1270-1289)
      const double e = core[atom], elow = m.ecut - m.decut;
      double fcut, dfcut;
      if (e >= m.ecut) {
        fcut = 0.0;
        dfcut = 0.0;
      } else if (e <= elow) {
        fcut = 1.0;
        dfcut = 0.0;
      } else {
        const double pi = 3.14159265358979323846264338327950288419;
        fcut = 0.5 * (1.0 + cos(pi * (e - elow) / m.decut));
        dfcut = -0.5 * sin(pi * (e - elow) / m.decut) * pi / m.decut;
      }
      edf_out[atom] = dfcut * energyi + 1.0;
      for (int d = 0; d < ND; ++d) {
        dE[d] = fcut * dE[d];
        s_dE[d] = dE[d];
        dedrho_out[static_cast<size_t>(atom) * 2 + d] = dE[d];
      }
      energy[atom] = fcut * energyi + e;
    }
    __syncthreads();
    C<R>* Wa = W + static_cast<size_t>(atom) * m.nW;
    for (int s = threadIdx.x; s < G.nslot; s += blockDim.x) {
      const int w = G.slot_weight[s];
      if (w < 0) continue;
      const R mu = R(G.slot_mult[s]);
      C<R> v = {R(0), R(0)};
      for (int d = 0; d < ND; ++d) {
        const R sc = mu * R(s_dE[d]);
        v.x += sc * tot[s * ND + d].x;
        v.y += sc * tot[s * ND + d].y;
      }
      Wa[w] = v;
    }
    __syncthreads();
  }
}

// ===========================================================================
// k_forces
// Shared memory: Ws[nW] (complex R), then per-thread feature columns (SoA,
// [feature][blockDim]) so that every thread's scratch is bank-conflict free.
template <class R>
__global__ void __launch_bounds__(kForceThreads)
    k_forces(DeviceModel m, int natom, const int* __restrict__ off, const double* __restrict__ rr,
             const double* __restrict__ ee, const double* __restrict__ magj, const double* __restrict__ mhj,
             const double* __restrict__ magi, const double* __restrict__ mhi, const C<R>* __restrict__ W,
             const double* __restrict__ edf_in, const double* __restrict__ dedrho, double* __restrict__ fij,
             double* __restrict__ tij, double* __restrict__ ti0, int* err) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int T = blockDim.x;
  C<R>* Ws = reinterpret_cast<C<R>*>(smem);
  C<R>* cY = Ws + ((m.nW + 1) & ~1);           // Ya full [lsa][T], then dYa [lsa][3][T]
  C<R>* cdY = cY + m.lsa * T;
  C<R>* cYm = cdY + m.lsa * 3 * T;              // Ym half [h2][T], dYm [h2][3][T]
  C<R>* cdYm = cYm + m.h2 * T;
  R* cg = reinterpret_cast<R*>(cdYm + m.h2 * 3 * T);  // g [nba][T], g' [nba][T]
  R* cgd = cg + m.nba * T;
  R* cR = cgd + m.nba * T;                      // R, R' [n3a*(l3a+1)][T]
  R* cRd = cR + m.n3a * (m.l3a + 1) * T;
  R* cM = cRd + m.n3a * (m.l3a + 1) * T;        // M, M' [n2m*(l2m+1)][T]
  R* cMd = cM + m.n2m * (m.l2m + 1) * T;
  const int t = threadIdx.x;
  const int nRl = m.n3a * (m.l3a + 1), nMl = m.n2m * (m.l2m + 1);

  for (int it = blockIdx.x; it < natom; it += gridDim.x) {
    const int atom = queue_atom(m, it);
    const C<R>* Wa = W + static_cast<size_t>(atom) * m.nW;
    for (int s = t; s < m.nW; s += T) Ws[s] = Wa[s];
    __syncthreads();
    const double edf = edf_in[atom];
    const int b0 = off[atom], b1 = off[atom + 1];
    for (int j = b0 + t; j < b1; j += T) {
      const double r = rr[j];
      const double ex = ee[3 * j], ey = ee[3 * j + 1], ez = ee[3 * j + 2];
      const double mg = magj[j];
      const double mx = mhj[3 * j], my = mhj[3 * j + 1], mz = mhj[3 * j + 2];
      // radial features with derivatives
      R tmpv[32], tmpd[32];
      double wl = 0.0;
      R cd = R(0);
      const int nla = atomic_bin(m, r, wl, err);
      if (nla > 0) {
        lut_eval<true>(pick<R>(m.lut_a, m.lut_a32), m.nfa, 0, m.nba, nla, R(wl), rscale_a<R>(m), tmpv, tmpd);
        for (int n = 0; n < m.nba; ++n) {
          cg[n * T + t] = tmpv[n];
          cgd[n * T + t] = tmpd[n];
        }
        lut_eval<true>(pick<R>(m.lut_a, m.lut_a32), m.nfa, m.nba, nRl, nla, R(wl), rscale_a<R>(m), tmpv, tmpd);
        for (int q = 0; q < nRl; ++q) {
          cR[q * T + t] = tmpv[q];
          cRd[q * T + t] = tmpd[q];
        }
        R cv[1], cdv[1];
        lut_eval<true>(pick<R>(m.lut_a, m.lut_a32), m.nfa, m.nba + nRl, 1, nla, R(wl), rscale_a<R>(m), cv, cdv);
        cd = cdv[0];
      } else {
        for (int n = 0; n < m.nba; ++n) cg[n * T + t] = cgd[n * T + t] = R(0);
        for (int q = 0; q < nRl; ++q) cR[q * T + t] = cRd[q * T + t] = R(0);
      }
      double wm = 0.0;
      const int nlm = magnetic_bin(m, mg, wm, err);
      if (nlm > 0) {
        lut_eval<true>(pick<R>(m.lut_m, m.lut_m32), m.nfm, 0, nMl, nlm, R(wm), rscale_m<R>(m), tmpv, tmpd);
        for (int q = 0; q < nMl; ++q) {
          cM[q * T + t] = tmpv[q];
          cMd[q * T + t] = tmpd[q];
        }
      } else {
        for (int q = 0; q < nMl; ++q) {
          cM[q * T + t] = R(nlm == 0 ? 1 : 0);
          cMd[q * T + t] = R(0);
        }
      }
      {
        C<R> Yh[kMaxHalf], dYh[kMaxHalf][3];
        ylm_half<R, true>(m.l3a, R(ex), R(ey), R(ez), Yh, dYh);
        for (int l = 0; l <= m.l3a; ++l)
          for (int mm = -l; mm <= l; ++mm) {
            const int lm = l * l + l + mm;
            cY[lm * T + t] = y_full(Yh, l, mm);
            for (int c = 0; c < 3; ++c) {
              C<R> d = dYh[ph(l, mm < 0 ? -mm : mm)][c];
              if (mm < 0) {
                const R s = R(parity(mm));
                d = {d.x * s, -d.y * s};
              }
              cdY[(lm * 3 + c) * T + t] = d;
            }
          }
        ylm_half<R, true>(m.l2m, R(mx), R(my), R(mz), Yh, dYh);
        for (int h = 0; h < m.h2; ++h) {
          cYm[h * T + t] = Yh[h];
          for (int c = 0; c < 3; ++c) cdYm[(h * 3 + c) * T + t] = dYh[h][c];
        }
      }
      // ---- force: dE_i / d(x_i - x_j)
      R fr = R(edf) * cd;  // radial (along e) part
      R ft[3] = {R(0), R(0), R(0)};
      const R invr = R(1.0 / r);
      // pair part: sum_n g'_n sum_{nr,h} Re(W2[n][nr][h] Q[nr][h])
      for (int nr = 0; nr < m.n2m; ++nr)
        for (int l = 0; l <= m.l2m; ++l) {
          const R Ml = cM[(nr * (m.l2m + 1) + l) * T + t];
          for (int mm = 0; mm <= l; ++mm) {
            const int h = ph(l, mm);
            const C<R> q = cscale(cYm[h * T + t], Ml);
            R s = R(0);
            for (int n = 0; n < m.nba; ++n) s += cgd[n * T + t] * re_mul(Ws[m.offW2 + (n * m.n2m + nr) * m.h2 + h], q);
            fr += s;
          }
        }
      // many-body part via U[n1][lma] = sum_{n2,h} WA Q
      for (int n1 = 0; n1 < m.n3a; ++n1)
        for (int l1 = 0; l1 <= m.l3a; ++l1)
          for (int m1 = -l1; m1 <= l1; ++m1) {
            const int lma = l1 * l1 + l1 + m1;
            const C<R>* wrow = Ws + (n1 * m.lsa + lma) * m.n3m * m.h3;
            C<R> U = {R(0), R(0)};
            for (int n2 = 0; n2 < m.n3m; ++n2)
              for (int l2 = 0; l2 <= m.l3m; ++l2) {
                const R Ml = cM[(n2 * (m.l2m + 1) + l2) * T + t];
                for (int m2 = 0; m2 <= l2; ++m2) {
                  const int h = ph(l2, m2);
                  const C<R> q = cscale(cYm[h * T + t], Ml);
                  const C<R> w = wrow[n2 * m.h3 + h];
                  U.x += w.x * q.x - w.y * q.y;
                  U.y += w.x * q.y + w.y * q.x;
                }
              }
            const R Rv = cR[(n1 * (m.l3a + 1) + l1) * T + t];
            const R Rd = cRd[(n1 * (m.l3a + 1) + l1) * T + t];
            fr += Rd * re_mul(U, cY[lma * T + t]);
            const R sc = invr * Rv;
            for (int c = 0; c < 3; ++c) ft[c] += sc * re_mul(U, cdY[(lma * 3 + c) * T + t]);
          }
      fij[3 * static_cast<size_t>(j) + 0] = static_cast<double>(fr * R(ex) + ft[0]);
      fij[3 * static_cast<size_t>(j) + 1] = static_cast<double>(fr * R(ey) + ft[1]);
      fij[3 * static_cast<size_t>(j) + 2] = static_cast<double>(fr * R(ez) + ft[2]);
      // ---- magnetic force: dE_i / dm_j
      R tr = R(0), tt[3] = {R(0), R(0), R(0)};
      const R invm = R(1.0 / mg);
      for (int nr = 0; nr < m.n2m; ++nr)
        for (int l = 0; l <= m.l2m; ++l)
          for (int mm = 0; mm <= l; ++mm) {
            const int h = ph(l, mm);
            C<R> V = {R(0), R(0)};
            for (int n = 0; n < m.nba; ++n) {
              const C<R> w = Ws[m.offW2 + (n * m.n2m + nr) * m.h2 + h];
              const R gv = cg[n * T + t];
              V.x += gv * w.x;
              V.y += gv * w.y;
            }
            if (nr < m.n3m && l <= m.l3m) {
              for (int n1 = 0; n1 < m.n3a; ++n1)
                for (int l1 = 0; l1 <= m.l3a; ++l1) {
                  const R Rv = cR[(n1 * (m.l3a + 1) + l1) * T + t];
                  for (int m1 = -l1; m1 <= l1; ++m1) {
                    const int lma = l1 * l1 + l1 + m1;
                    const C<R> ry = cscale(cY[lma * T + t], Rv);
                    const C<R> w = Ws[((n1 * m.lsa + lma) * m.n3m + nr) * m.h3 + h];
                    V.x += w.x * ry.x - w.y * ry.y;
                    V.y += w.x * ry.y + w.y * ry.x;
                  }
                }
            }
            const int q = nr * (m.l2m + 1) + l;
            tr += cMd[q * T + t] * re_mul(V, cYm[h * T + t]);
            const R sc = invm * cM[q * T + t];
            for (int c = 0; c < 3; ++c) tt[c] += sc * re_mul(V, cdYm[(h * 3 + c) * T + t]);
          }
      tij[3 * static_cast<size_t>(j) + 0] = static_cast<double>(tr * R(mx) + tt[0]);
      tij[3 * static_cast<size_t>(j) + 1] = static_cast<double>(tr * R(my) + tt[1]);
      tij[3 * static_cast<size_t>(j) + 2] = static_cast<double>(tr * R(mz) + tt[2]);
    }
    if (t == 0) {
      // on-site magnetic force dE_i/dm_i (src/forces.F90:690-749)
      const double mg = magi[atom];
      const double mx = mhi[3 * atom], my = mhi[3 * atom + 1], mz = mhi[3 * atom + 2];
      double wm = 0.0;
      const int nl = magnetic_bin(m, mg, wm, err);
      R Mv[32], Md[32], gm[32], gmd[32];
      if (nl > 0) {
        lut_eval<true>(pick<R>(m.lut_m, m.lut_m32), m.nfm, 0, nMl, nl, R(wm), rscale_m<R>(m), Mv, Md);
        lut_eval<true>(pick<R>(m.lut_m, m.lut_m32), m.nfm, nMl, m.nbm, nl, R(wm), rscale_m<R>(m), gm, gmd);
      } else {
        for (int q = 0; q < nMl; ++q) {
          Mv[q] = R(nl == 0 ? 1 : 0);
          Md[q] = R(0);
        }
        for (int q = 0; q < m.nbm; ++q) gmd[q] = R(0);
      }
      C<R> Yh[kMaxHalf], dYh[kMaxHalf][3];
      ylm_half<R, true>(m.l2m, R(mx), R(my), R(mz), Yh, dYh);
      double tr = 0.0, tt[3] = {0.0, 0.0, 0.0};
      for (int n = 0; n < m.nbm; ++n) {
        double wf1 = 0.0;
        for (int d = 0; d < m.nd; ++d) wf1 += dedrho[static_cast<size_t>(atom) * 2 + d] * m.c1[d * m.nbm + n];
        tr += wf1 * static_cast<double>(gmd[n]);
      }
      const double invm = 1.0 / mg;
      for (int nr = 0; nr < m.n2m; ++nr)
        for (int l = 0; l <= m.l2m; ++l)
          for (int mm = 0; mm <= l; ++mm) {
            const int h = ph(l, mm);
            const C<R> w = Ws[m.offW0 + nr * m.h2 + h];
            const int q = nr * (m.l2m + 1) + l;
            tr += static_cast<double>(Md[q] * re_mul(w, Yh[h]));
            const R sc = R(invm) * Mv[q];
            for (int c = 0; c < 3; ++c) tt[c] += static_cast<double>(sc * re_mul(w, dYh[h][c]));
          }
      ti0[3 * static_cast<size_t>(atom) + 0] = tr * mx + tt[0];
      ti0[3 * static_cast<size_t>(atom) + 1] = tr * my + tt[1];
      ti0[3 * static_cast<size_t>(atom) + 2] = tr * mz + tt[2];
    }
    __syncthreads();
  }
}

#include "kernels_fe.inl"

// ===========================================================================
// host-side launch helpers

void upload_ylm_constants(const double* alm, const double* blm, const double* cl, const double* dl) {
  cudaMemcpyToSymbol(c_alm, alm, sizeof(double) * kMaxHalf);
  cudaMemcpyToSymbol(c_blm, blm, sizeof(double) * kMaxHalf);
  cudaMemcpyToSymbol(c_cl, cl, sizeof(double) * (kMaxL + 1));
  cudaMemcpyToSymbol(c_dl, dl, sizeof(double) * (kMaxL + 1));
}

template <class R>
size_t abasis_smem(const DeviceModel& m) {
  const int TB = kAbasisTile;
  const size_t nacc = static_cast<size_t>(m.nWA) + static_cast<size_t>(m.nba) * m.n2m * m.h2;
  return sizeof(C<R>) * (nacc + static_cast<size_t>(m.n3a) * m.lsa * TB + static_cast<size_t>(m.n2m) * m.h2 * TB) +
         sizeof(R) * static_cast<size_t>(m.nba) * TB + sizeof(double) * TB + 64;
}

template <class R>
size_t density_smem(const DeviceModel& m) {
  const GatherView& g = m.g;
  return sizeof(C<R>) * (static_cast<size_t>((m.nF + 1) & ~1) + static_cast<size_t>((g.nseg * m.nd + 1) & ~1) +
                         static_cast<size_t>(g.nslot) * m.nd) + 64;
}

template <class R>
size_t forces_smem(const DeviceModel& m, int T) {
  const size_t nc = static_cast<size_t>((m.nW + 1) & ~1) + static_cast<size_t>(T) * (m.lsa * 4 + m.h2 * 4);
  const size_t nr = static_cast<size_t>(T) * (2 * m.nba + 2 * m.n3a * (m.l3a + 1) + 2 * m.n2m * (m.l2m + 1));
  return sizeof(C<R>) * nc + sizeof(R) * nr + 64;
}

// Whether the compile-time specialised kernels apply: the basis has the Fe
// layout, one density and no 5- or 6-body clusters, and MAGACE_GENERIC is
// not set.
bool use_specialised(const DeviceModel& m) {
  static const bool forced_generic = [] {
    const char* e = std::getenv("MAGACE_GENERIC");
    return e && e[0] == '1';
  }();
  return !forced_generic && m.nd == 1 && !m.high && dims_match<FeDims>(m);
}

// Opts a kernel into `bytes` of dynamic shared memory, once per kernel,
// device and size: the attribute call is skipped when a launch needs no more
// than was already set, so evaluations captured into a CUDA graph issue none.
template <class K>
void set_smem(K* kernel, size_t bytes, bool max_carveout = false) {
  static std::map<std::pair<const void*, int>, size_t> done;
  int dev = 0;
  cudaGetDevice(&dev);
  size_t& cur = done[{reinterpret_cast<const void*>(kernel), dev}];
  if (bytes > cur) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
    // all of the unified L1 as shared memory, so that the CTAs per SM the
    // kernel's registers allow also fit its shared memory
    if (max_carveout)
      cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    cur = bytes;
  }
}

// Multiprocessors of the current device (queried once per device).
int sm_count() {
  static std::map<int, int> done;
  int dev = 0;
  cudaGetDevice(&dev);
  int& n = done[dev];
  if (n == 0) {
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

// How k_b3_fe splits the last, partial wave of its 32-atom blocks (one CTA
// per SM): with every block on its own CTA, the blocks beyond the last whole
// wave are each divided among `parts` CTAs (2 to 8, as many as the idle SMs
// allow), unless that wave is more than half full.
struct B3Split {
  int nfull, ntail, parts;
};
B3Split b3_split(int nblk, int grid_cap) {
  B3Split s{nblk, 0, 1};
  if (nblk > grid_cap) return s;
  const int nsm = sm_count();
  const int nfull = nblk / nsm * nsm, ntail = nblk - nfull;
  const int parts = ntail > 0 ? std::min(8, nsm / ntail) : 1;
  if (parts >= 2) s = {nfull, ntail, parts};
  return s;
}

// The split-precision scratch (EvalBuffers::aux): rho_rest[natom] and
// rho3[natom] doubles, the 3-body gradients g3[natom][nc] (FP32 complex; a
// buffer of their own, because the 2-/4-body kernel may still be reading the
// factors F while the 3-body kernel finishes), then one record per tail block of the 3-body kernel's split tail (the
// blocks B3Split divides, 256-byte aligned): rho3[32] doubles, a ticket
// (padded to 16 bytes) and the gradients g[nc][32][2] floats. The records in
// use are zeroed before each evaluation that splits.
struct AuxLayout {
  size_t rho3;        // the 3-body density per atom
  size_t g3;          // the 3-body gradients [natom][nc], FP32 complex
  size_t tail0, rec;  // first record, bytes per record
  size_t end;
};
AuxLayout aux_layout(const DeviceModel& m, int natom) {
  const auto up = [](size_t x) { return (x + 255) & ~static_cast<size_t>(255); };
  const int nblk = (natom + 31) / 32;
  const B3Split sp = b3_split(nblk, nblk);  // as if every block had its own CTA
  const size_t ntail = sp.parts > 1 ? static_cast<size_t>(sp.ntail) : 0;
  AuxLayout L;
  L.rho3 = up(sizeof(double) * static_cast<size_t>(natom));
  L.g3 = L.rho3 + up(sizeof(double) * static_cast<size_t>(natom));
  L.tail0 = L.g3 + up(sizeof(float) * 2 * static_cast<size_t>(m.b3_nc) * static_cast<size_t>(natom));
  L.rec = up(kTailG + sizeof(float) * 64 * static_cast<size_t>(m.b3_nc));
  L.end = L.tail0 + L.rec * ntail;
  return L;
}

// The FP64 scratch of the specialised layout (EvalBuffers::aux):
// rho_rest[natom] doubles, then k_b3_fe64's 64-bit fixed-point sums (zeroed
// before each evaluation, one range): the 3-body density r3i[P] and the
// gradients g3i[nblk][nc][32][2]; then their scales g3s[P] and r3s[P], where
// nblk = ceil(natom/32) and P = 32 nblk queue positions.
struct AuxLayout64 {
  size_t r3i, g3i, g3s, r3s, end;
};
AuxLayout64 aux_layout64(const DeviceModel& m, int natom) {
  const auto up = [](size_t x) { return (x + 255) & ~static_cast<size_t>(255); };
  const size_t nblk = (static_cast<size_t>(natom) + 31) / 32;
  AuxLayout64 L;
  L.r3i = up(sizeof(double) * static_cast<size_t>(natom));
  L.g3i = L.r3i + up(sizeof(unsigned long long) * 32 * nblk);
  L.g3s = L.g3i + up(sizeof(unsigned long long) * 64 * static_cast<size_t>(m.b3_nc) * nblk);
  L.r3s = L.g3s + up(sizeof(double) * 32 * nblk);
  L.end = L.r3s + up(sizeof(double) * 32 * nblk);
  return L;
}

// Resident CTAs of `kernel` on this device (a persistent grid), computed
// once per kernel and device so that captured evaluations make no query.
template <class K>
int resident_grid(K* kernel, int threads, size_t smem_bytes) {
  static std::map<std::pair<const void*, int>, int> done;
  int dev = 0;
  cudaGetDevice(&dev);
  int& g = done[{reinterpret_cast<const void*>(kernel), dev}];
  if (g == 0) {
    int per_sm = 0, nsm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem_bytes);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    g = (per_sm > 0 ? per_sm : 1) * (nsm > 0 ? nsm : 1);
  }
  return g;
}

// The A-basis phase: factors F, rank-1 density and core energy per atom.
// Split-precision variants (DeviceModel::tune_abasis): 0 scalar, 1 packed
// FP32x2, 2 scalar with the bond tiles staged by TMA, 3 the same on a
// persistent grid, 4 the bond sums on the tensor cores with TMA-staged tiles
// on a persistent grid, 5 the tensor-core sums alone; 2-4 run only when the
// bond inputs are device memory (EvalBuffers::dev_inputs), else 0 (for 2, 3)
// or 5 (for 4) runs.
template <class R>
void launch_abasis(const DeviceModel& m, const EvalBuffers& b, cudaStream_t st, int grid, bool fe) {
  const int natom = b.natom;
  if (fe) {
    int v = 0;
    if constexpr (sizeof(R) == 4) v = m.tune_abasis;
    if ((v == 2 || v == 3) && !b.dev_inputs) v = 0;
    if (v == 4 && !b.dev_inputs) v = 5;
#define MAGACE_ABASIS(PK, TMA, PERSIST, TC)                                                                        \
  {                                                                                                                 \
    const size_t s1 = abasis_fe_smem<R, FeDims, TC>();                                                              \
    const size_t sm = TMA ? ((s1 + 15) & ~static_cast<size_t>(15)) + kTileBarBytes : s1;                           \
    set_smem(k_abasis_fe<R, FeDims, PK, TMA, TC>, sm);                                                             \
    int g = grid;                                                                                                   \
    if (PERSIST) {                                                                                                  \
      const int rg = resident_grid(k_abasis_fe<R, FeDims, PK, TMA, TC>, 64, sm);                                    \
      g = natom < rg ? natom : rg;                                                                                  \
    }                                                                                                               \
    k_abasis_fe<R, FeDims, PK, TMA, TC><<<g, 64, sm, st>>>(m, natom, b.off, b.r, b.e, b.magj, b.mhj, b.magi,        \
                                                           b.mhi, reinterpret_cast<C<R>*>(b.F), b.rho1, b.core,    \
                                                           static_cast<R*>(b.stage), b.err);                        \
  }
    if constexpr (sizeof(R) == 4) {
      switch (v) {
        case 1: MAGACE_ABASIS(true, false, false, false); break;
        case 2: MAGACE_ABASIS(false, true, false, false); break;
        case 3: MAGACE_ABASIS(false, true, true, false); break;
        case 4: MAGACE_ABASIS(false, true, true, true); break;
        case 5: MAGACE_ABASIS(false, false, false, true); break;
        default: MAGACE_ABASIS(false, false, false, false); break;
      }
    } else {
      MAGACE_ABASIS(false, false, false, false);
    }
#undef MAGACE_ABASIS
  } else {
    const size_t s1 = abasis_smem<R>(m);
    set_smem(k_abasis<R>, s1);
    k_abasis<R><<<grid, kAbasisThreads, s1, st>>>(m, natom, b.off, b.r, b.e, b.magj, b.mhj, b.magi, b.mhi,
                                                   reinterpret_cast<C<R>*>(b.F), b.rho1, b.core, b.err);
  }
}

// The density phase: in split precision with the specialised layout,
// k_density_fe (2- and 4-body terms, one CTA per atom) and then k_b3_fe
// (3-body terms, 32 atoms per CTA; embedding and weights); otherwise one
// generic k_density. Returns the number of kernels launched.
template <class R>
int launch_density(const DeviceModel& m, const EvalBuffers& b, cudaStream_t st, int grid, int grid_cap, bool fe,
                   cudaEvent_t ev_between, int* kernels) {
  const int natom = b.natom;
  if constexpr (sizeof(R) == 4) {
    if (fe) {
      double* rho_rest = static_cast<double*>(b.aux);
      const int nblk = (natom + 31) / 32;
      const int gb = nblk < grid_cap ? nblk : grid_cap;
      const auto* Fp = reinterpret_cast<const C<float>*>(b.F);
      auto* Wp = reinterpret_cast<C<float>*>(b.W);
      const int rw = kRestWarpChoices[m.tune_rest], bw = kB3WarpChoices[m.tune_b3];
      (void)bw;
      const size_t s2 = density_fe_smem(m, rw);
      const AuxLayout al = aux_layout(m, natom);
      double* rho3 = reinterpret_cast<double*>(static_cast<unsigned char*>(b.aux) + al.rho3);
      auto* G3 = reinterpret_cast<C<float>*>(static_cast<unsigned char*>(b.aux) + al.g3);
      // the 2-/4-body kernel and the 3-body kernel are independent: with a
      // side stream (EvalBuffers::side) the first runs there, forked from and
      // joined back into `st` by events, so that either fills the SMs the
      // other's last wave leaves idle; k_finish_fe then adds their densities
      const bool fork = b.side != nullptr;
      cudaStream_t sr = fork ? b.side : st;
      if (fork) {
        cudaEventRecord(b.ev_fork, st);
        cudaStreamWaitEvent(sr, b.ev_fork, 0);
      }
#define MAGACE_REST(NW, SM)                                                                                   \
  set_smem(k_density_fe<FeDims, NW, SM>, s2);                                                                 \
  k_density_fe<FeDims, NW, SM><<<gb, NW * 32, s2, sr>>>(m, natom, Fp, Wp, rho_rest)
      // variants: 32 or 16 warps; per-entry uniform loads, record streams
      // broadcast by shuffles, or record streams through shared memory
      switch (m.tune_rest) {
        case 1: MAGACE_REST(16, 0); break;
        case 2: MAGACE_REST(32, 1); break;
        case 3: MAGACE_REST(16, 1); break;
        case 4: MAGACE_REST(32, 2); break;
        case 5: MAGACE_REST(16, 2); break;
        default: MAGACE_REST(32, 0); break;
      }
#undef MAGACE_REST
      if (ev_between) cudaEventRecord(ev_between, st);
      const size_t sb = b3_fe_smem<FeDims>(m, bw);
      // the last partial wave split by task range (B3Split); the records of
      // the tail blocks start at zero
      const B3Split sp = b3_split(nblk, grid_cap);
      unsigned char* tails = static_cast<unsigned char*>(b.aux) + al.tail0;
      if (sp.parts > 1) cudaMemsetAsync(tails, 0, al.rec * sp.ntail, st);
      const int g3 = sp.parts > 1 ? sp.nfull + sp.ntail * sp.parts : gb;
#define MAGACE_B3(NW, LOOP)                                                                                  \
  set_smem(k_b3_fe<FeDims, NW, LOOP>, sb);                                                                   \
  k_b3_fe<FeDims, NW, LOOP><<<g3, NW * 32, sb, st>>>(m, natom, Fp, G3, rho3, b.err, sp.nfull, sp.parts, tails,  \
                                                     al.rec)
      // variants: (16 warps, n0' innermost), (12, innermost), (8, innermost),
      // (12, n0' outermost), (16, packed FP32x2), (12, packed FP32x2)
      switch (m.tune_b3) {
        case 1: MAGACE_B3(12, 0); break;
        case 2: MAGACE_B3(8, 0); break;
        case 3: MAGACE_B3(12, 1); break;
        case 4: MAGACE_B3(16, 2); break;
        case 5: MAGACE_B3(12, 2); break;
        default: MAGACE_B3(16, 0); break;
      }
#undef MAGACE_B3
      if (fork) {
        cudaEventRecord(b.ev_join, sr);
        cudaStreamWaitEvent(st, b.ev_join, 0);
      }
      // 64 threads per CTA: the FP64 embedding of every atom spread over all SMs
      const int gf = (natom + 63) / 64;
      k_finish_fe<<<gf, 64, 0, st>>>(m, natom, b.rho1, rho_rest, rho3, b.core, b.energy, b.edf, b.dedrho, b.err);
      if (kernels) *kernels += 3;
      return 2;
    }
  }
  if constexpr (sizeof(R) == 8) {
    if (fe) {
      // FP64, specialised layout: the 2-/4-body terms through the rest table
      // (k_rest64) on the side stream, beside the dense 3-body kernel
      // k_b3_fe64 on `st`; then k_finish_fe (density, embedding, inner cutoff)
      const AuxLayout64 al = aux_layout64(m, natom);
      unsigned char* aux = static_cast<unsigned char*>(b.aux);
      double* rho_rest = reinterpret_cast<double*>(aux);
      auto* r3i = reinterpret_cast<unsigned long long*>(aux + al.r3i);
      auto* g3i = reinterpret_cast<unsigned long long*>(aux + al.g3i);
      double* g3s = reinterpret_cast<double*>(aux + al.g3s);
      double* r3s = reinterpret_cast<double*>(aux + al.r3s);
      const bool fork = b.side != nullptr;
      cudaStream_t sr = fork ? b.side : st;
      if (fork) {
        cudaEventRecord(b.ev_fork, st);
        cudaStreamWaitEvent(sr, b.ev_fork, 0);
      }
      const size_t s2 = rest64_smem<FeDims>(m);
      set_smem(k_rest64<FeDims, kRestWarps64>, s2);
      const int nb16 = (natom + 15) / 16;
      k_rest64<FeDims, kRestWarps64><<<std::min(nb16, grid_cap), kRestWarps64 * 32, s2, sr>>>(
          m, natom, reinterpret_cast<const C<double>*>(b.F), reinterpret_cast<C<double>*>(b.W), rho_rest);
      if (ev_between) cudaEventRecord(ev_between, st);
      cudaMemsetAsync(r3i, 0, al.g3s - al.r3i, st);
      const size_t sb = b3_fe64_smem<FeDims>(m);
      set_smem(k_b3_fe64<FeDims, kB3Warps64>, sb);
      // one CTA per block, the last partial wave split by task range (B3Split)
      const int nblk = (natom + 31) / 32;
      const B3Split sp = b3_split(nblk, grid_cap);
      const int gb = sp.parts > 1 ? sp.nfull + sp.ntail * sp.parts : std::min(nblk, grid_cap);
      k_b3_fe64<FeDims, kB3Warps64><<<gb, kB3Warps64 * 32, sb, st>>>(
          m, natom, reinterpret_cast<const C<double>*>(b.F), g3i, g3s, r3i, r3s, b.err, sp.nfull, sp.parts);
      if (fork) {
        cudaEventRecord(b.ev_join, sr);
        cudaStreamWaitEvent(st, b.ev_join, 0);
      }
      const int gf = (natom + 63) / 64;
      k_finish_fe<<<gf, 64, 0, st>>>(m, natom, b.rho1, rho_rest, nullptr, b.core, b.energy, b.edf, b.dedrho, b.err,
                                     r3i, r3s);
      if (kernels) *kernels += 3;
      return 2;
    }
  }
  const size_t s2 = density_smem<R>(m);
  if (m.nd == 1) {
    set_smem(k_density<R, 1>, s2);
    k_density<R, 1><<<grid, kDensityThreads, s2, st>>>(m, natom, reinterpret_cast<const C<R>*>(b.F), b.rho1, b.core,
                                                       reinterpret_cast<C<R>*>(b.W), b.energy, b.edf, b.dedrho, b.err);
  } else {
    set_smem(k_density<R, 2>, s2);
    k_density<R, 2><<<grid, kDensityThreads, s2, st>>>(m, natom, reinterpret_cast<const C<R>*>(b.F), b.rho1, b.core,
                                                       reinterpret_cast<C<R>*>(b.W), b.energy, b.edf, b.dedrho, b.err);
  }
  if (kernels) *kernels += 1;
  return 1;
}

template <class R>
int launch_eval(const DeviceModel& m0, const EvalBuffers& b, cudaStream_t st, int grid_cap, cudaEvent_t* ev,
                int* kernels) {
  DeviceModel m = m0;
  m.order = b.order;
  const int natom = b.natom;
  if (natom <= 0) return 0;
  const int grid = natom < grid_cap ? natom : grid_cap;
  const bool fe = use_specialised(m);
  if (ev) cudaEventRecord(ev[0], st);
  launch_abasis<R>(m, b, st, grid, fe);
  if (ev) cudaEventRecord(ev[1], st);
  int nk = 2;  // the A-basis and force kernels
  const int nd = launch_density<R>(m, b, st, grid, grid_cap, fe, ev ? ev[2] : nullptr, &nk);
  const int nlaunch = 2 + nd;
  if (kernels) *kernels = nk;
  if (ev) cudaEventRecord(ev[1 + nd], st);
  if (fe) {
    // split precision: the 3-body kernel's part of the weights (g3 in aux)
    const C<float>* g3 =
        sizeof(R) == 4 ? reinterpret_cast<const C<float>*>(static_cast<unsigned char*>(b.aux) +
                                                           aux_layout(m, natom).g3)
                       : nullptr;
    // FP64: k_b3_fe64's fixed-point gradients and their block scales
    const unsigned long long* g3i = nullptr;
    const double* g3s = nullptr;
    if (sizeof(R) == 8) {
      const AuxLayout64 al = aux_layout64(m, natom);
      g3i = reinterpret_cast<const unsigned long long*>(static_cast<unsigned char*>(b.aux) + al.g3i);
      g3s = reinterpret_cast<const double*>(static_cast<unsigned char*>(b.aux) + al.g3s);
    }
    // outputs in host memory (acelib_ writing the caller's arrays directly):
    // the variants that store each tile's outputs as whole lines
#define MAGACE_FORCES_SO(MB, PK, SO)                                                                                \
  {                                                                                                                 \
    const size_t s3 = forces_fe_smem<R, FeDims>(SO);                                                                \
    set_smem(k_forces_fe<R, FeDims, MB, PK, SO, sizeof(R) == 8>, s3);                                               \
    k_forces_fe<R, FeDims, MB, PK, SO, sizeof(R) == 8><<<grid, 64, s3, st>>>(m, natom, b.off, b.r, b.e, b.magj,      \
                                                                           b.mhj, b.magi,                           \
                                                             b.mhi, reinterpret_cast<const C<R>*>(b.W), b.edf,      \
                                                             b.dedrho, b.fij, b.tij, b.ti0,                         \
                                                             static_cast<const R*>(b.stage), b.err, g3, g3i, g3s);  \
  }
#define MAGACE_FORCES(MB, PK)                 \
  if (b.host_outputs) {                       \
    MAGACE_FORCES_SO(MB, PK, true);           \
  } else {                                    \
    MAGACE_FORCES_SO(MB, PK, false);          \
  }
    // the contractions on the tensor cores (k_forces_tc, split precision only)
#define MAGACE_FORCES_TC_SO(MB, SO)                                                                                 \
  {                                                                                                                 \
    const size_t s3 = forces_tc_smem<FeDims>(SO);                                                                   \
    set_smem(k_forces_tc<FeDims, MB, SO>, s3, true);                                                                \
    k_forces_tc<FeDims, MB, SO><<<grid, 64, s3, st>>>(m, natom, b.off, b.r, b.e, b.magj, b.mhj, b.magi, b.mhi,      \
                                                      reinterpret_cast<const C<float>*>(b.W), b.edf, b.dedrho,      \
                                                      b.fij, b.tij, b.ti0, static_cast<const float*>(b.stage),      \
                                                      b.err, g3);                                                   \
  }
#define MAGACE_FORCES_TC(MB)                  \
  if (b.host_outputs) {                       \
    MAGACE_FORCES_TC_SO(MB, true);            \
  } else {                                    \
    MAGACE_FORCES_TC_SO(MB, false);           \
  }
    if constexpr (sizeof(R) == 8) {
      MAGACE_FORCES(4, false);
    } else {
      // variants: CTAs per SM 4 / 6 / 8, scalar then packed FP32x2; then
      // the tensor-core form at 5 / 6 CTAs per SM
      switch (m.tune_forces) {
        case 1: MAGACE_FORCES(6, false); break;
        case 2: MAGACE_FORCES(8, false); break;
        case 3: MAGACE_FORCES(4, true); break;
        case 4: MAGACE_FORCES(6, true); break;
        case 5: MAGACE_FORCES(8, true); break;
        case 6: MAGACE_FORCES_TC(5); break;
        case 7: MAGACE_FORCES_TC(6); break;
        default: MAGACE_FORCES(4, false); break;
      }
    }
#undef MAGACE_FORCES
#undef MAGACE_FORCES_SO
#undef MAGACE_FORCES_TC
#undef MAGACE_FORCES_TC_SO
  } else {
    const size_t s3 = forces_smem<R>(m, kForceThreads);
    set_smem(k_forces<R>, s3);
    k_forces<R><<<grid, kForceThreads, s3, st>>>(m, natom, b.off, b.r, b.e, b.magj, b.mhj, b.magi, b.mhi,
                                                  reinterpret_cast<const C<R>*>(b.W), b.edf, b.dedrho, b.fij, b.tij,
                                                  b.ti0, b.err);
  }
  if (ev) cudaEventRecord(ev[nlaunch], st);
  return nlaunch;
}

size_t eval_aux_bytes(const DeviceModel& m, int precision, int natom) {
  // the specialised kernels' per-atom densities and 3-body gradients
  // (aux_layout, aux_layout64)
  if (!use_specialised(m) || natom <= 0) return 0;
  return precision == 0 ? aux_layout64(m, natom).end : aux_layout(m, natom).end;
}

size_t eval_aux_bytes_bound(const DeviceModel& m, int precision, int natom) {
  // as eval_aux_bytes, with room for the most tail records any split can
  // use (a split tail has at most half an SM count of blocks, and never more
  // blocks than there are), so that the bound never falls as natom grows
  if (!use_specialised(m) || natom <= 0) return 0;
  if (precision == 0) return aux_layout64(m, natom).end;
  const AuxLayout L = aux_layout(m, natom);
  const size_t nblk = (static_cast<size_t>(natom) + 31) / 32;
  const size_t half = static_cast<size_t>(sm_count()) / 2;
  return L.tail0 + L.rec * (nblk < half ? nblk : half);
}

size_t eval_smem_bytes(const DeviceModel& m, int precision, int which) {
  if (use_specialised(m)) {
    if (precision == 0) {
      if (which == 0) return abasis_fe_smem<double, FeDims>();
      if (which == 1) {
        const size_t a = rest64_smem<FeDims>(m), b = b3_fe64_smem<FeDims>(m);
        return a > b ? a : b;
      }
      return forces_fe_smem<double, FeDims>(true);
    }
    if (which == 0) return abasis_fe_smem<float, FeDims, true>();
    if (which == 1) {
      const size_t a = density_fe_smem(m, 32), b = b3_fe_smem<FeDims>(m, 16);
      return a > b ? a : b;
    }
    return std::max(forces_fe_smem<float, FeDims>(true), forces_tc_smem<FeDims>(true));
  }
  if (precision == 0) {
    if (which == 0) return abasis_smem<double>(m);
    if (which == 1) return density_smem<double>(m);
    return forces_smem<double>(m, kForceThreads);
  }
  if (which == 0) return abasis_smem<float>(m);
  if (which == 1) return density_smem<float>(m);
  return forces_smem<float>(m, kForceThreads);
}

// ===========================================================================
// Work queue: atoms in order of decreasing bond count, so that the
// persistent CTAs, which take queue positions round-robin, meet the largest
// atoms first and similar ones in each round (a longest-first schedule for
// batches of uneven configurations). Counting sort; atoms of equal clipped
// count keep no particular order (each atom's result does not depend on it).
__global__ void k_queue_hist(int natom, const int* __restrict__ off, int* __restrict__ bins) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < natom; a += gridDim.x * blockDim.x) {
    const int c = min(off[a + 1] - off[a], kQueueBins - 1);
    atomicAdd(&bins[kQueueBins - 1 - c], 1);  // bin 0 holds the largest count
  }
}
__global__ void k_queue_scan(int* __restrict__ bins) {
  // one warp: exclusive prefix sum of kQueueBins counts into the cursors
  __shared__ int s[kQueueBins];
  for (int k = threadIdx.x; k < kQueueBins; k += blockDim.x) s[k] = bins[k];
  __syncwarp();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int k = 0; k < kQueueBins; ++k) {
      const int c = s[k];
      s[k] = run;
      run += c;
    }
  }
  __syncwarp();
  for (int k = threadIdx.x; k < kQueueBins; k += blockDim.x) bins[kQueueBins + k] = s[k];
}
__global__ void k_queue_place(int natom, const int* __restrict__ off, int* __restrict__ bins, int* __restrict__ order) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < natom; a += gridDim.x * blockDim.x) {
    const int c = min(off[a + 1] - off[a], kQueueBins - 1);
    order[atomicAdd(&bins[kQueueBins + kQueueBins - 1 - c], 1)] = a;
  }
}

void launch_work_queue(int natom, const int* off, int* order, int* bins, cudaStream_t st) {
  if (natom <= 0) return;
  cudaMemsetAsync(bins, 0, sizeof(int) * kQueueBins, st);
  const int blocks = (natom + 255) / 256 < 1024 ? (natom + 255) / 256 : 1024;
  k_queue_hist<<<blocks, 256, 0, st>>>(natom, off, bins);
  k_queue_scan<<<1, 32, 0, st>>>(bins);
  k_queue_place<<<blocks, 256, 0, st>>>(natom, off, bins, order);
}

// ===========================================================================
// k_descriptors: one CTA per atom, FP64. B[atom][k] for every cluster in
// coefficient order: rank 1, g_n(|m_i|) - 1 (src/b_basis.F90:74-83); ranks
// 2..6, Re sum over the cluster's m-terms of cf * F[o0] .. F[o5] (missing
// factors ONE; src/b_basis.F90:91-532 without the coefficients).
constexpr int kDescThreads = 128;

__global__ void __launch_bounds__(kDescThreads)
    k_descriptors(DeviceModel m, int natom, const C<double>* __restrict__ F, const double* __restrict__ magi,
                  double* __restrict__ B, int* err) {
  extern __shared__ __align__(16) unsigned char smem[];
  C<double>* Fs = reinterpret_cast<C<double>*>(smem);
  const int nB = m.d_nB, n1 = m.d_n1;
  for (int it = blockIdx.x; it < natom; it += gridDim.x) {
    const int atom = queue_atom(m, it);
    const C<double>* Fa = F + static_cast<size_t>(atom) * m.nF;
    for (int s = threadIdx.x; s < m.nF; s += blockDim.x) Fs[s] = Fa[s];
    __syncthreads();
    double* Ba = B + static_cast<size_t>(atom) * nB;
    for (int k = threadIdx.x; k < n1; k += blockDim.x) {
      double wl = 0.0, g = 1.0, dummy[1];
      const int nl = magnetic_bin(m, magi[atom], wl, err);
      if (nl > 0) {
        lut_eval<false>(m.lut_m, m.nfm, m.n2m * (m.l2m + 1) + m.d_rank1_n[k], 1, nl, wl, m.rscale_m, &g, dummy);
      } else if (nl < 0) {
        g = 0.0;
      }
      Ba[k] = g - 1.0;
    }
    for (int k = threadIdx.x; k < nB - n1; k += blockDim.x) {
      double acc = 0.0;
      for (int e = m.d_begin[k]; e < m.d_begin[k + 1]; ++e) {
        const uint4 q = __ldg(reinterpret_cast<const uint4*>(m.d_o + kDescFactors * static_cast<size_t>(e)));
        const C<double> p = cmul(cmul(cmul(Fs[q.x & 0xffffu], Fs[q.x >> 16]), cmul(Fs[q.y & 0xffffu], Fs[q.y >> 16])),
                                 cmul(Fs[q.z & 0xffffu], Fs[q.z >> 16]));
        acc += m.d_cf[e] * p.x;
      }
      Ba[n1 + k] = acc;
    }
    __syncthreads();
  }
}

int launch_descriptors(const DeviceModel& m0, const EvalBuffers& b, double* B, cudaStream_t st, int grid_cap) {
  DeviceModel m = m0;
  m.order = b.order;
  const int natom = b.natom;
  if (natom <= 0) return 0;
  const int grid = natom < grid_cap ? natom : grid_cap;
  launch_abasis<double>(m, b, st, grid, use_specialised(m));
  const size_t sd = sizeof(C<double>) * static_cast<size_t>(m.nF);
  set_smem(k_descriptors, sd);
  k_descriptors<<<grid, kDescThreads, sd, st>>>(m, natom, reinterpret_cast<const C<double>*>(b.F), b.magi, B, b.err);
  return 2;
}

// ===========================================================================
// Tangents for the coefficient gradients of force losses. Along a
// displacement field (bond-vector tangents dd_ij = u_i - u_j and moment
// tangents dm), k_abasis_tangent evaluates the factors F (as k_abasis in
// FP64) and their directional derivatives Fd, with
//   dr = e . dd,  d(R Y_lm(e)) = R' dr Y + R (dY . dd) / r,
//   d|m| = m_hat . dm,  d(M Y(m_hat)) = M' d|m| Y + M (dY . dm) / |m|,
// (dY the tangential gradient of ylm_half; the force kernels use the same
// derivatives), and the core energy and its derivative.
// k_descriptors_tangent then forms B and dB of every cluster by dual-number
// products: (p, dp) (f, df) = (p f, dp f + p df). One CTA per atom, FP64.
__global__ void __launch_bounds__(kAbasisThreads)
    k_abasis_tangent(DeviceModel m, int natom, const int* __restrict__ off, const double* __restrict__ rr,
                     const double* __restrict__ ee, const double* __restrict__ magj, const double* __restrict__ mhj,
                     const double* __restrict__ magi, const double* __restrict__ mhi, const double* __restrict__ dd,
                     const double* __restrict__ dmj, const double* __restrict__ dmi, C<double>* __restrict__ F,
                     C<double>* __restrict__ Fd, double* __restrict__ core_out, double* __restrict__ cored_out,
                     int* err) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int TB = kAbasisTile;
  const int nA2h = m.nba * m.n2m * m.h2;
  const int nacc = m.nWA + nA2h;
  const int nRY = m.n3a * m.lsa, nQ = m.n2m * m.h2;
  C<double>* acc = reinterpret_cast<C<double>*>(smem);  // [nacc] value, then [nacc] tangent
  C<double>* accd = acc + nacc;
  C<double>* sRY = accd + nacc;   // [nRY][TB]
  C<double>* sRYd = sRY + nRY * TB;
  C<double>* sQ = sRYd + nRY * TB;  // [nQ][TB]
  C<double>* sQd = sQ + nQ * TB;
  double* sg = reinterpret_cast<double*>(sQd + nQ * TB);  // [nba][TB]
  double* sgd = sg + m.nba * TB;
  double* score = sgd + m.nba * TB;  // [TB] value, then [TB] tangent
  __shared__ double s_core[2];
  for (int it = blockIdx.x; it < natom; it += gridDim.x) {
    const int atom = queue_atom(m, it);
    for (int s = threadIdx.x; s < 2 * nacc; s += blockDim.x) acc[s] = {0.0, 0.0};
    if (threadIdx.x == 0) s_core[0] = s_core[1] = 0.0;
    const int b0 = off[atom], b1 = off[atom + 1];
    __syncthreads();
    for (int t0 = b0; t0 < b1; t0 += TB) {
      const int nb = min(TB, b1 - t0);
      if (threadIdx.x < nb) {
        const int b = threadIdx.x, j = t0 + b;
        const double r = rr[j];
        const double e[3] = {ee[3 * j], ee[3 * j + 1], ee[3 * j + 2]};
        const double dv[3] = {dd[3 * j], dd[3 * j + 1], dd[3 * j + 2]};
        const double rdot = e[0] * dv[0] + e[1] * dv[1] + e[2] * dv[2];
        double g[kMaxFeat], gd[kMaxFeat], Rv[kMaxFeat], Rd[kMaxFeat], cv[1], cd[1], Mv[kMaxFeat], Md[kMaxFeat];
        double wl = 0.0;
        const int nla = atomic_bin(m, r, wl, err);
        const int nR = m.n3a * (m.l3a + 1), nM = m.n2m * (m.l2m + 1);
        if (nla > 0) {
          lut_eval<true>(m.lut_a, m.nfa, 0, m.nba, nla, wl, m.rscale_a, g, gd);
          lut_eval<true>(m.lut_a, m.nfa, m.nba, nR, nla, wl, m.rscale_a, Rv, Rd);
          lut_eval<true>(m.lut_a, m.nfa, m.nba + nR, 1, nla, wl, m.rscale_a, cv, cd);
        } else {
          for (int q = 0; q < m.nba; ++q) g[q] = gd[q] = 0.0;
          for (int q = 0; q < nR; ++q) Rv[q] = Rd[q] = 0.0;
          cv[0] = cd[0] = 0.0;
        }
        const double mg = magj[j];
        const double mh[3] = {mhj[3 * j], mhj[3 * j + 1], mhj[3 * j + 2]};
        const double dm[3] = {dmj[3 * j], dmj[3 * j + 1], dmj[3 * j + 2]};
        const double mgdot = mh[0] * dm[0] + mh[1] * dm[1] + mh[2] * dm[2];
        double wm = 0.0;
        const int nlm = magnetic_bin(m, mg, wm, err);
        if (nlm > 0) {
          lut_eval<true>(m.lut_m, m.nfm, 0, nM, nlm, wm, m.rscale_m, Mv, Md);
        } else {
          for (int q = 0; q < nM; ++q) {
            Mv[q] = nlm == 0 ? 1.0 : 0.0;
            Md[q] = 0.0;
          }
        }
        C<double> Ya[kMaxHalf], dYa[kMaxHalf][3], Ym[kMaxHalf], dYm[kMaxHalf][3];
        ylm_half<double, true>(m.l3a, e[0], e[1], e[2], Ya, dYa);
        ylm_half<double, true>(m.l2m, mh[0], mh[1], mh[2], Ym, dYm);
        const double ir = 1.0 / r, im = mg > 0.0 ? 1.0 / mg : 0.0;
        for (int l1 = 0; l1 <= m.l3a; ++l1)
          for (int m1 = -l1; m1 <= l1; ++m1) {
            const int k = ph(l1, m1 < 0 ? -m1 : m1);
            C<double> yd = {0.0, 0.0};
            for (int c = 0; c < 3; ++c) {
              yd.x = fma(dYa[k][c].x, dv[c], yd.x);
              yd.y = fma(dYa[k][c].y, dv[c], yd.y);
            }
            yd = cscale(yd, ir);
            if (m1 < 0) {
              const double sgn = parity(m1);
              yd = {yd.x * sgn, -yd.y * sgn};
            }
            const C<double> y = y_full(Ya, l1, m1);
            for (int n1 = 0; n1 < m.n3a; ++n1) {
              const int q = n1 * (m.l3a + 1) + l1, i = n1 * m.lsa + l1 * l1 + l1 + m1;
              sRY[i * TB + b] = cscale(y, Rv[q]);
              sRYd[i * TB + b] = {Rd[q] * rdot * y.x + Rv[q] * yd.x, Rd[q] * rdot * y.y + Rv[q] * yd.y};
            }
          }
        for (int l = 0; l <= m.l2m; ++l)
          for (int mm = 0; mm <= l; ++mm) {
            const int k = ph(l, mm);
            C<double> yd = {0.0, 0.0};
            for (int c = 0; c < 3; ++c) {
              yd.x = fma(dYm[k][c].x, dm[c], yd.x);
              yd.y = fma(dYm[k][c].y, dm[c], yd.y);
            }
            yd = cscale(yd, im);
            for (int nr = 0; nr < m.n2m; ++nr) {
              const int q = nr * (m.l2m + 1) + l, i = nr * m.h2 + k;
              sQ[i * TB + b] = cscale(Ym[k], Mv[q]);
              sQd[i * TB + b] = {Md[q] * mgdot * Ym[k].x + Mv[q] * yd.x, Md[q] * mgdot * Ym[k].y + Mv[q] * yd.y};
            }
          }
        for (int n = 0; n < m.nba; ++n) {
          sg[n * TB + b] = g[n];
          sgd[n * TB + b] = gd[n] * rdot;
        }
        score[b] = cv[0];
        score[TB + b] = cd[0] * rdot;
      }
      __syncthreads();
      for (int s = threadIdx.x; s < nacc; s += blockDim.x) {
        C<double> a = acc[s], ad = accd[s];
        if (s < m.nWA) {
          const int h = s % m.h3, q = s / m.h3, n2 = q % m.n3m, ia = q / m.n3m;
          const C<double>* ry = sRY + ia * TB;
          const C<double>* ryd = sRYd + ia * TB;
          const C<double>* qq = sQ + (n2 * m.h2 + h) * TB;
          const C<double>* qd = sQd + (n2 * m.h2 + h) * TB;
          for (int b = 0; b < nb; ++b) {
            cmac(a, ry[b], qq[b]);
            cmac(ad, ryd[b], qq[b]);
            cmac(ad, ry[b], qd[b]);
          }
        } else {
          const int t = s - m.nWA, h = t % m.h2, q = t / m.h2, nr = q % m.n2m, n = q / m.n2m;
          const double* gg = sg + n * TB;
          const double* ggd = sgd + n * TB;
          const C<double>* qq = sQ + (nr * m.h2 + h) * TB;
          const C<double>* qd = sQd + (nr * m.h2 + h) * TB;
          for (int b = 0; b < nb; ++b) {
            a.x = fma(gg[b], qq[b].x, a.x);
            a.y = fma(gg[b], qq[b].y, a.y);
            ad.x = fma(ggd[b], qq[b].x, fma(gg[b], qd[b].x, ad.x));
            ad.y = fma(ggd[b], qq[b].y, fma(gg[b], qd[b].y, ad.y));
          }
        }
        acc[s] = a;
        accd[s] = ad;
      }
      if (threadIdx.x == 0)
        for (int b = 0; b < nb; ++b) {
          s_core[0] += score[b];
          s_core[1] += score[TB + b];
        }
      __syncthreads();
    }
    // full A and A2 (m' < 0 by conjugate symmetry, linear: the same for the tangent)
    for (int pass = 0; pass < 2; ++pass) {
      const C<double>* src = pass ? accd : acc;
      C<double>* Fa = (pass ? Fd : F) + static_cast<size_t>(atom) * m.nF;
      const int nA = m.offA2 - m.offA;
      for (int s = threadIdx.x; s < nA; s += blockDim.x) {
        const int lmm = s % m.ls3, q = s / m.ls3, n2 = q % m.n3m, ia = q / m.n3m;
        const int n1 = ia / m.lsa, lma = ia % m.lsa;
        int l2 = 0;
        while ((l2 + 1) * (l2 + 1) <= lmm) ++l2;
        const int m2 = lmm - l2 * l2 - l2;
        int l1 = 0;
        while ((l1 + 1) * (l1 + 1) <= lma) ++l1;
        const int m1 = lma - l1 * l1 - l1;
        C<double> v;
        if (m2 >= 0) {
          v = src[((n1 * m.lsa + lma) * m.n3m + n2) * m.h3 + ph(l2, m2)];
        } else {
          const int lmb = l1 * l1 + l1 - m1;
          const C<double> w = src[((n1 * m.lsa + lmb) * m.n3m + n2) * m.h3 + ph(l2, -m2)];
          const double sgn = parity(m1 + m2);
          v = {w.x * sgn, -w.y * sgn};
        }
        Fa[m.offA + s] = v;
      }
      const int nA2 = m.offA0 - m.offA2;
      for (int s = threadIdx.x; s < nA2; s += blockDim.x) {
        const int lm = s % m.ls2, q = s / m.ls2;
        int l = 0;
        while ((l + 1) * (l + 1) <= lm) ++l;
        const int mm = lm - l * l - l;
        const C<double> w = src[m.nWA + q * m.h2 + ph(l, mm < 0 ? -mm : mm)];
        C<double> v = w;
        if (mm < 0) {
          const double sgn = parity(mm);
          v = {w.x * sgn, -w.y * sgn};
        }
        Fa[m.offA2 + s] = v;
      }
    }
    if (threadIdx.x == 0) {
      // on-site A0 and its tangent, the constants
      C<double>* Fa = F + static_cast<size_t>(atom) * m.nF;
      C<double>* Fda = Fd + static_cast<size_t>(atom) * m.nF;
      const double mg = magi[atom];
      const double mh[3] = {mhi[3 * atom], mhi[3 * atom + 1], mhi[3 * atom + 2]};
      const double dm[3] = {dmi[3 * atom], dmi[3 * atom + 1], dmi[3 * atom + 2]};
      const double mgdot = mh[0] * dm[0] + mh[1] * dm[1] + mh[2] * dm[2], im = mg > 0.0 ? 1.0 / mg : 0.0;
      double wl = 0.0, Mv[32], Md[32];
      const int nl = magnetic_bin(m, mg, wl, err);
      const int nM = m.n2m * (m.l2m + 1);
      if (nl > 0) {
        lut_eval<true>(m.lut_m, m.nfm, 0, nM, nl, wl, m.rscale_m, Mv, Md);
      } else {
        for (int q = 0; q < nM; ++q) {
          Mv[q] = nl == 0 ? 1.0 : 0.0;
          Md[q] = 0.0;
        }
      }
      C<double> Yi[kMaxHalf], dYi[kMaxHalf][3];
      ylm_half<double, true>(m.l2m, mh[0], mh[1], mh[2], Yi, dYi);
      for (int l = 0; l <= m.l2m; ++l)
        for (int mm = -l; mm <= l; ++mm) {
          const int k = ph(l, mm < 0 ? -mm : mm);
          C<double> yd = {0.0, 0.0};
          for (int c = 0; c < 3; ++c) {
            yd.x = fma(dYi[k][c].x, dm[c], yd.x);
            yd.y = fma(dYi[k][c].y, dm[c], yd.y);
          }
          yd = cscale(yd, im);
          if (mm < 0) {
            const double sgn = parity(mm);
            yd = {yd.x * sgn, -yd.y * sgn};
          }
          const C<double> y = y_full(Yi, l, mm);
          for (int nr = 0; nr < m.n2m; ++nr) {
            const int q = nr * (m.l2m + 1) + l, f = m.offA0 + nr * m.ls2 + l * l + l + mm;
            Fa[f] = cscale(y, Mv[q]);
            Fda[f] = {Md[q] * mgdot * y.x + Mv[q] * yd.x, Md[q] * mgdot * y.y + Mv[q] * yd.y};
          }
        }
      Fa[m.offOne] = {1.0, 0.0};
      Fa[m.offZero] = {0.0, 0.0};
      Fda[m.offOne] = {0.0, 0.0};
      Fda[m.offZero] = {0.0, 0.0};
      core_out[atom] = s_core[0];
      cored_out[atom] = s_core[1];
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kDescThreads)
    k_descriptors_tangent(DeviceModel m, int natom, const C<double>* __restrict__ F, const C<double>* __restrict__ Fd,
                          const double* __restrict__ magi, const double* __restrict__ mhi,
                          const double* __restrict__ dmi, double* __restrict__ B, double* __restrict__ Bd, int* err) {
  extern __shared__ __align__(16) unsigned char smem[];
  C<double>* Fs = reinterpret_cast<C<double>*>(smem);
  C<double>* Fds = Fs + m.nF;
  const int nB = m.d_nB, n1 = m.d_n1;
  for (int it = blockIdx.x; it < natom; it += gridDim.x) {
    const int atom = queue_atom(m, it);
    for (int s = threadIdx.x; s < m.nF; s += blockDim.x) {
      Fs[s] = F[static_cast<size_t>(atom) * m.nF + s];
      Fds[s] = Fd[static_cast<size_t>(atom) * m.nF + s];
    }
    __syncthreads();
    double* Ba = B + static_cast<size_t>(atom) * nB;
    double* Bda = Bd + static_cast<size_t>(atom) * nB;
    // rank 1: g_n(|m_i|) - 1 and g_n' (m_hat_i . dm_i)
    for (int k = threadIdx.x; k < n1; k += blockDim.x) {
      double wl = 0.0, g = 1.0, gd = 0.0;
      const int nl = magnetic_bin(m, magi[atom], wl, err);
      if (nl > 0) {
        lut_eval<true>(m.lut_m, m.nfm, m.n2m * (m.l2m + 1) + m.d_rank1_n[k], 1, nl, wl, m.rscale_m, &g, &gd);
      } else if (nl < 0) {
        g = 0.0;
      }
      const double mgdot =
          mhi[3 * atom] * dmi[3 * atom] + mhi[3 * atom + 1] * dmi[3 * atom + 1] + mhi[3 * atom + 2] * dmi[3 * atom + 2];
      Ba[k] = g - 1.0;
      Bda[k] = gd * mgdot;
    }
    for (int k = threadIdx.x; k < nB - n1; k += blockDim.x) {
      double acc = 0.0, accd = 0.0;
      for (int e = m.d_begin[k]; e < m.d_begin[k + 1]; ++e) {
        const uint4 q = __ldg(reinterpret_cast<const uint4*>(m.d_o + kDescFactors * static_cast<size_t>(e)));
        const unsigned o[6] = {q.x & 0xffffu, q.x >> 16, q.y & 0xffffu, q.y >> 16, q.z & 0xffffu, q.z >> 16};
        C<double> p = Fs[o[0]], pd = Fds[o[0]];
        for (int f = 1; f < 6; ++f) {
          const C<double> v = Fs[o[f]], vd = Fds[o[f]];
          pd = cmul(pd, v);
          cmac(pd, p, vd);
          p = cmul(p, v);
        }
        acc += m.d_cf[e] * p.x;
        accd += m.d_cf[e] * pd.x;
      }
      Ba[n1 + k] = acc;
      Bda[n1 + k] = accd;
    }
    __syncthreads();
  }
}

int launch_descriptors_tangent(const DeviceModel& m0, const EvalBuffers& b, const double* dd, const double* dmj,
                               const double* dmi, void* Fd, double* B, double* Bd, double* core, double* cored,
                               cudaStream_t st, int grid_cap) {
  DeviceModel m = m0;
  m.order = b.order;
  const int natom = b.natom;
  if (natom <= 0) return 0;
  const int grid = natom < grid_cap ? natom : grid_cap;
  const int TB = kAbasisTile;
  const size_t nacc = static_cast<size_t>(m.nWA) + static_cast<size_t>(m.nba) * m.n2m * m.h2;
  const size_t sa = sizeof(C<double>) * (2 * nacc + 2 * static_cast<size_t>(m.n3a) * m.lsa * TB +
                                         2 * static_cast<size_t>(m.n2m) * m.h2 * TB) +
                    sizeof(double) * (2 * static_cast<size_t>(m.nba) * TB + 2 * TB);
  set_smem(k_abasis_tangent, sa);
  k_abasis_tangent<<<grid, kAbasisThreads, sa, st>>>(m, natom, b.off, b.r, b.e, b.magj, b.mhj, b.magi, b.mhi, dd, dmj,
                                                     dmi, reinterpret_cast<C<double>*>(b.F),
                                                     reinterpret_cast<C<double>*>(Fd), core, cored, b.err);
  const size_t sd = 2 * sizeof(C<double>) * static_cast<size_t>(m.nF);
  set_smem(k_descriptors_tangent, sd);
  k_descriptors_tangent<<<grid, kDescThreads, sd, st>>>(m, natom, reinterpret_cast<const C<double>*>(b.F),
                                                        reinterpret_cast<const C<double>*>(Fd), b.magi, b.mhi, dmi, B,
                                                        Bd, b.err);
  return 2;
}

size_t descriptors_tangent_smem(const DeviceModel& m) {
  const int TB = kAbasisTile;
  const size_t nacc = static_cast<size_t>(m.nWA) + static_cast<size_t>(m.nba) * m.n2m * m.h2;
  return sizeof(C<double>) * (2 * nacc + 2 * static_cast<size_t>(m.n3a) * m.lsa * TB +
                              2 * static_cast<size_t>(m.n2m) * m.h2 * TB) +
         sizeof(double) * (2 * static_cast<size_t>(m.nba) * TB + 2 * TB);
}

int launch_eval_fp64(const DeviceModel& m, const EvalBuffers& b, cudaStream_t st, int grid_cap, cudaEvent_t* ev,
                     int* kernels) {
  return launch_eval<double>(m, b, st, grid_cap, ev, kernels);
}

}  // namespace magace

namespace magace {
int launch_eval_fp32(const DeviceModel& m, const EvalBuffers& b, cudaStream_t st, int grid_cap, cudaEvent_t* ev,
                     int* kernels) {
  return launch_eval<float>(m, b, st, grid_cap, ev, kernels);
}
}  // namespace magace
