// Device-resident spin-lattice molecular dynamics around the evaluation:
// cell-list neighbour list with a skin, per-step bond inputs, deterministic
// force and field assembly, velocity Verlet with spin precession, and an
// energy log, with each stretch of steps between two neighbour-list builds
// replayed from a CUDA graph.
//
// The reference leaves dynamics to LAMMPS (pair style spin/ace driven by
// fix nve/spin; lammps/pair_spin_ace.cpp). What this file keeps from it:
//  - bonds in the LAMMPS convention, d_ij = x_i - x_j(image), e = d/r
//    (lammps/pair_spin_ace.cpp:491-499); neighbours in the skin, beyond the
//    cutoff, contribute exactly zero (src/radial.F90:77-83);
//  - forces f_i -= dE/dd_ij, f_j += dE/dd_ij and the magnetic field
//    fm_i = -(mub/hbar) dE/dm_i with mub = 5.78901e-5 eV/T and hbar in eV ps
//    (lammps/pair_spin_ace.cpp:57,571-631,938-958);
//  - a zero moment points along z (neilist/neilist.F90:764-769).
// The integrator is this project's: per step, v += dt/2 F/m; x += dt v; each
// moment turns about its field by |fm| dt (Rodrigues, |m| kept); forces and
// fields at the new state; v += dt/2 F/m. One evaluation per step.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "magace.h"

namespace magace {
int runtime_error(int code, const char* msg);
}

namespace {

using magace::runtime_error;

constexpr double kMub = 5.78901e-5;         // eV/T (lammps/pair_spin_ace.cpp:57)
constexpr double kHbar = 6.582119569e-4;    // eV ps (metal units, hplanck / 2 pi)
constexpr double kAccel = 9648.53321233100; // (eV/A)/amu -> A/ps^2
constexpr int kMaxBondsPerAtom = 512;       // capacity guard of one atom's list
// atoms of one system: with at most kMaxBondsPerAtom per atom the 32-bit
// scan of the bond counts cannot overflow
constexpr int kMaxMdAtoms = std::numeric_limits<int>::max() / kMaxBondsPerAtom;

// --- small helpers -------------------------------------------------------
struct Cell {
  double h[9];     // rows are lattice vectors
  double hinv[9];  // inverse: s = x hinv
  int pbc[3];
  int nb[3];       // bins per axis
};

__device__ __forceinline__ void frac(const Cell& c, const double* x, double* s) {
  for (int b = 0; b < 3; ++b) s[b] = x[0] * c.hinv[0 * 3 + b] + x[1] * c.hinv[1 * 3 + b] + x[2] * c.hinv[2 * 3 + b];
}
__device__ __forceinline__ void cart(const Cell& c, const double* n, double* x) {
  for (int b = 0; b < 3; ++b) x[b] = n[0] * c.h[0 * 3 + b] + n[1] * c.h[1 * 3 + b] + n[2] * c.h[2 * 3 + b];
}
// image shifts packed as three biased bytes
__device__ __forceinline__ int pack_shift(int a, int b, int c) { return (a + 128) | ((b + 128) << 8) | ((c + 128) << 16); }
__device__ __forceinline__ void unpack_shift(int p, double* n) {
  n[0] = static_cast<double>((p & 0xff) - 128);
  n[1] = static_cast<double>(((p >> 8) & 0xff) - 128);
  n[2] = static_cast<double>(((p >> 16) & 0xff) - 128);
}
__device__ __forceinline__ int neg_shift(int p) {
  return pack_shift(128 - (p & 0xff), 128 - ((p >> 8) & 0xff), 128 - ((p >> 16) & 0xff));
}

// bin of an atom and its wrap count per axis (w = floor(s) on periodic axes)
__device__ __forceinline__ int bin_of(const Cell& c, const double* x, int* bin3, int* w) {
  double s[3];
  frac(c, x, s);
  for (int a = 0; a < 3; ++a) {
    double t = s[a];
    w[a] = 0;
    if (c.pbc[a]) {
      const double f = floor(t);
      w[a] = static_cast<int>(f);
      t -= f;
    }
    int b = static_cast<int>(t * c.nb[a]);
    b = b < 0 ? 0 : (b >= c.nb[a] ? c.nb[a] - 1 : b);
    bin3[a] = b;
  }
  return (bin3[0] * c.nb[1] + bin3[1]) * c.nb[2] + bin3[2];
}

// --- exclusive scan (three phases, any length) --------------------------
constexpr int kScanBlock = 1024;

__global__ void k_scan_blocks(const int* __restrict__ in, int* __restrict__ out, int* __restrict__ sums, int n) {
  __shared__ int s[kScanBlock];
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  const int v = i < n ? in[i] : 0;
  s[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < kScanBlock; o <<= 1) {
    const int t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) out[i] = s[threadIdx.x] - v;
  if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = s[threadIdx.x];
}
__global__ void k_scan_sums(int* __restrict__ sums, int nblk, int* __restrict__ total) {
  if (threadIdx.x == 0) {
    int run = 0;
    for (int b = 0; b < nblk; ++b) {
      const int v = sums[b];
      sums[b] = run;
      run += v;
    }
    *total = run;
  }
}
__global__ void k_scan_add(int* __restrict__ out, const int* __restrict__ sums, int n, const int* __restrict__ total,
                           int* __restrict__ last) {
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) out[i] += sums[blockIdx.x];
  if (i == 0 && last) *last = *total;
}
// out[0..n) = exclusive prefix sums of in[0..n); out[n] = total
void exclusive_scan(const int* in, int* out, int n, int* scratch, cudaStream_t st) {
  const int nblk = (n + kScanBlock - 1) / kScanBlock;
  int* sums = scratch;
  int* total = scratch + nblk;
  k_scan_blocks<<<nblk, kScanBlock, 0, st>>>(in, out, sums, n);
  k_scan_sums<<<1, 32, 0, st>>>(sums, nblk, total);
  k_scan_add<<<nblk, kScanBlock, 0, st>>>(out, sums, n, total, out + n);
}

// --- neighbour list -------------------------------------------------------
__global__ void k_nl_bin(int n, const double* __restrict__ x, Cell c, int* __restrict__ atom_cell,
                         int* __restrict__ cell_count) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int b3[3], w[3];
    const int id = bin_of(c, x + 3 * i, b3, w);
    atom_cell[i] = id;
    atomicAdd(&cell_count[id], 1);
  }
}
__global__ void k_nl_place(int n, const int* __restrict__ atom_cell, int* __restrict__ cursor,
                           int* __restrict__ cell_atoms) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    cell_atoms[atomicAdd(&cursor[atom_cell[i]], 1)] = i;
}
// atoms of each cell in index order, so that the lists do not depend on the
// order of the placement atomics
__global__ void k_nl_sort_cells(int ncell, const int* __restrict__ start, int* __restrict__ atoms) {
  for (int cidx = blockIdx.x * blockDim.x + threadIdx.x; cidx < ncell; cidx += gridDim.x * blockDim.x) {
    const int a = start[cidx], b = start[cidx + 1];
    for (int p = a + 1; p < b; ++p) {
      const int v = atoms[p];
      int q = p - 1;
      while (q >= a && atoms[q] > v) {
        atoms[q + 1] = atoms[q];
        --q;
      }
      atoms[q + 1] = v;
    }
  }
}

// Visits the candidate neighbours of atom i: the atoms of the 27 bins around
// its bin (periodic axes wrap, with the image count folded into the shift),
// calling fn(j, packed_shift, r2) for every pair closer than rlist.
template <class Fn>
__device__ __forceinline__ void for_each_pair(int i, const double* __restrict__ x, const Cell& c,
                                              const int* __restrict__ start, const int* __restrict__ atoms,
                                              double rlist2, Fn&& fn) {
  int bi[3], wi[3];
  bin_of(c, x + 3 * i, bi, wi);
  const double xi[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
  for (int da = -1; da <= 1; ++da)
    for (int db = -1; db <= 1; ++db)
      for (int dc = -1; dc <= 1; ++dc) {
        const int d3[3] = {da, db, dc};
        int nbin[3], img[3];
        bool skip = false;
        for (int a = 0; a < 3; ++a) {
          int t = bi[a] + d3[a];
          img[a] = 0;
          if (t < 0 || t >= c.nb[a]) {
            if (!c.pbc[a]) {
              skip = true;
              break;
            }
            img[a] = t < 0 ? -1 : 1;
            t -= img[a] * c.nb[a];
          }
          nbin[a] = t;
        }
        if (skip) continue;
        const int cid = (nbin[0] * c.nb[1] + nbin[1]) * c.nb[2] + nbin[2];
        for (int p = start[cid]; p < start[cid + 1]; ++p) {
          const int j = atoms[p];
          int bj[3], wj[3];
          bin_of(c, x + 3 * j, bj, wj);
          // x_j(image) = x_j - w_j h + w_i h + img h
          const int sh[3] = {img[0] + wi[0] - wj[0], img[1] + wi[1] - wj[1], img[2] + wi[2] - wj[2]};
          if (j == i && sh[0] == 0 && sh[1] == 0 && sh[2] == 0) continue;
          const double n[3] = {static_cast<double>(sh[0]), static_cast<double>(sh[1]), static_cast<double>(sh[2])};
          double t[3];
          cart(c, n, t);
          const double d0 = (xi[0] - x[3 * j]) - t[0], d1 = (xi[1] - x[3 * j + 1]) - t[1],
                       d2 = (xi[2] - x[3 * j + 2]) - t[2];
          const double r2 = d0 * d0 + d1 * d1 + d2 * d2;
          if (r2 < rlist2) fn(j, pack_shift(sh[0], sh[1], sh[2]), r2);
        }
      }
}

__global__ void k_nl_count(int n, const double* __restrict__ x, Cell c, const int* __restrict__ start,
                           const int* __restrict__ atoms, double rlist2, int* __restrict__ count, int* err) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int k = 0;
    for_each_pair(i, x, c, start, atoms, rlist2, [&](int, int, double) { ++k; });
    if (k > kMaxBondsPerAtom) {
      atomicCAS(err, 0, 1);
      k = kMaxBondsPerAtom;
    }
    count[i] = k;
  }
}

// fills atom i's bonds, then sorts them by (j, shift) so that the reverse of
// every bond is found by binary search
__global__ void k_nl_fill(int n, const double* __restrict__ x, Cell c, const int* __restrict__ start,
                          const int* __restrict__ atoms, double rlist2, const int* __restrict__ off,
                          unsigned long long* __restrict__ key) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int b0 = off[i], b1 = off[i + 1];
    int p = b0;
    for_each_pair(i, x, c, start, atoms, rlist2, [&](int j, int sh, double) {
      if (p < b1) key[p] = (static_cast<unsigned long long>(j) << 24) | static_cast<unsigned long long>(sh);
      ++p;
    });
    for (int q = b0 + 1; q < b1; ++q) {
      const unsigned long long v = key[q];
      int r = q - 1;
      while (r >= b0 && key[r] > v) {
        key[r + 1] = key[r];
        --r;
      }
      key[r + 1] = v;
    }
  }
}

__global__ void k_nl_split(int n, const int* __restrict__ off, const unsigned long long* __restrict__ key,
                           int* __restrict__ bj, int* __restrict__ bshift, int* __restrict__ bi) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int b = off[i]; b < off[i + 1]; ++b) {
      bj[b] = static_cast<int>(key[b] >> 24);
      bshift[b] = static_cast<int>(key[b] & 0xffffffull);
      bi[b] = i;
    }
}

// rev[b] = the bond (j -> i, -shift) of bond b = (i -> j, shift)
__global__ void k_nl_reverse(int nb, const int* __restrict__ off, const unsigned long long* __restrict__ key,
                             const int* __restrict__ bi, int* __restrict__ rev, int* err) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
    const int i = bi[b];
    const int j = static_cast<int>(key[b] >> 24);
    const int sh = static_cast<int>(key[b] & 0xffffffull);
    const unsigned long long want = (static_cast<unsigned long long>(i) << 24) |
                                    static_cast<unsigned long long>(neg_shift(sh));
    int lo = off[j], hi = off[j + 1] - 1, found = -1;
    while (lo <= hi) {
      const int mid = (lo + hi) >> 1;
      const unsigned long long v = key[mid];
      if (v == want) {
        found = mid;
        break;
      }
      if (v < want) lo = mid + 1;
      else hi = mid - 1;
    }
    if (found < 0) atomicCAS(err, 0, 2);
    rev[b] = found;
  }
}

// --- per-step kernels -----------------------------------------------------
// library inputs of every bond and atom from positions and moments
__global__ void k_bond_inputs(int nb, int n, const double* __restrict__ x, const double* __restrict__ m, Cell c,
                              const int* __restrict__ bi, const int* __restrict__ bj, const int* __restrict__ bsh,
                              double* __restrict__ r, double* __restrict__ e, double* __restrict__ magj,
                              double* __restrict__ mhj, double* __restrict__ magi, double* __restrict__ mhi) {
  const int stride = gridDim.x * blockDim.x;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += stride) {
    const int i = bi[b], j = bj[b];
    double nsh[3], t[3];
    unpack_shift(bsh[b], nsh);
    cart(c, nsh, t);
    const double d0 = (x[3 * i] - x[3 * j]) - t[0], d1 = (x[3 * i + 1] - x[3 * j + 1]) - t[1],
                 d2 = (x[3 * i + 2] - x[3 * j + 2]) - t[2];
    const double rr = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    r[b] = rr;
    e[3 * b] = d0 / rr;
    e[3 * b + 1] = d1 / rr;
    e[3 * b + 2] = d2 / rr;
    const double mx = m[3 * j], my = m[3 * j + 1], mz = m[3 * j + 2];
    const double mm = sqrt(mx * mx + my * my + mz * mz);
    magj[b] = mm;
    mhj[3 * b] = mm > 0.0 ? mx / mm : 0.0;
    mhj[3 * b + 1] = mm > 0.0 ? my / mm : 0.0;
    mhj[3 * b + 2] = mm > 0.0 ? mz / mm : 1.0;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double mx = m[3 * i], my = m[3 * i + 1], mz = m[3 * i + 2];
    const double mm = sqrt(mx * mx + my * my + mz * mz);
    magi[i] = mm;
    mhi[3 * i] = mm > 0.0 ? mx / mm : 0.0;
    mhi[3 * i + 1] = mm > 0.0 ? my / mm : 0.0;
    mhi[3 * i + 2] = mm > 0.0 ? mz / mm : 1.0;
  }
}

// F_i = sum_{bonds b of i} (-f_b + f_rev(b)),
// dE/dm_i = t0_i + sum_b t_rev(b), fm_i = -(mub/hbar) dE/dm_i;
// in bond order, without atomics
__global__ void k_assemble(int n, const int* __restrict__ off, const int* __restrict__ rev,
                           const double* __restrict__ fij, const double* __restrict__ tij,
                           const double* __restrict__ ti0, double* __restrict__ F, double* __restrict__ fm) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double f[3] = {0.0, 0.0, 0.0}, g[3] = {ti0[3 * i], ti0[3 * i + 1], ti0[3 * i + 2]};
    for (int b = off[i]; b < off[i + 1]; ++b) {
      const int q = rev[b];
      if (q < 0) continue;  // not reached: a list without every reverse bond is rejected
      for (int a = 0; a < 3; ++a) {
        f[a] += fij[3 * q + a] - fij[3 * b + a];
        g[a] += tij[3 * q + a];
      }
    }
    for (int a = 0; a < 3; ++a) {
      F[3 * i + a] = f[a];
      fm[3 * i + a] = -(kMub / kHbar) * g[a];
    }
  }
}

// v += dt/2 F/m
__global__ void k_kick(int n, double* __restrict__ v, const double* __restrict__ F, double h) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * n; i += gridDim.x * blockDim.x) v[i] += h * F[i];
}
// x += dt v; m turns about fm by |fm| dt
__global__ void k_drift_turn(int n, double* __restrict__ x, const double* __restrict__ v, double* __restrict__ m,
                             const double* __restrict__ fm, double dt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    for (int a = 0; a < 3; ++a) x[3 * i + a] += dt * v[3 * i + a];
    const double w0 = fm[3 * i], w1 = fm[3 * i + 1], w2 = fm[3 * i + 2];
    const double wn = sqrt(w0 * w0 + w1 * w1 + w2 * w2);
    if (wn == 0.0) continue;
    const double k0 = w0 / wn, k1 = w1 / wn, k2 = w2 / wn, th = wn * dt;
    const double cs = cos(th), sn = sin(th);
    const double m0 = m[3 * i], m1 = m[3 * i + 1], m2 = m[3 * i + 2];
    const double kd = k0 * m0 + k1 * m1 + k2 * m2;
    const double c0 = k1 * m2 - k2 * m1, c1 = k2 * m0 - k0 * m2, c2 = k0 * m1 - k1 * m0;
    m[3 * i] = m0 * cs + c0 * sn + k0 * kd * (1.0 - cs);
    m[3 * i + 1] = m1 * cs + c1 * sn + k1 * kd * (1.0 - cs);
    m[3 * i + 2] = m2 * cs + c2 * sn + k2 * kd * (1.0 - cs);
  }
}

// log[step] = (sum E_i, sum m v^2 / 2) with per-block partials summed in
// block order by the last kernel (deterministic)
constexpr int kLogThreads = 256;
__global__ void k_energy_partials(int n, const double* __restrict__ E, const double* __restrict__ v, double mass,
                                  double* __restrict__ part) {
  __shared__ double s[2][kLogThreads];
  double pe = 0.0, ke = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    pe += E[i];
    ke += v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2];
  }
  s[0][threadIdx.x] = pe;
  s[1][threadIdx.x] = ke * 0.5 * mass / kAccel;
  __syncthreads();
  for (int o = kLogThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s[0][threadIdx.x] += s[0][threadIdx.x + o];
      s[1][threadIdx.x] += s[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s[0][0];
    part[2 * blockIdx.x + 1] = s[1][0];
  }
}
__global__ void k_energy_log(const double* __restrict__ part, int nblk, double* __restrict__ log, int* __restrict__ step,
                             int cap) {
  if (threadIdx.x == 0) {
    double pe = 0.0, ke = 0.0;
    for (int b = 0; b < nblk; ++b) {
      pe += part[2 * b];
      ke += part[2 * b + 1];
    }
    const int k = *step;
    if (k < cap) {
      log[2 * k] = pe;
      log[2 * k + 1] = ke;
    }
    *step = k + 1;
  }
}

// --- state ----------------------------------------------------------------
template <class T>
struct Buf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t reserve(size_t want) {
    if (want <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    want = want ? want + want / 8 : 1;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), want * sizeof(T));
    if (e == cudaSuccess) n = want;
    return e;
  }
  ~Buf() {
    if (p) cudaFree(p);
  }
};

struct MdState {
  int natom = 0, nbond = 0, device = 0;
  double mass = 0, rcut = 0, skin = 0;
  Cell cell{};
  cudaStream_t st = nullptr;
  Buf<double> x, v, m, F, fm, E, ti0, magi, mhi, part, log;
  Buf<int> atom_cell, cell_count, cell_start, cell_atoms, cursor, count, off, scan, bi, bj, bsh, rev, flags, step;
  Buf<unsigned long long> key;
  Buf<double> r, e, magj, mhj, fij, tij;
  int nlog_blocks = 0;
  ~MdState() {
    if (st) cudaStreamDestroy(st);
  }
};

std::map<int, std::unique_ptr<MdState>>& states() {
  static std::map<int, std::unique_ptr<MdState>> s;
  return s;
}

int grid_for(int n, int threads) {
  const int b = (n + threads - 1) / threads;
  return b < 1 ? 1 : (b > 4096 ? 4096 : b);
}

#define MD_CUDA(x)                                                                  \
  do {                                                                              \
    cudaError_t e_ = (x);                                                           \
    if (e_ != cudaSuccess) return runtime_error(MAGACE_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

// neighbour list of the current positions (rcut + skin)
int build_list(MdState& S) {
  const int n = S.natom;
  cudaStream_t st = S.st;
  const int ncell = S.cell.nb[0] * S.cell.nb[1] * S.cell.nb[2];
  MD_CUDA(S.atom_cell.reserve(n));
  MD_CUDA(S.cell_count.reserve(ncell));
  MD_CUDA(S.cell_start.reserve(ncell + 1));
  MD_CUDA(S.cursor.reserve(ncell));
  MD_CUDA(S.cell_atoms.reserve(n));
  MD_CUDA(S.count.reserve(n));
  MD_CUDA(S.off.reserve(n + 1));
  const int maxn = n > ncell ? n : ncell;
  MD_CUDA(S.scan.reserve((maxn + kScanBlock - 1) / kScanBlock + 2));
  MD_CUDA(S.flags.reserve(1));
  MD_CUDA(cudaMemsetAsync(S.flags.p, 0, sizeof(int), st));
  MD_CUDA(cudaMemsetAsync(S.cell_count.p, 0, sizeof(int) * ncell, st));
  k_nl_bin<<<grid_for(n, 256), 256, 0, st>>>(n, S.x.p, S.cell, S.atom_cell.p, S.cell_count.p);
  exclusive_scan(S.cell_count.p, S.cell_start.p, ncell, S.scan.p, st);
  MD_CUDA(cudaMemcpyAsync(S.cursor.p, S.cell_start.p, sizeof(int) * ncell, cudaMemcpyDeviceToDevice, st));
  k_nl_place<<<grid_for(n, 256), 256, 0, st>>>(n, S.atom_cell.p, S.cursor.p, S.cell_atoms.p);
  k_nl_sort_cells<<<grid_for(ncell, 128), 128, 0, st>>>(ncell, S.cell_start.p, S.cell_atoms.p);
  const double rl = S.rcut + S.skin;
  k_nl_count<<<grid_for(n, 128), 128, 0, st>>>(n, S.x.p, S.cell, S.cell_start.p, S.cell_atoms.p, rl * rl, S.count.p,
                                               S.flags.p);
  exclusive_scan(S.count.p, S.off.p, n, S.scan.p, st);
  int nb = 0, flag = 0;
  MD_CUDA(cudaMemcpyAsync(&nb, S.off.p + n, sizeof(int), cudaMemcpyDeviceToHost, st));
  MD_CUDA(cudaMemcpyAsync(&flag, S.flags.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  MD_CUDA(cudaStreamSynchronize(st));
  if (flag) return runtime_error(MAGACE_ERR_ARGS, "more than 512 neighbours within rcut + skin for an atom");
  // the evaluation indexes per-bond vectors as 3 j with 32-bit j
  if (nb > std::numeric_limits<int>::max() / 3)
    return runtime_error(MAGACE_ERR_ARGS, "more than 715,827,882 bonds within rcut + skin");
  S.nbond = nb;
  MD_CUDA(S.key.reserve(nb));
  for (auto* b : {&S.bi, &S.bj, &S.bsh, &S.rev}) MD_CUDA(b->reserve(nb));
  for (auto* b : {&S.r, &S.magj}) MD_CUDA(b->reserve(nb));
  for (auto* b : {&S.e, &S.mhj, &S.fij, &S.tij}) MD_CUDA(b->reserve(3 * static_cast<size_t>(nb)));
  k_nl_fill<<<grid_for(n, 128), 128, 0, st>>>(n, S.x.p, S.cell, S.cell_start.p, S.cell_atoms.p, rl * rl, S.off.p,
                                              S.key.p);
  k_nl_split<<<grid_for(n, 256), 256, 0, st>>>(n, S.off.p, S.key.p, S.bj.p, S.bsh.p, S.bi.p);
  k_nl_reverse<<<grid_for(nb, 256), 256, 0, st>>>(nb, S.off.p, S.key.p, S.bi.p, S.rev.p, S.flags.p);
  MD_CUDA(cudaMemcpyAsync(&flag, S.flags.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  MD_CUDA(cudaStreamSynchronize(st));
  if (flag) return runtime_error(MAGACE_ERR_ARGS, "neighbour list is not symmetric (a reverse bond is missing)");
  return MAGACE_OK;
}

// library inputs, evaluation, forces and fields at the current state
int evaluate(MdState& S) {
  cudaStream_t st = S.st;
  const int n = S.natom, nb = S.nbond;
  k_bond_inputs<<<grid_for(nb > n ? nb : n, 256), 256, 0, st>>>(nb, n, S.x.p, S.m.p, S.cell, S.bi.p, S.bj.p, S.bsh.p,
                                                                S.r.p, S.e.p, S.magj.p, S.mhj.p, S.magi.p, S.mhi.p);
  int rc = ace_compute_device(n, nb, S.off.p, S.r.p, S.e.p, S.magj.p, S.mhj.p, S.magi.p, S.mhi.p, S.E.p, S.fij.p,
                              S.tij.p, S.ti0.p, st);
  if (rc) return rc;
  k_assemble<<<grid_for(n, 128), 128, 0, st>>>(n, S.off.p, S.rev.p, S.fij.p, S.tij.p, S.ti0.p, S.F.p, S.fm.p);
  return MAGACE_OK;
}

void log_energy(MdState& S, int cap) {
  k_energy_partials<<<S.nlog_blocks, kLogThreads, 0, S.st>>>(S.natom, S.E.p, S.v.p, S.mass, S.part.p);
  k_energy_log<<<1, 32, 0, S.st>>>(S.part.p, S.nlog_blocks, S.log.p, S.step.p, cap);
}

// one step after the forces of the current state are known
int step(MdState& S, double dt, int cap) {
  const int n = S.natom;
  const double h = 0.5 * dt * kAccel / S.mass;
  k_kick<<<grid_for(3 * n, 256), 256, 0, S.st>>>(n, S.v.p, S.F.p, h);
  k_drift_turn<<<grid_for(n, 256), 256, 0, S.st>>>(n, S.x.p, S.v.p, S.m.p, S.fm.p, dt);
  int rc = evaluate(S);
  if (rc) return rc;
  k_kick<<<grid_for(3 * n, 256), 256, 0, S.st>>>(n, S.v.p, S.F.p, h);
  log_energy(S, cap);
  return MAGACE_OK;
}

void invert3(const double* h, double* g) {
  const double det = h[0] * (h[4] * h[8] - h[5] * h[7]) - h[1] * (h[3] * h[8] - h[5] * h[6]) +
                     h[2] * (h[3] * h[7] - h[4] * h[6]);
  g[0] = (h[4] * h[8] - h[5] * h[7]) / det;
  g[1] = (h[2] * h[7] - h[1] * h[8]) / det;
  g[2] = (h[1] * h[5] - h[2] * h[4]) / det;
  g[3] = (h[5] * h[6] - h[3] * h[8]) / det;
  g[4] = (h[0] * h[8] - h[2] * h[6]) / det;
  g[5] = (h[2] * h[3] - h[0] * h[5]) / det;
  g[6] = (h[3] * h[7] - h[4] * h[6]) / det;
  g[7] = (h[1] * h[6] - h[0] * h[7]) / det;
  g[8] = (h[0] * h[4] - h[1] * h[3]) / det;
}

}  // namespace

extern "C" {

int ace_md_create(int natom, const double* x, const double* v, const double* m, const double* cell, const int* pbc,
                  double mass_amu, double rcut, double skin, int* handle) {
  if (natom <= 0 || !x || !v || !m || !cell || !pbc || !handle || mass_amu <= 0 || rcut <= 0 || skin < 0)
    return runtime_error(MAGACE_ERR_ARGS, "invalid MD arguments");
  if (natom > kMaxMdAtoms) return runtime_error(MAGACE_ERR_ARGS, "more than 4,194,303 atoms in one MD system");
  auto S = std::make_unique<MdState>();
  S->natom = natom;
  S->mass = mass_amu;
  S->rcut = rcut;
  S->skin = skin;
  std::memcpy(S->cell.h, cell, sizeof(double) * 9);
  invert3(S->cell.h, S->cell.hinv);
  const double vol = std::fabs(S->cell.h[0] * (S->cell.h[4] * S->cell.h[8] - S->cell.h[5] * S->cell.h[7]) -
                               S->cell.h[1] * (S->cell.h[3] * S->cell.h[8] - S->cell.h[5] * S->cell.h[6]) +
                               S->cell.h[2] * (S->cell.h[3] * S->cell.h[7] - S->cell.h[4] * S->cell.h[6]));
  for (int a = 0; a < 3; ++a) {
    S->cell.pbc[a] = pbc[a] ? 1 : 0;
    // width of the cell across axis a: volume over the area of the other two
    const double* b = S->cell.h + 3 * ((a + 1) % 3);
    const double* c = S->cell.h + 3 * ((a + 2) % 3);
    const double cx = b[1] * c[2] - b[2] * c[1], cy = b[2] * c[0] - b[0] * c[2], cz = b[0] * c[1] - b[1] * c[0];
    const double width = vol / std::sqrt(cx * cx + cy * cy + cz * cz);
    const int nb = static_cast<int>(std::floor(width / (rcut + skin)));
    if (S->cell.pbc[a] && nb < 3)
      return runtime_error(MAGACE_ERR_ARGS, "periodic cell narrower than 3 (rcut + skin): use a larger supercell");
    S->cell.nb[a] = nb < 1 ? 1 : (nb > 1024 ? 1024 : nb);
  }
  MD_CUDA(cudaGetDevice(&S->device));
  MD_CUDA(cudaStreamCreateWithFlags(&S->st, cudaStreamNonBlocking));
  const size_t n3 = 3 * static_cast<size_t>(natom);
  for (auto* b : {&S->x, &S->v, &S->m, &S->F, &S->fm, &S->ti0, &S->mhi}) MD_CUDA(b->reserve(n3));
  for (auto* b : {&S->E, &S->magi}) MD_CUDA(b->reserve(natom));
  S->nlog_blocks = grid_for(natom, kLogThreads) > 1024 ? 1024 : grid_for(natom, kLogThreads);
  MD_CUDA(S->part.reserve(2 * static_cast<size_t>(S->nlog_blocks)));
  MD_CUDA(S->step.reserve(1));
  MD_CUDA(cudaMemcpy(S->x.p, x, sizeof(double) * n3, cudaMemcpyHostToDevice));
  MD_CUDA(cudaMemcpy(S->v.p, v, sizeof(double) * n3, cudaMemcpyHostToDevice));
  MD_CUDA(cudaMemcpy(S->m.p, m, sizeof(double) * n3, cudaMemcpyHostToDevice));
  MD_CUDA(cudaMemset(S->fm.p, 0, sizeof(double) * n3));
  int rc = build_list(*S);
  if (rc) return rc;
  int id = 1;
  while (states().count(id)) ++id;
  states()[id] = std::move(S);
  *handle = id;
  return runtime_error(MAGACE_OK, "");
}

int ace_md_run(int handle, int nsteps, double dt_ps, int rebuild_every, int use_graph, double* log) {
  auto it = states().find(handle);
  if (it == states().end()) return runtime_error(MAGACE_ERR_ARGS, "unknown MD handle");
  MdState& S = *it->second;
  if (nsteps < 0 || rebuild_every <= 0 || !(dt_ps > 0)) return runtime_error(MAGACE_ERR_ARGS, "invalid MD run arguments");
  MD_CUDA(S.log.reserve(2 * static_cast<size_t>(nsteps) + 2));
  MD_CUDA(cudaMemsetAsync(S.step.p, 0, sizeof(int), S.st));
  // forces and fields of the starting state (logged as step 0)
  int rc = evaluate(S);
  if (rc) return rc;
  log_energy(S, nsteps + 1);
  int done = 0;
  while (done < nsteps) {
    if (done > 0) {
      rc = build_list(S);
      if (rc) return rc;
      rc = evaluate(S);  // forces on the new list (same state)
      if (rc) return rc;
    }
    const int k = nsteps - done < rebuild_every ? nsteps - done : rebuild_every;
    if (use_graph) {
      cudaGraph_t g = nullptr;
      cudaGraphExec_t ge = nullptr;
      MD_CUDA(cudaStreamBeginCapture(S.st, cudaStreamCaptureModeThreadLocal));
      rc = step(S, dt_ps, nsteps + 1);
      cudaError_t ce = cudaStreamEndCapture(S.st, &g);
      if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      MD_CUDA(ce);
      MD_CUDA(cudaGraphInstantiate(&ge, g, 0));
      for (int s = 0; s < k; ++s) MD_CUDA(cudaGraphLaunch(ge, S.st));
      cudaGraphExecDestroy(ge);
      cudaGraphDestroy(g);
    } else {
      for (int s = 0; s < k; ++s) {
        rc = step(S, dt_ps, nsteps + 1);
        if (rc) return rc;
      }
    }
    done += k;
  }
  MD_CUDA(cudaStreamSynchronize(S.st));
  rc = ace_device_status();
  if (rc) return rc;
  if (log) MD_CUDA(cudaMemcpy(log, S.log.p, sizeof(double) * 2 * (nsteps + 1), cudaMemcpyDeviceToHost));
  return runtime_error(MAGACE_OK, "");
}

int ace_md_state(int handle, double* x, double* v, double* m, double* F, double* fm) {
  auto it = states().find(handle);
  if (it == states().end()) return runtime_error(MAGACE_ERR_ARGS, "unknown MD handle");
  MdState& S = *it->second;
  MD_CUDA(cudaStreamSynchronize(S.st));
  const size_t bytes = sizeof(double) * 3 * static_cast<size_t>(S.natom);
  if (x) MD_CUDA(cudaMemcpy(x, S.x.p, bytes, cudaMemcpyDeviceToHost));
  if (v) MD_CUDA(cudaMemcpy(v, S.v.p, bytes, cudaMemcpyDeviceToHost));
  if (m) MD_CUDA(cudaMemcpy(m, S.m.p, bytes, cudaMemcpyDeviceToHost));
  if (F) MD_CUDA(cudaMemcpy(F, S.F.p, bytes, cudaMemcpyDeviceToHost));
  if (fm) MD_CUDA(cudaMemcpy(fm, S.fm.p, bytes, cudaMemcpyDeviceToHost));
  return runtime_error(MAGACE_OK, "");
}

int ace_md_bonds(int handle, int* nbond, int* off, int* j, int* shift, int* rev) {
  auto it = states().find(handle);
  if (it == states().end()) return runtime_error(MAGACE_ERR_ARGS, "unknown MD handle");
  MdState& S = *it->second;
  MD_CUDA(cudaStreamSynchronize(S.st));
  *nbond = S.nbond;
  const size_t nb = static_cast<size_t>(S.nbond);
  if (off) MD_CUDA(cudaMemcpy(off, S.off.p, sizeof(int) * (S.natom + 1), cudaMemcpyDeviceToHost));
  if (j) MD_CUDA(cudaMemcpy(j, S.bj.p, sizeof(int) * nb, cudaMemcpyDeviceToHost));
  if (shift) MD_CUDA(cudaMemcpy(shift, S.bsh.p, sizeof(int) * nb, cudaMemcpyDeviceToHost));
  if (rev) MD_CUDA(cudaMemcpy(rev, S.rev.p, sizeof(int) * nb, cudaMemcpyDeviceToHost));
  return runtime_error(MAGACE_OK, "");
}

int ace_md_destroy(int handle) {
  states().erase(handle);
  return runtime_error(MAGACE_OK, "");
}

}  // extern "C"
