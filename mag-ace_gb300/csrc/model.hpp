// Host-side model: the enumerated cluster basis of a potential, its
// coefficients, the generalized Clebsch-Gordan couplings folded into flat
// product-term tables, and the cubic-Hermite radial lookup tables, laid out
// for the device kernels.
//
// Per-atom data layout used by every kernel ("factor array", complex):
//   A   [n3a][(l3a+1)^2][n3m][(l3m+1)^2]   bond-sum basis R_nl Y_lm(r) M_n'l' Y_l'm'(m_j)
//   A2  [nba][n2m][(l2m+1)^2]              pair basis g_n(r) M_n'l' Y_l'm'(m_j)
//   A0  [n2m][(l2m+1)^2]                   on-site basis M_n'l'(|m_i|) Y_l'm'(m_i)
//   ONE, ZERO                               constants 1+0i and 0+0i
// with lm = l*l + l + m. The weight array (dE/dA for the half m' >= 0 that the
// force pass uses, already multiplied by dE/drho and by the half-plane
// multiplicity of the reference's force loops, src/forces.F90:460-614) is
//   WA  [n3a][(l3a+1)^2][n3m][h3]          h = l'(l'+1)/2 + m', m' >= 0
//   W2  [nba][n2m][h2]
//   W0  [n2m][h2]
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

#include "device_model.hpp"
#include "potential.hpp"

namespace magace {

struct FactorLayout {
  int n3a = 0, n3m = 0, l3a = 0, l3m = 0, nba = 0, n2m = 0, l2m = 0, nbm = 0;
  int lsa = 0, ls3 = 0, ls2 = 0, h3 = 0, h2 = 0;
  int offA = 0, offA2 = 0, offA0 = 0, offOne = 0, offZero = 0, nF = 0;
  int nWA = 0, offW2 = 0, offW0 = 0, nW = 0;

  int A(int n1, int l1, int m1, int n2, int l2, int m2) const;  // 0-based radial indices
  int A2(int n, int nr, int l, int m) const { return offA2 + (n * n2m + nr) * ls2 + l * l + l + m; }
  int A0(int nr, int l, int m) const { return offA0 + nr * ls2 + l * l + l + m; }
  int WA(int n1, int l1, int m1, int n2, int l2, int m2) const;   // -1 if not a stored slot
  int W2(int n, int nr, int l, int m) const { return offW2 + (n * n2m + nr) * h2 + l * (l + 1) / 2 + m; }
  int W0(int nr, int l, int m) const { return offW0 + nr * h2 + l * (l + 1) / 2 + m; }
};

// One gather entry: out_slot accumulates kappa * prod(F[o[k]]), k < arity.
struct Entry {
  double kappa[2];
  uint16_t o[kMaxArity];
};

// Device-ready gather table. Entries are grouped by output slot and cut into
// segments of at most kSegLen entries of one arity. Output slots are
//   [0, nG0)            one per A0 factor (all m): rho and W0
//   [nG0, nslot)        WA then W2 weight slots
// Segments of one slot have consecutive ids (slot_seg_begin). For the device,
// segments are packed 32 at a time into warp groups of one arity, sorted by
// length, and their entries interleaved so that entry e of lane l of group g
// sits at grp_first[g] + e*32 + l: one warp-wide load per entry is fully
// coalesced. Short segments are padded with kappa = 0 entries that point at
// the ZERO factor.
struct GatherTable {
  static const int kSegLen = 64;
  static const int kLanes = 32;
  int nslot = 0;
  int nG0 = 0;
  int nseg = 0;
  std::vector<int32_t> seg_slot;        // [nseg]
  std::vector<int32_t> slot_seg_begin;  // [nslot+1]
  int ngroup = 0;
  std::vector<int32_t> grp_arity, grp_len, grp_first;  // [ngroup]
  std::vector<int32_t> grp_seg;         // [ngroup*32], -1 for padding lanes
  // interleaved entries per arity (index 1..5): kappa per density, packed
  // factor indices o1 | o2 << 16, o3 | o4 << 16 (arity >= 3) and o5 (arity 5)
  std::vector<double> kap[kMaxArity + 1][2];
  std::vector<uint32_t> o12[kMaxArity + 1], o34[kMaxArity + 1];
  std::vector<uint16_t> o5;
  long entries[kMaxArity + 1] = {0, 0, 0, 0, 0, 0};  // real (unpadded) entries per arity
  // slot -> factor/weight index and multiplicity
  std::vector<int32_t> slot_factor;  // for G0 slots: A0 factor index
  std::vector<int32_t> slot_weight;  // weight index (or -1 when the slot stores no weight)
  std::vector<double> slot_mult;     // half-plane multiplicity applied to the weight
};

// Dense tables of the 3-body density for the specialised kernels (see
// build_dense_b3 in model.cpp). C is [combo][n0'][i][j], tasks are
// (combination, m-term) pairs with their coupling cf. The kernel keeps the
// half-plane factors the 3-body terms read (A with m' >= 0, then A0 with
// n' < n3m and m' >= 0: `nc` "compact" elements) and accumulates the
// gradient of the density with respect to the same elements. code[task][pos]
// addresses the factor a[NM], X[I], Y[I] of each task position: bits 0-13
// the compact element, bit 15 negates its real part and bit 14 its imaginary
// part (a factor with m' < 0 is (-1)^(m+m') times the conjugate of its
// mirror). Positions whose code has no sign bits are half-plane elements
// themselves and receive their gradient.
struct DenseB3 {
  int I = 0, NM = 0, ncombo = 0, ntask = 0, nc = 0;
  std::vector<std::array<int, 4>> combo_l;  // (l1, l0', l1', l2')
  std::vector<int32_t> pattern;             // 0: l1' == l2', 1: l1' > l2', 2: l1' < l2'
  std::vector<double> C;
  std::vector<int32_t> task_combo;
  std::vector<double> task_cf;
  std::vector<double> task_w;               // density weight: 2, or 1 for a task that is its own mirror
  std::vector<uint16_t> code;               // [ntask][NM + 2I]
  std::vector<uint16_t> code2;              // [ntask][NM + 2I] mirror-task gradient target (see build_dense_b3)
  std::vector<int32_t> factor_of;           // [nc] factor index of each compact element
  std::vector<int32_t> compact_of_weight;   // [nW] compact element of each weight, or -1
  std::vector<double> mult;                 // [nc] half-plane multiplicity of each element's weight
  // max over elements of the coefficient mass of the element's gradient:
  // sum over the (task, position) pairs that add to it of |cf| times the
  // sum of |C| over that position's products. With every factor bounded by
  // |x| + |y| <= f, every partial sum of a gradient is bounded by bound * f^2.
  double bound = 0.0;
  // the same for the density: sum over tasks of |cf * w| times the sum of
  // |C| over the task's products; every partial sum of the 3-body density
  // is bounded by bound_rho * f^3
  double bound_rho = 0.0;
};

// Per-cluster m-terms of the descriptors B_k, the basis functions that the
// expansion coefficients multiply (rho_d = sum_k c[d][k] B_k): for clusters
// of rank 2..6, B = Re sum_e cf_e F[o0] .. F[o5] with missing factors ONE;
// for rank 1, B = g_n(|m_i|) - 1. Clusters are in coefficient order (the
// file's record order, ranks 1..6).
struct DescriptorTable {
  int n1 = 0, nB = 0;            // rank-1 clusters; all clusters
  std::vector<int32_t> rank1_n;  // [n1] magnetic radial function of each rank-1 cluster
  std::vector<int32_t> begin;    // [nB - n1 + 1] first term of cluster n1 + k
  std::vector<double> cf;        // [terms] coupling
  std::vector<uint16_t> o;       // [terms][kDescFactors] factor indices
};

// The 2- and 4-body terms per output slot, for the split-precision kernel
// that holds 32 atoms in the lanes of a warp. Slot s (numbered as in
// GatherTable) adds kappa * prod F[factor_of[o_q]] over its entries
// [run[3s], run[3s+3]): arity 1 up to run[3s+1], arity 2 up to run[3s+2],
// arity 3 up to run[3s+3] (= run[3(s+1)]). An entry is one 16-byte record
// {kappa bits, o1 | o2 << 16, o3, 0}. Factors are renumbered into the `nfac`
// the terms use; slot_g0 is the compact A0 factor of a density slot. The
// slots are dealt to `nwarp` warps longest first: warp w takes
// warp_slots[warp_begin[w] .. warp_begin[w+1]).
struct RestTable {
  int nfac = 0, nslot = 0, nwarp = 0;
  std::vector<int32_t> factor_of;  // [nfac] factor index
  std::vector<int32_t> run;        // [3 * nslot + 1]
  std::vector<uint32_t> rec;       // [entries][4]
  std::vector<double> kap;         // [entries] kappa in FP64 (the plain-precision kernel)
  std::vector<int32_t> slot_g0;    // [nslot] compact A0 factor, or -1
  std::vector<int32_t> warp_begin; // [nwarp + 1]
  std::vector<int32_t> warp_slots; // [nslot]
  std::vector<int32_t> slot_weight; // [nslot] weight index, or -1
  std::vector<float> slot_mult;     // [nslot] half-plane multiplicity
  // The same entries as one record stream per warp, in schedule order:
  // {kappa bits, o1 | o2 << 16, o3, arity} per entry (two consecutive
  // one-factor entries as {kappa_a bits, o_a | o_b << 16, kappa_b bits,
  // kRestPair1}) and, after each slot's entries, {multiplicity bits, weight
  // index, A0 factor, kRestEnd | slot}.
  std::vector<uint32_t> stream;      // [records][4]
  std::vector<int32_t> stream_begin; // [nwarp + 1] first record of each warp
  // the FP64 kernel's schedule: slots dealt longest first to kRestWarps64
  // warps by that kernel's cost (half-warps take alternate entries)
  std::vector<int32_t> warp64_begin, warp64_slots;
  int nsplit = 0;                    // slots split in two stream items
  std::vector<int32_t> split_weight; // [nsplit] their weight index, or -1
};

struct RadialLUT {
  int nlut = 0;
  int nfa = 0;  // atomic: g_n (nba), R_nl (n3a*(l3a+1), index nr*(l3a+1)+l), core (1)
  int nfm = 0;  // magnetic: M_nl (n2m*(l2m+1), index nr*(l2m+1)+l), g_n (nbm)
  double rscale_a = 0, rscale_m = 0;
  std::vector<double> a, m;  // [(nlut+1)][nf][4] cubic coefficients per bin
};

struct Model {
  Potential pot;
  double cutoff = 0, cutoff_m = 0;
  FactorLayout L;
  int ndensity = 1, nfemb = 0;
  double par[2][2] = {{1, 1}, {1, 1}};
  double ecut = 0, decut = 0;
  double core_pre = 0, core_lambda = 0;
  // enumerated clusters in file layout, rank 1..6, with coefficients
  std::vector<std::vector<int>> rows[7];
  std::vector<std::array<double, 2>> coef[7];
  int unmatched_records = 0;
  long nterms[7] = {0, 0, 0, 0, 0, 0, 0};
  bool high = false;  // 5- or 6-body clusters: only the generic kernels and tables
  std::vector<double> c1[2];  // 1-body coefficient per magnetic radial function n
  GatherTable gt;        // every term (generic kernels)
  GatherTable gt_nob3;   // every term except the 3-body ones (specialised kernels)
  DenseB3 db3;           // 3-body terms in dense form (specialised kernels)
  RestTable rest;        // the other terms per slot (specialised split kernels)
  DescriptorTable desc;  // per-cluster terms without coefficients (descriptors)
  RadialLUT lut;
  bool ready = false;
};

// Builds the complete model (enumeration, couplings, tables, LUT) from a
// parsed potential. rcut / rcut_magnetic are the caller's global cutoffs,
// which set the LUT grid (src/radial.F90:198, :341).
int build_model(const Potential& pot, double rcut, double rcut_magnetic, Model& model, std::string& msg);

// Rebuilds the coefficient-dependent tables after M.coef changed.
int build_tables(Model& model, std::string& msg);

// Expansion coefficients as one vector [ndensity][num_coefficients], the
// clusters of ranks 1..4 in the file's record order.
int num_coefficients(const Model& model);
void get_coefficients(const Model& model, double* c);
int set_coefficients(Model& model, const double* c, std::string& msg);

// Clebsch-Gordan coefficient <j1 m1 j2 m2 | J M> by the Racah formula.
double clebsch_gordan(int j1, int j2, int J, int m1, int m2, int M);

}  // namespace magace
