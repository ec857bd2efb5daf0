// Plain-old-data view of the model for the kernels: sizes, constants and
// device pointers. Passed by value as a kernel argument.
#pragma once

#include <cstdint>

namespace magace {

// largest angular momentum the kernels' fixed-size scratch arrays support
constexpr int kMaxL = 4;
constexpr int kMaxHalf = (kMaxL + 1) * (kMaxL + 2) / 2;  // packed (l, m >= 0)
constexpr int kMaxFull = (kMaxL + 1) * (kMaxL + 1);      // packed (l, -l..l)

// warps of the split-precision rest kernel; its slot schedule is built for
// this many on the host
constexpr int kRestTableWarps = 32;
// flag of a slot's end record in the rest kernel's record stream
constexpr uint32_t kRestEnd = 0x80000000u;
// warps per CTA of the FP64 2-/4-body kernel (k_rest64), which walks its
// own slot schedule (RestTable::warp64_begin)
constexpr int kRestWarps64 = 16;
// record-stream tag of two one-factor entries in one record (see RestTable)
constexpr uint32_t kRestPair1 = 4u;
// end-record flag of one part of a split slot (low bits: 2 * split + part)
constexpr uint32_t kRestSplit = 0x40000000u;

// device-side error codes (first one wins)
enum DeviceError : int {
  kDevOk = 0,
  kDevSmallR = 1,  // r below the first LUT bin
  kDevMoment = 2,  // |m| negative, NaN or beyond the magnetic cutoff
  kDevNaN = 3,     // non-finite density
  kDevShape = 4,   // more bonds than a tile index can address
  kDevTimeout = 5, // a bulk copy of bond inputs did not complete within the wait limit
};

// largest number of other factors in one gather entry: a 6-body term
// A0 A1 .. A5 adds the product of five factors to each of its slots
constexpr int kMaxArity = 5;
// factor slots per descriptor term: six factors, ONE-padded to 16 bytes
constexpr int kDescFactors = 8;

// one gather table: group g has arity grp_arity[g], length grp_len[g] and its
// entries at grp_first[g] + e*32 + lane
struct GatherView {
  int nslot, nG0, nseg, ngroup;
  const int32_t* grp_arity;
  const int32_t* grp_len;
  const int32_t* grp_first;
  const int32_t* grp_seg;      // [ngroup*32] segment id per lane, -1 padding
  const double* kap[kMaxArity + 1];   // [arity][density * kstride[arity] + slot] FP64
  const float* kapf[kMaxArity + 1];   // FP32 copies (split path)
  int kstride[kMaxArity + 1];
  const uint32_t* o12[kMaxArity + 1]; // o1 | o2 << 16
  const uint32_t* o34[kMaxArity + 1]; // o3 | o4 << 16 (arity >= 3)
  const uint16_t* o5;                 // fifth factor of arity-5 entries
  const int32_t* slot_seg;     // [nslot+1]
  const int32_t* slot_factor;  // [nslot] (G0 slots only)
  const int32_t* slot_weight;  // [nslot]
  const double* slot_mult;     // [nslot]
  const float* slot_multf;     // FP32 copy (split path)
};

struct DeviceModel {
  // basis dims (see model.hpp for the layouts)
  int n3a, n3m, l3a, l3m, nba, n2m, l2m, nbm;
  int lsa, ls3, ls2, h3, h2;
  int offA, offA2, offA0, offOne, offZero, nF;
  int nWA, offW2, offW0, nW;
  int nd, nfemb;
  int high;  // the potential has 5- or 6-body clusters (generic kernels only)
  double par[2][2];  // embedding parameters [order][density]
  double ecut, decut;
  // radial lookup tables: [(nlut+1)][nf] double4 of cubic coefficients
  int nlut, nfa, nfm;
  double rscale_a, rscale_m;
  const double* lut_a;
  const double* lut_m;
  const float* lut_a32;  // FP32 copies for the split-precision path
  const float* lut_m32;
  // 1-body coefficients c1[d * nbm + n]
  const double* c1;
  // FP32 copies of the scale factors and 1-body coefficients (split path)
  float rscale_a_f, rscale_m_f;
  const float* c1f;
  // gather tables in warp groups (see model.hpp): g holds every term (generic
  // kernels), g2 every term except the 3-body ones (specialised kernels)
  GatherView g, g2;
  // dense 3-body tables of the specialised kernels (see model.hpp DenseB3)
  int b3_ntask, b3_ncombo, b3_nc;
  const float* b3_Cf;         // [combo][NM][I][I]
  const int32_t* b3_pattern;  // [combo]
  const int32_t* b3_combo;    // [task]
  const float* b3_cff;        // [task]
  const uint16_t* b3_code;    // [task][NM + 2I] compact element | sign bits
  const uint16_t* b3_code2;   // [task][NM + 2I] mirror-task gradient target, 0xffff for none
  const float* b3_cfw;        // [task] density weight (2 or 1) times the coupling
  const int32_t* b3_factor;   // [nc] factor index of each compact element
  const int32_t* b3_cw;       // [nW] compact element of each weight, or -1
  const float* b3_mult;       // [nc] half-plane multiplicity of each element's weight
  // FP64 copies for the plain-precision 3-body kernel, and the bound of its
  // gradients (model.hpp DenseB3::bound)
  const double* b3_C64;       // [combo][NM][I][I]
  const float* b3_Chl;        // [combo][NM][I][I][2] the same as hi + lo floats (float-float tasks)
  const double* b3_cf64;      // [task]
  const double* b3_cfw64;     // [task]
  double b3_bound, b3_bound_rho;
  // per-slot table of the 2- and 4-body terms (see model.hpp RestTable)
  int r_nfac, r_nslot;
  const int32_t* r_factor;
  const int32_t* r_run;         // [3 * nslot + 1]
  const uint32_t* r_rec;        // [entries][4]
  const double* r_kap64;        // [entries] kappa in FP64
  const float* r_kaphl;         // [entries][2] kappa as hi + lo floats (float-float entries)
  const int32_t* r_g0;
  const int32_t* r_warp_begin;  // [warps + 1]
  const int32_t* r_warp_slots;
  const uint32_t* r_stream;     // [records][4] per-warp record streams
  const int32_t* r_stream_begin;  // [warps + 1]
  const int32_t* r64_warp_begin;  // [kRestWarps64 + 1] the FP64 kernel's slot schedule
  const int32_t* r64_warp_slots;
  int r_nsplit;                 // slots split in two stream items
  const int32_t* r_split_w;     // [nsplit] their weight index, or -1
  // variants of the split-precision density kernels (indices into the
  // kernels.hpp choice tables)
  int tune_abasis, tune_rest, tune_b3, tune_forces;
  // work queue of this evaluation: atoms in order of decreasing bond count,
  // or null for the natural order (set per launch)
  const int32_t* order;
  // descriptor tables (see model.hpp DescriptorTable)
  int d_n1, d_nB;
  const int32_t* d_rank1_n;
  const int32_t* d_begin;
  const double* d_cf;
  const uint16_t* d_o;
};

}  // namespace magace
