// Kernels specialised at compile time for one basis layout: the layout of
// the reference's example Fe potential (example/Fe.pbe.in:6-13; 16/16 base
// functions, 4 atomic x 3 magnetic radial functions up to l = 1 / l' = 2,
// 5 magnetic pair functions up to l' = 2). Included by kernels.cu; the
// generic kernels there serve every other layout.
//
// With the dims known to the compiler, the per-bond and per-task loops fully
// unroll and their operands stay in registers:
//   k_abasis_fe  the bond sums A and A2 are small GEMMs over the bonds of an
//                atom; warp 0 owns 1 x 9 tiles of A, warp 1 1 x 15 tiles of A2.
//   k_density_fe the 2- and 4-body terms through the rest table (split
//                precision; FP64 uses the generic k_density).
//   k_b3_fe      the 3-body density and its gradients as dense
//                contractions per (angular combination, m-term) task,
//                C[n0'][i][j] a X Y, exploiting the triangular cluster
//                order, with 32 atoms in the lanes of each warp.
//   k_finish_fe  per atom, the total density, the embedding and the energy.
//   k_forces_fe  the weights dE/drho (W + g3), then per bond U = W_A Q and
//                V = W2 g + W_A^T RY with the weights transposed in shared
//                memory for 16-byte loads.

// byte offsets in a split tail block's record of accumulators (aux_layout):
// 3-body density [32] doubles, ticket, 3-body gradients [nc][32][2] floats
constexpr size_t kTailRho3 = 0, kTailTickets = 256, kTailG = 272;

template <int NA_, int LA_, int NM_, int LM_, int NB_, int N2_, int L2_, int NBM_>
struct Dims {
  static constexpr int NA = NA_, LA = LA_, NM = NM_, LM = LM_, NB = NB_, N2 = N2_, L2 = L2_, NBM = NBM_;
  static constexpr int LSA = (LA + 1) * (LA + 1), LS3 = (LM + 1) * (LM + 1), LS2 = (L2 + 1) * (L2 + 1);
  static constexpr int HA = (LA + 1) * (LA + 2) / 2, H3 = (LM + 1) * (LM + 2) / 2, H2 = (L2 + 1) * (L2 + 2) / 2;
  static constexpr int NR = NA * (LA + 1);  // atomic radial functions R_nl
  static constexpr int NMF = N2 * (L2 + 1); // magnetic radial functions M_nl
  static constexpr int NRY = NA * LSA;      // R_nl Y_lm products (rows of A)
  static constexpr int NQ = N2 * H2;        // M_nl Y_lm (m >= 0) products
  static constexpr int NQ3 = NM * H3;       // the subset used by A
  static constexpr int NWA = NRY * NQ3;
  static constexpr int NA2H = NB * NQ;
  static constexpr int I = NA * NM;         // dense 3-body index (n, n')
  static constexpr int NPOS = NM + 2 * I;   // outputs of one 3-body task
  static constexpr int NFA = NB + NR + 1;
  static constexpr int NFM = NMF + NBM;
};
using FeDims = Dims<4, 1, 3, 2, 16, 5, 2, 16>;

template <class D>
bool dims_match(const DeviceModel& m) {
  return m.n3a == D::NA && m.l3a == D::LA && m.n3m == D::NM && m.l3m == D::LM && m.nba == D::NB &&
         m.n2m == D::N2 && m.l2m == D::L2 && m.nbm == D::NBM && m.nfa == D::NFA && m.nfm == D::NFM;
}

__host__ __device__ constexpr int l_of_h(int h) { return h == 0 ? 0 : (h < 3 ? 1 : (h < 6 ? 2 : (h < 10 ? 3 : 4))); }
__host__ __device__ constexpr int l_of_lm(int lm) { return lm == 0 ? 0 : (lm < 4 ? 1 : (lm < 9 ? 2 : (lm < 16 ? 3 : 4))); }

// bond-row strides of k_abasis_fe's tiles: RY (complex), q (complex) and g;
// the tensor-core form pads them so that its fragment loads are free of
// bank conflicts
template <class D, bool TC>
struct AbasisRows {
  static constexpr int RY = TC ? D::NRY + 4 : D::NRY, Q = TC ? D::NQ + 6 : D::NQ, G = TC ? D::NB + 8 : D::NB;
};
// dynamic shared memory of k_abasis_fe without the staged tile
template <class R, class D, bool TC = false>
__host__ __device__ constexpr size_t abasis_fe_smem() {
  using S = AbasisRows<D, TC>;
  // sQ holds S::Q complex or, packed, 2 x 32 floats per bond
  const size_t q = sizeof(C<R>) * S::Q > sizeof(float) * 64 ? sizeof(C<R>) * S::Q : sizeof(float) * 64;
  return sizeof(C<R>) * 64 * S::RY + q * 64 + sizeof(R) * 64 * (S::G + 1) + 64;
}

// ===========================================================================
// Bond tiles staged by the Tensor Memory Accelerator. One thread issues, per
// input array, a bulk copy (cp.async.bulk) of a tile's bond segment into
// shared memory; the copies signal one mbarrier with their byte count and
// the CTA waits on its phase. A bulk copy needs 16-byte aligned addresses
// and a multiple of 16 bytes, and the caller's arrays are only 8-byte
// aligned, so each copy covers the 16-byte aligned interior of the segment
// and the at most two FP64 elements outside it are read from global memory
// by the threads that use them. An element g of the segment [e0, e1) sits
// at shared index g - e0 + h (h = 1 when element e0 starts 8 bytes past a
// 16-byte boundary), which keeps the interior's start 16-byte aligned.
// Every wait is bounded: after ~2^32 SM cycles it returns false and the
// kernel reports kDevTimeout instead of hanging.
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_to_smem(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
// L2 eviction priorities for single loads and stores: the weights the
// 3-body kernel writes are kept (evict-last) for the force kernel, which
// reads them once (evict-first), as does the 3-body kernel its factors
__device__ __forceinline__ uint64_t l2_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ void st_l2(C<float>* a, C<float> v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(__cvta_generic_to_global(a)), "f"(v.x),
               "f"(v.y), "l"(pol)
               : "memory");
}
__device__ __forceinline__ C<float> ld_l2(const C<float>* a, uint64_t pol) {
  C<float> v;
  asm volatile("ld.global.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;"
               : "=f"(v.x), "=f"(v.y)
               : "l"(__cvta_generic_to_global(a)), "l"(pol));
  return v;
}
__device__ __forceinline__ C<double> ld_l2(const C<double>* a, uint64_t pol) {
  C<double> v;
  asm volatile("ld.global.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;"
               : "=d"(v.x), "=d"(v.y)
               : "l"(__cvta_generic_to_global(a)), "l"(pol));
  return v;
}

// one bond's 8 inputs in the working precision, with an L2 policy
__device__ __forceinline__ void st8_l2(float* a, const float* v, uint64_t pol) {
  const size_t g = __cvta_generic_to_global(a);
  asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(g), "f"(v[0]), "f"(v[1]),
               "f"(v[2]), "f"(v[3]), "l"(pol)
               : "memory");
  asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(g + 16), "f"(v[4]), "f"(v[5]),
               "f"(v[6]), "f"(v[7]), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void st8_l2(double* a, const double* v, uint64_t) {
  for (int q = 0; q < 8; ++q) a[q] = v[q];
}
__device__ __forceinline__ void ld8_l2(const float* a, float* v, uint64_t pol) {
  const size_t g = __cvta_generic_to_global(a);
  asm volatile("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
               : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3])
               : "l"(g), "l"(pol));
  asm volatile("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
               : "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
               : "l"(g + 16), "l"(pol));
}
__device__ __forceinline__ void ld8_l2(const double* a, double* v, uint64_t) {
  for (int q = 0; q < 8; ++q) v[q] = a[q];
}

// a bulk prefetch of [src, src + bytes) into L2 (16-byte aligned, 16-byte multiple)
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}
// L2 prefetch of atom slot `a` of 32-atom block `b`'s row of an [atom][row]
// array (the row's whole 16-byte units, so nothing past the array is touched)
__device__ __forceinline__ void prefetch_row(const DeviceModel& m, int natom, const void* base, size_t row_bytes, int b,
                                             int a) {
  if (b * 32 + a >= natom) return;
  const int atom = queue_atom(m, b * 32 + a);
  const uintptr_t p0 = reinterpret_cast<uintptr_t>(base) + row_bytes * static_cast<size_t>(atom);
  const uintptr_t lo = (p0 + 15) & ~static_cast<uintptr_t>(15), hi = (p0 + row_bytes) & ~static_cast<uintptr_t>(15);
  if (hi > lo) bulk_prefetch_l2(reinterpret_cast<const void*>(lo), static_cast<uint32_t>(hi - lo));
}
// Blocks between this CTA's block and the next one to start on this SM, for
// a kernel of one CTA per SM: the grid stride on a persistent grid, else
// the SM count (CTAs start in block order as SMs free up)
__device__ __forceinline__ int next_stride() {
  unsigned nsm;
  asm("mov.u32 %0, %%nsmid;" : "=r"(nsm));
  return gridDim.x <= nsm ? static_cast<int>(gridDim.x) : static_cast<int>(nsm);
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const long long end = clock64() + (1ll << 32);
  while (!mbar_test(bar, parity))
    if (clock64() > end) return false;
  return true;
}

// the part of the segment [e0, e1) of array g that one bulk copy moves
struct TileWindow {
  int lo, hi, h;
};
__device__ __forceinline__ TileWindow tile_window(const double* g, int e0, int e1) {
  TileWindow w;
  w.h = (reinterpret_cast<uintptr_t>(g + e0) & 8u) ? 1 : 0;
  w.lo = e0 + w.h;
  w.hi = e1 - ((reinterpret_cast<uintptr_t>(g + e1) & 8u) ? 1 : 0);
  if (w.hi < w.lo) w.hi = w.lo;
  return w;
}
__device__ __forceinline__ double tile_value(const double* sbuf, const double* g, const TileWindow& w, int e0, int idx) {
  return (idx >= w.lo && idx < w.hi) ? sbuf[idx - e0 + w.h] : g[idx];
}

// shared-memory layout of one staged tile of up to 64 bonds: r, e[3], |m|,
// m-hat[3] as FP64, each array padded to keep the next one 16-byte aligned
constexpr int kTileR = 66, kTileE = 194;
constexpr int kTileDoubles = 2 * kTileR + 2 * kTileE;
constexpr size_t kTileBytes = sizeof(double) * kTileDoubles;
constexpr size_t kTileBarBytes = 16;  // the mbarrier and the staged tile's first bond

struct BondTile {
  double* r;
  double* e;
  double* mg;
  double* mh;
  uint64_t* bar;
  int* first;
  // p: kTileBytes, 16-byte aligned; q: kTileBarBytes, 8-byte aligned
  __device__ BondTile(unsigned char* p, unsigned char* q)
      : r(reinterpret_cast<double*>(p)), e(r + kTileR), mg(e + kTileE), mh(mg + kTileR),
        bar(reinterpret_cast<uint64_t*>(q)), first(reinterpret_cast<int*>(bar + 1)) {}
  // issues the copies of bonds [j0, j0 + nb) (one thread)
  __device__ void issue(const double* rr, const double* ee, const double* magj, const double* mhj, int j0, int nb) {
    const TileWindow w0 = tile_window(rr, j0, j0 + nb), w1 = tile_window(ee, 3 * j0, 3 * (j0 + nb)),
                     w2 = tile_window(magj, j0, j0 + nb), w3 = tile_window(mhj, 3 * j0, 3 * (j0 + nb));
    const uint32_t b0 = 8u * (w0.hi - w0.lo), b1 = 8u * (w1.hi - w1.lo), b2 = 8u * (w2.hi - w2.lo),
                   b3 = 8u * (w3.hi - w3.lo);
    *first = j0;
    // the buffer was last written and read through the generic proxy (the
    // caller passed a CTA barrier since): order those accesses before the
    // bulk copies' writes
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(bar, b0 + b1 + b2 + b3);
    if (b0) bulk_to_smem(r + 2 * w0.h, rr + w0.lo, b0, bar);
    if (b1) bulk_to_smem(e + 2 * w1.h, ee + w1.lo, b1, bar);
    if (b2) bulk_to_smem(mg + 2 * w2.h, magj + w2.lo, b2, bar);
    if (b3) bulk_to_smem(mh + 2 * w3.h, mhj + w3.lo, b3, bar);
  }
};

// the first tile of the first atom with bonds at queue position it, it +
// gridDim.x, ...: (j0, nb), nb = 0 when there is none
__device__ __forceinline__ int2 next_atom_tile(const DeviceModel& m, const int* __restrict__ off, int it, int natom,
                                               int tb) {
  for (; it < natom; it += gridDim.x) {
    const int a = queue_atom(m, it);
    const int c0 = off[a], c1 = off[a + 1];
    if (c1 > c0) return make_int2(c0, c1 - c0 < tb ? c1 - c0 : tb);
  }
  return make_int2(0, 0);
}

// ===========================================================================
// TF32 operands for mma.sync: x = hi + lo, hi the TF32 truncation of x (its
// low 13 mantissa bits cleared), lo = x - hi exactly (|lo| < 2^-10 |x|; the
// tensor cores read its TF32 part, so the products' error is below 2^-20
// relative). d += a b in the 3xTF32 split: lo hi' + hi lo' + hi hi'.
__device__ __forceinline__ void tf32_split(float x, uint32_t& hi, uint32_t& lo) {
  hi = __float_as_uint(x) & 0xffffe000u;
  lo = __float_as_uint(x - __uint_as_float(hi));
}
__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ void mma_3xtf32(float (&d)[4], const uint32_t (&ah)[4], const uint32_t (&al)[4],
                                           uint32_t bh0, uint32_t bh1, uint32_t bl0, uint32_t bl1) {
  mma_tf32(d, al, bh0, bh1);
  mma_tf32(d, ah, bl0, bl1);
  mma_tf32(d, ah, bh0, bh1);
}

// ---------------------------------------------------------------------------
// Float-float arithmetic for the FP64 path's contractions (FF). A double x is
// carried as hi + lo with hi = x rounded to FP32 and lo = x - hi rounded
// (48 bits of x). A dot product accumulates in (s, c): each product a b is
// split exactly into p + e (p = a.hi b.hi, e its FMA residual plus the cross
// terms a.hi b.lo + a.lo b.hi), s takes p by an error-free two-sum whose
// error, with e, goes to c; the result is s + c in FP64 (Ogita, Rump and
// Oishi's compensated dot product, "Dot2"). Its error is about 2^-48 of the
// sum of |products|, against 2^-53 in FP64, and it runs on the FP32 pipe,
// which on this part issues 64 times the FP64 pipe's operations.
struct FFv {
  float hi, lo;
};
__device__ __forceinline__ FFv ff_of(double x) {
  const float h = d2f(x);
  return {h, d2f(x - f2d(h))};  // x - h is exact in FP64
}
__device__ __forceinline__ double ff_d(float s, float c) { return f2d(s) + f2d(c); }
// (s, c) += a b
__device__ __forceinline__ void ff_dot(float& s, float& c, FFv a, FFv b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const float t = s + p, z = t - s;
  c += ((s - (t - z)) + (p - z)) + e;
  s = t;
}
__device__ __forceinline__ FFv ff_neg(FFv a) { return {-a.hi, -a.lo}; }
// a[h] for an h that differs across the lanes, by selection (no local memory)
template <int N, class V>
__device__ __forceinline__ V pick_of(const V (&a)[N], int h) {
  V v = a[0];
#pragma unroll
  for (int j = 1; j < N; ++j)
    if (h == j) v = a[j];
  return v;
}
// a complex weight staged as float-float in the 16 bytes of a C<double>
struct FFc {
  FFv x, y;
};
// a compensated sum (s, c) as hi + lo, and acc += a b for complex
// float-float a, b into (Re s, Re c, Im s, Im c)
__device__ __forceinline__ FFv ff_norm(float s, float c) {
  const float h = s + c;
  return {h, c - (h - s)};
}
__device__ __forceinline__ void ff_cmac(float (&acc)[4], FFc a, FFc b) {
  ff_dot(acc[0], acc[1], a.x, b.x);
  ff_dot(acc[0], acc[1], ff_neg(a.y), b.y);
  ff_dot(acc[2], acc[3], a.x, b.y);
  ff_dot(acc[2], acc[3], a.y, b.x);
}

// ===========================================================================
// PACKED (split precision only): the M Y tile is stored as real and
// imaginary planes of 32 columns, and the lanes accumulate column pairs with
// packed FP32x2 FMAs (warp 0: five pairs of the 18 A columns per half-row,
// warp 1: eight pairs of the 30 A2 columns; padding pairs are discarded).
//
// TMA (device-resident inputs only): each CTA's bond tiles staged into
// shared memory by bulk copies (BondTile); the copy of the CTA's next tile
// is issued as soon as the current tile's features are computed, so that it
// overlaps the bond sums and the completion of A (on a persistent grid every
// tile after a CTA's first arrives this way).
//
// TC (split precision only): the bond sums as GEMMs over the tile's bonds
// (K) on the tensor cores, mma.sync m16n8k8 TF32 in the 3xTF32 split.
// Warp 0: D1 = [Re RY; Im RY]^T (32 x K) times Q (K x 40, Re and Im of q_k
// interleaved), so that each lane holds Re and Im of both parts of A_ik:
// A = (D1[Re][Re q] - D1[Im][Im q], D1[Re][Im q] + D1[Im][Re q]). Warp 1:
// D2 = g^T (16 x K) times Q (K x 64) is A2 itself. Bonds past the atom's
// last are zero rows of both operands.
template <class R, class D, bool PACKED, bool TMA = false, bool TC = false>
__global__ void __launch_bounds__(64)
    k_abasis_fe(DeviceModel m, int natom, const int* __restrict__ off, const double* __restrict__ rr,
                const double* __restrict__ ee, const double* __restrict__ magj, const double* __restrict__ mhj,
                const double* __restrict__ magi, const double* __restrict__ mhi, C<R>* __restrict__ F,
                double* __restrict__ rho1, double* __restrict__ core_out, R* __restrict__ stage, int* err) {
  constexpr int TB = 64;
  static_assert(D::NRY == 16 && D::NB == 16 && D::NQ3 == 18 && D::NQ == 30, "tile shapes assume the Fe layout");
  extern __shared__ __align__(16) unsigned char smem[];
  using S = AbasisRows<D, TC>;
  // FP64 path: the bond sums as float-float dot products on the FP32 pipe
  constexpr bool FF = sizeof(R) == 8 && !PACKED && !TC;
  static_assert(!FF || sizeof(FFc) == sizeof(C<R>), "float-float tiles reuse the FP64 rows");
  C<R>* sRY = reinterpret_cast<C<R>*>(smem);             // [TB][S::RY]
  C<R>* sQ = sRY + TB * S::RY;                            // [TB][S::Q] (PACKED: 2 x [TB][32] floats)
  constexpr size_t kQBytes = sizeof(C<R>) * S::Q > sizeof(float) * 64 ? sizeof(C<R>) * S::Q : sizeof(float) * 64;
  R* sg = reinterpret_cast<R*>(reinterpret_cast<unsigned char*>(sQ) + TB * kQBytes);  // [TB][S::G]
  R* score = sg + TB * S::G;                              // [TB]
  float* sQx = reinterpret_cast<float*>(sQ);              // PACKED: [TB][32] real, then imaginary
  float* sQy = sQx + TB * 32;
  C<R>* accA = sRY;                                       // reuse after the tiles: [NRY][NQ3]
  C<R>* accA2 = accA + D::NWA;                            // [NB][NQ]
  double core_acc = 0.0;  // warp 1: the atom's core energy, over its bond tiles
  static_assert(!PACKED || (sizeof(R) == 4 && D::H3 == D::H2 && D::NQ <= 32), "packed tiles: FP32, Fe layout");
  static_assert(!TC || (sizeof(R) == 4 && !PACKED && D::H3 == D::H2), "tensor-core sums: FP32, Fe layout");
  static_assert(D::NWA + D::NA2H <= TB * S::RY, "A and A2 fit in the RY tile");
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int row = lane >> 1, cb = lane & 1;
  const uint64_t pol_f = l2_evict_first();  // split path: the factors are read once per density kernel
  // TMA: the staged tile lives in the M Y tile's space (sQ), which is not
  // read between the end of a tile's bond sums and the next tile's
  // features; its mbarrier after the other buffers
  static_assert(sizeof(C<R>) * D::NQ * 64 >= kTileBytes || sizeof(float) * 64 * 64 >= kTileBytes,
                "the staged tile fits in the M Y tile");
  BondTile tile(reinterpret_cast<unsigned char*>(sQ),
                smem + ((abasis_fe_smem<R, D, TC>() + 15) & ~static_cast<size_t>(15)));
  constexpr int kIssuer = 32;  // lane 0 of warp 1 issues the copies
  uint32_t phase = 0;
  bool timed_out = false;
  uint32_t timeout_parity = 0;
  if constexpr (TMA) {
    if (t == kIssuer) {
      mbar_init(tile.bar, 1);
      const int2 first = next_atom_tile(m, off, blockIdx.x, natom, TB);
      if (first.y > 0) tile.issue(rr, ee, magj, mhj, first.x, first.y);
    }
    __syncthreads();
  }

  for (int it = blockIdx.x; it < natom; it += gridDim.x) {
    const int atom = queue_atom(m, it);
    C<R> acc[15];
#pragma unroll
    for (int c = 0; c < 15; ++c) acc[c] = {R(0), R(0)};
    float2 accx[8], accy[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) accx[c] = accy[c] = make_float2(0.f, 0.f);
    float dacc[10][4];  // TC: warp 0 D1 tiles [m-tile * 5 + n-tile], warp 1 D2 tiles [n-tile]
    float ffa[15][4];   // FF: per column (Re sum, Re compensation, Im sum, Im compensation)
#pragma unroll
    for (int c = 0; c < 15; ++c) ffa[c][0] = ffa[c][1] = ffa[c][2] = ffa[c][3] = 0.f;
#pragma unroll
    for (int u = 0; u < 10; ++u)
#pragma unroll
      for (int e = 0; e < 4; ++e) dacc[u][e] = 0.f;
    core_acc = 0.0;
    const int b0 = off[atom], b1 = off[atom + 1];
    for (int t0 = b0; t0 < b1; t0 += TB) {
      const int nb = min(TB, b1 - t0);
      __syncthreads();
      if constexpr (TMA) {
        // a later tile of this atom: the previous tile's bond sums are done
        if (t0 > b0 && t == kIssuer) tile.issue(rr, ee, magj, mhj, t0, nb);
        if (!mbar_wait(tile.bar, phase)) {
          raise_error(err, kDevTimeout);
          timed_out = true;
          timeout_parity = phase;
        }
        phase ^= 1u;
      }
      // the bond's inputs
      double dr = 0.0, dex = 0.0, dey = 0.0, dez = 0.0, dmg = 0.0, dmx = 0.0, dmy = 0.0, dmz = 0.0;
      if (t < nb) {
        const int j = t0 + t;
        if constexpr (TMA) {
          if (*tile.first != t0) raise_error(err, kDevShape);  // the staged tile is always this one
          const int e0 = 3 * t0, e1 = 3 * (t0 + nb);
          const TileWindow w0 = tile_window(rr, t0, t0 + nb), w1 = tile_window(ee, e0, e1),
                           w2 = tile_window(magj, t0, t0 + nb), w3 = tile_window(mhj, e0, e1);
          dr = tile_value(tile.r, rr, w0, t0, j);
          dex = tile_value(tile.e, ee, w1, e0, 3 * j);
          dey = tile_value(tile.e, ee, w1, e0, 3 * j + 1);
          dez = tile_value(tile.e, ee, w1, e0, 3 * j + 2);
          dmg = tile_value(tile.mg, magj, w2, t0, j);
          dmx = tile_value(tile.mh, mhj, w3, e0, 3 * j);
          dmy = tile_value(tile.mh, mhj, w3, e0, 3 * j + 1);
          dmz = tile_value(tile.mh, mhj, w3, e0, 3 * j + 2);
        } else {
          dr = rr[j];
          dex = ee[3 * j];
          dey = ee[3 * j + 1];
          dez = ee[3 * j + 2];
          dmg = magj[j];
          dmx = mhj[3 * j];
          dmy = mhj[3 * j + 1];
          dmz = mhj[3 * j + 2];
        }
      }
      if constexpr (TMA) __syncthreads();  // the staged tile is read: sQ may be written
      if (t < nb) {
        const int j = t0 + t;
        // the bond's inputs in the working precision; with `stage`, also
        // kept in device memory for the force kernel (8 values per bond)
        const R br = to_r<R>(dr);
        const R bex = to_r<R>(dex), bey = to_r<R>(dey), bez = to_r<R>(dez);
        const R bmg = to_r<R>(dmg);
        const R bmx = to_r<R>(dmx), bmy = to_r<R>(dmy), bmz = to_r<R>(dmz);
        if (stage) {
          const R sv[8] = {br, bex, bey, bez, bmg, bmx, bmy, bmz};
          st8_l2(stage + 8 * static_cast<size_t>(j), sv, l2_evict_last());  // kept in L2 for the force kernel
        }
        R g[D::NB], Rv[D::NR], Mv[D::NMF], cv[1], dummy[1];
        R wl = R(0);
        const int nla = atomic_bin_r<R>(m, br, wl, err);
        if (nla > 0) {
          lut_eval<false>(pick<R>(m.lut_a, m.lut_a32), D::NFA, 0, D::NB, nla, wl, rscale_a<R>(m), g, dummy);
          lut_eval<false>(pick<R>(m.lut_a, m.lut_a32), D::NFA, D::NB, D::NR, nla, wl, rscale_a<R>(m), Rv, dummy);
          lut_eval<false>(pick<R>(m.lut_a, m.lut_a32), D::NFA, D::NB + D::NR, 1, nla, wl, rscale_a<R>(m), cv, dummy);
        } else {
#pragma unroll
          for (int q = 0; q < D::NB; ++q) g[q] = R(0);
#pragma unroll
          for (int q = 0; q < D::NR; ++q) Rv[q] = R(0);
          cv[0] = R(0);
        }
        R wm = R(0);
        const int nlm = magnetic_bin_r<R>(m, bmg, wm, err);
        if (nlm > 0) {
          lut_eval<false>(pick<R>(m.lut_m, m.lut_m32), D::NFM, 0, D::NMF, nlm, wm, rscale_m<R>(m), Mv, dummy);
        } else {
#pragma unroll
          for (int q = 0; q < D::NMF; ++q) Mv[q] = R(nlm == 0 ? 1 : 0);
        }
        C<R> Ya[D::HA], Ym[D::H2];
        ylm_half<R, false>(D::LA, bex, bey, bez, Ya, nullptr);
        ylm_half<R, false>(D::L2, bmx, bmy, bmz, Ym, nullptr);
#pragma unroll
        for (int n1 = 0; n1 < D::NA; ++n1)
#pragma unroll
          for (int lm = 0; lm < D::LSA; ++lm) {
            const int l = l_of_lm(lm), mm = lm - l * l - l;
            const C<R> ry = cscale(y_full(Ya, l, mm), Rv[n1 * (D::LA + 1) + l]);
            if constexpr (FF) {
              reinterpret_cast<FFc*>(sRY)[t * S::RY + n1 * D::LSA + lm] = {ff_of(ry.x), ff_of(ry.y)};
            } else {
              sRY[t * S::RY + n1 * D::LSA + lm] = ry;
            }
          }
#pragma unroll
        for (int nr = 0; nr < D::N2; ++nr)
#pragma unroll
          for (int h = 0; h < D::H2; ++h) {
            const C<R> q = cscale(Ym[h], Mv[nr * (D::L2 + 1) + l_of_h(h)]);
            if constexpr (PACKED) {
              sQx[t * 32 + nr * D::H2 + h] = q.x;
              sQy[t * 32 + nr * D::H2 + h] = q.y;
            } else {
              if constexpr (FF) {
                reinterpret_cast<FFc*>(sQ)[t * S::Q + nr * D::H2 + h] = {ff_of(q.x), ff_of(q.y)};
              } else {
                sQ[t * S::Q + nr * D::H2 + h] = q;
              }
            }
          }
        if constexpr (PACKED) {
          for (int k = D::NQ; k < 32; ++k) sQx[t * 32 + k] = sQy[t * 32 + k] = 0.f;
        }
#pragma unroll
        for (int n = 0; n < D::NB; ++n) {
          if constexpr (FF) {
            reinterpret_cast<FFv*>(sg)[t * S::G + n] = ff_of(g[n]);
          } else {
            sg[t * S::G + n] = g[n];
          }
        }
        score[t] = cv[0];
      } else if constexpr (TC) {
        // a bond past the atom's last: zero rows (the GEMMs sum over all 64)
#pragma unroll
        for (int i = 0; i < D::NRY; ++i) sRY[t * S::RY + i] = {R(0), R(0)};
#pragma unroll
        for (int k = 0; k < D::NQ; ++k) sQ[t * S::Q + k] = {R(0), R(0)};
#pragma unroll
        for (int n = 0; n < D::NB; ++n) sg[t * S::G + n] = R(0);
      }
      __syncthreads();
      if constexpr (TC) {
        const int gid = lane >> 2, tig = lane & 3;
        const int nks = (nb + 7) >> 3;  // k-steps of 8 bonds holding a bond
        const float* Qf = reinterpret_cast<const float*>(sQ);  // [TB][2 S::Q]: Re, Im interleaved
        if (warp == 0) {
          const float2* RYf = reinterpret_cast<const float2*>(sRY);
          for (int ks = 0; ks < nks; ++ks) {
            const int k0 = 8 * ks + tig;
            // A fragments of both m-tiles (Re RY rows, Im RY rows): rows gid, gid + 8
            const float2 r00 = RYf[k0 * S::RY + gid], r10 = RYf[k0 * S::RY + gid + 8];
            const float2 r01 = RYf[(k0 + 4) * S::RY + gid], r11 = RYf[(k0 + 4) * S::RY + gid + 8];
            uint32_t ah[2][4], al[2][4];
            tf32_split(r00.x, ah[0][0], al[0][0]);
            tf32_split(r10.x, ah[0][1], al[0][1]);
            tf32_split(r01.x, ah[0][2], al[0][2]);
            tf32_split(r11.x, ah[0][3], al[0][3]);
            tf32_split(r00.y, ah[1][0], al[1][0]);
            tf32_split(r10.y, ah[1][1], al[1][1]);
            tf32_split(r01.y, ah[1][2], al[1][2]);
            tf32_split(r11.y, ah[1][3], al[1][3]);
#pragma unroll
            for (int nt = 0; nt < 5; ++nt) {
              uint32_t bh0, bl0, bh1, bl1;
              tf32_split(Qf[k0 * 2 * S::Q + 8 * nt + gid], bh0, bl0);
              tf32_split(Qf[(k0 + 4) * 2 * S::Q + 8 * nt + gid], bh1, bl1);
              mma_3xtf32(dacc[nt], ah[0], al[0], bh0, bh1, bl0, bl1);
              mma_3xtf32(dacc[5 + nt], ah[1], al[1], bh0, bh1, bl0, bl1);
            }
          }
        } else {
          for (int ks = 0; ks < nks; ++ks) {
            const int k0 = 8 * ks + tig;
            uint32_t ah[4], al[4];
            tf32_split(sg[k0 * S::G + gid], ah[0], al[0]);
            tf32_split(sg[k0 * S::G + gid + 8], ah[1], al[1]);
            tf32_split(sg[(k0 + 4) * S::G + gid], ah[2], al[2]);
            tf32_split(sg[(k0 + 4) * S::G + gid + 8], ah[3], al[3]);
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
              uint32_t bh0, bl0, bh1, bl1;
              tf32_split(Qf[k0 * 2 * S::Q + 8 * nt + gid], bh0, bl0);
              tf32_split(Qf[(k0 + 4) * 2 * S::Q + 8 * nt + gid], bh1, bl1);
              mma_3xtf32(dacc[nt], ah, al, bh0, bh1, bl0, bl1);
            }
          }
        }
      } else if constexpr (PACKED) {
        if (warp == 0) {
          // A[row][10cb .. 10cb+9] (columns 18, 19 padding)
          for (int b = 0; b < nb; ++b) {
            const C<R> ry = sRY[b * S::RY + row];
            const float2 rxx = make_float2(ry.x, ry.x), ryy = make_float2(ry.y, ry.y),
                         ryn = make_float2(-ry.y, -ry.y);
            const float2* qx = reinterpret_cast<const float2*>(sQx + b * 32 + 10 * cb);
            const float2* qy = reinterpret_cast<const float2*>(sQy + b * 32 + 10 * cb);
#pragma unroll
            for (int c = 0; c < 5; ++c) {
              const float2 a = qx[c], d = qy[c];
              accx[c] = __ffma2_rn(ryn, d, __ffma2_rn(rxx, a, accx[c]));
              accy[c] = __ffma2_rn(ryy, a, __ffma2_rn(rxx, d, accy[c]));
            }
          }
        } else {
          // A2[row][16cb .. 16cb+15] (columns 30, 31 padding)
          for (int b = 0; b < nb; ++b) {
            const R gv = sg[b * S::G + row];
            const float2 gg = make_float2(gv, gv);
            const float2* qx = reinterpret_cast<const float2*>(sQx + b * 32 + 16 * cb);
            const float2* qy = reinterpret_cast<const float2*>(sQy + b * 32 + 16 * cb);
#pragma unroll
            for (int c = 0; c < 8; ++c) {
              accx[c] = __ffma2_rn(gg, qx[c], accx[c]);
              accy[c] = __ffma2_rn(gg, qy[c], accy[c]);
            }
          }
        }
      } else if constexpr (FF) {
        // FP64 path: the same sums as compensated float-float dot products
        // (the tile's features were split into hi/lo floats as they were
        // written): ffa[c] = (Re sum, Re compensation, Im sum, Im compensation)
        const FFc* RYf = reinterpret_cast<const FFc*>(sRY);
        const FFc* Qf = reinterpret_cast<const FFc*>(sQ);
        if (warp == 0) {
          for (int b = 0; b < nb; ++b) {
            const FFc ry = RYf[b * S::RY + row];
            const FFv ryn = ff_neg(ry.y);
#pragma unroll
            for (int c = 0; c < 9; ++c) {
              const int k3 = 9 * cb + c;
              const FFc q = Qf[b * S::Q + (k3 / D::H3) * D::H2 + k3 % D::H3];
              ff_dot(ffa[c][0], ffa[c][1], ry.x, q.x);
              ff_dot(ffa[c][0], ffa[c][1], ryn, q.y);
              ff_dot(ffa[c][2], ffa[c][3], ry.x, q.y);
              ff_dot(ffa[c][2], ffa[c][3], ry.y, q.x);
            }
          }
        } else {
          const FFv* gf = reinterpret_cast<const FFv*>(sg);
          for (int b = 0; b < nb; ++b) {
            const FFv gv = gf[b * S::G + row];
#pragma unroll
            for (int c = 0; c < 15; ++c) {
              const FFc q = Qf[b * S::Q + 15 * cb + c];
              ff_dot(ffa[c][0], ffa[c][1], gv, q.x);
              ff_dot(ffa[c][2], ffa[c][3], gv, q.y);
            }
          }
        }
      } else if (warp == 0) {
        // A[row][9cb .. 9cb+8], row = (n1, l1 m1), column = (n2, l2 m2 >= 0)
        for (int b = 0; b < nb; ++b) {
          const C<R> ry = sRY[b * S::RY + row];
#pragma unroll
          for (int c = 0; c < 9; ++c) {
            const int k3 = 9 * cb + c;
            const C<R> q = sQ[b * S::Q + (k3 / D::H3) * D::H2 + k3 % D::H3];
            cmac(acc[c], ry, q);
          }
        }
      } else {
        // A2[row][15cb .. 15cb+14], row = n, column = (n', l' m' >= 0)
        for (int b = 0; b < nb; ++b) {
          const R gv = sg[b * S::G + row];
#pragma unroll
          for (int c = 0; c < 15; ++c) {
            const C<R> q = sQ[b * S::Q + 15 * cb + c];
            acc[c].x = fma(gv, q.x, acc[c].x);
            acc[c].y = fma(gv, q.y, acc[c].y);
          }
        }
      }
      if (warp == 1) {
        double cs = (lane < nb ? static_cast<double>(score[lane]) : 0.0) +
                    (lane + 32 < nb ? static_cast<double>(score[lane + 32]) : 0.0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cs += __shfl_xor_sync(0xffffffffu, cs, o);
        core_acc += cs;
      }
    }
    __syncthreads();
    if constexpr (TMA) {
      // the bond sums are done (sQ is free): stage the CTA's next atom's
      // first tile while A is completed and written
      if (b1 > b0 && t == kIssuer) {
        const int2 nx = next_atom_tile(m, off, it + gridDim.x, natom, TB);
        if (nx.y > 0) tile.issue(rr, ee, magj, mhj, nx.x, nx.y);
      }
    }
    if constexpr (TC) {
      // fragment c0..c3 = rows (gid, gid, gid + 8, gid + 8), columns (2 tig, 2 tig + 1) of n-tile nt
      const int gid = lane >> 2, tig = lane & 3;
      if (warp == 0) {
#pragma unroll
        for (int nt = 0; nt < 5; ++nt) {
          const int k = 4 * nt + tig;
          if (k < D::NQ3) {
            const float* re = dacc[nt];
            const float* im = dacc[5 + nt];
            accA[gid * D::NQ3 + k] = {re[0] - im[1], re[1] + im[0]};
            accA[(gid + 8) * D::NQ3 + k] = {re[2] - im[3], re[3] + im[2]};
          }
        }
      } else {
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
          const int k = 4 * nt + tig;
          if (k < D::NQ) {
            accA2[gid * D::NQ + k] = {dacc[nt][0], dacc[nt][1]};
            accA2[(gid + 8) * D::NQ + k] = {dacc[nt][2], dacc[nt][3]};
          }
        }
      }
    } else if constexpr (PACKED) {
      if (warp == 0) {
#pragma unroll
        for (int c = 0; c < 10; ++c) {
          const int k3 = 10 * cb + c;
          const float2 x = accx[c / 2], y = accy[c / 2];
          if (k3 < D::NQ3) accA[row * D::NQ3 + k3] = (c & 1) ? C<R>{x.y, y.y} : C<R>{x.x, y.x};
        }
      } else {
#pragma unroll
        for (int c = 0; c < 16; ++c) {
          const int k = 16 * cb + c;
          const float2 x = accx[c / 2], y = accy[c / 2];
          if (k < D::NQ) accA2[row * D::NQ + k] = (c & 1) ? C<R>{x.y, y.y} : C<R>{x.x, y.x};
        }
      }
    } else if constexpr (FF) {
      if (warp == 0) {
#pragma unroll
        for (int c = 0; c < 9; ++c)
          accA[row * D::NQ3 + 9 * cb + c] = {ff_d(ffa[c][0], ffa[c][1]), ff_d(ffa[c][2], ffa[c][3])};
      } else {
#pragma unroll
        for (int c = 0; c < 15; ++c)
          accA2[row * D::NQ + 15 * cb + c] = {ff_d(ffa[c][0], ffa[c][1]), ff_d(ffa[c][2], ffa[c][3])};
      }
    } else if (warp == 0) {
#pragma unroll
      for (int c = 0; c < 9; ++c) accA[row * D::NQ3 + 9 * cb + c] = acc[c];
    } else {
#pragma unroll
      for (int c = 0; c < 15; ++c) accA2[row * D::NQ + 15 * cb + c] = acc[c];
    }
    __syncthreads();
    // complete the m' < 0 half by A(m1,m2) = (-1)^(m1+m2) conj A(-m1,-m2) and write F
    C<R>* Fa = F + static_cast<size_t>(atom) * m.nF;
    constexpr int nA = D::NRY * D::NM * D::LS3;
    if constexpr (sizeof(R) == 4) {
      // split path: only the elements the density kernels read, A with
      // m' >= 0 (the 3-body codes reach the other half as mirrors) and A2
      // with m' <= 0 (the folded 2-body entries)
      for (int q = t; q < D::NRY * D::NM * D::H3; q += blockDim.x) {
        const int h = q % D::H3, l2 = l_of_h(h), m2 = h - l2 * (l2 + 1) / 2;
        st_l2(Fa + m.offA + (q / D::H3) * D::LS3 + l2 * l2 + l2 + m2, accA[q], pol_f);
      }
      for (int q = t; q < D::NB * D::N2 * D::H2; q += blockDim.x) {
        const int h = q % D::H2, l = l_of_h(h), mh = h - l * (l + 1) / 2;
        const C<R> w = accA2[q];
        const R sgn = R(parity(mh));
        st_l2(Fa + m.offA2 + (q / D::H2) * D::LS2 + l * l + l - mh, mh ? C<R>{w.x * sgn, -w.y * sgn} : w, pol_f);
      }
    }
    for (int s = t; s < (sizeof(R) == 4 ? 0 : nA); s += blockDim.x) {
      const int lmm = s % D::LS3, q = s / D::LS3, n2 = q % D::NM, ia = q / D::NM;
      const int lma = ia % D::LSA;
      const int l2 = l_of_lm(lmm), m2 = lmm - l2 * l2 - l2;
      const int l1 = l_of_lm(lma), m1 = lma - l1 * l1 - l1;
      C<R> v;
      if (m2 >= 0) {
        v = accA[ia * D::NQ3 + n2 * D::H3 + ph(l2, m2)];
      } else {
        const int ib = ia - lma + (l1 * l1 + l1 - m1);
        const C<R> w = accA[ib * D::NQ3 + n2 * D::H3 + ph(l2, -m2)];
        const R sgn = R(parity(m1 + m2));
        v = {w.x * sgn, -w.y * sgn};
      }
      Fa[m.offA + s] = v;
    }
    constexpr int nA2 = D::NB * D::N2 * D::LS2;
    for (int s = t; s < (sizeof(R) == 4 ? 0 : nA2); s += blockDim.x) {
      const int lm = s % D::LS2, q = s / D::LS2;  // q = n*N2 + nr
      const int l = l_of_lm(lm), mm = lm - l * l - l;
      const C<R> w = accA2[(q / D::N2) * D::NQ + (q % D::N2) * D::H2 + ph(l, mm < 0 ? -mm : mm)];
      C<R> v = w;
      if (mm < 0) {
        const R sgn = R(parity(mm));
        v = {w.x * sgn, -w.y * sgn};
      }
      Fa[m.offA2 + s] = v;
    }
    if (warp == 1) {
      // on-site A0 and the 1-body density in the working precision, one
      // magnetic function per lane: lane q < NMF holds M_q, lane NMF + n the
      // 1-body function g_n
      static_assert(D::NMF + D::NBM <= 32 && D::N2 * D::LS2 <= 64, "one function per lane");
      R wl = R(0);
      const int nl = magnetic_bin_r<R>(m, to_r<R>(magi[atom]), wl, err);
      R v = R(nl == 0 ? 1 : 0), dummy[1];
      if (nl > 0 && lane < D::NMF + D::NBM)
        lut_eval<false>(pick<R>(m.lut_m, m.lut_m32), D::NFM, lane, 1, nl, wl, rscale_m<R>(m), &v, dummy);
      C<R> Yi[D::H2];
      ylm_half<R, false>(D::L2, to_r<R>(mhi[3 * atom]), to_r<R>(mhi[3 * atom + 1]), to_r<R>(mhi[3 * atom + 2]), Yi,
                         nullptr);
#pragma unroll
      for (int k0 = 0; k0 < D::N2 * D::LS2; k0 += 32) {
        const int k = k0 + lane;
        const int nr = k / D::LS2, lm = k % D::LS2, l = l_of_lm(lm), mm = lm - l * l - l;
        const R mv = __shfl_sync(0xffffffffu, v, k < D::N2 * D::LS2 ? nr * (D::L2 + 1) + l : 0);
        if (k < D::N2 * D::LS2) {
          // y_full with (l, m) that differ across the lanes: Y by selection
          C<R> yv = pick_of(Yi, ph(l, mm < 0 ? -mm : mm));
          if (mm < 0) {
            const R sg = R(parity(mm));
            yv = {yv.x * sg, -yv.y * sg};
          }
          Fa[m.offA0 + k] = cscale(yv, mv);
        }
      }
      if (lane == 0) {
        Fa[m.offOne] = {R(1), R(0)};
        Fa[m.offZero] = {R(0), R(0)};
        core_out[atom] = core_acc;
      }
      for (int d = 0; d < m.nd; ++d) {
        const int n = lane - D::NMF;
        double s1 = n >= 0 && n < D::NBM ? static_cast<double>(c1_of<R>(m, d * D::NBM + n) * (v - R(1))) : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        if (lane == 0) rho1[static_cast<size_t>(atom) * 2 + d] = s1;
      }
    }
    __syncthreads();
  }
  if constexpr (TMA) {
    if (timed_out) mbar_wait(tile.bar, timeout_parity);  // a copy still in flight: wait once more, bounded
  }
}

// ===========================================================================
// The split-precision density phase of the specialised layout, three
// kernels; the first two are independent and may run side by side:
//
// k_density_fe (32 atoms per CTA, one per lane) evaluates the 2- and 4-body
// terms through the rest table and writes, per atom, their density rho_rest
// and the unscaled weights mult * dRho_rest/dF into W.
//
// k_b3_fe (32 atoms per CTA, one per lane) evaluates the 3-body terms as
// dense contractions per (angular combination, m-term) task and writes, per
// atom, their density rho3 and the gradients mult * dRho3/dF into g3.
//
// k_finish_fe (one atom per thread) adds rho = rho1 + rho_rest + rho3 and
// evaluates the embedding and energy in FP64; the force kernel then forms
// the weights W = dE/drho * (W + g3).

// Global loads of the staging and weight loops are issued kBatch at a time,
// so that each thread has that many in flight.
constexpr int kBatch = 8;


// k_density_fe: 32 atoms per CTA, one per lane; every warp walks its share
// of the output slots of the rest table (dealt longest first on the host).
// All lanes of a warp read the same 16-byte entry records (uniform loads)
// and apply them to their own atom's factors, staged in shared memory as
// Fs[factor][atom]. Slot totals are FP32 sums in entry order; the density
// terms of the A0 slots add up per lane in FP64, and the per-warp partials
// in warp order.
constexpr int kRestStride = 33;  // row stride of Fs in complex elements

template <int A>
__device__ __forceinline__ void rest_run(const uint4* __restrict__ rec, int e0, int e1, const C<float>* Fs, int lane,
                                         float& vx, float& vy) {
#pragma unroll 4
  for (int e = e0; e < e1; ++e) {
    const uint4 r = __ldg(rec + e);
    const float k = __uint_as_float(r.x);
    C<float> p = Fs[(r.y & 0xffffu) * kRestStride + lane];
    if (A >= 2) p = cmul(p, Fs[(r.y >> 16) * kRestStride + lane]);
    if (A >= 3) p = cmul(p, Fs[r.z * kRestStride + lane]);
    vx += k * p.x;
    vy += k * p.y;
  }
}

// NW warps per CTA (a divisor of kRestTableWarps): warp w walks the slots
// the host schedule gave to warps w, w + NW, ... With STREAM the warp reads
// its slots as one record stream, 32 records per coalesced load, and
// broadcasts record q to every lane with warp shuffles (STREAM 1) or, 16
// records at a time, through a per-warp shared-memory buffer read with one
// uniform 16-byte load per record (STREAM 2), instead of one warp-uniform
// global load per entry (STREAM 0).
template <class D, int NW, int STREAM>
__global__ void __launch_bounds__(NW * 32, 1)
    k_density_fe(DeviceModel m, int natom, const C<float>* __restrict__ F, C<float>* __restrict__ W,
                 double* __restrict__ rho_rest) {
  static_assert(kRestTableWarps % NW == 0, "the slot schedule is dealt to kRestTableWarps warps");
  extern __shared__ __align__(16) unsigned char smem[];
  const int nf = m.r_nfac, nW = m.nW;
  const uint64_t pol_last = l2_evict_last();  // the weights are read by the force kernel
  const GatherView& g = m.g2;  // slot weights and multiplicities (same slot numbering)
  C<float>* Fs = reinterpret_cast<C<float>*>(smem);                   // [nf][33]
  double* rpart = reinterpret_cast<double*>(Fs + nf * kRestStride);   // [NW][32]
  __shared__ int s_atom[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nblk = (natom + 31) / 32;
  const uint4* rec = reinterpret_cast<const uint4*>(m.r_rec);

  for (int blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int a0 = blk * 32;
    const int na = min(32, natom - a0);
    __syncthreads();
    if (threadIdx.x < na) s_atom[threadIdx.x] = queue_atom(m, a0 + threadIdx.x);
    __syncthreads();
    // stage: thread c takes factor c of every atom, kBatch atoms in flight
    for (int c = threadIdx.x; c < nf; c += blockDim.x) {
      const int fc = __ldg(m.r_factor + c);
      for (int ab = 0; ab < 32; ab += kBatch) {
        C<float> v[kBatch];
#pragma unroll
        for (int b = 0; b < kBatch; ++b)
          v[b] = ab + b < na ? F[static_cast<size_t>(s_atom[ab + b]) * m.nF + fc] : C<float>{0.f, 0.f};
#pragma unroll
        for (int b = 0; b < kBatch; ++b) Fs[c * kRestStride + ab + b] = v[b];
      }
    }
    __syncthreads();
    // the factors of the block that follows this one on the SM, into L2
    if (warp == NW - 1) prefetch_row(m, natom, F, sizeof(C<float>) * m.nF, blk + next_stride(), lane);
    const int atom = lane < na ? s_atom[lane] : -1;
    double rloc = 0.0;
    if constexpr (STREAM > 0) {
      const uint4* srec = reinterpret_cast<const uint4*>(m.r_stream);
      constexpr int CH = STREAM == 1 ? 32 : 16;  // records per load
      uint4* rbuf = reinterpret_cast<uint4*>(rpart + NW * 32) + warp * 16;  // STREAM 2
      C<float>* psum = reinterpret_cast<C<float>*>(reinterpret_cast<uint4*>(rpart + NW * 32) + NW * 16);
      for (int sw = warp; sw < kRestTableWarps; sw += NW) {
        const int e0 = __ldg(m.r_stream_begin + sw), e1 = __ldg(m.r_stream_begin + sw + 1);
        float vx = 0.f, vy = 0.f;
        for (int base = e0; base < e1; base += CH) {
          uint4 mine = make_uint4(0u, 0u, 0u, 0u);
          if (lane < CH && base + lane < e1) mine = __ldg(srec + base + lane);
          if constexpr (STREAM == 2) {
            if (lane < 16) rbuf[lane] = mine;
            __syncwarp();
          }
          const int n = min(CH, e1 - base);
          for (int q = 0; q < n; ++q) {
            unsigned rx, ry, rz, rw;
            if constexpr (STREAM == 2) {
              const uint4 t = rbuf[q];
              rx = t.x;
              ry = t.y;
              rz = t.z;
              rw = t.w;
            } else {
              rx = __shfl_sync(0xffffffffu, mine.x, q);
              ry = __shfl_sync(0xffffffffu, mine.y, q);
              rz = __shfl_sync(0xffffffffu, mine.z, q);
              rw = __shfl_sync(0xffffffffu, mine.w, q);
            }
            if (rw & kRestEnd) {
              // end of a slot (or of one part of a split slot): density
              // term and unscaled weight (a part's into psum)
              const int g0 = static_cast<int>(rz), w = static_cast<int>(ry);
              if (g0 >= 0) {
                const C<float> f = Fs[g0 * kRestStride + lane];
                rloc += f2d(f.x * vx) - f2d(f.y * vy);
              }
              const float mu = __uint_as_float(rx);
              if (rw & kRestSplit) {
                psum[(rw & 0xffffu) * 32 + lane] = {vx * mu, vy * mu};
              } else if (w >= 0 && atom >= 0) {
                st_l2(W + static_cast<size_t>(atom) * nW + w, {vx * mu, vy * mu}, pol_last);
              }
              vx = vy = 0.f;
            } else if (rw == kRestPair1) {
              // two one-factor entries, applied in order
              const C<float> fa = Fs[(ry & 0xffffu) * kRestStride + lane], fb = Fs[(ry >> 16) * kRestStride + lane];
              const float ka = __uint_as_float(rx), kb = __uint_as_float(rz);
              vx += ka * fa.x;
              vy += ka * fa.y;
              vx += kb * fb.x;
              vy += kb * fb.y;
            } else {
              const float k = __uint_as_float(rx);
              C<float> p = Fs[(ry & 0xffffu) * kRestStride + lane];
              if (rw >= 2u) p = cmul(p, Fs[(ry >> 16) * kRestStride + lane]);
              if (rw == 3u) p = cmul(p, Fs[rz * kRestStride + lane]);
              vx += k * p.x;
              vy += k * p.y;
            }
          }
          if constexpr (STREAM == 2) __syncwarp();
        }
      }
    } else {
      for (int sw = warp; sw < kRestTableWarps; sw += NW)
        for (int q = __ldg(m.r_warp_begin + sw); q < __ldg(m.r_warp_begin + sw + 1); ++q) {
          const int s = __ldg(m.r_warp_slots + q);
          float vx = 0.f, vy = 0.f;
          rest_run<1>(rec, __ldg(m.r_run + 3 * s), __ldg(m.r_run + 3 * s + 1), Fs, lane, vx, vy);
          rest_run<2>(rec, __ldg(m.r_run + 3 * s + 1), __ldg(m.r_run + 3 * s + 2), Fs, lane, vx, vy);
          rest_run<3>(rec, __ldg(m.r_run + 3 * s + 2), __ldg(m.r_run + 3 * s + 3), Fs, lane, vx, vy);
          const int g0 = __ldg(m.r_g0 + s);
          if (g0 >= 0) {
            const C<float> f = Fs[g0 * kRestStride + lane];
            rloc += f2d(f.x * vx) - f2d(f.y * vy);
          }
          const int w = __ldg(g.slot_weight + s);
          if (w >= 0 && atom >= 0) {
            const float mu = __ldg(g.slot_multf + s);
            st_l2(W + static_cast<size_t>(atom) * nW + w, {vx * mu, vy * mu}, pol_last);
          }
        }
    }
    rpart[warp * 32 + lane] = rloc;
    __syncthreads();
    if (warp == 0 && lane < na) {
      double r = 0.0;
      for (int w = 0; w < NW; ++w) r += rpart[w * 32 + lane];
      rho_rest[atom] = r;
    }
    if constexpr (STREAM > 0) {
      // the split slots' weights: the sum of their two parts
      const C<float>* psum = reinterpret_cast<const C<float>*>(reinterpret_cast<const uint4*>(rpart + NW * 32) + NW * 16);
      for (int q = threadIdx.x - 32; q >= 0 && q < m.r_nsplit * 32; q += blockDim.x - 32) {
        const int sp = q >> 5, a = q & 31, w = __ldg(m.r_split_w + sp);
        if (a < na && w >= 0) {
          const C<float> p0 = psum[(2 * sp) * 32 + a], p1 = psum[(2 * sp + 1) * 32 + a];
          st_l2(W + static_cast<size_t>(s_atom[a]) * nW + w, {p0.x + p1.x, p0.y + p1.y}, pol_last);
        }
      }
    }
  }
}

// k_rest64: the 2- and 4-body terms in FP64 (the plain precision) through
// the rest table, 16 atoms per CTA: lane & 15 is the atom, and the two
// half-warps take alternate entries of the same slot, so that both follow
// the same path; a shuffle adds their sums. Warp w walks the slots the host
// schedule gave it (RestTable::warp64_begin) in order, so every sum has a
// fixed order. Writes rho_rest and the unscaled weights mult * dRho_rest/dF.
constexpr int kRestStride64 = 17;  // row stride of Fs in complex elements
// (kRestWarps64, the warps per CTA of k_rest64, is in device_model.hpp)

// the entries [e0, e1) (every second one) of arity A in float-float: the
// factors staged as hi/lo floats (Fs), the coefficients as hi/lo pairs
// (kap), the slot sums compensated (vx, vy: sum, compensation); a product of
// two or three factors is formed as a compensated complex product and
// rounded to hi/lo before the next
template <int A>
__device__ __forceinline__ void rest_run64(const uint4* __restrict__ rec, const float* __restrict__ kap, int e0,
                                           int e1, const FFc* Fs, int al, float (&vx)[2], float (&vy)[2]) {
#pragma unroll 2
  for (int e = e0; e < e1; e += 2) {
    const uint4 r = __ldg(rec + e);
    const float2 kk = __ldg(reinterpret_cast<const float2*>(kap) + e);
    const FFv k = {kk.x, kk.y};
    FFc p = Fs[(r.y & 0xffffu) * kRestStride64 + al];
    if (A >= 2) {
      float t[4] = {0.f, 0.f, 0.f, 0.f};
      ff_cmac(t, p, Fs[(r.y >> 16) * kRestStride64 + al]);
      p = {ff_norm(t[0], t[1]), ff_norm(t[2], t[3])};
    }
    if (A >= 3) {
      float t[4] = {0.f, 0.f, 0.f, 0.f};
      ff_cmac(t, p, Fs[r.z * kRestStride64 + al]);
      p = {ff_norm(t[0], t[1]), ff_norm(t[2], t[3])};
    }
    ff_dot(vx[0], vx[1], k, p.x);
    ff_dot(vy[0], vy[1], k, p.y);
  }
}
// (s, c) += (s2, c2), error-free in s
__device__ __forceinline__ void ff_add_sum(float& s, float& c, float s2, float c2) {
  const float t = s + s2, z = t - s;
  c += ((s - (t - z)) + (s2 - z)) + c2;
  s = t;
}

template <class D, int NW>
__global__ void __launch_bounds__(NW * 32, 1)
    k_rest64(DeviceModel m, int natom, const C<double>* __restrict__ F, C<double>* __restrict__ W,
             double* __restrict__ rho_rest) {
  static_assert(NW == kRestWarps64, "the FP64 slot schedule is dealt to kRestWarps64 warps");
  extern __shared__ __align__(16) unsigned char smem[];
  const int nf = m.r_nfac, nW = m.nW;
  const GatherView& g = m.g2;  // slot weights and multiplicities (same slot numbering)
  C<double>* Fs = reinterpret_cast<C<double>*>(smem);                    // [nf][17] (as hi/lo floats)
  const FFc* Ff = reinterpret_cast<const FFc*>(Fs);
  double* rpart = reinterpret_cast<double*>(Fs + nf * kRestStride64);    // [NW][16]
  __shared__ int s_atom[16];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, al = lane & 15, half = lane >> 4;
  const int nblk = (natom + 15) / 16;
  const uint4* rec = reinterpret_cast<const uint4*>(m.r_rec);
  for (int blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int a0 = blk * 16;
    const int na = min(16, natom - a0);
    if (threadIdx.x < na) s_atom[threadIdx.x] = queue_atom(m, a0 + threadIdx.x);
    __syncthreads();
    // stage: thread c takes factor c of every atom
    for (int c = threadIdx.x; c < nf; c += blockDim.x) {
      const int fc = __ldg(m.r_factor + c);
      C<double> v[16];
#pragma unroll
      for (int b = 0; b < 16; ++b)
        v[b] = b < na ? F[static_cast<size_t>(s_atom[b]) * m.nF + fc] : C<double>{0.0, 0.0};
#pragma unroll
      for (int b = 0; b < 16; ++b) reinterpret_cast<FFc*>(Fs)[c * kRestStride64 + b] = {ff_of(v[b].x), ff_of(v[b].y)};
    }
    __syncthreads();
    const int atom = al < na ? s_atom[al] : -1;
    double rloc = 0.0;
    for (int q = __ldg(m.r64_warp_begin + warp); q < __ldg(m.r64_warp_begin + warp + 1); ++q) {
      const int s = __ldg(m.r64_warp_slots + q);
      float vx[2] = {0.f, 0.f}, vy[2] = {0.f, 0.f};
      rest_run64<1>(rec, m.r_kaphl, __ldg(m.r_run + 3 * s) + half, __ldg(m.r_run + 3 * s + 1), Ff, al, vx, vy);
      rest_run64<2>(rec, m.r_kaphl, __ldg(m.r_run + 3 * s + 1) + half, __ldg(m.r_run + 3 * s + 2), Ff, al, vx,
                    vy);
      rest_run64<3>(rec, m.r_kaphl, __ldg(m.r_run + 3 * s + 2) + half, __ldg(m.r_run + 3 * s + 3), Ff, al, vx,
                    vy);
      // the other half-warp's sums (lanes 16-31 add lanes 0-15's, and the
      // reverse; only lanes 0-15 use the result)
      ff_add_sum(vx[0], vx[1], __shfl_xor_sync(0xffffffffu, vx[0], 16), __shfl_xor_sync(0xffffffffu, vx[1], 16));
      ff_add_sum(vy[0], vy[1], __shfl_xor_sync(0xffffffffu, vy[0], 16), __shfl_xor_sync(0xffffffffu, vy[1], 16));
      const C<double> v = {ff_d(vx[0], vx[1]), ff_d(vy[0], vy[1])};
      if (half == 0) {
        const int g0 = __ldg(m.r_g0 + s);
        if (g0 >= 0) {
          const FFc f = Ff[g0 * kRestStride64 + al];
          rloc = re_mac(rloc, C<double>{f2d(f.x.hi) + f2d(f.x.lo), f2d(f.y.hi) + f2d(f.y.lo)}, v);
        }
        const int w = __ldg(g.slot_weight + s);
        if (w >= 0 && atom >= 0) {
          const double mu = __ldg(g.slot_mult + s);
          W[static_cast<size_t>(atom) * nW + w] = {mu * v.x, mu * v.y};
        }
      }
    }
    if (half == 0) rpart[warp * 16 + al] = rloc;
    __syncthreads();
    if (threadIdx.x < na) {
      double r = 0.0;
      for (int w = 0; w < NW; ++w) r += rpart[w * 16 + threadIdx.x];
      rho_rest[s_atom[threadIdx.x]] = r;
    }
    __syncthreads();
  }
}
template <class D>
size_t rest64_smem(const DeviceModel& m) {
  return sizeof(C<double>) * static_cast<size_t>(m.r_nfac) * kRestStride64 + sizeof(double) * kRestWarps64 * 16;
}

constexpr int kB3Stride = 33;  // row stride of Xs/Gs in complex elements

// pairs (i, j) the enumeration keeps for pattern PAT (0: l1' == l2' keeps
// (n1,n1') >= (n2,n2'); 1: l1' > l2' keeps n1 >= n2; 2: keeps n1 > n2),
// as the j bound of row i
template <int PAT, int I, int NM>
__device__ __forceinline__ constexpr int jmax_of(int i) {
  return PAT == 0 ? i + 1 : (PAT == 1 ? (i / NM + 1) * NM : (i / NM) * NM);
}

// factor of a task position: the compact element (low 13 bits) with its
// sign bits (0x8000 real, 0x4000 imaginary) applied; 0x2000 marks a directly
// read element whose gradient is not needed (weight multiplicity 0)
__device__ __forceinline__ C<float> b3_load(const C<float>* Xs, unsigned code, int lane) {
  const C<float> v = Xs[(code & 0x1fffu) * kB3Stride + lane];
  return {__uint_as_float(__float_as_uint(v.x) ^ ((code & 0x8000u) << 16)),
          __uint_as_float(__float_as_uint(v.y) ^ ((code & 0x4000u) << 17))};
}
// gradient of task position `pos`: dRho_T/dF to the element read directly
// there (a factor read through a mirror code gets nothing: its element's
// weight collects the mirror task's gradient instead), and the mirror task's
// gradient s conj(dRho_T/dF) to the element that task reads directly there
__device__ __forceinline__ void b3_add(C<float>* Gs, const uint16_t* __restrict__ code,
                                       const uint16_t* __restrict__ code2, int pos, int lane, C<float> v, float cf) {
  const unsigned c = __ldg(code + pos);
  if (!(c & 0xe000u)) {
    C<float>* g = Gs + c * kB3Stride + lane;
    atomicAdd(&g->x, cf * v.x);
    atomicAdd(&g->y, cf * v.y);
  }
  const unsigned c2 = __ldg(code2 + pos);
  if (c2 != 0xffffu) {
    const float s = (c2 & 0x8000u) ? -cf : cf;
    C<float>* g = Gs + (c2 & 0x3fffu) * kB3Stride + lane;
    atomicAdd(&g->x, s * v.x);
    atomicAdd(&g->y, -s * v.y);
  }
}

// One task on the lane's atom: the density term cf * sum C[p][i][j] a_p X_i Y_j
// (returned) and its gradient, added into Gs. Cs points at the combination's
// coefficients [NM][I][I] in shared memory; rows are read four at a time.
template <int PAT, class D>
__device__ __forceinline__ float b3_task(const float* __restrict__ Cs, const C<float>* Xs, C<float>* Gs,
                                         const uint16_t* __restrict__ code, const uint16_t* __restrict__ code2, float cf,
                                         int lane) {
  constexpr int I = D::I, NM = D::NM;
  static_assert(I % 4 == 0, "rows of C are read as float4");
  constexpr int JUSED = jmax_of<PAT, I, NM>(I - 1);  // largest j bound (rows grow with i)
  C<float> Y[I], gY[I], a[NM], ga[NM];
#pragma unroll
  for (int j = 0; j < I; ++j) {
    Y[j] = j < JUSED ? b3_load(Xs, __ldg(code + NM + I + j), lane) : C<float>{0.f, 0.f};
    gY[j] = {0.f, 0.f};
  }
#pragma unroll
  for (int p = 0; p < NM; ++p) {
    a[p] = b3_load(Xs, __ldg(code + p), lane);
    ga[p] = {0.f, 0.f};
  }
  float rt = 0.f;
#pragma unroll
  for (int i = 0; i < I; ++i) {
    const int jm = jmax_of<PAT, I, NM>(i);
    if (jm == 0) continue;
    const unsigned cx = __ldg(code + NM + i);
    const C<float> x = b3_load(Xs, cx, lane);
    C<float> az = {0.f, 0.f};
#pragma unroll
    for (int p = 0; p < NM; ++p) {
      C<float> z = {0.f, 0.f};
      const C<float> ax = cmul(a[p], x);
      const float4* crow = reinterpret_cast<const float4*>(Cs + (p * I + i) * I);
#pragma unroll
      for (int j4 = 0; j4 < (jm + 3) / 4; ++j4) {
        const float4 c4 = crow[j4];
        const float cv[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int j = 4 * j4 + u;
          if (j < jm) {
            z.x += cv[u] * Y[j].x;
            z.y += cv[u] * Y[j].y;
            gY[j].x += cv[u] * ax.x;
            gY[j].y += cv[u] * ax.y;
          }
        }
      }
      const C<float> t = cmul(a[p], z);
      az.x += t.x;
      az.y += t.y;
      const C<float> u = cmul(x, z);
      ga[p].x += u.x;
      ga[p].y += u.y;
    }
    rt += re_mul(x, az);
    b3_add(Gs, code, code2, NM + i, lane, az, cf);
  }
#pragma unroll
  for (int j = 0; j < JUSED; ++j) b3_add(Gs, code, code2, NM + I + j, lane, gY[j], cf);
#pragma unroll
  for (int p = 0; p < NM; ++p) b3_add(Gs, code, code2, p, lane, ga[p], cf);
  return rt;
}

// The same task with packed FP32x2 arithmetic (__ffma2_rn, two FMAs per
// instruction): Y and dY are held as pairs of consecutive j, (Y_j, Y_j+1) for
// the real and the imaginary parts, so that a row of C multiplies two j at a
// time, and z is summed in two halves. Row lengths round up to even; the
// coefficient after a row's last allowed j is zero in C.
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

template <int PAT, class D>
__device__ __forceinline__ float b3_task_x2(const float* __restrict__ Cs, const C<float>* Xs, C<float>* Gs,
                                            const uint16_t* __restrict__ code, const uint16_t* __restrict__ code2, float cf,
                                         int lane) {
  constexpr int I = D::I, NM = D::NM, H = I / 2;
  static_assert(I % 4 == 0, "rows of C are read as float4");
  constexpr int JUSED = jmax_of<PAT, I, NM>(I - 1);
  constexpr int HUSED = (JUSED + 1) / 2;
  float2 Yx[H], Yy[H], gYx[H], gYy[H];
  C<float> a[NM], ga[NM];
#pragma unroll
  for (int h = 0; h < H; ++h) {
    C<float> y0 = {0.f, 0.f}, y1 = {0.f, 0.f};
    if (h < HUSED) {
      y0 = b3_load(Xs, __ldg(code + NM + I + 2 * h), lane);
      y1 = b3_load(Xs, __ldg(code + NM + I + 2 * h + 1), lane);
    }
    Yx[h] = f2(y0.x, y1.x);
    Yy[h] = f2(y0.y, y1.y);
    gYx[h] = f2(0.f, 0.f);
    gYy[h] = f2(0.f, 0.f);
  }
#pragma unroll
  for (int p = 0; p < NM; ++p) {
    a[p] = b3_load(Xs, __ldg(code + p), lane);
    ga[p] = {0.f, 0.f};
  }
  float rt = 0.f;
#pragma unroll
  for (int i = 0; i < I; ++i) {
    const int jm = jmax_of<PAT, I, NM>(i);
    if (jm == 0) continue;
    const int hm = (jm + 1) / 2;
    const unsigned cx = __ldg(code + NM + i);
    const C<float> x = b3_load(Xs, cx, lane);
    C<float> az = {0.f, 0.f};
#pragma unroll
    for (int p = 0; p < NM; ++p) {
      const C<float> ax = cmul(a[p], x);
      const float2 axx = f2(ax.x, ax.x), axy = f2(ax.y, ax.y);
      float2 zx = f2(0.f, 0.f), zy = f2(0.f, 0.f);
      const float4* crow = reinterpret_cast<const float4*>(Cs + (p * I + i) * I);
#pragma unroll
      for (int h4 = 0; h4 < (hm + 1) / 2; ++h4) {
        const float4 c4 = crow[h4];
        const float2 cp[2] = {f2(c4.x, c4.y), f2(c4.z, c4.w)};
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int h = 2 * h4 + u;
          if (h < hm) {
            zx = __ffma2_rn(cp[u], Yx[h], zx);
            zy = __ffma2_rn(cp[u], Yy[h], zy);
            gYx[h] = __ffma2_rn(cp[u], axx, gYx[h]);
            gYy[h] = __ffma2_rn(cp[u], axy, gYy[h]);
          }
        }
      }
      const C<float> z = {zx.x + zx.y, zy.x + zy.y};
      const C<float> t = cmul(a[p], z);
      az.x += t.x;
      az.y += t.y;
      const C<float> u = cmul(x, z);
      ga[p].x += u.x;
      ga[p].y += u.y;
    }
    rt += re_mul(x, az);
    b3_add(Gs, code, code2, NM + i, lane, az, cf);
  }
#pragma unroll
  for (int h = 0; h < H; ++h) {
    if (2 * h < JUSED) b3_add(Gs, code, code2, NM + I + 2 * h, lane, C<float>{gYx[h].x, gYy[h].x}, cf);
    if (2 * h + 1 < JUSED) b3_add(Gs, code, code2, NM + I + 2 * h + 1, lane, C<float>{gYx[h].y, gYy[h].y}, cf);
  }
#pragma unroll
  for (int p = 0; p < NM; ++p) b3_add(Gs, code, code2, p, lane, ga[p], cf);
  return rt;
}

// The same task with the n0' loop outermost and not unrolled: X, Y, dX and
// dY stay in registers across it (more registers, a third of the code).
template <int PAT, class D>
__device__ __forceinline__ float b3_task_po(const float* __restrict__ Cs, const C<float>* Xs, C<float>* Gs,
                                            const uint16_t* __restrict__ code, const uint16_t* __restrict__ code2, float cf,
                                         int lane) {
  constexpr int I = D::I, NM = D::NM;
  constexpr int JUSED = jmax_of<PAT, I, NM>(I - 1);
  C<float> X[I], Y[I], aZ[I], gY[I];
#pragma unroll
  for (int i = 0; i < I; ++i) {
    X[i] = b3_load(Xs, __ldg(code + NM + i), lane);
    Y[i] = i < JUSED ? b3_load(Xs, __ldg(code + NM + I + i), lane) : C<float>{0.f, 0.f};
    aZ[i] = {0.f, 0.f};
    gY[i] = {0.f, 0.f};
  }
#pragma unroll 1
  for (int p = 0; p < NM; ++p) {
    const unsigned cp = __ldg(code + p);
    const C<float> a = b3_load(Xs, cp, lane);
    C<float> ga = {0.f, 0.f};
#pragma unroll
    for (int i = 0; i < I; ++i) {
      const int jm = jmax_of<PAT, I, NM>(i);
      if (jm == 0) continue;
      C<float> z = {0.f, 0.f};
      const C<float> ax = cmul(a, X[i]);
      const float4* crow = reinterpret_cast<const float4*>(Cs + (p * I + i) * I);
#pragma unroll
      for (int j4 = 0; j4 < (jm + 3) / 4; ++j4) {
        const float4 c4 = crow[j4];
        const float cv[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int j = 4 * j4 + u;
          if (j < jm) {
            z.x += cv[u] * Y[j].x;
            z.y += cv[u] * Y[j].y;
            gY[j].x += cv[u] * ax.x;
            gY[j].y += cv[u] * ax.y;
          }
        }
      }
      const C<float> t = cmul(a, z);
      aZ[i].x += t.x;
      aZ[i].y += t.y;
      const C<float> u = cmul(X[i], z);
      ga.x += u.x;
      ga.y += u.y;
    }
    b3_add(Gs, code, code2, p, lane, ga, cf);
  }
  float rt = 0.f;
#pragma unroll
  for (int i = 0; i < I; ++i) {
    if (jmax_of<PAT, I, NM>(i) == 0) continue;
    rt += re_mul(X[i], aZ[i]);
    b3_add(Gs, code, code2, NM + i, lane, aZ[i], cf);
  }
#pragma unroll
  for (int j = 0; j < JUSED; ++j) b3_add(Gs, code, code2, NM + I + j, lane, gY[j], cf);
  return rt;
}

// k_b3_fe. Shared memory: Cs (all combinations' coefficients), Xs[nc][33]
// (the CTA's factors, element-major), Gs[nc][33] (their density gradient),
// the per-warp density partials, the atoms' dE/drho, and the element and
// weight maps.
//
// Split tail (parts > 1, one CTA per block): CTAs below `nfull` evaluate
// their block whole. The remaining blocks, the last partial wave of one CTA
// per SM, are each divided among `parts` CTAs by task range. Each such CTA
// adds its 3-body density and its gradients [nc][32] (re, im) into the tail
// block's record in `tails` (tail_rec bytes per block) with global atomics,
// then takes a ticket; the CTA that takes the last ticket loads the totals
// and completes the block (its rho3 and g3). No CTA waits on
// another. The records are zeroed before the launch.
template <class D, int NW, int LOOP>
__global__ void __launch_bounds__(NW * 32, 1)
    k_b3_fe(DeviceModel m, int natom, const C<float>* __restrict__ F, C<float>* __restrict__ G3,
            double* __restrict__ rho3, int* err, int nfull, int parts, unsigned char* __restrict__ tails,
            size_t tail_rec) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NPOS = D::NPOS, I = D::I, NM = D::NM;
  const int nc = m.b3_nc;
  const int ncoef = m.b3_ncombo * NM * I * I;
  float* Cs = reinterpret_cast<float*>(smem);
  C<float>* Xs = reinterpret_cast<C<float>*>(Cs + ((ncoef + 3) & ~3));
  C<float>* Gs = Xs + nc * kB3Stride;
  double* rpart = reinterpret_cast<double*>(Gs + nc * kB3Stride);  // [NW][32]
  float* s_mult = reinterpret_cast<float*>(rpart + NW * 32);      // [nc]
  int* s_fac = reinterpret_cast<int*>(s_mult + nc);                // [nc]
  __shared__ int s_atom[32];                                       // the block's atoms
  __shared__ int s_next;                                           // next task to take
  __shared__ int s_last;                                           // split tail: this CTA completes the block
  const uint64_t pol_first = l2_evict_first(), pol_last = l2_evict_last();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nblk = (natom + 31) / 32;
  // this CTA's blocks and task range
  int blk_first = blockIdx.x, blk_stride = gridDim.x, task0 = 0, task1 = m.b3_ntask, tail = -1;
  if (parts > 1) {
    blk_stride = nblk;  // one block per CTA
    if (static_cast<int>(blockIdx.x) >= nfull) {
      const int q = (blockIdx.x - nfull) / parts, p = (blockIdx.x - nfull) % parts;
      tail = q;
      blk_first = nfull + q;
      task0 = m.b3_ntask * p / parts;
      task1 = m.b3_ntask * (p + 1) / parts;
    }
  }
  for (int t = threadIdx.x; t < ncoef / 4; t += blockDim.x)
    reinterpret_cast<float4*>(Cs)[t] = __ldg(reinterpret_cast<const float4*>(m.b3_Cf) + t);
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    s_mult[c] = __ldg(m.b3_mult + c);
    s_fac[c] = __ldg(m.b3_factor + c);
  }
  __syncthreads();
  for (int blk = blk_first; blk < nblk; blk += blk_stride) {
    const int a0 = blk * 32;
    const int na = min(32, natom - a0);
    if (threadIdx.x < na) s_atom[threadIdx.x] = queue_atom(m, a0 + threadIdx.x);
    if (threadIdx.x == 0) s_next = task0 + NW;
    __syncthreads();
    // stage: thread c takes element c of every atom, kBatch atoms in flight
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
      const int fc = s_fac[c];
      for (int ab = 0; ab < 32; ab += kBatch) {
        C<float> v[kBatch];
#pragma unroll
        for (int b = 0; b < kBatch; ++b)
          v[b] = ab + b < na ? ld_l2(F + static_cast<size_t>(s_atom[ab + b]) * m.nF + fc, pol_first) : C<float>{0.f, 0.f};
#pragma unroll
        for (int b = 0; b < kBatch; ++b) {
          Xs[c * kB3Stride + ab + b] = v[b];
          Gs[c * kB3Stride + ab + b] = {0.f, 0.f};
        }
      }
    }
    __syncthreads();
    double rloc = 0.0;
    // tasks from a shared counter (dynamic balance between the warps)
    int tk = task0 + warp;
#pragma unroll 1
    while (tk < task1) {
      const int k = __ldg(m.b3_combo + tk);
      const int pat = __ldg(m.b3_pattern + k);
      const float cf = __ldg(m.b3_cff + tk);
      const uint16_t* code = m.b3_code + tk * NPOS;
      const uint16_t* code2 = m.b3_code2 + tk * NPOS;
      const float* Ck = Cs + k * NM * I * I;
      float r;
      if constexpr (LOOP == 0) {
        if (pat == 0) r = b3_task<0, D>(Ck, Xs, Gs, code, code2, cf, lane);
        else if (pat == 1) r = b3_task<1, D>(Ck, Xs, Gs, code, code2, cf, lane);
        else r = b3_task<2, D>(Ck, Xs, Gs, code, code2, cf, lane);
      } else if constexpr (LOOP == 2) {
        if (pat == 0) r = b3_task_x2<0, D>(Ck, Xs, Gs, code, code2, cf, lane);
        else if (pat == 1) r = b3_task_x2<1, D>(Ck, Xs, Gs, code, code2, cf, lane);
        else r = b3_task_x2<2, D>(Ck, Xs, Gs, code, code2, cf, lane);
      } else {
        if (pat == 0) r = b3_task_po<0, D>(Ck, Xs, Gs, code, code2, cf, lane);
        else if (pat == 1) r = b3_task_po<1, D>(Ck, Xs, Gs, code, code2, cf, lane);
        else r = b3_task_po<2, D>(Ck, Xs, Gs, code, code2, cf, lane);
      }
      rloc += f2d(__ldg(m.b3_cfw + tk) * r);
      int nx = 0;
      if (lane == 0) nx = atomicAdd(&s_next, 1);
      tk = __shfl_sync(0xffffffffu, nx, 0);
    }
    rpart[warp * 32 + lane] = rloc;
    __syncthreads();
    if (tail >= 0) {
      // split tail: add this part into the block's accumulators
      unsigned char* rec = tails + tail * tail_rec;
      double* rho3_acc = reinterpret_cast<double*>(rec + kTailRho3);
      if (warp == 0 && lane < na) {
        double r3 = 0.0;
        for (int w = 0; w < NW; ++w) r3 += rpart[w * 32 + lane];
        atomicAdd(rho3_acc + lane, r3);
      }
      float* ga = reinterpret_cast<float*>(rec + kTailG);
      for (int q = threadIdx.x; q < nc * 32; q += blockDim.x) {
        const int c = q >> 5, a = q & 31;
        if (a < na) {
          const C<float> g = Gs[c * kB3Stride + a];
          atomicAdd(ga + 2 * q, g.x);
          atomicAdd(ga + 2 * q + 1, g.y);
        }
      }
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) s_last = atomicAdd(reinterpret_cast<int*>(rec + kTailTickets), 1) == parts - 1;
      __syncthreads();
      if (!s_last) break;  // another part completes the block
      __threadfence();
      // the last part: the block's totals replace this part's own
      for (int q = threadIdx.x; q < nc * 32; q += blockDim.x) {
        const int c = q >> 5, a = q & 31;
        Gs[c * kB3Stride + a] = {__ldcg(ga + 2 * q), __ldcg(ga + 2 * q + 1)};
      }
      for (int q = threadIdx.x; q < NW * 32; q += blockDim.x)
        rpart[q] = q < 32 ? __ldcg(rho3_acc + q) : 0.0;
      __syncthreads();
    }
    // the 3-body density of the block's atoms (k_finish_fe adds the parts)
    if (warp == 0 && lane < na) {
      double r3 = 0.0;
      for (int w = 0; w < NW; ++w) r3 += rpart[w * 32 + lane];
      rho3[s_atom[lane]] = r3;
    }
    // the block's 3-body gradients times their multiplicities, g3[atom][c]:
    // the force kernel assembles W = dE/drho (W_rest + g3) from them;
    // atom-major, so that consecutive threads store consecutive elements
    for (int q = threadIdx.x; q < nc * 32; q += blockDim.x) {
      const int a = q / nc, c = q - a * nc;
      if (a < na) {
        const C<float> gv = Gs[c * kB3Stride + a];
        const float mu = s_mult[c];
        st_l2(G3 + static_cast<size_t>(s_atom[a]) * nc + c, {mu * gv.x, mu * gv.y}, pol_last);
      }
    }
    __syncthreads();
  }
}

// ===========================================================================
// k_b3_fe64: the 3-body density and its gradients in FP64 (the plain
// precision), the same dense tasks as k_b3_fe with 32 atoms in the lanes of
// each warp; the coefficients C are read from global memory (one uniform
// load serves the warp) and the factors Xs[nc][33] are staged in shared
// memory. Warps take tasks from a shared counter.
//
// Every sum is exact integer arithmetic, so no result depends on which warp
// or CTA took which task or in which order the atomics arrive: the FP64 path
// stays bitwise reproducible, and an atom gets the same result in any batch
// and any order. Each contribution v is rounded once to a 64-bit integer
// q = rint(v * 2^e) and added with integer atomics: the gradients into
// G3i[block][c][lane] (re, im), the density into R3i[position]. The
// exponents of an atom follow from bounds of every partial sum: with f = max
// over the atom's factors of |x| + |y|, every gradient is at most
// b3_bound * f^2 and the density at most b3_bound_rho * f^3 (model.hpp
// DenseB3), so e = 61 - ceil(log2(bound)) keeps the sums below 2^61;
// G3s[position] and R3s[position] receive 2^-e. The rounding error of a sum
// is at most its number of contributions times 2^-e / 2, about 1e-17 of its
// bound.
//
// Split tail (parts > 1, one CTA per block): CTAs below `nfull` evaluate
// their block whole; the remaining blocks, the last partial wave of one CTA
// per SM, are each divided among `parts` CTAs by task range. The parts add
// into the same integer sums, so nothing else is needed to combine them.
constexpr int kB3Stride64 = 33;  // row stride of Xs in complex elements

// one fixed-point contribution (v already scaled by 2^e)
__device__ __forceinline__ void red_fix(unsigned long long* p, double v) {
  atomicAdd(p, static_cast<unsigned long long>(__double2ll_rn(v)));
}

// as b3_add, into the fixed-point gradients of the lane's atom: G points at
// element 0 of the lane ([c][32 lanes][2] words), cfs = cf * 2^e
__device__ __forceinline__ void b3_add64(unsigned long long* G, const uint16_t* __restrict__ code,
                                         const uint16_t* __restrict__ code2, int pos, C<double> v, double cfs) {
  const unsigned c = __ldg(code + pos);
  if (!(c & 0xe000u)) {
    unsigned long long* g = G + 64 * static_cast<size_t>(c);
    red_fix(g, cfs * v.x);
    red_fix(g + 1, cfs * v.y);
  }
  const unsigned c2 = __ldg(code2 + pos);
  if (c2 != 0xffffu) {
    const double sc = (c2 & 0x8000u) ? -cfs : cfs;
    unsigned long long* g = G + 64 * static_cast<size_t>(c2 & 0x3fffu);
    red_fix(g, sc * v.x);
    red_fix(g + 1, -sc * v.y);
  }
}

__device__ __forceinline__ FFc b3_load_ff(const FFc* Xs, unsigned code, int lane) {
  FFc v = Xs[(code & 0x1fffu) * kB3Stride64 + lane];
  const unsigned sx = (code & 0x8000u) << 16, sy = (code & 0x4000u) << 17;
  v.x = {__uint_as_float(__float_as_uint(v.x.hi) ^ sx), __uint_as_float(__float_as_uint(v.x.lo) ^ sx)};
  v.y = {__uint_as_float(__float_as_uint(v.y.hi) ^ sy), __uint_as_float(__float_as_uint(v.y.lo) ^ sy)};
  return v;
}

// b3_task64 with its arithmetic in float-float (the factors staged as hi/lo
// floats, the coefficients Chl [NM][I][I] as hi/lo pairs): every sum a
// compensated dot product on the FP32 pipe, the fixed-point contributions
// formed in FP64 from them as before. One body serves the three patterns:
// the loop over i is not unrolled and the row bounds are run-time values
// (uniform over the warp), so that the code stays within the instruction
// cache; Y and its gradient stay in registers (the loops over j unrolled).
template <class D>
__device__ __forceinline__ int jmax_rt(int pat, int i) {
  constexpr int NM = D::NM;
  return pat == 0 ? i + 1 : (pat == 1 ? (i / NM + 1) * NM : (i / NM) * NM);
}
template <class D>
__device__ __forceinline__ double b3_task64_ff(int pat, const float* __restrict__ Chl, const FFc* Xs,
                                               unsigned long long* G, const uint16_t* __restrict__ code,
                                               const uint16_t* __restrict__ code2, double cfs, int lane) {
  constexpr int I = D::I, NM = D::NM;
  static_assert(I % 2 == 0, "rows of C are read two coefficients at a time");
  const int jused = jmax_rt<D>(pat, I - 1);
  FFc Y[I], a[NM];
  float gY[I][4], ga[NM][4];
#pragma unroll
  for (int j = 0; j < I; ++j) {
    Y[j] = j < jused ? b3_load_ff(Xs, __ldg(code + NM + I + j), lane) : FFc{{0.f, 0.f}, {0.f, 0.f}};
    gY[j][0] = gY[j][1] = gY[j][2] = gY[j][3] = 0.f;
  }
#pragma unroll
  for (int p = 0; p < NM; ++p) {
    a[p] = b3_load_ff(Xs, __ldg(code + p), lane);
    ga[p][0] = ga[p][1] = ga[p][2] = ga[p][3] = 0.f;
  }
  float rts = 0.f, rtc = 0.f;
#pragma unroll 1
  for (int i = 0; i < I; ++i) {
    const int jm = jmax_rt<D>(pat, i);
    if (jm == 0) continue;
    const FFc x = b3_load_ff(Xs, __ldg(code + NM + i), lane);
    float az[4] = {0.f, 0.f, 0.f, 0.f};
    // the n0' loop is not unrolled either (a by selection, ga by a guarded
    // update): the body then fits the instruction cache
#pragma unroll 1
    for (int p = 0; p < NM; ++p) {
      const FFc ap = pick_of(a, p);
      float t[4] = {0.f, 0.f, 0.f, 0.f};
      ff_cmac(t, ap, x);
      const FFc ax = {ff_norm(t[0], t[1]), ff_norm(t[2], t[3])};
      float z[4] = {0.f, 0.f, 0.f, 0.f};
      const float4* crow = reinterpret_cast<const float4*>(Chl + 2 * (p * I + i) * I);
#pragma unroll
      for (int j2 = 0; j2 < I / 2; ++j2) {
        if (2 * j2 >= jm) break;
        const float4 c4 = __ldg(crow + j2);
        const FFv cv[2] = {{c4.x, c4.y}, {c4.z, c4.w}};
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int j = 2 * j2 + u;
          if (j < jm) {
            ff_dot(z[0], z[1], cv[u], Y[j].x);
            ff_dot(z[2], z[3], cv[u], Y[j].y);
            ff_dot(gY[j][0], gY[j][1], cv[u], ax.x);
            ff_dot(gY[j][2], gY[j][3], cv[u], ax.y);
          }
        }
      }
      const FFc zf = {ff_norm(z[0], z[1]), ff_norm(z[2], z[3])};
      ff_cmac(az, ap, zf);
#pragma unroll
      for (int q = 0; q < NM; ++q)
        if (q == p) ff_cmac(ga[q], x, zf);
    }
    const FFc azf = {ff_norm(az[0], az[1]), ff_norm(az[2], az[3])};
    ff_dot(rts, rtc, x.x, azf.x);
    ff_dot(rts, rtc, ff_neg(x.y), azf.y);
    b3_add64(G, code, code2, NM + i, C<double>{ff_d(az[0], az[1]), ff_d(az[2], az[3])}, cfs);
  }
#pragma unroll
  for (int j = 0; j < I; ++j)
    if (j < jused)
      b3_add64(G, code, code2, NM + I + j, C<double>{ff_d(gY[j][0], gY[j][1]), ff_d(gY[j][2], gY[j][3])}, cfs);
#pragma unroll
  for (int p = 0; p < NM; ++p)
    b3_add64(G, code, code2, p, C<double>{ff_d(ga[p][0], ga[p][1]), ff_d(ga[p][2], ga[p][3])}, cfs);
  return ff_d(rts, rtc);
}

// Shared memory: Xs[nc][33] (complex FP64) and the factor map [nc]. G3i is
// [ceil(natom/32)][nc][32][2] words and R3i [ceil(natom/32) * 32], both
// zeroed before the launch; G3s and R3s [ceil(natom/32) * 32]; blocks are 32
// consecutive queue positions.
template <class D, int NW>
__global__ void __launch_bounds__(NW * 32, 1)
    k_b3_fe64(DeviceModel m, int natom, const C<double>* __restrict__ F, unsigned long long* __restrict__ G3i,
              double* __restrict__ G3s, unsigned long long* __restrict__ R3i, double* __restrict__ R3s, int* err,
              int nfull, int parts) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NPOS = D::NPOS, I = D::I, NM = D::NM;
  const int nc = m.b3_nc;
  C<double>* Xs = reinterpret_cast<C<double>*>(smem);
  int* s_fac = reinterpret_cast<int*>(Xs + nc * kB3Stride64);  // [nc]
  __shared__ int s_atom[32];
  // per atom, the largest |x| + |y| of its factors (non-negative doubles
  // order as their bit patterns)
  __shared__ unsigned long long s_fm[32];
  __shared__ int s_next;  // next task to take
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nblk = (natom + 31) / 32;
  // this CTA's blocks and task range
  int blk_first = blockIdx.x, blk_stride = gridDim.x, task0 = 0, task1 = m.b3_ntask;
  if (parts > 1) {
    blk_stride = nblk;  // one block per CTA
    if (static_cast<int>(blockIdx.x) >= nfull) {
      const int q = (blockIdx.x - nfull) / parts, p = (blockIdx.x - nfull) % parts;
      blk_first = nfull + q;
      task0 = m.b3_ntask * p / parts;
      task1 = m.b3_ntask * (p + 1) / parts;
    }
  }
  for (int c = threadIdx.x; c < nc; c += blockDim.x) s_fac[c] = __ldg(m.b3_factor + c);
  __syncthreads();
  for (int blk = blk_first; blk < nblk; blk += blk_stride) {
    const int a0 = blk * 32;
    const int na = min(32, natom - a0);
    if (threadIdx.x < 32) {
      if (threadIdx.x < na) s_atom[threadIdx.x] = queue_atom(m, a0 + threadIdx.x);
      s_fm[threadIdx.x] = 0ull;
    }
    if (threadIdx.x == 0) s_next = task0 + NW;
    __syncthreads();
    // stage: thread c takes element c of every atom
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
      const int fc = s_fac[c];
      for (int ab = 0; ab < 32; ab += kBatch) {
        C<double> v[kBatch];
#pragma unroll
        for (int b = 0; b < kBatch; ++b)
          v[b] = ab + b < na ? F[static_cast<size_t>(s_atom[ab + b]) * m.nF + fc] : C<double>{0.0, 0.0};
#pragma unroll
        for (int b = 0; b < kBatch; ++b) {
          // staged as hi/lo floats for the float-float tasks
          reinterpret_cast<FFc*>(Xs)[c * kB3Stride64 + ab + b] = {ff_of(v[b].x), ff_of(v[b].y)};
          const double f = fabs(v[b].x) + fabs(v[b].y);
          // NaN compares as the largest pattern and is caught below
          atomicMax(&s_fm[ab + b], static_cast<unsigned long long>(__double_as_longlong(f)));
        }
      }
    }
    __syncthreads();
    // this lane's atom: the fixed-point exponents of its gradients and density
    double gscale, rscale;
    {
      const double f = __longlong_as_double(static_cast<long long>(s_fm[lane]));
      const double bg = m.b3_bound * f * f, br = m.b3_bound_rho * f * f * f;
      int eg = 0, er = 0;
      if (!(bg < 1e300) || !(br < 1e300)) {  // non-finite factors
        if (lane < na) raise_error(err, kDevNaN);
        eg = er = 1100;
      } else {
        if (bg > 0.0) frexp(bg, &eg);  // bound < 2^eg
        if (br > 0.0) frexp(br, &er);
      }
      eg = max(-1000, min(1000, 61 - eg));
      er = max(-1000, min(1000, 61 - er));
      gscale = ldexp(1.0, eg);
      rscale = ldexp(1.0, er);
      if (warp == 0) {  // every part of a split block writes the same values
        G3s[a0 + lane] = ldexp(1.0, -eg);
        R3s[a0 + lane] = ldexp(1.0, -er);
      }
    }
    unsigned long long* G = G3i + static_cast<size_t>(blk) * nc * 64 + 2 * lane;
    long long racc = 0;
    int tk = task0 + warp;
#pragma unroll 1
    while (tk < task1) {
      const int k = __ldg(m.b3_combo + tk);
      const int pat = __ldg(m.b3_pattern + k);
      const double cfs = __ldg(m.b3_cf64 + tk) * gscale;
      const uint16_t* code = m.b3_code + tk * NPOS;
      const uint16_t* code2 = m.b3_code2 + tk * NPOS;
      const float* Ck = m.b3_Chl + 2 * static_cast<size_t>(k) * NM * I * I;
      const FFc* Xf = reinterpret_cast<const FFc*>(Xs);
      const double r = b3_task64_ff<D>(pat, Ck, Xf, G, code, code2, cfs, lane);
      racc += __double2ll_rn(__ldg(m.b3_cfw64 + tk) * rscale * r);
      int nx = 0;
      if (lane == 0) nx = atomicAdd(&s_next, 1);
      tk = __shfl_sync(0xffffffffu, nx, 0);
    }
    if (lane < na) atomicAdd(R3i + a0 + lane, static_cast<unsigned long long>(racc));
    __syncthreads();
  }
}

// k_finish_fe: per atom (one per thread) rho = rho1 + rho_rest + rho3, the
// FP64 embedding and the inner cutoff on the core energy; the energy, edf and
// dE/drho outputs (the two density kernels before it may run side by side).
// With R3i (FP64), the 3-body density is the fixed-point sum of k_b3_fe64 at
// the atom's queue position times its scale R3s.
__global__ void __launch_bounds__(256) k_finish_fe(DeviceModel m, int natom, const double* __restrict__ rho1,
                                                   const double* __restrict__ rho_rest,
                                                   const double* __restrict__ rho3, const double* __restrict__ core,
                                                   double* __restrict__ energy, double* __restrict__ edf_out,
                                                   double* __restrict__ dedrho_out, int* err,
                                                   const unsigned long long* __restrict__ R3i = nullptr,
                                                   const double* __restrict__ R3s = nullptr) {
  for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < natom; it += gridDim.x * blockDim.x) {
    const int atom = R3i ? queue_atom(m, it) : it;
    const double r3 = R3i ? static_cast<double>(static_cast<long long>(R3i[it])) * R3s[it] : rho3[atom];
    const double rho = rho1[static_cast<size_t>(atom) * 2] + rho_rest[atom] + r3;
    if (!isfinite(rho)) raise_error(err, kDevNaN);
    double Fd, dFd;
    embed(m.nfemb, rho, m.par[0][0], m.par[1][0], Fd, dFd);
    const double e = core[atom], elow = m.ecut - m.decut;
    double fcut = 1.0, dfcut = 0.0;
    if (e >= m.ecut) {
      fcut = 0.0;
    } else if (e > elow) {
      const double pi = 3.14159265358979323846264338327950288419;
      fcut = 0.5 * (1.0 + cos(pi * (e - elow) / m.decut));
      dfcut = -0.5 * sin(pi * (e - elow) / m.decut) * pi / m.decut;
    }
    edf_out[atom] = dfcut * Fd + 1.0;
    dedrho_out[static_cast<size_t>(atom) * 2] = fcut * dFd;
    energy[atom] = fcut * Fd + e;
  }
}

// Writes v[0 .. 3n) to dst[3 j0 .. 3 (j0 + n)) with 16-byte stores wherever
// the destination is 16-byte aligned (the CTA's threads in turn).
__device__ __forceinline__ void store_tile(double* __restrict__ dst, const double* v, int j0, int n) {
  double* d = dst + 3 * static_cast<size_t>(j0);
  const int cnt = 3 * n;
  const int h = (reinterpret_cast<uintptr_t>(d) & 8u) ? 1 : 0;
  const int np = (cnt - h) >> 1;
  double2* d2 = reinterpret_cast<double2*>(d + h);
  for (int q = threadIdx.x; q < np; q += blockDim.x) d2[q] = make_double2(v[h + 2 * q], v[h + 2 * q + 1]);
  if (threadIdx.x == 0 && h) d[0] = v[0];
  if (threadIdx.x == blockDim.x - 1 && ((cnt - h) & 1)) d[cnt - 1] = v[cnt - 1];
}

// ===========================================================================
// k_forces_fe: one thread per bond. Weights transposed into shared memory:
// W2T[k][n] and WAT[k3][i], so the inner loops read 16-byte pairs. MINB is
// the CTAs per SM the register allocation must allow (a tuning variant).
// PACKED (split precision only) stores the transposed weights as separate
// real and imaginary planes and runs the contractions two n (or i) at a
// time with packed FP32x2 FMAs.
//
// SOUT: each tile's f_ij and t_ij go through shared memory and are written
// as contiguous 16-byte stores (whole lines); chosen when the outputs are
// host memory read over NVLink-C2C, where scattered 8-byte stores cost far
// more than in device memory.
template <class R, class D, int MINB, bool PACKED, bool SOUT = false, bool FF = false>
__global__ void __launch_bounds__(64, MINB)
    k_forces_fe(DeviceModel m, int natom, const int* __restrict__ off, const double* __restrict__ rr,
                const double* __restrict__ ee, const double* __restrict__ magj, const double* __restrict__ mhj,
                const double* __restrict__ magi, const double* __restrict__ mhi, const C<R>* __restrict__ W,
                const double* __restrict__ edf_in, const double* __restrict__ dedrho, double* __restrict__ fij,
                double* __restrict__ tij, double* __restrict__ ti0, const R* __restrict__ stage, int* err,
                const C<float>* __restrict__ g3, const unsigned long long* __restrict__ g3i = nullptr,
                const double* __restrict__ g3s = nullptr) {
  constexpr int T = 64;
  extern __shared__ __align__(16) unsigned char smem[];
  C<R>* W2T = reinterpret_cast<C<R>*>(smem);   // [NQ][NB]
  C<R>* WAT = W2T + D::NQ * D::NB;             // [NQ3][NRY]
  C<R>* W0s = WAT + D::NQ3 * D::NRY;           // [N2*H2]
  // per-thread feature columns [feature][T]
  R* cgd = reinterpret_cast<R*>(W0s + D::NQ + 2);
  R* cR = cgd + D::NB * T;
  R* cRd = cR + D::NR * T;
  R* cM = cRd + D::NR * T;
  R* cMd = cM + D::NMF * T;
  C<R>* cYa = reinterpret_cast<C<R>*>(cMd + D::NMF * T);  // full [LSA]
  double* sOut = reinterpret_cast<double*>(cYa + D::LSA * T);  // SOUT: the tile's f_ij [T][3], then t_ij [T][3]
  const int t = threadIdx.x;
  static_assert(!PACKED || sizeof(R) == 4, "packed contractions are FP32");
  static_assert(D::NB % 4 == 0 && D::NRY % 4 == 0, "planes are read four floats at a time");
  // planar views of the same shared memory (PACKED): [k][n] real, then imaginary
  float* W2x = reinterpret_cast<float*>(W2T);
  float* W2y = W2x + D::NQ * D::NB;
  float* WAx = reinterpret_cast<float*>(WAT);
  float* WAy = WAx + D::NQ3 * D::NRY;
  const uint64_t pol_first = l2_evict_first();  // the weights are read once

  for (int it = blockIdx.x; it < natom; it += gridDim.x) {
    const int atom = queue_atom(m, it);
    const C<R>* Wa = W + static_cast<size_t>(atom) * m.nW;
    if constexpr (sizeof(R) == 4) {
      // the weights of the atom a CTA starting about one CTA lifetime later
      // takes (MINB CTAs per SM resident), into L2
      if (t == 0) {
        unsigned nsm;
        asm("mov.u32 %0, %%nsmid;" : "=r"(nsm));
        const int ahead = it + MINB * static_cast<int>(nsm);
        if (ahead < natom) {
          const int a2 = queue_atom(m, ahead);
          const size_t wb = sizeof(C<R>) * static_cast<size_t>(m.nW);
          if (wb % 16 == 0) bulk_prefetch_l2(W + static_cast<size_t>(a2) * m.nW, static_cast<uint32_t>(wb));
          const size_t gb = sizeof(C<float>) * static_cast<size_t>(m.b3_nc);
          if (g3 && gb % 16 == 0) bulk_prefetch_l2(g3 + static_cast<size_t>(a2) * m.b3_nc, static_cast<uint32_t>(gb));
        }
      }
    }
    // with g3 (split path, Fe layout): W holds the 2-/4-body part of the
    // unscaled weights and g3 [atom][nc] the 3-body part per compact element;
    // the weight is dE/drho (W + g3)
    const C<float>* Ga = g3 ? g3 + static_cast<size_t>(atom) * m.b3_nc : nullptr;
    // with g3i (FP64, Fe layout): the 3-body part as fixed-point words of
    // the atom's queue position, times the block's scale and the element's
    // multiplicity
    const unsigned long long* Gi = g3i ? g3i + static_cast<size_t>(it >> 5) * m.b3_nc * 64 + 2 * (it & 31) : nullptr;
    const double gs = g3i ? g3s[it] : 0.0;
    const R sc = (g3 || g3i) ? to_r<R>(dedrho[static_cast<size_t>(atom) * 2]) : R(1);
    // weight w with its 3-body element c (-1: none); the A weights are the
    // first compact elements in the same order (c = w), the 2-body weights
    // have none, the on-site ones are looked up
    const auto weight = [&](int w, int c) {
      C<R> v = ld_l2(Wa + w, pol_first);
      if constexpr (sizeof(R) == 4) {
        if (Ga) {
          if (c >= 0) {
            const C<float> gv = ld_l2(Ga + c, pol_first);
            v.x += gv.x;
            v.y += gv.y;
          }
          v.x *= sc;
          v.y *= sc;
        }
      } else {
        if (Gi) {
          if (c >= 0) {
            const double mu = gs * static_cast<double>(__ldg(m.b3_mult + c));
            const unsigned long long* q = Gi + 64 * static_cast<size_t>(c);
            v.x += mu * static_cast<double>(static_cast<long long>(q[0]));
            v.y += mu * static_cast<double>(static_cast<long long>(q[1]));
          }
          v.x *= sc;
          v.y *= sc;
        }
      }
      return v;
    };
    for (int s = t; s < D::NA2H; s += T) {  // W2[n][k] -> W2T[k][n]
      const int n = s / D::NQ, k = s % D::NQ;
      const C<R> w = weight(m.offW2 + s, -1);
      if constexpr (PACKED) {
        W2x[k * D::NB + n] = w.x;
        W2y[k * D::NB + n] = w.y;
      } else if constexpr (FF) {
        reinterpret_cast<FFc*>(W2T)[k * D::NB + n] = {ff_of(w.x), ff_of(w.y)};
      } else {
        W2T[k * D::NB + n] = w;
      }
    }
    for (int s = t; s < D::NWA; s += T) {   // WA[i][k3] -> WAT[k3][i]
      const int i = s / D::NQ3, k3 = s % D::NQ3;
      const C<R> w = weight(s, s);
      if constexpr (PACKED) {
        WAx[k3 * D::NRY + i] = w.x;
        WAy[k3 * D::NRY + i] = w.y;
      } else if constexpr (FF) {
        reinterpret_cast<FFc*>(WAT)[k3 * D::NRY + i] = {ff_of(w.x), ff_of(w.y)};
      } else {
        WAT[k3 * D::NRY + i] = w;
      }
    }
    for (int s = t; s < D::NQ; s += T) W0s[s] = weight(m.offW0 + s, (Ga || Gi) ? __ldg(m.b3_cw + m.offW0 + s) : -1);
    __syncthreads();
    const R edf = to_r<R>(edf_in[atom]);
    const int b0 = off[atom], b1 = off[atom + 1];
    // bonds in tiles of T, uniform over the CTA (SOUT: each tile's outputs
    // are written from shared memory after the tile)
    for (int jt = b0; jt < b1; jt += T) {
      const int j = jt + t;
      if (j < b1) {
        R r, ex, ey, ez, mg, mx, my, mz;
        if (stage) {  // the A-basis kernel's copy in device memory
          R sp[8];
          ld8_l2(stage + 8 * static_cast<size_t>(j), sp, pol_first);
          r = sp[0];
          ex = sp[1];
          ey = sp[2];
          ez = sp[3];
          mg = sp[4];
          mx = sp[5];
          my = sp[6];
          mz = sp[7];
        } else {
          r = to_r<R>(rr[j]);
          ex = to_r<R>(ee[3 * j]);
          ey = to_r<R>(ee[3 * j + 1]);
          ez = to_r<R>(ee[3 * j + 2]);
          mg = to_r<R>(magj[j]);
          mx = to_r<R>(mhj[3 * j]);
          my = to_r<R>(mhj[3 * j + 1]);
          mz = to_r<R>(mhj[3 * j + 2]);
        }
        R g[D::NB];
        R cdv = R(0);
        {
          R tv[D::NR], td[D::NR], gd[D::NB], cv[1];
          R wl = R(0);
          const int nla = atomic_bin_r<R>(m, r, wl, err);
          if (nla > 0) {
            lut_eval<true>(pick<R>(m.lut_a, m.lut_a32), D::NFA, 0, D::NB, nla, wl, rscale_a<R>(m), g, gd);
            lut_eval<true>(pick<R>(m.lut_a, m.lut_a32), D::NFA, D::NB, D::NR, nla, wl, rscale_a<R>(m), tv, td);
            R cd1[1];
            lut_eval<true>(pick<R>(m.lut_a, m.lut_a32), D::NFA, D::NB + D::NR, 1, nla, wl, rscale_a<R>(m), cv, cd1);
            cdv = cd1[0];
          } else {
  #pragma unroll
            for (int q = 0; q < D::NB; ++q) g[q] = gd[q] = R(0);
  #pragma unroll
            for (int q = 0; q < D::NR; ++q) tv[q] = td[q] = R(0);
          }
  #pragma unroll
          for (int q = 0; q < D::NB; ++q) cgd[q * T + t] = gd[q];
  #pragma unroll
          for (int q = 0; q < D::NR; ++q) {
            cR[q * T + t] = tv[q];
            cRd[q * T + t] = td[q];
          }
        }
        {
          R mv[D::NMF], Md[D::NMF];
          R wm = R(0);
          const int nlm = magnetic_bin_r<R>(m, mg, wm, err);
          if (nlm > 0) {
            lut_eval<true>(pick<R>(m.lut_m, m.lut_m32), D::NFM, 0, D::NMF, nlm, wm, rscale_m<R>(m), mv, Md);
          } else {
  #pragma unroll
            for (int q = 0; q < D::NMF; ++q) {
              mv[q] = R(nlm == 0 ? 1 : 0);
              Md[q] = R(0);
            }
          }
  #pragma unroll
          for (int q = 0; q < D::NMF; ++q) {
            cM[q * T + t] = mv[q];
            cMd[q * T + t] = Md[q];
          }
        }
        C<R> Ym[D::H2], dYm[D::H2][3];
        {
          C<R> Ya[D::HA];
          ylm_half<R, false>(D::LA, ex, ey, ez, Ya, nullptr);
  #pragma unroll
          for (int lm = 0; lm < D::LSA; ++lm) {
            const int l = l_of_lm(lm), mm = lm - l * l - l;
            cYa[lm * T + t] = y_full(Ya, l, mm);
          }
          ylm_half<R, true>(D::L2, mx, my, mz, Ym, dYm);
        }
        // ---- force
        R fr = edf * cdv, ft[3] = {R(0), R(0), R(0)};
        {
          R sp[D::NB];
          C<R> U[D::NRY];
          if constexpr (PACKED) {
            float2 sp2[D::NB / 2], Ux2[D::NRY / 2], Uy2[D::NRY / 2];
  #pragma unroll
            for (int n = 0; n < D::NB / 2; ++n) sp2[n] = make_float2(0.f, 0.f);
  #pragma unroll
            for (int i = 0; i < D::NRY / 2; ++i) Ux2[i] = Uy2[i] = make_float2(0.f, 0.f);
  #pragma unroll 1
            for (int nr = 0; nr < D::N2; ++nr)
  #pragma unroll
              for (int h = 0; h < D::H2; ++h) {
                const int k = nr * D::H2 + h;
                const C<R> q = cscale(Ym[h], cM[(nr * (D::L2 + 1) + l_of_h(h)) * T + t]);
                const float2 qxx = make_float2(q.x, q.x), qyy = make_float2(q.y, q.y), qyn = make_float2(-q.y, -q.y);
                const float4* w2x = reinterpret_cast<const float4*>(W2x + k * D::NB);
                const float4* w2y = reinterpret_cast<const float4*>(W2y + k * D::NB);
  #pragma unroll
                for (int n4 = 0; n4 < D::NB / 4; ++n4) {
                  const float4 a = w2x[n4], b = w2y[n4];
                  sp2[2 * n4] = __ffma2_rn(make_float2(a.x, a.y), qxx, sp2[2 * n4]);
                  sp2[2 * n4] = __ffma2_rn(make_float2(b.x, b.y), qyn, sp2[2 * n4]);
                  sp2[2 * n4 + 1] = __ffma2_rn(make_float2(a.z, a.w), qxx, sp2[2 * n4 + 1]);
                  sp2[2 * n4 + 1] = __ffma2_rn(make_float2(b.z, b.w), qyn, sp2[2 * n4 + 1]);
                }
                if (nr < D::NM && h < D::H3) {
                  const int k3 = nr * D::H3 + h;
                  const float4* wax = reinterpret_cast<const float4*>(WAx + k3 * D::NRY);
                  const float4* way = reinterpret_cast<const float4*>(WAy + k3 * D::NRY);
  #pragma unroll
                  for (int i4 = 0; i4 < D::NRY / 4; ++i4) {
                    const float4 a = wax[i4], b = way[i4];
                    const float2 a0 = make_float2(a.x, a.y), a1 = make_float2(a.z, a.w);
                    const float2 b0 = make_float2(b.x, b.y), b1 = make_float2(b.z, b.w);
                    Ux2[2 * i4] = __ffma2_rn(b0, qyn, __ffma2_rn(a0, qxx, Ux2[2 * i4]));
                    Uy2[2 * i4] = __ffma2_rn(b0, qxx, __ffma2_rn(a0, qyy, Uy2[2 * i4]));
                    Ux2[2 * i4 + 1] = __ffma2_rn(b1, qyn, __ffma2_rn(a1, qxx, Ux2[2 * i4 + 1]));
                    Uy2[2 * i4 + 1] = __ffma2_rn(b1, qxx, __ffma2_rn(a1, qyy, Uy2[2 * i4 + 1]));
                  }
                }
              }
  #pragma unroll
            for (int n = 0; n < D::NB / 2; ++n) {
              sp[2 * n] = sp2[n].x;
              sp[2 * n + 1] = sp2[n].y;
            }
  #pragma unroll
            for (int i = 0; i < D::NRY / 2; ++i) {
              U[2 * i] = {Ux2[i].x, Uy2[i].x};
              U[2 * i + 1] = {Ux2[i].y, Uy2[i].y};
            }
          } else if constexpr (FF) {
            static_assert(sizeof(R) == 8 && sizeof(FFc) == sizeof(C<double>), "float-float contractions: FP64 path");
            // compensated float-float dot products (sum, compensation)
            float sps[D::NB], spc[D::NB], uxs[D::NRY], uxc[D::NRY], uys[D::NRY], uyc[D::NRY];
  #pragma unroll
            for (int n = 0; n < D::NB; ++n) sps[n] = spc[n] = 0.f;
  #pragma unroll
            for (int i = 0; i < D::NRY; ++i) uxs[i] = uxc[i] = uys[i] = uyc[i] = 0.f;
            // one magnetic product per iteration, not unrolled (the float-float
            // loops unrolled over h overflow the instruction cache)
  #pragma unroll 1
            for (int k = 0; k < D::NQ; ++k) {
              const int nr = k / D::H2, h = k - nr * D::H2;
              {
                const C<R> qd = cscale(pick_of(Ym, h), cM[(nr * (D::L2 + 1) + l_of_h(h)) * T + t]);
                const FFv qx = ff_of(qd.x), qy = ff_of(qd.y), qyn = ff_neg(qy);
                const FFc* w2 = reinterpret_cast<const FFc*>(W2T) + k * D::NB;
  #pragma unroll
                for (int n = 0; n < D::NB; ++n) {
                  const FFc w = w2[n];
                  ff_dot(sps[n], spc[n], w.x, qx);
                  ff_dot(sps[n], spc[n], w.y, qyn);
                }
                if (nr < D::NM && h < D::H3) {
                  const FFc* wa = reinterpret_cast<const FFc*>(WAT) + (nr * D::H3 + h) * D::NRY;
  #pragma unroll
                  for (int i = 0; i < D::NRY; ++i) {
                    const FFc w = wa[i];
                    ff_dot(uxs[i], uxc[i], w.x, qx);
                    ff_dot(uxs[i], uxc[i], w.y, qyn);
                    ff_dot(uys[i], uyc[i], w.x, qy);
                    ff_dot(uys[i], uyc[i], w.y, qx);
                  }
                }
              }
            }
  #pragma unroll
            for (int n = 0; n < D::NB; ++n) sp[n] = ff_d(sps[n], spc[n]);
  #pragma unroll
            for (int i = 0; i < D::NRY; ++i) U[i] = {ff_d(uxs[i], uxc[i]), ff_d(uys[i], uyc[i])};
          } else {
  #pragma unroll
            for (int n = 0; n < D::NB; ++n) sp[n] = R(0);
  #pragma unroll
            for (int i = 0; i < D::NRY; ++i) U[i] = {R(0), R(0)};
  #pragma unroll 1
            for (int nr = 0; nr < D::N2; ++nr)
  #pragma unroll
              for (int h = 0; h < D::H2; ++h) {
                const int k = nr * D::H2 + h;
                const C<R> q = cscale(Ym[h], cM[(nr * (D::L2 + 1) + l_of_h(h)) * T + t]);
                const C<R>* w2 = W2T + k * D::NB;
  #pragma unroll
                for (int n = 0; n < D::NB; ++n) sp[n] = re_mac(sp[n], w2[n], q);
                if (nr < D::NM && h < D::H3) {
                  const C<R>* wa = WAT + (nr * D::H3 + h) * D::NRY;
  #pragma unroll
                  for (int i = 0; i < D::NRY; ++i) cmac(U[i], wa[i], q);
                }
              }
          }
  #pragma unroll
          for (int n = 0; n < D::NB; ++n) fr = fma(cgd[n * T + t], sp[n], fr);
          const R invr = rcp(r);
          // the angular part: S_lm = sum_n1 U R_n1,l / r, contracted once
          // with dY_lm (recomputed here rather than kept per bond)
          C<R> S[D::LSA];
  #pragma unroll
          for (int lm = 0; lm < D::LSA; ++lm) S[lm] = {R(0), R(0)};
  #pragma unroll
          for (int i = 0; i < D::NRY; ++i) {
            const int n1 = i / D::LSA, lma = i % D::LSA, l1 = l_of_lm(lma);
            fr = fma(cRd[(n1 * (D::LA + 1) + l1) * T + t], re_mul(U[i], cYa[lma * T + t]), fr);
            const C<R> su = cscale(U[i], invr * cR[(n1 * (D::LA + 1) + l1) * T + t]);
            S[lma].x += su.x;
            S[lma].y += su.y;
          }
          C<R> Ya[D::HA], dYa[D::HA][3];
          ylm_half<R, true>(D::LA, ex, ey, ez, Ya, dYa);
  #pragma unroll
          for (int lm = 0; lm < D::LSA; ++lm) {
            const int l = l_of_lm(lm), mm = lm - l * l - l;
  #pragma unroll
            for (int c = 0; c < 3; ++c) {
              C<R> d = dYa[ph(l, mm < 0 ? -mm : mm)][c];
              if (mm < 0) {
                const R s = R(parity(mm));
                d = {d.x * s, -d.y * s};
              }
              ft[c] = re_mac(ft[c], S[lm], d);
            }
          }
        }
        *(SOUT ? sOut + 3 * t + 0 : fij + 3 * static_cast<size_t>(j) + 0) = to_d(fr * ex + ft[0]);
        *(SOUT ? sOut + 3 * t + 1 : fij + 3 * static_cast<size_t>(j) + 1) = to_d(fr * ey + ft[1]);
        *(SOUT ? sOut + 3 * t + 2 : fij + 3 * static_cast<size_t>(j) + 2) = to_d(fr * ez + ft[2]);
        // ---- magnetic force
        R tr = R(0), tt[3] = {R(0), R(0), R(0)};
        {
          C<R> RY[D::NRY];
  #pragma unroll
          for (int i = 0; i < D::NRY; ++i) {
            const int n1 = i / D::LSA, lma = i % D::LSA;
            RY[i] = cscale(cYa[lma * T + t], cR[(n1 * (D::LA + 1) + l_of_lm(lma)) * T + t]);
          }
          const R invm = rcp(mg);
          // V[k] = sum_n g_n W2[n][k] + sum_i W_A[i][k] RY_i, contracted per k
          const auto contract = [&](int nr, int h, C<R> V) {
            const int q = nr * (D::L2 + 1) + l_of_h(h);
            tr = fma(cMd[q * T + t], re_mul(V, Ym[h]), tr);
            const C<R> sv = cscale(V, invm * cM[q * T + t]);
  #pragma unroll
            for (int c = 0; c < 3; ++c) tt[c] = re_mac(tt[c], sv, dYm[h][c]);
          };
          if constexpr (PACKED) {
            float2 g2[D::NB / 2], RYx2[D::NRY / 2], RYy2[D::NRY / 2], RYyn2[D::NRY / 2];
  #pragma unroll
            for (int n = 0; n < D::NB / 2; ++n) g2[n] = make_float2(g[2 * n], g[2 * n + 1]);
  #pragma unroll
            for (int i = 0; i < D::NRY / 2; ++i) {
              RYx2[i] = make_float2(RY[2 * i].x, RY[2 * i + 1].x);
              RYy2[i] = make_float2(RY[2 * i].y, RY[2 * i + 1].y);
              RYyn2[i] = make_float2(-RY[2 * i].y, -RY[2 * i + 1].y);
            }
  #pragma unroll 1
            for (int nr = 0; nr < D::N2; ++nr)
  #pragma unroll
              for (int h = 0; h < D::H2; ++h) {
                const int k = nr * D::H2 + h;
                float2 vx2 = make_float2(0.f, 0.f), vy2 = make_float2(0.f, 0.f);
                const float4* w2x = reinterpret_cast<const float4*>(W2x + k * D::NB);
                const float4* w2y = reinterpret_cast<const float4*>(W2y + k * D::NB);
  #pragma unroll
                for (int n4 = 0; n4 < D::NB / 4; ++n4) {
                  const float4 a = w2x[n4], b = w2y[n4];
                  vx2 = __ffma2_rn(g2[2 * n4], make_float2(a.x, a.y), vx2);
                  vx2 = __ffma2_rn(g2[2 * n4 + 1], make_float2(a.z, a.w), vx2);
                  vy2 = __ffma2_rn(g2[2 * n4], make_float2(b.x, b.y), vy2);
                  vy2 = __ffma2_rn(g2[2 * n4 + 1], make_float2(b.z, b.w), vy2);
                }
                if (nr < D::NM && h < D::H3) {
                  const int k3 = nr * D::H3 + h;
                  const float4* wax = reinterpret_cast<const float4*>(WAx + k3 * D::NRY);
                  const float4* way = reinterpret_cast<const float4*>(WAy + k3 * D::NRY);
  #pragma unroll
                  for (int i4 = 0; i4 < D::NRY / 4; ++i4) {
                    const float4 a = wax[i4], b = way[i4];
                    const float2 a0 = make_float2(a.x, a.y), a1 = make_float2(a.z, a.w);
                    const float2 b0 = make_float2(b.x, b.y), b1 = make_float2(b.z, b.w);
                    vx2 = __ffma2_rn(b0, RYyn2[2 * i4], __ffma2_rn(a0, RYx2[2 * i4], vx2));
                    vy2 = __ffma2_rn(b0, RYx2[2 * i4], __ffma2_rn(a0, RYy2[2 * i4], vy2));
                    vx2 = __ffma2_rn(b1, RYyn2[2 * i4 + 1], __ffma2_rn(a1, RYx2[2 * i4 + 1], vx2));
                    vy2 = __ffma2_rn(b1, RYx2[2 * i4 + 1], __ffma2_rn(a1, RYy2[2 * i4 + 1], vy2));
                  }
                }
                contract(nr, h, C<R>{vx2.x + vx2.y, vy2.x + vy2.y});
              }
          } else if constexpr (FF) {
            FFv gf[D::NB], rx[D::NRY], ry[D::NRY];
  #pragma unroll
            for (int n = 0; n < D::NB; ++n) gf[n] = ff_of(g[n]);
  #pragma unroll
            for (int i = 0; i < D::NRY; ++i) {
              rx[i] = ff_of(RY[i].x);
              ry[i] = ff_of(RY[i].y);
            }
            // per h, Z = sum_nr M_q V_k and Zd = sum_nr M'_q V_k (q = nr (L2 + 1)
            // + l(h), k = nr H2 + h), then one contraction with Y_h, dY_h:
            // tr += Re(Zd Y_h), tt += Re(Z dY_h) / |m|
  #pragma unroll 1
            for (int h = 0; h < D::H2; ++h) {
              C<R> Z = {R(0), R(0)}, Zd = {R(0), R(0)};
  #pragma unroll 1
              for (int nr = 0; nr < D::N2; ++nr) {
                const int k = nr * D::H2 + h;
                const FFc* w2 = reinterpret_cast<const FFc*>(W2T) + k * D::NB;
                float vxs = 0.f, vxc = 0.f, vys = 0.f, vyc = 0.f;
  #pragma unroll
                for (int n = 0; n < D::NB; ++n) {
                  const FFc w = w2[n];
                  ff_dot(vxs, vxc, gf[n], w.x);
                  ff_dot(vys, vyc, gf[n], w.y);
                }
                if (nr < D::NM && h < D::H3) {
                  const FFc* wa = reinterpret_cast<const FFc*>(WAT) + (nr * D::H3 + h) * D::NRY;
  #pragma unroll
                  for (int i = 0; i < D::NRY; ++i) {
                    const FFc w = wa[i];
                    ff_dot(vxs, vxc, w.x, rx[i]);
                    ff_dot(vxs, vxc, ff_neg(w.y), ry[i]);
                    ff_dot(vys, vyc, w.x, ry[i]);
                    ff_dot(vys, vyc, w.y, rx[i]);
                  }
                }
                const R vx = ff_d(vxs, vxc), vy = ff_d(vys, vyc);
                const int q = nr * (D::L2 + 1) + l_of_h(h);
                const R s = cM[q * T + t], sd = cMd[q * T + t];
                Z.x = fma(s, vx, Z.x);
                Z.y = fma(s, vy, Z.y);
                Zd.x = fma(sd, vx, Zd.x);
                Zd.y = fma(sd, vy, Zd.y);
              }
              tr += re_mul(Zd, pick_of(Ym, h));
              const C<R> sz = cscale(Z, invm);
  #pragma unroll
              for (int c = 0; c < 3; ++c) {
                C<R> d = dYm[0][c];
  #pragma unroll
                for (int j = 1; j < D::H2; ++j)
                  if (h == j) d = dYm[j][c];
                tt[c] = re_mac(tt[c], sz, d);
              }
            }
          } else {
  #pragma unroll 1
            for (int nr = 0; nr < D::N2; ++nr)
  #pragma unroll
              for (int h = 0; h < D::H2; ++h) {
                const int k = nr * D::H2 + h;
                const C<R>* w2 = W2T + k * D::NB;
                C<R> V = {R(0), R(0)};
  #pragma unroll
                for (int n = 0; n < D::NB; ++n) {
                  V.x = fma(g[n], w2[n].x, V.x);
                  V.y = fma(g[n], w2[n].y, V.y);
                }
                if (nr < D::NM && h < D::H3) {
                  const C<R>* wa = WAT + (nr * D::H3 + h) * D::NRY;
  #pragma unroll
                  for (int i = 0; i < D::NRY; ++i) cmac(V, wa[i], RY[i]);
                }
                contract(nr, h, V);
              }
          }
        }
        *(SOUT ? sOut + 3 * T + 3 * t + 0 : tij + 3 * static_cast<size_t>(j) + 0) = to_d(tr * mx + tt[0]);
        *(SOUT ? sOut + 3 * T + 3 * t + 1 : tij + 3 * static_cast<size_t>(j) + 1) = to_d(tr * my + tt[1]);
        *(SOUT ? sOut + 3 * T + 3 * t + 2 : tij + 3 * static_cast<size_t>(j) + 2) = to_d(tr * mz + tt[2]);
      }
      if constexpr (SOUT) {
        __syncthreads();
        store_tile(fij, sOut, jt, min(T, b1 - jt));
        store_tile(tij, sOut + 3 * T, jt, min(T, b1 - jt));
        __syncthreads();
      }
    }
    if (t >= 32) {
      // on-site magnetic force dE_i/dm_i (src/forces.F90:690-749), in the
      // working precision, on warp 1: lane q < NMF evaluates M_q, lane
      // NMF + n the 1-body function g_n (values and derivatives); lane k <
      // NQ takes the on-site weight W0[k]; the terms are summed by shuffles
      static_assert(D::NMF + D::NBM <= 32 && D::NQ <= 32, "one function and one weight per lane");
      const int lane = t - 32;
      const R mg = to_r<R>(magi[atom]);
      const R mx = to_r<R>(mhi[3 * atom]), my = to_r<R>(mhi[3 * atom + 1]), mz = to_r<R>(mhi[3 * atom + 2]);
      R wm = R(0);
      const int nl = magnetic_bin_r<R>(m, mg, wm, err);
      R v = R(nl == 0 ? 1 : 0), dv = R(0);
      if (nl > 0 && lane < D::NMF + D::NBM)
        lut_eval<true>(pick<R>(m.lut_m, m.lut_m32), D::NFM, lane, 1, nl, wm, rscale_m<R>(m), &v, &dv);
      C<R> Yh[D::H2], dYh[D::H2][3];
      ylm_half<R, true>(D::L2, mx, my, mz, Yh, dYh);
      R tr = R(0), tt[3] = {R(0), R(0), R(0)};
      const int n = lane - D::NMF;
      if (n >= 0 && n < D::NBM) tr = to_r<R>(dedrho[static_cast<size_t>(atom) * 2]) * c1_of<R>(m, n) * dv;
      const int k = lane < D::NQ ? lane : 0;
      const int nr = k / D::H2, h = k % D::H2, q = nr * (D::L2 + 1) + l_of_h(h);
      const R Mq = __shfl_sync(0xffffffffu, v, q), Mdq = __shfl_sync(0xffffffffu, dv, q);
      if (lane < D::NQ) {
        // Y_h and its gradient by selection (h differs across the lanes)
        C<R> y = Yh[0], dy[3] = {dYh[0][0], dYh[0][1], dYh[0][2]};
#pragma unroll
        for (int hh = 1; hh < D::H2; ++hh)
          if (h == hh) {
            y = Yh[hh];
#pragma unroll
            for (int c = 0; c < 3; ++c) dy[c] = dYh[hh][c];
          }
        const C<R> w = W0s[k];
        const R invm = rcp(mg);
        tr += Mdq * re_mul(w, y);
        const R sc = invm * Mq;
#pragma unroll
        for (int c = 0; c < 3; ++c) tt[c] += sc * re_mul(w, dy[c]);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        tr += __shfl_xor_sync(0xffffffffu, tr, o);
#pragma unroll
        for (int c = 0; c < 3; ++c) tt[c] += __shfl_xor_sync(0xffffffffu, tt[c], o);
      }
      if (lane == 0) {
        ti0[3 * static_cast<size_t>(atom) + 0] = to_d(tr * mx + tt[0]);
        ti0[3 * static_cast<size_t>(atom) + 1] = to_d(tr * my + tt[1]);
        ti0[3 * static_cast<size_t>(atom) + 2] = to_d(tr * mz + tt[2]);
      }
    }
    __syncthreads();
  }
}

// ===========================================================================
// k_forces_tc (split precision): the contractions of k_forces_fe as GEMMs on
// the tensor cores (mma.sync m16n8k8 TF32 in the 3xTF32 split: each FP32
// operand x = hi + lo with hi, lo TF32, products lo*hi + hi*lo + hi*hi
// accumulated in FP32, so the error stays near FP32's), per 64-bond tile of
// one atom, bonds as the M dimension, one warp per 32 bonds (two m16 tiles):
//   F1  sp[b][n]         = sum_K Q[b][K] B1[K][n]    K = 64 (Re, Im of q_k), N = 16
//   F2  U[b][2i + c]     = sum_K Q[b][K] B2[K][..]   K = 40 (Re, Im of q_k, k < NQ3), N = 32
//   T   V[b][2k + c]     = sum_K G[b][K] B3[K][..]   K = 48 (g_n, Re, Im of RY_i), N = 64
// with q_k = M_nl(|m_j|) Y_lm(m-hat_j) (m >= 0), RY_i = R_nl(r) Y_lm(e) and
// B1..B3 the atom's weights (dE/drho (W + g3)) laid out as the real GEMMs of
// the complex products: sp_n = Re sum_k W2[n][k] q_k, U_i = sum_k W_A[i][k] q_k,
// V_k = sum_n g_n W2[n][k] + sum_i W_A[i][k] RY_i. The weights are arranged
// once per atom in the order of the B fragments; each warp's Q and G rows and
// its D results share one shared-memory row per bond. The per-bond features
// stay in the registers of the bond's thread; the epilogues (f_ij from sp and
// U, t_ij from V) are k_forces_fe's.
//
// Q row columns: Re q_k (k < 18), Im q_k (k < 18), Re q_k (k >= 18), Im q_k
// (k >= 18), four zeros; G row: g_n, Re RY_i, Im RY_i.
constexpr int kTcRow = 68;      // floats per bond row (64 + 4: conflict-free fragment loads)
constexpr int kTcF1 = 8 * 2;    // B fragments of F1 (k-steps x n-tiles)
constexpr int kTcF2 = 5 * 4;    // of F2
constexpr int kTcT = 5 * 6 + 3 * 2;  // of T (n-tiles 5-7 hold k >= 20 only: the 2 k-steps of g)
constexpr int kTcFrags = kTcF1 + kTcF2 + kTcT;


template <class D>
size_t forces_tc_smem(bool sout) {
  return sizeof(float2) * kTcFrags * 32 + sizeof(C<float>) * 32 + sizeof(float) * 64 * kTcRow +
         (sout ? sizeof(double) * 6 * 64 : 0);
}

template <class D, int MINB, bool SOUT>
__global__ void __launch_bounds__(64, MINB)
    k_forces_tc(DeviceModel m, int natom, const int* __restrict__ off, const double* __restrict__ rr,
                const double* __restrict__ ee, const double* __restrict__ magj, const double* __restrict__ mhj,
                const double* __restrict__ magi, const double* __restrict__ mhi, const C<float>* __restrict__ W,
                const double* __restrict__ edf_in, const double* __restrict__ dedrho, double* __restrict__ fij,
                double* __restrict__ tij, double* __restrict__ ti0, const float* __restrict__ stage, int* err,
                const C<float>* __restrict__ g3) {
  using R = float;
  constexpr int T = 64;
  static_assert(D::NQ3 == 18 && D::NQ == 30 && D::NB == 16 && D::NRY == 16 && D::H3 == D::H2,
                "fragment shapes assume the Fe layout");
  extern __shared__ __align__(16) unsigned char smem[];
  float2* Bf = reinterpret_cast<float2*>(smem);                       // [kTcFrags][32 lanes]
  C<float>* W0s = reinterpret_cast<C<float>*>(Bf + kTcFrags * 32);   // [32]
  float* QA = reinterpret_cast<float*>(W0s + 32);                     // [64 bonds][kTcRow]
  double* sOut = reinterpret_cast<double*>(QA + 64 * kTcRow);  // SOUT: f_ij [T][3], then t_ij [T][3]
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31, gid = lane >> 2, tig = lane & 3;
  const uint64_t pol_first = l2_evict_first();

  for (int it = blockIdx.x; it < natom; it += gridDim.x) {
    const int atom = queue_atom(m, it);
    const C<float>* Wa = W + static_cast<size_t>(atom) * m.nW;
    if (t == 0) {
      // the weights of the atom a CTA starting about one CTA lifetime later
      // takes (MINB CTAs per SM resident), into L2
      unsigned nsm;
      asm("mov.u32 %0, %%nsmid;" : "=r"(nsm));
      const int ahead = it + MINB * static_cast<int>(nsm);
      if (ahead < natom) {
        const int a2 = queue_atom(m, ahead);
        const size_t wb = sizeof(C<float>) * static_cast<size_t>(m.nW);
        if (wb % 16 == 0) bulk_prefetch_l2(W + static_cast<size_t>(a2) * m.nW, static_cast<uint32_t>(wb));
        const size_t gb = sizeof(C<float>) * static_cast<size_t>(m.b3_nc);
        if (g3 && gb % 16 == 0) bulk_prefetch_l2(g3 + static_cast<size_t>(a2) * m.b3_nc, static_cast<uint32_t>(gb));
      }
    }
    // the weight is dE/drho (W + g3): W the 2-/4-body part, g3 [atom][nc]
    // the 3-body part per compact element c (-1: none)
    const C<float>* Ga = g3 ? g3 + static_cast<size_t>(atom) * m.b3_nc : nullptr;
    const R sc = g3 ? to_r<R>(dedrho[static_cast<size_t>(atom) * 2]) : R(1);
    const auto weight = [&](int w, int c) {
      C<R> v = ld_l2(Wa + w, pol_first);
      if (Ga) {
        if (c >= 0) {
          const C<float> gv = ld_l2(Ga + c, pol_first);
          v.x += gv.x;
          v.y += gv.y;
        }
        v.x *= sc;
        v.y *= sc;
      }
      return v;
    };
    // the B fragments: lane L of fragment (k-step s, n-tile u) holds
    // B[8 s + L % 4][8 u + L / 4] and B[8 s + L % 4 + 4][8 u + L / 4]. Each
    // weight goes to its places in F1 and T (W2[n][k]) or F2 and T
    // (W_A[i][k]); the padding places stay zero.
    // (the weights are staged in the rows' space first, then scattered)
    C<R>* raw = reinterpret_cast<C<R>*>(QA);  // W2[n][k], then W_A[i][k]
    static_assert(sizeof(C<R>) * (D::NA2H + D::NWA) <= sizeof(float) * 64 * kTcRow, "the weights fit in the rows");
    // the atom's bond range and scalars, then every weight load of the
    // thread in flight at once, then the first tile's bond inputs (their
    // latency hidden behind the weights' stores and scatter)
    const R edf = to_r<R>(edf_in[atom]);
    const int b0 = off[atom], b1 = off[atom + 1];
    constexpr int N1 = (D::NA2H + T - 1) / T, N2 = (D::NWA + T - 1) / T;
    {
      C<R> v1[N1], v2[N2];
#pragma unroll
      for (int u = 0; u < N1; ++u)
        v1[u] = t + u * T < D::NA2H ? weight(m.offW2 + t + u * T, -1) : C<R>{R(0), R(0)};
#pragma unroll
      for (int u = 0; u < N2; ++u) v2[u] = t + u * T < D::NWA ? weight(t + u * T, t + u * T) : C<R>{R(0), R(0)};
      if (t < D::NQ) W0s[t] = weight(m.offW0 + t, Ga ? __ldg(m.b3_cw + m.offW0 + t) : -1);
#pragma unroll
      for (int u = 0; u < N1; ++u)
        if (t + u * T < D::NA2H) raw[t + u * T] = v1[u];
#pragma unroll
      for (int u = 0; u < N2; ++u)
        if (t + u * T < D::NWA) raw[D::NA2H + t + u * T] = v2[u];
    }
    R sp0[8];
    if (stage && b0 + t < b1) ld8_l2(stage + 8 * static_cast<size_t>(b0 + t), sp0, pol_first);
    float* Bs = reinterpret_cast<float*>(Bf);
    for (int q = t; q < kTcFrags * 16; q += T) reinterpret_cast<float4*>(Bs)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    const auto place = [&](int f, int K, int n) { return f * 64 + ((n & 7) * 4 + (K & 3)) * 2 + ((K >> 2) & 1); };
    const auto put1 = [&](int K, int n, float v) { Bs[place((K >> 3) * 2 + (n >> 3), K, n)] = v; };
    const auto put2 = [&](int K, int n, float v) { Bs[place(kTcF1 + (K >> 3) * 4 + (n >> 3), K, n)] = v; };
    const auto put3 = [&](int K, int n, float v) {
      const int u = n >> 3, sk = K >> 3;
      Bs[place(kTcF1 + kTcF2 + (u < 5 ? 6 * u + sk : 30 + 2 * (u - 5) + sk), K, n)] = v;
    };
#pragma unroll 1
    for (int q = t; q < D::NA2H; q += T) {
      const C<R> w = raw[q];
      const int n = q / D::NQ, k = q % D::NQ;
      put1(k < D::NQ3 ? k : D::NQ3 + k, n, w.x);            // Re q_k column
      put1(k < D::NQ3 ? D::NQ3 + k : D::NQ + k, n, -w.y);   // Im q_k column
      put3(n, 2 * k, w.x);
      put3(n, 2 * k + 1, w.y);
    }
#pragma unroll 1
    for (int q = t; q < D::NWA; q += T) {
      const C<R> w = raw[D::NA2H + q];
      const int i = q / D::NQ3, k = q % D::NQ3;
      put2(k, 2 * i, w.x);
      put2(D::NQ3 + k, 2 * i, -w.y);
      put2(k, 2 * i + 1, w.y);
      put2(D::NQ3 + k, 2 * i + 1, w.x);
      put3(D::NB + i, 2 * k, w.x);
      put3(D::NB + i, 2 * k + 1, w.y);
      put3(D::NB + D::NRY + i, 2 * k, -w.y);
      put3(D::NB + D::NRY + i, 2 * k + 1, w.x);
    }
    __syncthreads();  // the fragments are built; the rows are free
    float* row = QA + t * kTcRow;                  // this thread's bond row
    const float* wrows = QA + warp * 32 * kTcRow;  // the warp's 32 rows
    for (int jt = b0; jt < b1; jt += T) {
      const int j = jt + t;
      const bool live = j < b1;
      // ---- the bond's inputs, and its magnetic functions M_nl, M'_nl (kept
      // in registers to the magnetic epilogue) with the Q row
      R r = R(1), ex = R(0), ey = R(0), ez = R(1), mg = R(1), mx = R(0), my = R(0), mz = R(1);
      R mv[D::NMF], Md[D::NMF];
      {
        if (live) {
          if (stage) {  // the A-basis kernel's copy in device memory
            R sp[8];
            if (jt == b0) {
#pragma unroll
              for (int q = 0; q < 8; ++q) sp[q] = sp0[q];
            } else {
              ld8_l2(stage + 8 * static_cast<size_t>(j), sp, pol_first);
            }
            r = sp[0];
            ex = sp[1];
            ey = sp[2];
            ez = sp[3];
            mg = sp[4];
            mx = sp[5];
            my = sp[6];
            mz = sp[7];
          } else {
            r = to_r<R>(rr[j]);
            ex = to_r<R>(ee[3 * j]);
            ey = to_r<R>(ee[3 * j + 1]);
            ez = to_r<R>(ee[3 * j + 2]);
            mg = to_r<R>(magj[j]);
            mx = to_r<R>(mhj[3 * j]);
            my = to_r<R>(mhj[3 * j + 1]);
            mz = to_r<R>(mhj[3 * j + 2]);
          }
        }
        R wm = R(0);
        const int nlm = live ? magnetic_bin_r<R>(m, mg, wm, err) : -1;
        if (nlm > 0) {
          lut_eval<true>(m.lut_m32, D::NFM, 0, D::NMF, nlm, wm, rscale_m<R>(m), mv, Md);
        } else {
#pragma unroll
          for (int q = 0; q < D::NMF; ++q) {
            mv[q] = R(nlm == 0 ? 1 : 0);
            Md[q] = R(0);
          }
        }
        // the Q row: q_k = M_{n, l(h)} Y_h(m-hat), k = n H2 + h, in the
        // column order Re (k < 18), Im (k < 18), Re (k >= 18), Im (k >= 18), 0
        C<R> Ym[D::H2];
        ylm_half<R, false>(D::L2, mx, my, mz, Ym, nullptr);
        const auto qcol = [&](int c) -> float {
          const int k = c < 2 * D::NQ3 ? c % D::NQ3 : (c < D::NQ3 + D::NQ ? c - D::NQ3 : c - D::NQ);
          const bool im = c < 2 * D::NQ3 ? c >= D::NQ3 : c >= D::NQ3 + D::NQ;
          if (c >= 2 * D::NQ) return 0.f;
          const int nr = k / D::H2, h = k % D::H2;
          const R mq = mv[nr * (D::L2 + 1) + l_of_h(h)];
          return im ? Ym[h].y * mq : Ym[h].x * mq;
        };
#pragma unroll
        for (int c = 0; c < 2 * D::NQ + 4; c += 4)
          *reinterpret_cast<float4*>(row + c) = make_float4(qcol(c), qcol(c + 1), qcol(c + 2), qcol(c + 3));
      }
      __syncwarp();
      // ---- force GEMMs F1 (sp) and F2 (U) over the warp's two m16 tiles
      {
        float s1[2][2][4], s2[2][4][4];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
          for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              s2[a][u][e] = 0.f;
              if (u < 2) s1[a][u][e] = 0.f;
            }
#pragma unroll
        for (int s = 0; s < 8; ++s) {
          uint32_t ah[2][4], al[2][4];
#pragma unroll
          for (int a = 0; a < 2; ++a) {
            const float* ra = wrows + (16 * a + gid) * kTcRow + 8 * s + tig;
            tf32_split(ra[0], ah[a][0], al[a][0]);
            tf32_split(ra[8 * kTcRow], ah[a][1], al[a][1]);
            tf32_split(ra[4], ah[a][2], al[a][2]);
            tf32_split(ra[8 * kTcRow + 4], ah[a][3], al[a][3]);
          }
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const float2 bv = Bf[(2 * s + u) * 32 + lane];
            uint32_t bh0, bl0, bh1, bl1;
            tf32_split(bv.x, bh0, bl0);
            tf32_split(bv.y, bh1, bl1);
#pragma unroll
            for (int a = 0; a < 2; ++a) mma_3xtf32(s1[a][u], ah[a], al[a], bh0, bh1, bl0, bl1);
          }
          if (s < 5) {
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const float2 bv = Bf[(kTcF1 + 4 * s + u) * 32 + lane];
              uint32_t bh0, bl0, bh1, bl1;
              tf32_split(bv.x, bh0, bl0);
              tf32_split(bv.y, bh1, bl1);
#pragma unroll
              for (int a = 0; a < 2; ++a) mma_3xtf32(s2[a][u], ah[a], al[a], bh0, bh1, bl0, bl1);
            }
          }
        }
        __syncwarp();  // every lane's Q fragments are read: the rows take the results
#pragma unroll
        for (int a = 0; a < 2; ++a) {
          float* r0 = const_cast<float*>(wrows) + (16 * a + gid) * kTcRow + 2 * tig;
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            *reinterpret_cast<float2*>(r0 + 8 * u) = make_float2(s1[a][u][0], s1[a][u][1]);
            *reinterpret_cast<float2*>(r0 + 8 * kTcRow + 8 * u) = make_float2(s1[a][u][2], s1[a][u][3]);
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            *reinterpret_cast<float2*>(r0 + D::NB + 8 * u) = make_float2(s2[a][u][0], s2[a][u][1]);
            *reinterpret_cast<float2*>(r0 + 8 * kTcRow + D::NB + 8 * u) = make_float2(s2[a][u][2], s2[a][u][3]);
          }
        }
        __syncwarp();
      }
      // ---- the atomic functions g_n, R_nl and the core term with derivatives
      R g[D::NB], gd[D::NB], tv[D::NR], td[D::NR], cdv = R(0);
      {
        R wl = R(0);
        const int nla = live ? atomic_bin_r<R>(m, r, wl, err) : 0;
        if (nla > 0) {
          R cv[1], cd1[1];
          lut_eval<true>(m.lut_a32, D::NFA, 0, D::NB, nla, wl, rscale_a<R>(m), g, gd);
          lut_eval<true>(m.lut_a32, D::NFA, D::NB, D::NR, nla, wl, rscale_a<R>(m), tv, td);
          lut_eval<true>(m.lut_a32, D::NFA, D::NB + D::NR, 1, nla, wl, rscale_a<R>(m), cv, cd1);
          cdv = cd1[0];
        } else {
#pragma unroll
          for (int q = 0; q < D::NB; ++q) g[q] = gd[q] = R(0);
#pragma unroll
          for (int q = 0; q < D::NR; ++q) tv[q] = td[q] = R(0);
        }
      }
      // ---- force epilogue (k_forces_fe's): the row holds sp_n, then (Re U_i, Im U_i)
      C<R> Ya[D::HA], dYa[D::HA][3];
      ylm_half<R, true>(D::LA, ex, ey, ez, Ya, dYa);
      if (live) {
        R fr = edf * cdv, ft[3] = {R(0), R(0), R(0)};
#pragma unroll
        for (int n = 0; n < D::NB; n += 4) {
          const float4 v = *reinterpret_cast<const float4*>(row + n);
          fr = fma(gd[n], v.x, fr);
          fr = fma(gd[n + 1], v.y, fr);
          fr = fma(gd[n + 2], v.z, fr);
          fr = fma(gd[n + 3], v.w, fr);
        }
        const R invr = rcp(r);
#pragma unroll
        for (int i = 0; i < D::NRY; i += 2) {
          const float4 v = *reinterpret_cast<const float4*>(row + D::NB + 2 * i);
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const C<R> U = e ? C<R>{v.z, v.w} : C<R>{v.x, v.y};
            const int ii = i + e, n1 = ii / D::LSA, lma = ii % D::LSA, l1 = l_of_lm(lma);
            const int mm = lma - l1 * l1 - l1;
            fr = fma(td[n1 * (D::LA + 1) + l1], re_mul(U, y_full(Ya, l1, mm)), fr);
            const C<R> su = cscale(U, invr * tv[n1 * (D::LA + 1) + l1]);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              C<R> d = dYa[ph(l1, mm < 0 ? -mm : mm)][c];
              if (mm < 0) {
                const R sg = R(parity(mm));
                d = {d.x * sg, -d.y * sg};
              }
              ft[c] = re_mac(ft[c], su, d);
            }
          }
        }
        *(SOUT ? sOut + 3 * t + 0 : fij + 3 * static_cast<size_t>(j) + 0) = to_d(fr * ex + ft[0]);
        *(SOUT ? sOut + 3 * t + 1 : fij + 3 * static_cast<size_t>(j) + 1) = to_d(fr * ey + ft[1]);
        *(SOUT ? sOut + 3 * t + 2 : fij + 3 * static_cast<size_t>(j) + 2) = to_d(fr * ez + ft[2]);
      }
      __syncwarp();  // the row's results are read: it takes the G row
      {
        // the G row: g_n, then Re and Im of RY_i = R_{n1, l} Y_lm(e), i = n1 LSA + lm
        const auto gcol = [&](int c) -> float {
          if (c < D::NB) return g[c];
          const int i = (c - D::NB) % D::NRY, n1 = i / D::LSA, lma = i % D::LSA, l1 = l_of_lm(lma);
          const C<R> y = y_full(Ya, l1, lma - l1 * l1 - l1);
          return (c < D::NB + D::NRY ? y.x : y.y) * tv[n1 * (D::LA + 1) + l1];
        };
#pragma unroll
        for (int c = 0; c < D::NB + 2 * D::NRY; c += 4)
          *reinterpret_cast<float4*>(row + c) = make_float4(gcol(c), gcol(c + 1), gcol(c + 2), gcol(c + 3));
      }
      __syncwarp();
      // ---- magnetic GEMM T (V) over all eight n-tiles (n-tiles 5-7 hold
      // k >= 20, which has no W_A terms: two k-steps)
      {
        float s3[2][8][4];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
          for (int u = 0; u < 8; ++u)
#pragma unroll
            for (int e = 0; e < 4; ++e) s3[a][u][e] = 0.f;
#pragma unroll
        for (int s = 0; s < 6; ++s) {
          uint32_t ah[2][4], al[2][4];
#pragma unroll
          for (int a = 0; a < 2; ++a) {
            const float* ra = wrows + (16 * a + gid) * kTcRow + 8 * s + tig;
            tf32_split(ra[0], ah[a][0], al[a][0]);
            tf32_split(ra[8 * kTcRow], ah[a][1], al[a][1]);
            tf32_split(ra[4], ah[a][2], al[a][2]);
            tf32_split(ra[8 * kTcRow + 4], ah[a][3], al[a][3]);
          }
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            if (u >= 5 && s >= 2) continue;
            const int f = kTcF1 + kTcF2 + (u < 5 ? 6 * u + s : 30 + 2 * (u - 5) + s);
            const float2 bv = Bf[f * 32 + lane];
            uint32_t bh0, bl0, bh1, bl1;
            tf32_split(bv.x, bh0, bl0);
            tf32_split(bv.y, bh1, bl1);
#pragma unroll
            for (int a = 0; a < 2; ++a) mma_3xtf32(s3[a][u], ah[a], al[a], bh0, bh1, bl0, bl1);
          }
        }
        __syncwarp();  // every lane's G fragments are read: the rows take V
#pragma unroll
        for (int a = 0; a < 2; ++a) {
          float* r0 = const_cast<float*>(wrows) + (16 * a + gid) * kTcRow + 2 * tig;
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            *reinterpret_cast<float2*>(r0 + 8 * u) = make_float2(s3[a][u][0], s3[a][u][1]);
            *reinterpret_cast<float2*>(r0 + 8 * kTcRow + 8 * u) = make_float2(s3[a][u][2], s3[a][u][3]);
          }
        }
        __syncwarp();
      }
      // ---- magnetic epilogue (k_forces_fe's): the row holds (Re V_k, Im V_k)
      if (live) {
        C<R> Ym[D::H2], dYm[D::H2][3];
        ylm_half<R, true>(D::L2, mx, my, mz, Ym, dYm);
        const R invm = rcp(mg);
        R tr = R(0), tt[3] = {R(0), R(0), R(0)};
#pragma unroll
        for (int k = 0; k < D::NQ; k += 2) {
          const float4 v = *reinterpret_cast<const float4*>(row + 2 * k);
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const C<R> V = e ? C<R>{v.z, v.w} : C<R>{v.x, v.y};
            const int kk = k + e, nr = kk / D::H2, h = kk % D::H2, q = nr * (D::L2 + 1) + l_of_h(h);
            tr = fma(Md[q], re_mul(V, Ym[h]), tr);
            const C<R> sv = cscale(V, invm * mv[q]);
#pragma unroll
            for (int c = 0; c < 3; ++c) tt[c] = re_mac(tt[c], sv, dYm[h][c]);
          }
        }
        *(SOUT ? sOut + 3 * T + 3 * t + 0 : tij + 3 * static_cast<size_t>(j) + 0) = to_d(tr * mx + tt[0]);
        *(SOUT ? sOut + 3 * T + 3 * t + 1 : tij + 3 * static_cast<size_t>(j) + 1) = to_d(tr * my + tt[1]);
        *(SOUT ? sOut + 3 * T + 3 * t + 2 : tij + 3 * static_cast<size_t>(j) + 2) = to_d(tr * mz + tt[2]);
      }
      if constexpr (SOUT) {
        __syncthreads();
        store_tile(fij, sOut, jt, min(T, b1 - jt));
        store_tile(tij, sOut + 3 * T, jt, min(T, b1 - jt));
        __syncthreads();
      }
      __syncwarp();  // the row is read before the next tile's Q row
    }
    if (t >= 32) {
      // on-site magnetic force dE_i/dm_i (src/forces.F90:690-749) on warp 1,
      // as in k_forces_fe
      static_assert(D::NMF + D::NBM <= 32 && D::NQ <= 32, "one function and one weight per lane");
      const R mg = to_r<R>(magi[atom]);
      const R mx = to_r<R>(mhi[3 * atom]), my = to_r<R>(mhi[3 * atom + 1]), mz = to_r<R>(mhi[3 * atom + 2]);
      R wm = R(0);
      const int nl = magnetic_bin_r<R>(m, mg, wm, err);
      R v = R(nl == 0 ? 1 : 0), dv = R(0);
      if (nl > 0 && lane < D::NMF + D::NBM) lut_eval<true>(m.lut_m32, D::NFM, lane, 1, nl, wm, rscale_m<R>(m), &v, &dv);
      C<R> Yh[D::H2], dYh[D::H2][3];
      ylm_half<R, true>(D::L2, mx, my, mz, Yh, dYh);
      R tr = R(0), tt[3] = {R(0), R(0), R(0)};
      const int n = lane - D::NMF;
      if (n >= 0 && n < D::NBM) tr = to_r<R>(dedrho[static_cast<size_t>(atom) * 2]) * c1_of<R>(m, n) * dv;
      const int k = lane < D::NQ ? lane : 0;
      const int nr = k / D::H2, h = k % D::H2, q = nr * (D::L2 + 1) + l_of_h(h);
      const R Mq = __shfl_sync(0xffffffffu, v, q), Mdq = __shfl_sync(0xffffffffu, dv, q);
      if (lane < D::NQ) {
        // Y_h and its gradient by selection (h differs across the lanes)
        C<R> y = Yh[0], dy[3] = {dYh[0][0], dYh[0][1], dYh[0][2]};
#pragma unroll
        for (int hh = 1; hh < D::H2; ++hh)
          if (h == hh) {
            y = Yh[hh];
#pragma unroll
            for (int c = 0; c < 3; ++c) dy[c] = dYh[hh][c];
          }
        const C<R> w = W0s[k];
        const R invm = rcp(mg);
        tr += Mdq * re_mul(w, y);
        const R s = invm * Mq;
#pragma unroll
        for (int c = 0; c < 3; ++c) tt[c] += s * re_mul(w, dy[c]);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        tr += __shfl_xor_sync(0xffffffffu, tr, o);
#pragma unroll
        for (int c = 0; c < 3; ++c) tt[c] += __shfl_xor_sync(0xffffffffu, tt[c], o);
      }
      if (lane == 0) {
        ti0[3 * static_cast<size_t>(atom) + 0] = to_d(tr * mx + tt[0]);
        ti0[3 * static_cast<size_t>(atom) + 1] = to_d(tr * my + tt[1]);
        ti0[3 * static_cast<size_t>(atom) + 2] = to_d(tr * mz + tt[2]);
      }
    }
    __syncthreads();  // the fragments, W0 and the rows are free for the next atom
  }
}

inline size_t density_fe_smem(const DeviceModel& m, int nw) {
  // factors, per-warp density partials, per-warp 16-record buffers, the
  // split slots' part weights
  return sizeof(C<float>) * static_cast<size_t>(m.r_nfac) * kRestStride + sizeof(double) * nw * 32 +
         sizeof(uint4) * 16 * nw + sizeof(C<float>) * 64 * static_cast<size_t>(m.r_nsplit);
}
template <class D>
size_t b3_fe_smem(const DeviceModel& m, int nw) {
  const size_t ncoef = static_cast<size_t>(m.b3_ncombo) * D::NM * D::I * D::I;
  return sizeof(float) * ((ncoef + 3) & ~static_cast<size_t>(3)) +
         sizeof(C<float>) * 2 * static_cast<size_t>(m.b3_nc) * kB3Stride + sizeof(double) * nw * 32 +
         sizeof(float) * m.b3_nc + sizeof(int) * m.b3_nc;
}
constexpr int kB3Warps64 = 8;  // warps per CTA of k_b3_fe64
template <class D>
size_t b3_fe64_smem(const DeviceModel& m) {
  return sizeof(C<double>) * static_cast<size_t>(m.b3_nc) * kB3Stride64 + sizeof(int) * m.b3_nc;
}
template <class R, class D>
size_t forces_fe_smem(bool sout) {
  return sizeof(C<R>) * (D::NQ * D::NB + D::NQ3 * D::NRY + D::NQ + 2) +
         sizeof(R) * 64 * (D::NB + 2 * D::NR + 2 * D::NMF) + sizeof(C<R>) * 64 * D::LSA +
         (sout ? sizeof(double) * 6 * 64 : 0) + 64;
}
