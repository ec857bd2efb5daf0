// C ABI and runtime: the drop-in acelibini_/acelib_ entry points, the
// extended ace_* API, device-table upload and device work buffers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <limits>
#include <string>
#include <vector>

#include "device_model.hpp"
#include "kernels.hpp"
#include "magace.h"
#include "model.hpp"
#include "potential.hpp"

namespace magace {
namespace {

// element symbols indexed by atomic number + 1 - 1 (index 0 is the
// placeholder 'X'; the caller passes atomic number + 1, src/ace.F90:30-37)
const char* const kElements[] = {
    "X",  "H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg", "Al", "Si", "P",  "S",
    "Cl", "Ar", "K",  "Ca", "Sc", "Ti", "V",  "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As",
    "Se", "Br", "Kr", "Rb", "Sr", "Y",  "Zr", "Nb", "Mo", "Tc", "Ru", "Rh", "Pd", "Ag", "Cd", "In", "Sn",
    "Sb", "Te", "I",  "Xe", "Cs", "Ba", "La", "Ce", "Pr", "Nd", "Pm", "Sm", "Eu", "Gd", "Tb", "Dy", "Ho",
    "Er", "Tm", "Yb", "Lu", "Hf", "Ta", "W",  "Re", "Os", "Ir", "Pt", "Au", "Hg", "Tl", "Pb", "Bi", "Po",
    "At", "Rn", "Fr", "Ra", "Ac", "Th", "Pa", "U",  "Np", "Pu", "Am", "Cm", "Bk", "Cf", "Es", "Fm", "Md",
    "No", "Lr"};
const int kNumElements = sizeof(kElements) / sizeof(kElements[0]);

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t reserve(size_t count) {
    if (count <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    size_t want = std::max<size_t>(count, 1);
    want += want / 4;  // geometric headroom for growing systems
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), want * sizeof(T));
    if (e == cudaSuccess) n = want;
    return e;
  }
  cudaError_t upload(const std::vector<T>& v) {
    cudaError_t e = reserve(v.size());
    if (e != cudaSuccess) return e;
    if (!v.empty()) e = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

struct Runtime {
  Model model;
  bool ready = false;
  bool ini_done = false;  // acelibini_ succeeded once (src/util.F90:29-33)
  int precision = 0;
  int last_error = MAGACE_OK;
  std::string last_msg;
  int last_launches = 0;  // timed slots of the last evaluation (ace_kernel_times)
  int last_kernels = 0;   // kernels it launched
  // the side stream and fork/join events of the density kernels (EvalBuffers::side)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  bool overlap = true;  // MAGACE_OVERLAP=0 keeps every kernel on the launch stream
  int last_natom = -1;  // atoms of the last evaluation (ace_density_gradient_device)
  bool work_queue = false;  // neighbour-count-sorted work queue
  // kernel variants (ace_autotune_device, ace_set_tuning)
  int tune_abasis = kDefaultTuning[0], tune_rest = kDefaultTuning[1], tune_b3 = kDefaultTuning[2],
      tune_forces = kDefaultTuning[3];
  DevBuf<int> order, queue_bins;

  // device tables
  bool dev_tables = false;
  int device = -1;
  cudaStream_t stream = nullptr;
  DevBuf<double> lut_a, lut_m, c1;
  DevBuf<float> c1f;
  DevBuf<float> lut_a32, lut_m32;
  struct GatherBufs {
    DevBuf<double> kap[kMaxArity + 1], slot_mult;
    DevBuf<float> kapf[kMaxArity + 1], slot_multf;
    DevBuf<uint32_t> o12[kMaxArity + 1], o34[kMaxArity + 1];
    DevBuf<uint16_t> o5;
    DevBuf<int32_t> grp_arity, grp_len, grp_first, grp_seg, slot_seg, slot_factor, slot_weight;
    void release() {
      for (int a = 0; a <= kMaxArity; ++a) {
        kap[a].release();
        kapf[a].release();
        o12[a].release();
        o34[a].release();
      }
      slot_mult.release();
      slot_multf.release();
      o5.release();
      for (auto* b : {&grp_arity, &grp_len, &grp_first, &grp_seg, &slot_seg, &slot_factor, &slot_weight}) b->release();
    }
  } gb1, gb2;
  DevBuf<float> b3_Cf, b3_cff, b3_mult, b3_cfw, b3_Chl, r_kaphl;
  DevBuf<double> b3_C64, b3_cf64, b3_cfw64, r_kap64;
  DevBuf<int32_t> b3_pattern, b3_combo, b3_factor, b3_cw;
  DevBuf<uint16_t> b3_code, b3_code2;
  DevBuf<int32_t> d_rank1_n, d_begin;
  DevBuf<int32_t> r_factor, r_run, r_g0, r_warp_begin, r_warp_slots;
  DevBuf<uint32_t> r_rec, r_stream;
  DevBuf<int32_t> r_stream_begin, r_split_w, r64_warp_begin, r64_warp_slots;
  DevBuf<double> d_cf;
  DevBuf<uint16_t> d_o;
  DeviceModel dm{};
  int grid_cap = 0;

  // work buffers
  DevBuf<int> off, err;
  DevBuf<double> r, e, magj, mhj, magi, mhi, energy, fij, tij, ti0, rho1, core, edf, dedrho;
  DevBuf<unsigned char> F, W, aux, bstage, Fd;
  std::vector<int> h_off;

  // pinned staging for host transfers, and whether the GPU reads pageable
  // host memory directly (Grace: NVLink-C2C with the host page tables)
  unsigned char* pinned = nullptr;
  size_t pinned_bytes = 0;
  int pageable_access = -1;  // -1 unknown, 0 no, 1 yes

  // optional kernel-boundary events of the last evaluation
  bool timing = false;
  cudaEvent_t ev[kMaxLaunches + 1] = {};
  bool ev_recorded = false;
};

Runtime& rt() {
  static Runtime r;
  return r;
}

int set_error(int code, const std::string& msg) {
  Runtime& R = rt();
  R.last_error = code;
  R.last_msg = msg;
  if (code != MAGACE_OK) std::fprintf(stderr, "magace: %s\n", msg.c_str());
  return code;
}

int cuda_error(cudaError_t e, const char* what) {
  return set_error(MAGACE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// The kernels index the per-bond and per-atom vectors as 3 j with 32-bit j,
// so one call takes at most INT_MAX / 3 = 715,827,882 bonds (and atoms).
constexpr int kMaxCallSize = std::numeric_limits<int>::max() / 3;

int check_sizes(int natom, int nei) {
  if (natom < 0 || nei < 0) return set_error(MAGACE_ERR_ARGS, "negative sizes");
  if (natom > kMaxCallSize || nei > kMaxCallSize)
    return set_error(MAGACE_ERR_ARGS, "more than 715,827,882 atoms or bonds in one call (32-bit indices): split the call");
  return MAGACE_OK;
}

#define CUDA_TRY(call)                                \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return cuda_error(e_, #call); \
  } while (0)

void ylm_constants(double* alm, double* blm, double* cl, double* dl) {
  // recurrence constants of src/spherical.F90:18-49, indexed by l(l+1)/2 + m
  for (int i = 0; i < kMaxHalf; ++i) alm[i] = blm[i] = 0.0;
  for (int l = 0; l <= kMaxL; ++l) cl[l] = dl[l] = 0.0;
  for (int l = 1; l <= kMaxL; ++l) {
    const double lsq = l * l, ld = 2 * l, l1 = 4 * lsq - 1, l2 = lsq - ld + 1;
    for (int m = 0; m <= l - 2; ++m) {
      const double msq = m * m;
      alm[l * (l + 1) / 2 + m] = std::sqrt(l1 / (lsq - msq));
      blm[l * (l + 1) / 2 + m] = -std::sqrt((l2 - msq) / (4 * l2 - 1));
    }
    cl[l] = -std::sqrt(1.0 + 0.5 / static_cast<double>(l));
    dl[l] = std::sqrt(2.0 * (l - 1) + 3.0);
  }
}

template <class T>
std::vector<float> to_float(const std::vector<T>& v) {
  return std::vector<float>(v.begin(), v.end());
}

int upload_gather(const GatherTable& g, Runtime::GatherBufs& B, GatherView& v) {
  for (int a = 1; a <= kMaxArity; ++a) {
    std::vector<double> k(g.kap[a][0]);
    k.insert(k.end(), g.kap[a][1].begin(), g.kap[a][1].end());
    CUDA_TRY(B.kap[a].upload(k));
    CUDA_TRY(B.kapf[a].upload(to_float(k)));
    CUDA_TRY(B.o12[a].upload(g.o12[a]));
    CUDA_TRY(B.o34[a].upload(g.o34[a]));
  }
  CUDA_TRY(B.o5.upload(g.o5));
  CUDA_TRY(B.grp_arity.upload(g.grp_arity));
  CUDA_TRY(B.grp_len.upload(g.grp_len));
  CUDA_TRY(B.grp_first.upload(g.grp_first));
  CUDA_TRY(B.grp_seg.upload(g.grp_seg));
  CUDA_TRY(B.slot_seg.upload(g.slot_seg_begin));
  CUDA_TRY(B.slot_factor.upload(g.slot_factor));
  CUDA_TRY(B.slot_weight.upload(g.slot_weight));
  CUDA_TRY(B.slot_mult.upload(g.slot_mult));
  CUDA_TRY(B.slot_multf.upload(to_float(g.slot_mult)));
  v.nslot = g.nslot;
  v.nG0 = g.nG0;
  v.nseg = g.nseg;
  v.ngroup = g.ngroup;
  v.grp_arity = B.grp_arity.p;
  v.grp_len = B.grp_len.p;
  v.grp_first = B.grp_first.p;
  v.grp_seg = B.grp_seg.p;
  v.kap[0] = nullptr;
  v.kapf[0] = nullptr;
  v.o12[0] = nullptr;
  v.o34[0] = nullptr;
  v.kstride[0] = 0;
  for (int a = 1; a <= kMaxArity; ++a) {
    v.kap[a] = B.kap[a].p;
    v.kapf[a] = B.kapf[a].p;
    v.o12[a] = B.o12[a].p;
    v.o34[a] = B.o34[a].p;
    v.kstride[a] = static_cast<int>(g.kap[a][0].size());
  }
  v.o5 = B.o5.p;
  v.slot_seg = B.slot_seg.p;
  v.slot_factor = B.slot_factor.p;
  v.slot_weight = B.slot_weight.p;
  v.slot_mult = B.slot_mult.p;
  v.slot_multf = B.slot_multf.p;
  return MAGACE_OK;
}

int upload_tables() {
  Runtime& R = rt();
  if (!R.ready) return set_error(MAGACE_ERR_NOT_INIT, "no potential initialised");
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  if (R.dev_tables && R.device == dev) return MAGACE_OK;
  R.device = dev;
  if (!R.stream) CUDA_TRY(cudaStreamCreateWithFlags(&R.stream, cudaStreamNonBlocking));
  if (!R.side) {
    CUDA_TRY(cudaStreamCreateWithFlags(&R.side, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreateWithFlags(&R.ev_fork, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&R.ev_join, cudaEventDisableTiming));
    const char* e = std::getenv("MAGACE_OVERLAP");
    R.overlap = !(e && e[0] == '0');
  }
  const Model& M = R.model;
  const GatherTable& g = M.gt;
  CUDA_TRY(R.lut_a.upload(M.lut.a));
  CUDA_TRY(R.lut_m.upload(M.lut.m));
  CUDA_TRY(R.lut_a32.upload(to_float(M.lut.a)));
  CUDA_TRY(R.lut_m32.upload(to_float(M.lut.m)));
  std::vector<double> c1(2 * M.L.nbm);
  for (int d = 0; d < 2; ++d)
    for (int n = 0; n < M.L.nbm; ++n) c1[d * M.L.nbm + n] = M.c1[d][n];
  CUDA_TRY(R.c1.upload(c1));
  CUDA_TRY(R.c1f.upload(to_float(c1)));
  {
    int st = upload_gather(M.gt, R.gb1, R.dm.g);
    if (st) return st;
    if (M.ndensity == 1 && !M.high) {
      st = upload_gather(M.gt_nob3, R.gb2, R.dm.g2);
      if (st) return st;
      const DenseB3& D = M.db3;
      CUDA_TRY(R.b3_Cf.upload(to_float(D.C)));
      CUDA_TRY(R.b3_cff.upload(to_float(D.task_cf)));
      CUDA_TRY(R.b3_pattern.upload(D.pattern));
      CUDA_TRY(R.b3_combo.upload(D.task_combo));
      CUDA_TRY(R.b3_code.upload(D.code));
      CUDA_TRY(R.b3_code2.upload(D.code2));
      {
        std::vector<double> cfw(D.ntask);
        for (int t = 0; t < D.ntask; ++t) cfw[t] = D.task_cf[t] * D.task_w[t];
        CUDA_TRY(R.b3_cfw.upload(to_float(cfw)));
        CUDA_TRY(R.b3_cfw64.upload(cfw));
      }
      CUDA_TRY(R.b3_C64.upload(D.C));
      {
        std::vector<float> hl(2 * D.C.size());
        for (size_t q = 0; q < D.C.size(); ++q) {
          hl[2 * q] = static_cast<float>(D.C[q]);
          hl[2 * q + 1] = static_cast<float>(D.C[q] - static_cast<double>(hl[2 * q]));
        }
        CUDA_TRY(R.b3_Chl.upload(hl));
      }
      CUDA_TRY(R.b3_cf64.upload(D.task_cf));
      CUDA_TRY(R.b3_factor.upload(D.factor_of));
      CUDA_TRY(R.b3_cw.upload(D.compact_of_weight));
      CUDA_TRY(R.b3_mult.upload(to_float(D.mult)));
      const RestTable& T = M.rest;
      CUDA_TRY(R.r_factor.upload(T.factor_of));
      CUDA_TRY(R.r_run.upload(T.run));
      CUDA_TRY(R.r_g0.upload(T.slot_g0));
      CUDA_TRY(R.r_rec.upload(T.rec));
      CUDA_TRY(R.r_kap64.upload(T.kap));
      {
        std::vector<float> hl(2 * T.kap.size());
        for (size_t q = 0; q < T.kap.size(); ++q) {
          hl[2 * q] = static_cast<float>(T.kap[q]);
          hl[2 * q + 1] = static_cast<float>(T.kap[q] - static_cast<double>(hl[2 * q]));
        }
        CUDA_TRY(R.r_kaphl.upload(hl));
      }
      CUDA_TRY(R.r_warp_begin.upload(T.warp_begin));
      CUDA_TRY(R.r_warp_slots.upload(T.warp_slots));
      CUDA_TRY(R.r_stream.upload(T.stream));
      CUDA_TRY(R.r_stream_begin.upload(T.stream_begin));
      if (T.nsplit) CUDA_TRY(R.r_split_w.upload(T.split_weight));
      CUDA_TRY(R.r64_warp_begin.upload(T.warp64_begin));
      CUDA_TRY(R.r64_warp_slots.upload(T.warp64_slots));
    } else {
      R.dm.g2 = R.dm.g;
    }
  }
  {
    const DescriptorTable& T = M.desc;
    CUDA_TRY(R.d_rank1_n.upload(T.rank1_n));
    CUDA_TRY(R.d_begin.upload(T.begin));
    CUDA_TRY(R.d_cf.upload(T.cf));
    CUDA_TRY(R.d_o.upload(T.o));
  }
  double alm[kMaxHalf], blm[kMaxHalf], cl[kMaxL + 1], dl[kMaxL + 1];
  ylm_constants(alm, blm, cl, dl);
  upload_ylm_constants(alm, blm, cl, dl);

  DeviceModel& d = R.dm;
  const FactorLayout& L = M.L;
  d.n3a = L.n3a; d.n3m = L.n3m; d.l3a = L.l3a; d.l3m = L.l3m;
  d.nba = L.nba; d.n2m = L.n2m; d.l2m = L.l2m; d.nbm = L.nbm;
  d.lsa = L.lsa; d.ls3 = L.ls3; d.ls2 = L.ls2; d.h3 = L.h3; d.h2 = L.h2;
  d.offA = L.offA; d.offA2 = L.offA2; d.offA0 = L.offA0; d.offOne = L.offOne; d.offZero = L.offZero;
  d.nF = L.nF; d.nWA = L.nWA; d.offW2 = L.offW2; d.offW0 = L.offW0; d.nW = L.nW;
  d.nd = M.ndensity;
  d.nfemb = M.nfemb;
  d.high = M.high ? 1 : 0;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) d.par[a][b] = M.par[a][b];
  d.ecut = M.ecut;
  d.decut = M.decut;
  d.nlut = M.lut.nlut;
  d.nfa = M.lut.nfa;
  d.nfm = M.lut.nfm;
  d.rscale_a = M.lut.rscale_a;
  d.rscale_m = M.lut.rscale_m;
  d.lut_a = R.lut_a.p;
  d.lut_m = R.lut_m.p;
  d.lut_a32 = R.lut_a32.p;
  d.lut_m32 = R.lut_m32.p;
  d.c1 = R.c1.p;
  d.c1f = R.c1f.p;
  d.rscale_a_f = static_cast<float>(d.rscale_a);
  d.rscale_m_f = static_cast<float>(d.rscale_m);
  d.b3_ntask = M.db3.ntask;
  d.b3_ncombo = M.db3.ncombo;
  d.b3_nc = M.db3.nc;
  d.b3_Cf = R.b3_Cf.p;
  d.b3_pattern = R.b3_pattern.p;
  d.b3_combo = R.b3_combo.p;
  d.b3_cff = R.b3_cff.p;
  d.b3_code = R.b3_code.p;
  d.b3_code2 = R.b3_code2.p;
  d.b3_cfw = R.b3_cfw.p;
  d.b3_factor = R.b3_factor.p;
  d.b3_cw = R.b3_cw.p;
  d.b3_mult = R.b3_mult.p;
  d.b3_C64 = R.b3_C64.p;
  d.b3_Chl = R.b3_Chl.p;
  d.b3_cf64 = R.b3_cf64.p;
  d.b3_cfw64 = R.b3_cfw64.p;
  d.b3_bound = M.db3.bound;
  d.b3_bound_rho = M.db3.bound_rho;
  d.tune_abasis = R.tune_abasis;
  d.tune_rest = R.tune_rest;
  d.tune_b3 = R.tune_b3;
  d.tune_forces = R.tune_forces;
  d.r_nfac = M.rest.nfac;
  d.r_nslot = M.rest.nslot;
  d.r_factor = R.r_factor.p;
  d.r_run = R.r_run.p;
  d.r_rec = R.r_rec.p;
  d.r_kap64 = R.r_kap64.p;
  d.r_kaphl = R.r_kaphl.p;
  d.r_g0 = R.r_g0.p;
  d.r_warp_begin = R.r_warp_begin.p;
  d.r_warp_slots = R.r_warp_slots.p;
  d.r_stream = R.r_stream.p;
  d.r_stream_begin = R.r_stream_begin.p;
  d.r_nsplit = M.rest.nsplit;
  d.r64_warp_begin = R.r64_warp_begin.p;
  d.r64_warp_slots = R.r64_warp_slots.p;
  d.r_split_w = R.r_split_w.p;
  d.d_n1 = M.desc.n1;
  d.d_nB = M.desc.nB;
  d.d_rank1_n = R.d_rank1_n.p;
  d.d_begin = R.d_begin.p;
  d.d_cf = R.d_cf.p;
  d.d_o = R.d_o.p;
  int sms = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  R.grid_cap = std::max(1, sms) * 64;
  int smem_max = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  for (int p = 0; p < 2; ++p)
    for (int w = 0; w < 3; ++w)
      if (eval_smem_bytes(d, p, w) > static_cast<size_t>(smem_max))
        return set_error(MAGACE_ERR_UNSUPPORTED, "basis too large for the kernels' shared-memory tiles");
  R.dev_tables = true;
  return MAGACE_OK;
}

int reserve_work(int natom, int nei, int precision) {
  Runtime& R = rt();
  const size_t na = static_cast<size_t>(natom), nb = static_cast<size_t>(nei);
  const size_t csz = precision == 0 ? 16 : 8;
  CUDA_TRY(R.off.reserve(na + 1));
  CUDA_TRY(R.err.reserve(1));
  CUDA_TRY(R.energy.reserve(na));
  CUDA_TRY(R.rho1.reserve(2 * na));
  CUDA_TRY(R.core.reserve(na));
  CUDA_TRY(R.edf.reserve(na));
  CUDA_TRY(R.dedrho.reserve(2 * na));
  CUDA_TRY(R.F.reserve(na * R.dm.nF * csz));
  CUDA_TRY(R.W.reserve(na * R.dm.nW * csz));
  CUDA_TRY(R.aux.reserve(eval_aux_bytes(R.dm, precision, natom)));
  CUDA_TRY(R.bstage.reserve(nb * 8 * (precision == 0 ? sizeof(double) : sizeof(float))));
  return MAGACE_OK;
}

int run_eval(EvalBuffers& b, cudaStream_t st) {
  Runtime& R = rt();
  b.F = R.F.p;
  b.W = R.W.p;
  b.rho1 = R.rho1.p;
  b.core = R.core.p;
  b.edf = R.edf.p;
  b.dedrho = R.dedrho.p;
  b.err = R.err.p;
  b.aux = R.aux.p;
  b.stage = R.bstage.p;
  CUDA_TRY(cudaMemsetAsync(R.err.p, 0, sizeof(int), st));
  if (R.work_queue && b.natom > 0) {
    CUDA_TRY(R.order.reserve(static_cast<size_t>(b.natom)));
    CUDA_TRY(R.queue_bins.reserve(2 * kQueueBins));
    launch_work_queue(b.natom, b.off, R.order.p, R.queue_bins.p, st);
    b.order = R.order.p;
  }
  cudaEvent_t* ev = nullptr;
  if (R.timing) {
    for (auto& e : R.ev)
      if (!e) CUDA_TRY(cudaEventCreate(&e));
    ev = R.ev;
  }
  if (!ev && R.overlap && R.side) {
    b.side = R.side;
    b.ev_fork = R.ev_fork;
    b.ev_join = R.ev_join;
  }
  R.last_launches = R.precision == 0 ? launch_eval_fp64(R.dm, b, st, R.grid_cap, ev, &R.last_kernels)
                                     : launch_eval_fp32(R.dm, b, st, R.grid_cap, ev, &R.last_kernels);
  R.ev_recorded = ev != nullptr && R.last_launches >= 3;
  R.last_natom = b.natom;
  CUDA_TRY(cudaGetLastError());
  return MAGACE_OK;
}

int device_error_to_status(int dev) {
  switch (dev) {
    case kDevOk: return MAGACE_OK;
    case kDevSmallR: return set_error(MAGACE_ERR_SMALL_R, "encountered a very small distance");
    case kDevMoment: return set_error(MAGACE_ERR_MOMENT, "moment magnitude negative, NaN or beyond the magnetic cutoff");
    case kDevNaN: return set_error(MAGACE_ERR_NAN, "non-finite density");
    case kDevTimeout: return set_error(MAGACE_ERR_CUDA, "a bulk copy of bond inputs did not complete");
    default: return set_error(MAGACE_ERR_ARGS, "inconsistent bond tile");
  }
}

enum HostAccess { kHostCopy = 0, kHostPinned = 1, kHostDirect = 2 };

// How acelib_ moves the caller's host arrays. MAGACE_HOST_ACCESS selects
// "direct" (kernels read and write the caller's pageable memory, possible
// when the GPU uses the host page tables, as on Grace with NVLink-C2C),
// "pinned" (staged through a pinned buffer) or "copy" (plain pageable
// copies); the default "auto" takes direct when available, else pinned.
int host_access_mode() {
  Runtime& R = rt();
  if (R.pageable_access < 0) {
    int a = 0, b = 0;
    if (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, R.device) != cudaSuccess) a = 0;
    if (cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, R.device) != cudaSuccess) b = 0;
    R.pageable_access = (a && b) ? 1 : 0;
  }
  const char* env = std::getenv("MAGACE_HOST_ACCESS");
  const std::string m = env ? env : "auto";
  if (m == "copy") return kHostCopy;
  if (m == "pinned") return kHostPinned;
  if (m == "direct" && R.pageable_access == 1) return kHostDirect;
  return R.pageable_access == 1 ? kHostDirect : kHostPinned;
}

int reserve_pinned(size_t bytes) {
  Runtime& R = rt();
  if (bytes <= R.pinned_bytes && R.pinned) return MAGACE_OK;
  if (R.pinned) cudaFreeHost(R.pinned);
  R.pinned = nullptr;
  R.pinned_bytes = 0;
  size_t want = bytes + bytes / 4;
  CUDA_TRY(cudaHostAlloc(reinterpret_cast<void**>(&R.pinned), want, cudaHostAllocDefault));
  R.pinned_bytes = want;
  return MAGACE_OK;
}

int init_file(const char* path, const char* element, double rcut, double rcut_magnetic, double smear,
              int xcnumber) {
  Runtime& R = rt();
  std::string xc;
  if (xcnumber == 1) xc = "pbe";
  else if (xcnumber == 2) xc = "lda";
  else return set_error(MAGACE_ERR_ARGS, "unknown XC functional received by acelibini");
  Potential pot;
  std::string msg;
  int st = read_potential(path, element, xc, smear, pot, msg);
  if (st) return set_error(st, msg);
  Model mdl;
  st = build_model(pot, rcut, rcut_magnetic, mdl, msg);
  if (st) return set_error(st, msg);
  const FactorLayout& L = mdl.L;
  if (L.l3a > kMaxL || L.l2m > kMaxL || L.nba > kMaxFeat || L.nbm > kMaxFeat ||
      L.n3a * (L.l3a + 1) > kMaxFeat || L.n2m * (L.l2m + 1) > kMaxFeat)
    return set_error(MAGACE_ERR_UNSUPPORTED, "basis exceeds the kernels' compile-time limits (l <= 4, <= 32 radial functions)");
  R.model = std::move(mdl);
  R.ready = true;
  R.dev_tables = false;
  return set_error(MAGACE_OK, "");
}

}  // namespace

// Read-only view of the runtime for the allocation-free entry point
// (noalloc.cu): the device model of the current device, if its tables are
// already resident there, and the selected precision.
int runtime_snapshot(DeviceModel* dm, int* precision, int* grid_cap) {
  Runtime& R = rt();
  if (!R.ready) return set_error(MAGACE_ERR_NOT_INIT, "no potential initialised");
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  if (!R.dev_tables || R.device != dev)
    return set_error(MAGACE_ERR_NOT_INIT,
                     "the potential's tables are not on this device yet; an ace_compute_device call "
                     "(natom = 0 is enough) places them");
  *dm = R.dm;
  *precision = R.precision;
  *grid_cap = R.grid_cap;
  return MAGACE_OK;
}

int runtime_error(int code, const char* msg) { return set_error(code, msg); }

int runtime_check_sizes(int natom, int nei) { return check_sizes(natom, nei); }

bool runtime_device_resident(const void* r, const void* e, const void* mag_j, const void* mhat_j);

int runtime_device_error(int dev_err) { return dev_err ? device_error_to_status(dev_err) : set_error(MAGACE_OK, ""); }

void runtime_set_launches(int slots, int kernels) {
  rt().last_launches = slots;
  rt().last_kernels = kernels;
}

}  // namespace magace

using namespace magace;

// True when every non-null pointer is device memory, 8-byte aligned: the
// bond arrays the TMA-staged A-basis variants read with bulk copies.
static bool device_resident(std::initializer_list<const void*> ptrs) {
  for (const void* p : ptrs) {
    if (!p) continue;
    if (reinterpret_cast<uintptr_t>(p) & 7u) return false;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    if (a.type != cudaMemoryTypeDevice) return false;
  }
  return true;
}


namespace magace {
// The same check for the allocation-free entry point (noalloc.cu).
bool runtime_device_resident(const void* r, const void* e, const void* mag_j, const void* mhat_j) {
  return device_resident({r, e, mag_j, mhat_j});
}
}  // namespace magace

extern "C" {

int ace_last_error(void) { return rt().last_error; }

const char* ace_last_error_message(void) { return rt().last_msg.c_str(); }

void ace_clear_error(void) {
  rt().last_error = MAGACE_OK;
  rt().last_msg.clear();
}

const char* ace_error_string(int code) {
  switch (code) {
    case MAGACE_OK: return "ok";
    case MAGACE_ERR_FILE: return "potential file missing or unreadable";
    case MAGACE_ERR_FORMAT: return "malformed or inconsistent potential file";
    case MAGACE_ERR_UNSUPPORTED: return "unsupported potential or argument";
    case MAGACE_ERR_SMALL_R: return "bond shorter than one lookup-table bin";
    case MAGACE_ERR_MOMENT: return "moment magnitude out of the tabulated range";
    case MAGACE_ERR_NOT_INIT: return "not initialised";
    case MAGACE_ERR_ARGS: return "inconsistent arguments";
    case MAGACE_ERR_CUDA: return "CUDA runtime failure";
    case MAGACE_ERR_NAN: return "non-finite density";
    default: return "unknown error";
  }
}

int ace_init_file(const char* path, const char* element, double rcut, double rcut_magnetic, double smear,
                  int xcnumber) {
  if (!path || !element) return set_error(MAGACE_ERR_ARGS, "null path or element");
  return init_file(path, element, rcut, rcut_magnetic, smear, xcnumber);
}

void acelibini_(int* nele, double* rcut, double* rcut_magnetic, double* smear, int* xcnumber, int* elenumbers) {
  Runtime& R = rt();
  if (R.ini_done) return;  // later calls are no-ops, as in src/util.F90:29-33
  if (!nele || *nele != 1) {
    set_error(MAGACE_ERR_UNSUPPORTED, "multiple elements require fixing acelibini call first");
    return;
  }
  const int idx = elenumbers ? elenumbers[0] - 1 : -1;
  if (idx < 1 || idx >= kNumElements) {
    set_error(MAGACE_ERR_ARGS, "element number out of range");
    return;
  }
  const char* el = kElements[idx];
  const char* xc = *xcnumber == 1 ? "pbe" : (*xcnumber == 2 ? "lda" : "");
  std::string path = std::string(el) + "." + xc + ".in";
  if (init_file(path.c_str(), el, *rcut, *rcut_magnetic, *smear, *xcnumber) == MAGACE_OK) R.ini_done = true;
}

int ace_set_precision(int mode) {
  if (mode != 0 && mode != 1) return set_error(MAGACE_ERR_ARGS, "precision mode must be 0 or 1");
  rt().precision = mode;
  return MAGACE_OK;
}

int ace_get_precision(void) { return rt().precision; }

int ace_basis_sizes(int* out) {
  Runtime& R = rt();
  if (!R.ready) return set_error(MAGACE_ERR_NOT_INIT, "no potential initialised");
  for (int r = 1; r <= 4; ++r) out[r - 1] = static_cast<int>(R.model.rows[r].size());
  out[4] = static_cast<int>(R.model.nterms[2]);
  out[5] = static_cast<int>(R.model.nterms[3]);
  out[6] = static_cast<int>(R.model.nterms[4]);
  out[7] = R.model.unmatched_records;
  return MAGACE_OK;
}

int ace_basis_rows(int rank, int* out) {
  Runtime& R = rt();
  if (!R.ready) return set_error(MAGACE_ERR_NOT_INIT, "no potential initialised");
  if (rank < 1 || rank > 6) return set_error(MAGACE_ERR_ARGS, "rank must be 1..6");
  size_t k = 0;
  for (const auto& row : R.model.rows[rank])
    for (int v : row) out[k++] = v;
  return MAGACE_OK;
}

int ace_basis_count(int rank, int* count) {
  Runtime& R = rt();
  if (!R.ready) return set_error(MAGACE_ERR_NOT_INIT, "no potential initialised");
  if (rank < 1 || rank > 6 || !count) return set_error(MAGACE_ERR_ARGS, "rank must be 1..6");
  *count = static_cast<int>(R.model.rows[rank].size());
  return set_error(MAGACE_OK, "");
}

int ace_last_launch_count(void) { return rt().last_kernels; }

int ace_host_access_mode(void) {
  int st = upload_tables();
  if (st) return -1;
  return host_access_mode();
}

int ace_set_kernel_timing(int on) {
  rt().timing = on != 0;
  return MAGACE_OK;
}

int ace_kernel_times(float* ms) {
  Runtime& R = rt();
  if (!R.ev_recorded) return set_error(MAGACE_ERR_ARGS, "no timed evaluation recorded");
  const int n = R.last_launches;
  CUDA_TRY(cudaEventSynchronize(R.ev[n]));
  for (int k = 0; k < kMaxLaunches; ++k) {
    ms[k] = 0.0f;
    if (k < n) CUDA_TRY(cudaEventElapsedTime(&ms[k], R.ev[k], R.ev[k + 1]));
  }
  return MAGACE_OK;
}

int ace_table_stats(long long* out) {
  Runtime& R = rt();
  if (!R.ready) return set_error(MAGACE_ERR_NOT_INIT, "no potential initialised");
  const GatherTable& g = R.model.gt;
  const FactorLayout& L = R.model.L;
  out[0] = g.entries[1];
  out[1] = g.entries[2];
  out[2] = g.entries[3];
  out[3] = g.nseg;
  out[4] = g.nslot;
  out[5] = L.nF;
  out[6] = L.nW;
  out[7] = L.nWA;
  out[8] = static_cast<long long>(L.nba) * L.n2m * L.h2;  // A2 half slots
  out[9] = R.model.lut.nfa;
  out[10] = R.model.lut.nfm;
  const int dims[10] = {L.nba, L.nbm, L.n2m, L.l2m, L.n3a, L.n3m, L.l3a, L.l3m, L.h2, L.h3};
  for (int k = 0; k < 10; ++k) out[11 + k] = dims[k];
  out[21] = R.model.db3.ntask;
  out[22] = R.model.db3.ncombo;
  out[23] = R.model.db3.nc;
  out[24] = R.model.gt_nob3.nseg;
  out[25] = R.model.gt_nob3.entries[1] + R.model.gt_nob3.entries[2] + R.model.gt_nob3.entries[3];
  for (int a = 1; a <= 3; ++a) out[25 + a] = R.model.gt_nob3.entries[a];
  // (i, j) coefficient pairs the dense 3-body contraction visits per atom
  const DenseB3& D = R.model.db3;
  long long pairs = 0;
  for (int t = 0; t < D.ntask; ++t) {
    const int pat = D.pattern[D.task_combo[t]];
    for (int i = 0; i < D.I; ++i)
      pairs += D.NM * (pat == 0 ? i + 1 : (pat == 1 ? (i / D.NM + 1) * D.NM : (i / D.NM) * D.NM));
  }
  out[29] = pairs;
  out[30] = R.model.rest.nfac;
  return MAGACE_OK;
}

int ace_compute_device(int natom, int nei, const int* bond_offset, const double* r, const double* e,
                       const double* mag_j, const double* mhat_j, const double* mag_i, const double* mhat_i,
                       double* energy, double* fij, double* tij, double* ti0, void* stream) {
  Runtime& R = rt();
  if (int st0 = check_sizes(natom, nei)) return st0;
  int st = upload_tables();
  if (st) return st;
  st = reserve_work(natom, nei, R.precision);
  if (st) return st;
  EvalBuffers b;
  b.natom = natom;
  b.nei = nei;
  b.off = bond_offset;
  b.r = r;
  b.e = e;
  b.magj = mag_j;
  b.mhj = mhat_j;
  b.magi = mag_i;
  b.mhi = mhat_i;
  b.energy = energy;
  b.fij = fij;
  b.tij = tij;
  b.ti0 = ti0;
  b.dev_inputs = device_resident({r, e, mag_j, mhat_j});
  return run_eval(b, stream ? static_cast<cudaStream_t>(stream) : R.stream);
}

int ace_set_work_queue(int on) {
  rt().work_queue = on != 0;
  return set_error(MAGACE_OK, "");
}

int ace_autotune_device(int natom, int nei, const int* bond_offset, const double* r, const double* e,
                        const double* mag_j, const double* mhat_j, const double* mag_i, const double* mhat_i,
                        void* stream, int* rest_warps, int* b3_warps, int* force_blocks) {
  Runtime& R = rt();
  if (int st0 = check_sizes(natom, nei)) return st0;
  int st = upload_tables();
  if (st) return st;
  st = reserve_work(natom, nei, R.precision);
  if (st) return st;
  CUDA_TRY(R.energy.reserve(natom));
  CUDA_TRY(R.ti0.reserve(3 * static_cast<size_t>(natom)));
  CUDA_TRY(R.fij.reserve(3 * static_cast<size_t>(nei)));
  CUDA_TRY(R.tij.reserve(3 * static_cast<size_t>(nei)));
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : R.stream;
  EvalBuffers b;
  b.natom = natom;
  b.nei = nei;
  b.off = bond_offset;
  b.r = r;
  b.e = e;
  b.magj = mag_j;
  b.mhj = mhat_j;
  b.magi = mag_i;
  b.mhi = mhat_i;
  b.energy = R.energy.p;
  b.fij = R.fij.p;
  b.tij = R.tij.p;
  b.ti0 = R.ti0.p;
  b.dev_inputs = device_resident({r, e, mag_j, mhat_j});
  // variant v of every kernel at once (each kernel's own choice list,
  // clamped), warmed up, then timed kernel by kernel; each kernel keeps its
  // fastest variant
  const bool timing = R.timing;
  R.timing = true;
  for (auto& ev : R.ev)
    if (!ev) CUDA_TRY(cudaEventCreate(&ev));
  const int nr = static_cast<int>(sizeof(kRestWarpChoices) / sizeof(int));
  const int nbw = static_cast<int>(sizeof(kB3WarpChoices) / sizeof(int));
  const int nfv = static_cast<int>(sizeof(kForceMinBlocksChoices) / sizeof(int));
  float best[4] = {1e30f, 1e30f, 1e30f, 1e30f};  // A basis, density, b3, forces
  int pick[4] = {R.tune_abasis, R.tune_rest, R.tune_b3, R.tune_forces};
  for (int v = 0; v < std::max(nr, std::max(nbw, nfv)); ++v) {
    R.dm.tune_abasis = std::min(v, kAbasisVariants - 1);
    R.dm.tune_rest = std::min(v, nr - 1);
    R.dm.tune_b3 = std::min(v, nbw - 1);
    R.dm.tune_forces = std::min(v, nfv - 1);
    st = run_eval(b, s);
    if (st) break;
    st = run_eval(b, s);
    if (st) break;
    if (R.last_launches != 4) break;  // not the split-precision specialised path: nothing to tune
    float ms[kMaxLaunches];
    CUDA_TRY(cudaEventSynchronize(R.ev[R.last_launches]));
    for (int k = 0; k < R.last_launches; ++k) CUDA_TRY(cudaEventElapsedTime(&ms[k], R.ev[k], R.ev[k + 1]));
    const int idx[4] = {R.dm.tune_abasis, R.dm.tune_rest, R.dm.tune_b3, R.dm.tune_forces};
    for (int q = 0; q < 4; ++q)
      if (ms[q] < best[q]) {
        best[q] = ms[q];
        pick[q] = idx[q];
      }
  }
  R.timing = timing;
  R.tune_abasis = R.dm.tune_abasis = pick[0];
  R.tune_rest = R.dm.tune_rest = pick[1];
  R.tune_b3 = R.dm.tune_b3 = pick[2];
  R.tune_forces = R.dm.tune_forces = pick[3];
  const int best_r = pick[1], best_b = pick[2];
  if (st) return st;
  if (rest_warps) *rest_warps = kRestWarpChoices[best_r];
  if (b3_warps) *b3_warps = kB3WarpChoices[best_b];
  if (force_blocks) *force_blocks = kForceMinBlocksChoices[pick[3]];
  return ace_device_status();
}

int ace_get_tuning(int* variants) {
  Runtime& R = rt();
  variants[0] = R.tune_abasis;
  variants[1] = R.tune_rest;
  variants[2] = R.tune_b3;
  variants[3] = R.tune_forces;
  return set_error(MAGACE_OK, "");
}

int ace_set_tuning(const int* variants) {
  Runtime& R = rt();
  const int count[4] = {kAbasisVariants, static_cast<int>(sizeof(kRestWarpChoices) / sizeof(int)),
                        static_cast<int>(sizeof(kB3WarpChoices) / sizeof(int)),
                        static_cast<int>(sizeof(kForceMinBlocksChoices) / sizeof(int))};
  if (!variants) return set_error(MAGACE_ERR_ARGS, "null variants");
  for (int k = 0; k < 4; ++k)
    if (variants[k] < 0 || variants[k] >= count[k]) return set_error(MAGACE_ERR_ARGS, "kernel variant out of range");
  R.tune_abasis = R.dm.tune_abasis = variants[0];
  R.tune_rest = R.dm.tune_rest = variants[1];
  R.tune_b3 = R.dm.tune_b3 = variants[2];
  R.tune_forces = R.dm.tune_forces = variants[3];
  return set_error(MAGACE_OK, "");
}

int ace_num_coefficients(int* ncoef, int* ndensity) {
  Runtime& R = rt();
  if (!R.ready) return set_error(MAGACE_ERR_NOT_INIT, "no potential initialised");
  *ncoef = num_coefficients(R.model);
  *ndensity = R.model.ndensity;
  return set_error(MAGACE_OK, "");
}

int ace_get_coefficients(double* c) {
  Runtime& R = rt();
  if (!R.ready) return set_error(MAGACE_ERR_NOT_INIT, "no potential initialised");
  get_coefficients(R.model, c);
  return set_error(MAGACE_OK, "");
}

int ace_set_coefficients(const double* c) {
  Runtime& R = rt();
  if (!R.ready) return set_error(MAGACE_ERR_NOT_INIT, "no potential initialised");
  std::string msg;
  const int st = set_coefficients(R.model, c, msg);
  if (st) return set_error(st, msg);
  R.dev_tables = false;  // the next device call uploads the new tables
  return set_error(MAGACE_OK, "");
}

int ace_descriptors_device(int natom, int nei, const int* bond_offset, const double* r, const double* e,
                           const double* mag_j, const double* mhat_j, const double* mag_i, const double* mhat_i,
                           double* B, void* stream) {
  Runtime& R = rt();
  if (int st0 = check_sizes(natom, nei)) return st0;
  int st = upload_tables();
  if (st) return st;
  st = reserve_work(natom, nei, 0);
  if (st) return st;
  EvalBuffers b;
  b.natom = natom;
  b.nei = nei;
  b.off = bond_offset;
  b.r = r;
  b.e = e;
  b.magj = mag_j;
  b.mhj = mhat_j;
  b.magi = mag_i;
  b.mhi = mhat_i;
  b.F = R.F.p;
  b.rho1 = R.rho1.p;
  b.core = R.core.p;
  b.err = R.err.p;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : R.stream;
  CUDA_TRY(cudaMemsetAsync(R.err.p, 0, sizeof(int), s));
  R.last_launches = R.last_kernels = launch_descriptors(R.dm, b, B, s, R.grid_cap);
  R.ev_recorded = false;
  CUDA_TRY(cudaGetLastError());
  return set_error(MAGACE_OK, "");
}

int ace_descriptors_tangent_device(int natom, int nei, const int* bond_offset, const double* r, const double* e,
                                   const double* mag_j, const double* mhat_j, const double* mag_i,
                                   const double* mhat_i, const double* dd, const double* dm_j, const double* dm_i,
                                   double* B, double* Bdot, double* core, double* core_dot, void* stream) {
  Runtime& R = rt();
  if (int st0 = check_sizes(natom, nei)) return st0;
  if (natom > 0 && (!B || !Bdot || !core || !core_dot || !dm_i || (nei > 0 && (!dd || !dm_j))))
    return set_error(MAGACE_ERR_ARGS, "null tangent or output array");
  int st = upload_tables();
  if (st) return st;
  st = reserve_work(natom, nei, 0);
  if (st) return st;
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  int smem_max = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (descriptors_tangent_smem(R.dm) > static_cast<size_t>(smem_max))
    return set_error(MAGACE_ERR_UNSUPPORTED, "basis too large for the tangent kernel's shared-memory tiles");
  CUDA_TRY(R.Fd.reserve(static_cast<size_t>(natom) * R.dm.nF * 16));
  EvalBuffers b;
  b.natom = natom;
  b.nei = nei;
  b.off = bond_offset;
  b.r = r;
  b.e = e;
  b.magj = mag_j;
  b.mhj = mhat_j;
  b.magi = mag_i;
  b.mhi = mhat_i;
  b.F = R.F.p;
  b.err = R.err.p;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : R.stream;
  CUDA_TRY(cudaMemsetAsync(R.err.p, 0, sizeof(int), s));
  R.last_launches = R.last_kernels =
      launch_descriptors_tangent(R.dm, b, dd, dm_j, dm_i, R.Fd.p, B, Bdot, core, core_dot, s, R.grid_cap);
  R.ev_recorded = false;
  CUDA_TRY(cudaGetLastError());
  return set_error(MAGACE_OK, "");
}

int ace_embedding(int* nfemb, double* par, double* inner_cutoff) {
  Runtime& R = rt();
  if (!R.ready) return set_error(MAGACE_ERR_NOT_INIT, "no potential initialised");
  if (nfemb) *nfemb = R.model.nfemb;
  if (par)
    for (int a = 0; a < 2; ++a)
      for (int d = 0; d < 2; ++d) par[2 * a + d] = R.model.par[a][d];
  if (inner_cutoff) {
    inner_cutoff[0] = R.model.ecut;
    inner_cutoff[1] = R.model.decut;
  }
  return set_error(MAGACE_OK, "");
}

int ace_density_gradient_device(int natom, double* dedrho, void* stream) {
  Runtime& R = rt();
  if (natom < 0 || natom > R.last_natom)
    return set_error(MAGACE_ERR_ARGS, "natom exceeds the atoms of the last evaluation");
  if (natom == 0) return set_error(MAGACE_OK, "");
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : R.stream;
  CUDA_TRY(cudaMemcpyAsync(dedrho, R.dedrho.p, sizeof(double) * 2 * static_cast<size_t>(natom),
                           cudaMemcpyDeviceToDevice, s));
  return set_error(MAGACE_OK, "");
}

int ace_device_status(void) {
  Runtime& R = rt();
  if (!R.err.p) return MAGACE_OK;
  int dev = 0;
  CUDA_TRY(cudaDeviceSynchronize());
  CUDA_TRY(cudaMemcpy(&dev, R.err.p, sizeof(int), cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemset(R.err.p, 0, sizeof(int)));
  return device_error_to_status(dev);
}

void ace_release_device(void) {
  Runtime& R = rt();
  for (auto* b : {&R.lut_a, &R.lut_m, &R.c1, &R.r, &R.e, &R.magj, &R.mhj, &R.magi, &R.mhi, &R.energy, &R.fij,
                  &R.tij, &R.ti0, &R.rho1, &R.core, &R.edf, &R.dedrho})
    b->release();
  for (auto* b : {&R.lut_a32, &R.lut_m32, &R.b3_Cf, &R.b3_cff, &R.b3_mult, &R.c1f, &R.b3_Chl, &R.r_kaphl}) b->release();
  for (auto* b : {&R.b3_pattern, &R.b3_combo, &R.b3_factor, &R.b3_cw}) b->release();
  R.b3_code.release();
  R.b3_code2.release();
  R.b3_cfw.release();
  for (auto* b : {&R.b3_C64, &R.b3_cf64, &R.b3_cfw64, &R.r_kap64}) b->release();
  for (auto* b : {&R.d_rank1_n, &R.d_begin, &R.r_factor, &R.r_run, &R.r_g0, &R.r_warp_begin, &R.r_warp_slots})
    b->release();
  R.r_rec.release();
  R.r_stream.release();
  R.r_stream_begin.release();
  R.r_split_w.release();
  R.r64_warp_begin.release();
  R.r64_warp_slots.release();
  R.d_cf.release();
  R.d_o.release();
  R.gb1.release();
  R.gb2.release();
  R.off.release();
  R.err.release();
  R.F.release();
  R.Fd.release();
  R.aux.release();
  R.bstage.release();
  R.order.release();
  R.queue_bins.release();
  R.W.release();
  if (R.stream) cudaStreamDestroy(R.stream);
  R.stream = nullptr;
  if (R.side) cudaStreamDestroy(R.side);
  if (R.ev_fork) cudaEventDestroy(R.ev_fork);
  if (R.ev_join) cudaEventDestroy(R.ev_join);
  R.side = nullptr;
  R.ev_fork = R.ev_join = nullptr;
  if (R.pinned) cudaFreeHost(R.pinned);
  R.pinned = nullptr;
  R.pinned_bytes = 0;
  R.dev_tables = false;
}

void acelib_(int* natom_p, int* nall, int* nei_p, int* nlist, int* occ, int* occlist, int* nstart, int* nstop,
             double* eout, double* dlist, double* elist, double* flist, double* dlist_momi, double* elist_momi,
             double* dlist_mom, double* elist_mom, double* tlist, double* tlist0) {
  (void)nall;
  (void)nlist;
  Runtime& R = rt();
  const int natom = natom_p ? *natom_p : -1, nei = nei_p ? *nei_p : -1;
  // total packed bonds and contiguity of the caller's ranges
  auto fail = [&](int code, const char* msg, long npacked) {
    set_error(code, msg);
    const double nan = std::numeric_limits<double>::quiet_NaN();
    if (natom > 0) {
      std::fill(eout, eout + natom, nan);
      std::fill(tlist0, tlist0 + 3L * natom, nan);
    }
    if (npacked > 0) {
      std::fill(flist, flist + 3 * npacked, nan);
      std::fill(tlist, tlist + 3 * npacked, nan);
    }
  };
  if (check_sizes(natom, nei)) return;
  if (!R.ready) return fail(MAGACE_ERR_NOT_INIT, "acelib_ called before a successful acelibini_", 0);
  std::vector<int>& off = R.h_off;
  off.assign(natom + 1, 0);
  bool contiguous = true;
  for (int i = 0; i < natom; ++i) {
    const int cnt = nstop[i] >= nstart[i] ? nstop[i] - nstart[i] + 1 : 0;
    if (cnt > 0 && (nstart[i] < 1 || nstop[i] > nei)) return fail(MAGACE_ERR_ARGS, "bond range outside 1..nei", 0);
    if (occ && occ[i] != 1) return fail(MAGACE_ERR_ARGS, "element index other than 1 (single element)", 0);
    if (cnt > 0 && nstart[i] != off[i] + 1) contiguous = false;
    if (cnt > kMaxCallSize - off[i]) return fail(MAGACE_ERR_ARGS, "the bond ranges hold more than 715,827,882 bonds", 0);
    off[i + 1] = off[i] + cnt;
  }
  const long npacked = off[natom];
  // the neighbour elements must all be 1; the scan runs on the host while
  // the GPU evaluates, and a failure is reported once the stream is idle
  const auto occlist_bad = [&]() {
    unsigned bad = 0;  // a branch-free scan the compiler vectorises
    if (occlist)
      for (int j = 0; j < nei; ++j) bad |= static_cast<unsigned>(occlist[j] ^ 1);
    return bad != 0;
  };
  const char* occ_msg = "neighbour element index other than 1";
  int st = upload_tables();
  if (st) return fail(st, R.last_msg.c_str(), npacked);
  st = reserve_work(natom, static_cast<int>(npacked), R.precision);
  if (st) return fail(st, R.last_msg.c_str(), npacked);
  const size_t na = natom, nb = npacked;
  cudaStream_t s = R.stream;
  // inputs; non-contiguous ranges are gathered into atom order first
  std::vector<double> gr, ge, gm, gmh;
  const double *pr = dlist, *pe = elist, *pm = dlist_mom, *pmh = elist_mom;
  if (!contiguous) {
    gr.resize(nb);
    ge.resize(3 * nb);
    gm.resize(nb);
    gmh.resize(3 * nb);
    for (int i = 0; i < natom; ++i)
      for (int k = 0; k < off[i + 1] - off[i]; ++k) {
        const size_t src = nstart[i] - 1 + k, dst = off[i] + k;
        gr[dst] = dlist[src];
        gm[dst] = dlist_mom[src];
        for (int c = 0; c < 3; ++c) {
          ge[3 * dst + c] = elist[3 * src + c];
          gmh[3 * dst + c] = elist_mom[3 * src + c];
        }
      }
    pr = gr.data();
    pe = ge.data();
    pm = gm.data();
    pmh = gmh.data();
  }
  const int mode = host_access_mode();
  cudaError_t ce = cudaSuccess;
  EvalBuffers b;
  b.natom = natom;
  b.nei = static_cast<int>(npacked);
  if (mode == kHostDirect) {
    // the kernels read the caller's arrays and write its outputs in place
    b.off = off.data();
    b.r = pr;
    b.e = pe;
    b.magj = pm;
    b.mhj = pmh;
    b.magi = dlist_momi;
    b.mhi = elist_momi;
    b.energy = eout;
    b.fij = flist;
    b.tij = tlist;
    b.ti0 = tlist0;
    b.host_outputs = true;
    if (run_eval(b, s)) return fail(R.last_error, R.last_msg.c_str(), npacked);
    if (occlist_bad()) {
      cudaStreamSynchronize(s);
      return fail(MAGACE_ERR_ARGS, occ_msg, npacked);
    }
  } else {
    auto res = [&](DevBuf<double>& bb, size_t n) { return bb.reserve(n) == cudaSuccess; };
    if (!(res(R.r, nb) && res(R.e, 3 * nb) && res(R.magj, nb) && res(R.mhj, 3 * nb) && res(R.magi, na) &&
          res(R.mhi, 3 * na) && res(R.fij, 3 * nb) && res(R.tij, 3 * nb) && res(R.ti0, 3 * na)) ||
        R.off.reserve(na + 1) != cudaSuccess)
      return fail(MAGACE_ERR_CUDA, "device allocation failed", npacked);
    // host side of every transfer: the caller's memory, or a pinned copy of it
    struct Xfer {
      void* dev;
      const void* host;
      size_t bytes;
    };
    const Xfer in[] = {{R.off.p, off.data(), (na + 1) * sizeof(int)},
                       {R.r.p, pr, nb * sizeof(double)},
                       {R.e.p, pe, 3 * nb * sizeof(double)},
                       {R.magj.p, pm, nb * sizeof(double)},
                       {R.mhj.p, pmh, 3 * nb * sizeof(double)},
                       {R.magi.p, dlist_momi, na * sizeof(double)},
                       {R.mhi.p, elist_momi, 3 * na * sizeof(double)}};
    const Xfer out[] = {{R.energy.p, eout, na * sizeof(double)},
                        {R.fij.p, flist, 3 * nb * sizeof(double)},
                        {R.tij.p, tlist, 3 * nb * sizeof(double)},
                        {R.ti0.p, tlist0, 3 * na * sizeof(double)}};
    size_t in_bytes = 0, out_bytes = 0;
    for (const auto& x : in) in_bytes += (x.bytes + 255) & ~static_cast<size_t>(255);
    for (const auto& x : out) out_bytes += (x.bytes + 255) & ~static_cast<size_t>(255);
    bool pinned = mode == kHostPinned && reserve_pinned(std::max(in_bytes, out_bytes)) == MAGACE_OK;
    size_t o = 0;
    for (const auto& x : in) {
      const void* src = x.host;
      if (pinned && x.bytes) {
        std::memcpy(R.pinned + o, x.host, x.bytes);
        src = R.pinned + o;
        o += (x.bytes + 255) & ~static_cast<size_t>(255);
      }
      if (ce == cudaSuccess && x.bytes) ce = cudaMemcpyAsync(x.dev, src, x.bytes, cudaMemcpyHostToDevice, s);
    }
    if (ce != cudaSuccess) return fail(MAGACE_ERR_CUDA, cudaGetErrorString(ce), npacked);
    b.off = R.off.p;
    b.r = R.r.p;
    b.e = R.e.p;
    b.magj = R.magj.p;
    b.mhj = R.mhj.p;
    b.dev_inputs = true;  // the library's own device buffers
    b.magi = R.magi.p;
    b.mhi = R.mhi.p;
    b.energy = R.energy.p;
    b.fij = R.fij.p;
    b.tij = R.tij.p;
    b.ti0 = R.ti0.p;
    if (run_eval(b, s)) return fail(R.last_error, R.last_msg.c_str(), npacked);
    o = 0;
    for (const auto& x : out) {
      void* dst = const_cast<void*>(x.host);
      if (pinned && x.bytes) {
        dst = R.pinned + o;
        o += (x.bytes + 255) & ~static_cast<size_t>(255);
      }
      if (ce == cudaSuccess && x.bytes) ce = cudaMemcpyAsync(dst, x.dev, x.bytes, cudaMemcpyDeviceToHost, s);
    }
    const bool bad_elements = occlist_bad();
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (bad_elements) return fail(MAGACE_ERR_ARGS, occ_msg, npacked);
    if (ce != cudaSuccess) return fail(MAGACE_ERR_CUDA, cudaGetErrorString(ce), npacked);
    if (pinned) {
      o = 0;
      for (const auto& x : out)
        if (x.bytes) {
          std::memcpy(const_cast<void*>(x.host), R.pinned + o, x.bytes);
          o += (x.bytes + 255) & ~static_cast<size_t>(255);
        }
    }
  }
  int dev_err = 0;
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(&dev_err, R.err.p, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return fail(MAGACE_ERR_CUDA, cudaGetErrorString(ce), npacked);
  if (dev_err) {
    const int code = device_error_to_status(dev_err);
    return fail(code, R.last_msg.c_str(), npacked);
  }
  set_error(MAGACE_OK, "");
}

}  // extern "C"
