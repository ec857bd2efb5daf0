// Launch interface of the hot-path kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

#include "device_model.hpp"

namespace magace {

constexpr int kAbasisThreads = 128;
constexpr int kAbasisTile = 64;  // bonds per feature tile
constexpr int kDensityThreads = 256;
constexpr int kForceThreads = 64;
constexpr int kMaxFeat = 32;     // per-bond radial functions of one kind
constexpr int kMaxLaunches = 4;  // kernels of one evaluation
// variants of the split-precision A-basis kernel: scalar, packed FP32x2,
// scalar with TMA-staged bond tiles, the same on a persistent grid, the bond
// sums on the tensor cores with TMA-staged tiles on a persistent grid, the
// tensor-core sums alone (DeviceModel::tune_abasis)
constexpr int kAbasisVariants = 6;
// warps per CTA of the split-precision density kernels, chosen by
// DeviceModel::tune_rest / tune_b3 (ace_autotune_device picks them)
// (2/3: record streams broadcast by shuffles, 4/5: through shared memory)
constexpr int kRestWarpChoices[6] = {32, 16, 32, 16, 32, 16};
// (b3 variants 3: n0' loop outermost; 4 and 5: packed FP32x2 arithmetic)
constexpr int kB3WarpChoices[6] = {16, 12, 8, 12, 16, 12};
// CTAs per SM the split-precision force kernel's registers must allow, for
// its scalar (variants 0-2) and packed FP32x2 (3-5) forms, and for the form
// with its contractions on the tensor cores (6-7) (DeviceModel::tune_forces)
constexpr int kForceMinBlocksChoices[8] = {4, 6, 8, 4, 6, 8, 5, 6};
// the variants used until ace_autotune_device or ace_set_tuning picks
// others: the fastest on a 15,840-atom bcc Fe workload (A-basis bond sums on
// the tensor cores, with bulk-copied bond tiles on a persistent grid where
// the inputs are in device memory; record streams through shared memory;
// packed FP32x2 3-body sums; force contractions on the tensor cores)
constexpr int kDefaultTuning[4] = {4, 4, 4, 6};

// Device arrays of one evaluation. F and W are complex arrays of the selected
// precision (FP64: 16 bytes per entry, FP32: 8 bytes).
struct EvalBuffers {
  int natom = 0, nei = 0;
  const int* off = nullptr;  // [natom+1] bond offsets
  const double* r = nullptr;
  const double* e = nullptr;
  const double* magj = nullptr;
  const double* mhj = nullptr;
  const double* magi = nullptr;
  const double* mhi = nullptr;
  void* F = nullptr;          // [natom][nF]
  void* W = nullptr;          // [natom][nW]
  double* rho1 = nullptr;     // [natom][2]
  double* core = nullptr;     // [natom]
  double* edf = nullptr;      // [natom]
  double* dedrho = nullptr;   // [natom][2]
  double* energy = nullptr;   // [natom]
  double* fij = nullptr;      // [3*nei]
  double* tij = nullptr;      // [3*nei]
  double* ti0 = nullptr;      // [3*natom]
  int* err = nullptr;         // device error word
  void* aux = nullptr;        // [eval_aux_bytes] scratch of the specialised split-precision kernels
  const int* order = nullptr; // [natom] work queue (atoms by decreasing bond count) or null
  void* stage = nullptr;      // [nei][8] bond inputs in the working precision (specialised kernels), or null
  bool dev_inputs = false;    // r, e, magj, mhj are device memory (bulk copies may read them)
  bool host_outputs = false;  // fij, tij are host memory (written as whole lines)
  // a second stream for the 2-/4-body density kernel beside the 3-body one,
  // with the events that fork it from and join it back into the launch
  // stream; null: everything runs on the launch stream
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

// Work queue of one evaluation: the atoms sorted by decreasing bond count
// (counting sort over counts clipped to kQueueBins - 1), into order[natom];
// scratch bins[2 * kQueueBins] ints. Three small kernels on `st`.
constexpr int kQueueBins = 256;
void launch_work_queue(int natom, const int* off, int* order, int* bins, cudaStream_t st);

void upload_ylm_constants(const double* alm, const double* blm, const double* cl, const double* dl);
size_t eval_smem_bytes(const DeviceModel& m, int precision, int which);
// Size of EvalBuffers::aux for natom atoms (0 when the kernels need none).
size_t eval_aux_bytes(const DeviceModel& m, int precision, int natom);
// An upper bound of eval_aux_bytes that never decreases as natom grows.
size_t eval_aux_bytes_bound(const DeviceModel& m, int precision, int natom);
// Launches the A-basis, density and force phases on `st` and returns the
// number n of timed slots: 3 (A basis, density, forces) or, when the
// split-precision density runs its 3-body part in kernels of its own, 4 (the
// third slot is the 3-body kernel and k_finish_fe). With `ev` (kMaxLaunches +
// 1 events) ev[k] is recorded before slot k and ev[n] after the last one;
// callers that time pass no side stream, so that the slots do not overlap.
// `kernels` receives the number of kernels launched.
// Descriptors: the FP64 A-basis phase into b.F, then B[natom][nB] (see
// model.hpp DescriptorTable); returns the number of kernels launched.
int launch_descriptors(const DeviceModel& m, const EvalBuffers& b, double* B, cudaStream_t st, int grid_cap);
// Descriptors B and their directional derivatives Bd along the tangents dd
// [nei][3] (of the bond vectors x_i - x_j), dmj [nei][3] (of the neighbours'
// moments) and dmi [natom][3] (of the atoms' moments), FP64: factors into b.F
// and their tangents into Fd ([natom][nF] complex), then B and Bd
// [natom][nB]; core and cored [natom] receive the core energy and its
// derivative. Returns the number of kernels launched.
int launch_descriptors_tangent(const DeviceModel& m, const EvalBuffers& b, const double* dd, const double* dmj,
                               const double* dmi, void* Fd, double* B, double* Bd, double* core, double* cored,
                               cudaStream_t st, int grid_cap);
size_t descriptors_tangent_smem(const DeviceModel& m);
int launch_eval_fp64(const DeviceModel& m, const EvalBuffers& b, cudaStream_t st, int grid_cap, cudaEvent_t* ev,
                     int* kernels = nullptr);
int launch_eval_fp32(const DeviceModel& m, const EvalBuffers& b, cudaStream_t st, int grid_cap, cudaEvent_t* ev,
                     int* kernels = nullptr);

}  // namespace magace
