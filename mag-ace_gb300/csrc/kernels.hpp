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
};

void upload_ylm_constants(const double* alm, const double* blm, const double* cl, const double* dl);
size_t eval_smem_bytes(const DeviceModel& m, int precision, int which);
// Launches k_abasis, k_density and k_forces on `st`; returns the number of
// kernels launched. With `ev` (4 events) the kernel boundaries are recorded.
int launch_eval_fp64(const DeviceModel& m, const EvalBuffers& b, cudaStream_t st, int grid_cap, cudaEvent_t* ev);
int launch_eval_fp32(const DeviceModel& m, const EvalBuffers& b, cudaStream_t st, int grid_cap, cudaEvent_t* ev);

}  // namespace magace
