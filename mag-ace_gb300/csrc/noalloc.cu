// Allocation-free evaluation entry point.
//
// Some callers cannot allocate device memory at the point where they
// evaluate the potential: code running inside a memory pool or allocator
// they do not own, real-time MD drivers that forbid allocation after set-up,
// or hosts whose device allocator is disabled in the evaluation phase. For
// them, ace_compute_device_noalloc runs the same kernels as
// ace_compute_device, but its per-atom scratch (the factor array F, the
// weight array W, the per-atom density, core energy and embedding
// derivatives, and the 3-body scratch of the split-precision kernels) lives in one fixed file-scope device array instead of
// library-allocated buffers. The caller still passes the inputs and outputs.
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdio>

#include "device_model.hpp"
#include "kernels.hpp"
#include "magace.h"

namespace magace {

int runtime_snapshot(DeviceModel* dm, int* precision, int* grid_cap);
int runtime_check_sizes(int natom, int nei);
bool runtime_device_resident(const void* r, const void* e, const void* mag_j, const void* mhat_j);
int runtime_error(int code, const char* msg);
int runtime_device_error(int dev_err);
void runtime_set_launches(int slots, int kernels);

namespace {

// Capacity of the shared scratch: 64 MiB on every device that loads the
// library, held until the process exits.
constexpr size_t kScratchBytes = static_cast<size_t>(64) << 20;

// The scratch itself. In host code this name is only a stand-in for the
// device symbol; its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {nullptr};  // device address per device

size_t round256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

// Byte offsets of one call's arrays in the scratch. Every size is an upper
// bound that never falls as natom grows, so the atoms that fit form one
// range 0..max_atoms().
struct ScratchLayout {
  size_t err, F, W, rho1, core, edf, dedrho, aux, aux_bytes, end;
};
ScratchLayout scratch_layout(const DeviceModel& dm, int precision, int natom) {
  const size_t csz = precision == 0 ? 16 : 8;  // complex FP64 / FP32
  const size_t na = static_cast<size_t>(natom);
  ScratchLayout L;
  size_t off = 0;
  L.err = off;
  off += 256;
  L.F = off;
  off += round256(na * dm.nF * csz);
  L.W = off;
  off += round256(na * dm.nW * csz);
  L.rho1 = off;
  off += round256(na * 2 * sizeof(double));
  L.core = off;
  off += round256(na * sizeof(double));
  L.edf = off;
  off += round256(na * sizeof(double));
  L.dedrho = off;
  off += round256(na * 2 * sizeof(double));
  L.aux = off;
  L.aux_bytes = eval_aux_bytes_bound(dm, precision, natom);
  off += round256(L.aux_bytes);
  L.end = off;
  return L;
}

// The largest natom whose layout fits the scratch.
int max_atoms(const DeviceModel& dm, int precision) {
  int lo = 0, hi = 1;
  while (scratch_layout(dm, precision, hi).end <= kScratchBytes) hi *= 2;
  while (hi - lo > 1) {
    const int mid = lo + (hi - lo) / 2;
    (scratch_layout(dm, precision, mid).end <= kScratchBytes ? lo : hi) = mid;
  }
  return lo;
}

}  // namespace
}  // namespace magace

using namespace magace;

extern "C" int ace_compute_device_noalloc(int natom, int nei, const int* bond_offset, const double* r,
                                          const double* e, const double* mag_j, const double* mhat_j,
                                          const double* mag_i, const double* mhat_i, double* energy,
                                          double* fij, double* tij, double* ti0, void* stream) {
  // the same per-call limits as ace_compute_device (32-bit bond indexing)
  if (int st0 = runtime_check_sizes(natom, nei)) return st0;
  DeviceModel dm;
  int precision = 0, grid_cap = 1;
  int st = runtime_snapshot(&dm, &precision, &grid_cap);
  if (st) return st;
  int dev = -1;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return runtime_error(MAGACE_ERR_CUDA, cudaGetErrorString(ce));
  if (dev < 0 || dev >= kMaxDevices) return runtime_error(MAGACE_ERR_CUDA, "device index beyond 64");
  // the call reads its status back and synchronizes, so it cannot be part of
  // a captured graph: refuse before any device work, which leaves the
  // caller's capture intact
  if (stream) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cs) == cudaSuccess &&
        cs != cudaStreamCaptureStatusNone)
      return runtime_error(MAGACE_ERR_ARGS,
                           "ace_compute_device_noalloc is synchronous and cannot run in a stream capture");
  }
  // one-time set-up per device, with that device current: the device
  // address of the scratch array
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (ce != cudaSuccess || !p) return runtime_error(MAGACE_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed");
    g_scratch_addr[dev] = p;
  }
  unsigned char* base = static_cast<unsigned char*>(g_scratch_addr[dev]);
  const ScratchLayout L = scratch_layout(dm, precision, natom);
  if (L.end > kScratchBytes) {
    static char msg[200];
    snprintf(msg, sizeof(msg),
             "natom = %d exceeds the allocation-free scratch: at most %d atoms fit in its 64 MiB for this "
             "potential and precision",
             natom, max_atoms(dm, precision));
    return runtime_error(MAGACE_ERR_ARGS, msg);
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int* err = reinterpret_cast<int*>(base + L.err);
  // every call shares the scratch; only the error word must start at zero,
  // the kernels overwrite every other entry they read
  ce = cudaMemsetAsync(err, 0, sizeof(int), s);
  if (ce != cudaSuccess) return runtime_error(MAGACE_ERR_CUDA, cudaGetErrorString(ce));
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
  b.F = base + L.F;
  b.W = base + L.W;
  b.rho1 = reinterpret_cast<double*>(base + L.rho1);
  b.core = reinterpret_cast<double*>(base + L.core);
  b.edf = reinterpret_cast<double*>(base + L.edf);
  b.dedrho = reinterpret_cast<double*>(base + L.dedrho);
  b.err = err;
  b.aux = L.aux_bytes ? base + L.aux : nullptr;
  // device-memory bond arrays let the A-basis kernel variants that stage
  // bond tiles with bulk copies run, as in ace_compute_device
  b.dev_inputs = runtime_device_resident(r, e, mag_j, mhat_j);
  int nk = 0;
  const int n = precision == 0 ? launch_eval_fp64(dm, b, s, grid_cap, nullptr, &nk)
                               : launch_eval_fp32(dm, b, s, grid_cap, nullptr, &nk);
  runtime_set_launches(n, nk);
  ce = cudaGetLastError();
  if (ce != cudaSuccess) return runtime_error(MAGACE_ERR_CUDA, cudaGetErrorString(ce));
  // the call completes before it returns, so that the device error word of
  // this call can be reported
  int dev_err = 0;
  ce = cudaMemcpyAsync(&dev_err, err, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return runtime_error(MAGACE_ERR_CUDA, cudaGetErrorString(ce));
  return runtime_device_error(dev_err);
}
