// Allocation-free variant of mlipg_compute_device.
//
// Some callers cannot let a library call cudaMalloc: an MD engine or
// service whose device memory is owned by its own pool or budget hands the
// library only buffers it allocated itself, and latency-critical loops must
// not enter the CUDA allocator (cudaMalloc can synchronise the device and
// take milliseconds).  mlipg_compute_device_noalloc serves them: the fused
// kernel's scratch (its per-CTA partial sums of energy and virial, and the
// status word) lives in the file-scope array below instead of in buffers
// the handle allocates on demand.  Inputs and outputs are still the
// caller's device buffers; the model tables were allocated once by
// mlipg_create.
//
// Limits and sharing:
//  * the array holds kNoAllocSlots CTA slots (8 doubles each, 128 KiB) plus
//    the status word; a launch that would need more CTAs is rejected with
//    MLIPG_ECAPACITY (GB300 runs at most 152 SMs x 8 resident CTAs = 1216);
//  * every GPU that loads this library keeps the array until the process
//    exits;
//  * every call shares the array and it keeps the last call's contents:
//    the status word is cleared on each call and each launched CTA
//    overwrites its own slot, so calls that overlap on the GPU (on
//    different streams, or from different handles) race on it.
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (host code cannot use the symbol itself) and keeps
//    it for that device; make that first call before any stream capture.
//    The kept address belongs to the device's current context: after a
//    cudaDeviceReset it is stale, so reload the library (or restart the
//    process) before calling again;
//  * the call runs on the handle's device: the calling thread's current
//    device must be that device (MLIPG_EINVAL otherwise), so that the
//    scratch address and the handle's stream belong to the same GPU;
//  * the launch's status bits are written to d_out8[7] as for
//    mlipg_compute_device.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/mlipg.h"

namespace {

constexpr int kNoAllocSlots = 2048;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocSlots * 8 + 32];

std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

}  // namespace

// defined in capi.cpp: launches the fused kernel and the finalize reduction
// with caller-provided scratch, without allocating
int mlipg_internal_launch_scratch(mlipg_handle* h, int ncenters, const void* d_x4,
                                  const int* d_centers, const int* d_nbr_off,
                                  const int* d_nbr_idx, const int* d_img, const double* d_cell,
                                  const int* d_center_cell, const int* d_fold, int nb_cap,
                                  double* d_f, double* d_eatom, double* d_vatom, double* d_out8,
                                  double* partials, int partial_slots, int* status);
int mlipg_internal_fail(mlipg_handle* h, int code, const char* msg);
int mlipg_internal_handle_device(const mlipg_handle* h);

extern "C" int mlipg_compute_device_noalloc(mlipg_handle* h, int ncenters, const void* d_x4,
                                            const int* d_centers, const int* d_nbr_off,
                                            const int* d_nbr_idx, const int* d_img,
                                            const double* d_cell, const int* d_center_cell,
                                            const int* d_fold, int nb_cap, double* d_f,
                                            double* d_eatom, double* d_vatom, double* d_out8) {
  if (!h) return mlipg_internal_fail(nullptr, MLIPG_EINVAL, "null handle");
  const int dev = mlipg_internal_handle_device(h);
  if (dev < 0 || dev >= kMaxDevices)
    return mlipg_internal_fail(h, MLIPG_ENOGPU, "no usable CUDA device for the scratch array");
  int cur = -1;
  if (cudaGetDevice(&cur) != cudaSuccess) {
    cudaGetLastError();
    return mlipg_internal_fail(h, MLIPG_ENOGPU, "cudaGetDevice failed");
  }
  if (cur != dev)
    return mlipg_internal_fail(h, MLIPG_EINVAL,
                               "the current device differs from the handle's device");
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p)
        return mlipg_internal_fail(h, MLIPG_ECUDA,
                                   "cudaGetSymbolAddress of the no-allocation scratch failed");
      g_addr[dev] = p;
    }
    base = g_addr[dev];
  }
  double* partials = static_cast<double*>(base);
  int* status = reinterpret_cast<int*>(partials + (size_t)kNoAllocSlots * 8);
  return mlipg_internal_launch_scratch(h, ncenters, d_x4, d_centers, d_nbr_off, d_nbr_idx, d_img,
                                       d_cell, d_center_cell, d_fold, nb_cap, d_f, d_eatom,
                                       d_vatom, d_out8, partials, kNoAllocSlots, status);
}
