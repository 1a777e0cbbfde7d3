// Precision dispatch and the deterministic partial-sum reduction.
#include "kernels.cuh"

namespace mlipg {

static_assert(sizeof(DeviceTerm) == 16, "DeviceTerm must be 16 bytes");
static_assert(kBlock / 32 == kCtaWarps, "schedules are dealt to the CTA's warps");
static_assert(sizeof(DeviceUnit) == 32, "DeviceUnit must be 32 bytes");
static_assert(sizeof(DevicePoly) == 32, "DevicePoly must be 32 bytes");

size_t fused_smem_bytes(int variant, int T, int L, int nb_cap, int nl_cap, int lh64) {
  switch (variant) {
    case kVariantF64: return f64::smem_bytes(T, L, nb_cap, nl_cap, 0);
    case kVariantF64DF: return f64df::smem_bytes(T, L, nb_cap, nl_cap, 0);
    default: return f32::smem_bytes(T, L, nb_cap, nl_cap, lh64);
  }
}

int fused_max_blocks_per_sm(int variant, int L, size_t smem) {
  switch (variant) {
    case kVariantF64: return f64::max_blocks(L, smem);
    case kVariantF64DF: return f64df::max_blocks(L, smem);
    default: return f32::max_blocks(L, smem);
  }
}

cudaError_t launch_fused(int variant, int L, const KernelArgs& a, int grid, size_t smem,
                         cudaStream_t s) {
  switch (variant) {
    case kVariantF64: return f64::launch(L, a, grid, smem, s);
    case kVariantF64DF: return f64df::launch(L, a, grid, smem, s);
    default: return f32::launch(L, a, grid, smem, s);
  }
}

cudaError_t init_device_constants() {
  cudaError_t e = f64::init_constants();
  if (e == cudaSuccess) e = f64df::init_constants();
  if (e != cudaSuccess) return e;
  return f32::init_constants();
}

// Sums the per-CTA partials [nparts][8] in a fixed order (deterministic);
// slot 7 of the output carries the launch's status bits.
__global__ void finalize_kernel(const double* __restrict__ parts, int nparts,
                                const int* __restrict__ status, double* out) {
  __shared__ double red[8][33];
  const int q = threadIdx.y;        // 0..7
  const int lane = threadIdx.x;     // 0..31
  double s = 0.0;
  for (int p = lane; p < nparts; p += 32) s += parts[(size_t)p * 8 + q];
  red[q][lane] = s;
  __syncthreads();
  if (lane == 0) {
    double t = 0.0;
    for (int k = 0; k < 32; ++k) t += red[q][k];
    out[q] = q == 7 ? (double)*status : t;
  }
}

cudaError_t launch_finalize(const double* partials, int nparts, const int* status, double* out8,
                            cudaStream_t s) {
  finalize_kernel<<<1, dim3(32, 8), 0, s>>>(partials, nparts, status, out8);
  return cudaGetLastError();
}

}  // namespace mlipg
