// FP32 / FP64 FMA throughput microkernels.  The fused MLIP kernels are bound
// by the CUDA-core FP32 pipe (mixed and double-float kernels) or the FP64 pipe
// (the all-FP64 kernel), whose peaks are
// not among the copy / tensor-core peaks measured for the machine; these
// kernels measure them live on the same device so the roofline fraction has
// a measured denominator.
#include <cuda_runtime.h>

#include "../../include/mlipg.h"

namespace {

template <typename T>
__global__ void fma_chain(T* out, int iters, T a, T b) {
  // 8 independent chains per thread hide the FMA latency
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
    x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  const T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == T(-1.2345)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
int measure(double* tflops, int iters) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int block = 256, grid = sms * 8;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * block * grid) != cudaSuccess) return MLIPG_ENOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chain<T><<<grid, block>>>(out, iters / 10, T(0.999), T(0.001));
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0);
    fma_chain<T><<<grid, block>>>(out, iters, T(0.999), T(0.001));
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess) return MLIPG_ECUDA;
  *tflops = 2.0 * 8.0 * iters * (double)block * grid / (best * 1e-3) / 1e12;
  return MLIPG_OK;
}

}  // namespace

extern "C" int mlipg_measure_fma_peak(int fp64, double* tflops) {
  if (!tflops) return MLIPG_EINVAL;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return MLIPG_ENOGPU;
  return fp64 ? measure<double>(tflops, 4096) : measure<float>(tflops, 65536);
}
