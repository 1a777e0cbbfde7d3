// FP64 instantiation of the fused kernel (plain path).
#define MLIPG_REAL double
#define MLIPG_TAG f64
#include "kernel_impl.cuh"
