// All-FP64 instantiation of the fused kernel (MLIPG_PREC_FP64_NATIVE, and
// MLIPG_PREC_FP64 for potentials outside the double-float kernel's range or
// shared memory): every product and sum in FP64.
#define MLIPG_REAL double
#define MLIPG_TAG f64
#include "kernel_impl.cuh"
