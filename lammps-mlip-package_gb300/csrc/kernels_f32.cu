// FP32-product instantiation of the fused kernel (mixed path: radial, Y_lm,
// invariant and adjoint products in FP32; order-parameter sums, forces,
// energies and virial accumulated in FP64).
#define MLIPG_REAL float
#define MLIPG_TAG f32
#include "kernel_impl.cuh"
