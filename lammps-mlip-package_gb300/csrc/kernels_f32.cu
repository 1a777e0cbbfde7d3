// FP32-product instantiation of the fused kernel (the mixed precisions):
// radial functions, Y_lm, invariant and adjoint products in FP32;
// order-parameter neighbour sums in Kahan-compensated FP32, or in plain FP64
// FMAs for MLIPG_PREC_MIXED_A64; the polynomial's input features and their
// energy, and forces, energies and virial accumulated in FP64.
#define MLIPG_REAL float
#define MLIPG_TAG f32
#include "kernel_impl.cuh"
