// FP64 instantiation of the fused kernel with the invariant/adjoint phase in
// double-float arithmetic (FP32 pairs on the FP32 pipe) and the adjoint in
// exact four-word fixed point; order parameters, the polynomial, forces,
// energies and virial in FP64.
#define MLIPG_REAL double
#define MLIPG_TAG f64df
#define MLIPG_DF 1
#include "kernel_impl.cuh"
