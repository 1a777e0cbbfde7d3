// Device-side interface of the fused MLIP kernel (see kernel_impl.cuh).
#pragma once

#include <cuda_runtime.h>

#include "model.hpp"

namespace mlipg {

constexpr int kBlock = 256;      // threads per CTA (8 warps)
constexpr int kChunk = 32;       // neighbours staged per order-parameter chunk
constexpr int kLhMax = (kMaxL + 1) * (kMaxL + 2) / 2;

// Status bits raised by the kernel (read back by the host after each call).
enum StatusBits : int {
  kStatusNeighbourCapacity = 1,  // an atom had more neighbours inside rc than nb_cap
  kStatusBadType = 2,            // an element index outside [0, T) in the inputs
  kStatusAdjointRange = 4,       // fixed-point paths: adjoint flushes out of the range
};

struct KernelArgs {
  // geometry (device pointers)
  const double4* x4;      // [nall] position + element index (as double, <0 = skip)
  const int* centers;     // [ncenters] atom indices whose energy/adjoint is evaluated
  const int* nbr_off;     // [ncenters + 1] CSR into nbr_idx (indexed by centre position)
  const int* nbr_idx;     // neighbour atom indices into x4
  const int* img;         // optional per-pair packed image shift (null = none)
  const double* cell;     // optional per-centre-cell lattice [ncell][9] (rows a1,a2,a3)
  const int* center_cell; // optional cell id per centre (null = none)
  const int* fold;        // optional atom -> force index (null = identity)
  int ncenters;
  // model (device pointers)
  const DeviceTerm* terms;
  const DeviceTerm* terms64;  // the table with FP64 coefficients (the mixed path's
                              // FP64 evaluation of the polynomial's input features)
  const DeviceUnit* units;
  const int* unit_off;    // [T + 1]
  const DeviceIrrUnit* iunits;  // batched-tuple units
  const int* iunit_off;          // [T + 1]
  const DeviceTuple* tuples;
  const DeviceUnit* nl_units;
  const int* nl_off;      // [T + 1]
  const DevicePoly* poly;
  const int* poly_off;    // [T + 1]
  const int* adj_base;    // [T]: first entry of each element's adj_off rows
  const int* adj_off;     // polynomial adjoint gather lists (global CSR)
  const DeviceAdj* adj;   // (term weight, other factors) per gather entry
  const double* w_lin;    // [n_itc][16]
  const float* w_lin_f;   // [n_itc][16], FP32 copy for the mixed path
  const float2* w_lin_df; // [n_itc][16], (high, low) FP32 pairs for the double-float path
  const double* radial;   // [F][2] (beta, mu)
  // radial-only descriptor (pair potentials, pair.cu)
  const DevicePairTerm* pair_terms;
  const int* pair_term_off;      // [T + 1]
  const DevicePairAdj* pair_adj;
  const int* pair_adj_off;       // [T * pair_nd + 1]
  const int* type_pairs;         // [T][T] -> type pair index
  int pair_nd;                   // features: type pairs x radial functions
  // Optional recurrence of the FP64 radial functions for a common beta
  // (null: one exp per function): f_{n+1}/fc = f_n/fc * exp(rec_q r) *
  // K_n * (1 + eps_n r), radial_rec[n] = (K_n, eps_n)
  const double* radial_rec;
  double rec_q;
  int T, F, L, Lh, nb_cap, nl_cap;
  double rc;
  float g_bound;          // fixed-point paths: largest adjoint flush (power of two)
  int* gexp_cache;        // fixed-point paths: [kMaxTypes] scale exponents to start from
  int unit_dyn;           // 1: warps take batched units from a shared counter
  int sum64;              // mixed path: order-parameter sums in plain FP64 FMAs
  int lh64;               // mixed path: rows of FP64 order parameters (0 = none)
  // outputs
  double* f;              // [nforce][3], accumulated with atomics
  double* eatom;          // [ncenters] (may be null)
  double* vatom;          // [ncenters][6] centre virial, LAMMPS order xx yy zz xy xz yz (may be null)
  double* partials;       // [gridDim.x][8]: energy, virial(6, reference order), spare
  int* status;            // [1]
  unsigned long long* phase_clocks;  // optional [8]: SM cycles spent per phase (P1..P6)
};

// Instantiations of the fused kernel: FP32 products (the mixed
// precisions), FP64 throughout, and FP64 with the invariant/adjoint phase in
// double-float arithmetic.
enum KernelVariant { kVariantF32 = 0, kVariantF64 = 1, kVariantF64DF = 2 };
size_t fused_smem_bytes(int variant, int T, int L, int nb_cap, int nl_cap, int lh64);
int fused_max_blocks_per_sm(int variant, int L, size_t smem);
cudaError_t launch_fused(int variant, int L, const KernelArgs& a, int grid, size_t smem,
                         cudaStream_t s);
// Sums the per-CTA partials in a fixed order into out8[0..6] and writes the
// launch's status bits (as a double) into out8[7].
cudaError_t launch_finalize(const double* partials, int nparts, const int* status, double* out8,
                            cudaStream_t s);
cudaError_t init_device_constants();

// radial-only descriptor kernel (pair.cu)
size_t pair_smem_bytes(int F, int nd);
int pair_max_blocks(size_t smem);
cudaError_t launch_pair(const KernelArgs& a, int grid, size_t smem, cudaStream_t s);

}  // namespace mlipg

namespace mlipg {
#define MLIPG_DECL_PREC(tag)                                                           \
  namespace tag {                                                                      \
  size_t smem_bytes(int T, int L, int nb_cap, int nl_cap, int lh64);                     \
  int max_blocks(int L, size_t smem);                                                  \
  cudaError_t launch(int L, const KernelArgs& a, int grid, size_t smem, cudaStream_t s); \
  cudaError_t init_constants();                                                        \
  }
MLIPG_DECL_PREC(f64)
MLIPG_DECL_PREC(f64df)
MLIPG_DECL_PREC(f32)
#undef MLIPG_DECL_PREC
}  // namespace mlipg
