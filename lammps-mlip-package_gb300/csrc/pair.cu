// Energy, forces and virial of the radial-only descriptor (potentials with
// des_type "pair", the reference's `pair_style mlip_pair`,
// src/USER-MLIP/pair_mlip_pair.cpp:56-264), in FP64 for every precision.
//
// One CTA per centre atom (persistent grid-stride loop), neighbours staged
// 128 at a time:
//   1. dn[tc][n] = sum_j f_n(r_ij) over the neighbours of type pair tc
//      (one thread per neighbour evaluates its radial functions; one thread
//      per feature sums them in list order, so the sums are deterministic);
//   2. E_i = sum_k c_k prod dn over the terms valid for the centre's element
//      (threads over terms, fixed-order block reduction);
//   3. H[f] = dE_i/d dn[f], gathered from per-feature (weight, other
//      factors) records, slices summed in order;
//   4. per neighbour f_ij = sum_n f_n'(r) H[tc][n] r_hat, F_i += f, F_j -= f,
//      virial -= r_ij (x) f (owner computes: the pair's other half comes from
//      the neighbour's own centre).
// Per-CTA partial sums (energy, virial in the order xx yy zz yz zx xy) and
// the status word follow the fused kernel's contract, so the same finalize
// kernel and host paths serve both.
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace mlipg {
namespace {

constexpr int kPairChunk = 128;

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// displacement of list entry k of centre c (image shift for batched cells)
__device__ __forceinline__ void pdisp(const KernelArgs& A, int c, int k, const double4& xi,
                                      const double4& xj, double& dx, double& dy, double& dz) {
  dx = xj.x - xi.x;
  dy = xj.y - xi.y;
  dz = xj.z - xi.z;
  if (A.img != nullptr) {
    const int code = __ldg(A.img + k);
    if (code != 0) {
      const double n1 = (double)((code & 1023) - 512);
      const double n2 = (double)(((code >> 10) & 1023) - 512);
      const double n3 = (double)(((code >> 20) & 1023) - 512);
      const double* L = A.cell + 9 * __ldg(A.center_cell + c);
      dx += n1 * L[0] + n2 * L[3] + n3 * L[6];
      dy += n1 * L[1] + n2 * L[4] + n3 * L[7];
      dz += n1 * L[2] + n2 * L[5] + n3 * L[8];
    }
  }
}

// block reduction of v (one value per thread) in a fixed order
__device__ __forceinline__ double block_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum_d(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < kBlock / 32; ++w) s += red[w];
  return s;
}

__global__ void __launch_bounds__(kBlock) pair_kernel(const __grid_constant__ KernelArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int F = A.F, T = A.T, nd = A.pair_nd;
  double* fst = reinterpret_cast<double*>(smem);              // [kPairChunk][F]
  double* dn = fst + kPairChunk * F;                          // [nd]
  double* H = dn + nd;                                        // [nd]
  double* part = H + nd;                                      // [kBlock] slices of H
  double* red = part + kBlock;                                // [8][8]
  int* tcj = reinterpret_cast<int*>(red + 64);                // [kPairChunk]
  const int tid = threadIdx.x;
  double ecta = 0.0, vir[6] = {0, 0, 0, 0, 0, 0};
  const double rc2 = A.rc * A.rc;
  for (int c = blockIdx.x; c < A.ncenters; c += gridDim.x) {
    const int i = __ldg(A.centers + c);
    const double4 xi = A.x4[i];
    const int ti = (int)xi.w;
    if (ti < 0 || ti >= T) {
      if (tid == 0) {
        if (A.eatom) A.eatom[c] = 0.0;
        if (A.vatom)
          for (int q = 0; q < 6; ++q) A.vatom[(size_t)c * 6 + q] = 0.0;
        if (ti >= T) atomicOr(A.status, kStatusBadType);
      }
      continue;
    }
    const int o0 = __ldg(A.nbr_off + c), o1 = __ldg(A.nbr_off + c + 1);
    // 1. features
    double acc = 0.0;
    const int etc = tid < nd ? tid / F : -1, en = tid < nd ? tid % F : 0;
    for (int cb = o0; cb < o1; cb += kPairChunk) {
      const int csz = min(kPairChunk, o1 - cb);
      if (tid < csz) {
        const int k = cb + tid;
        const int j = __ldg(A.nbr_idx + k);
        const double4 xj = A.x4[j];
        const int tj = (int)xj.w;
        double dx, dy, dz;
        pdisp(A, c, k, xi, xj, dx, dy, dz);
        const double r2 = dx * dx + dy * dy + dz * dz;
        int tc = -1;
        if (tj >= T) atomicOr(A.status, kStatusBadType);
        if (tj >= 0 && tj < T && r2 < rc2 && r2 > 0.0) {
          tc = __ldg(A.type_pairs + ti * T + tj);
          const double r = sqrt(r2);
          double sn, cs;
          sincospi(r / A.rc, &sn, &cs);
          const double fc = 0.5 * (cs + 1.0);
          for (int n = 0; n < F; ++n) {
            const double dr = r - __ldg(A.radial + 2 * n + 1);
            fst[tid * F + n] = exp(-__ldg(A.radial + 2 * n) * dr * dr) * fc;
          }
        }
        tcj[tid] = tc;
      }
      __syncthreads();
      if (etc >= 0)
        for (int kk = 0; kk < csz; ++kk)
          if (tcj[kk] == etc) acc += fst[kk * F + en];
      __syncthreads();
    }
    if (tid < nd) dn[tid] = acc;
    __syncthreads();
    // 2. energy
    const int t0 = __ldg(A.pair_term_off + ti), t1 = __ldg(A.pair_term_off + ti + 1);
    double e = 0.0;
    for (int k = t0 + tid; k < t1; k += kBlock) {
      const DevicePairTerm tm = A.pair_terms[k];
      double v = tm.c;
      for (int q = 0; q < tm.order; ++q) v *= dn[tm.f[q]];
      e += v;
    }
    const double Ei = block_sum(e, red);
    // 3. dE/d dn, each feature's records cut into S contiguous slices
    const int* aoff = A.pair_adj_off + (size_t)ti * nd;
    const int S = nd >= kBlock ? 1 : kBlock / nd;
    for (int w = tid; w < nd * S; w += kBlock) {
      const int f = w % nd, sl = w / nd;
      const int x0 = __ldg(aoff + f), len = __ldg(aoff + f + 1) - x0;
      const int xs = x0 + (len * sl) / S, xe = x0 + (len * (sl + 1)) / S;
      double h = 0.0;
      for (int x = xs; x < xe; ++x) {
        const DevicePairAdj r = A.pair_adj[x];
        double v = r.c;
        if (r.other[0] >= 0) v *= dn[r.other[0]];
        if (r.other[1] >= 0) v *= dn[r.other[1]];
        h += v;
      }
      if (S == 1) H[f] = h;
      else part[w] = h;
    }
    __syncthreads();
    if (S > 1) {
      for (int f = tid; f < nd; f += kBlock) {
        double h = 0.0;
        for (int sl = 0; sl < S; ++sl) h += part[sl * nd + f];
        H[f] = h;
      }
      __syncthreads();
    }
    // 4. forces and virial
    double fx = 0.0, fy = 0.0, fz = 0.0, va[6] = {0, 0, 0, 0, 0, 0};
    for (int k = o0 + tid; k < o1; k += kBlock) {
      const int j = __ldg(A.nbr_idx + k);
      const double4 xj = A.x4[j];
      const int tj = (int)xj.w;
      if (tj < 0 || tj >= T) continue;
      double dx, dy, dz;
      pdisp(A, c, k, xi, xj, dx, dy, dz);
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (!(r2 < rc2 && r2 > 0.0)) continue;
      const double r = sqrt(r2), ir = 1.0 / r;
      const int tc = __ldg(A.type_pairs + ti * T + tj);
      double sn, cs;
      sincospi(r / A.rc, &sn, &cs);
      const double fc = 0.5 * (cs + 1.0);
      const double fcd = -0.5 * 3.14159265358979323846 / A.rc * sn;
      double g = 0.0;
      for (int n = 0; n < F; ++n) {
        const double beta = __ldg(A.radial + 2 * n), dr = r - __ldg(A.radial + 2 * n + 1);
        const double bf = exp(-beta * dr * dr);
        g += ((-2.0 * beta * dr * bf) * fc + bf * fcd) * H[tc * F + n];
      }
      const double gx = g * dx * ir, gy = g * dy * ir, gz = g * dz * ir;
      fx += gx; fy += gy; fz += gz;
      const int fj = A.fold ? __ldg(A.fold + j) : j;
      atomicAdd(A.f + 3 * (size_t)fj, -gx);
      atomicAdd(A.f + 3 * (size_t)fj + 1, -gy);
      atomicAdd(A.f + 3 * (size_t)fj + 2, -gz);
      // order xx yy zz yz zx xy
      va[0] -= dx * gx; va[1] -= dy * gy; va[2] -= dz * gz;
      va[3] -= dy * gz; va[4] -= dz * gx; va[5] -= dx * gy;
    }
    const double Fx = block_sum(fx, red), Fy = block_sum(fy, red), Fz = block_sum(fz, red);
    double V[6];
    for (int q = 0; q < 6; ++q) V[q] = block_sum(va[q], red);
    if (tid == 0) {
      const int fi = A.fold ? __ldg(A.fold + i) : i;
      atomicAdd(A.f + 3 * (size_t)fi, Fx);
      atomicAdd(A.f + 3 * (size_t)fi + 1, Fy);
      atomicAdd(A.f + 3 * (size_t)fi + 2, Fz);
      if (A.eatom) A.eatom[c] = Ei;
      if (A.vatom) {
        // LAMMPS order xx yy zz xy xz yz
        double* v = A.vatom + (size_t)c * 6;
        v[0] = V[0]; v[1] = V[1]; v[2] = V[2]; v[3] = V[5]; v[4] = V[4]; v[5] = V[3];
      }
    }
    ecta += Ei;
    for (int q = 0; q < 6; ++q) vir[q] += V[q];
    __syncthreads();
  }
  if (tid < 8) A.partials[(size_t)blockIdx.x * 8 + tid] = tid == 0 ? ecta : (tid < 7 ? vir[tid - 1] : 0.0);
}

}  // namespace

size_t pair_smem_bytes(int F, int nd) {
  return (size_t)kPairChunk * F * sizeof(double) + 2 * (size_t)nd * sizeof(double) +
         (size_t)kBlock * sizeof(double) + 64 * sizeof(double) + kPairChunk * sizeof(int);
}

int pair_max_blocks(size_t smem) {
  if (cudaFuncSetAttribute(pair_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pair_kernel, kBlock, smem) != cudaSuccess)
    return 0;
  return nb;
}

cudaError_t launch_pair(const KernelArgs& a, int grid, size_t smem, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(pair_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  pair_kernel<<<grid, kBlock, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace mlipg
