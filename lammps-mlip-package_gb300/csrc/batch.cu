// Many independent periodic cells evaluated in one persistent launch.
//
// Each cell's atoms are wrapped into its cell and get a full neighbour list
// of owned atoms whose entries carry packed periodic image codes (no ghost
// atoms; small cells see their own images).  All cells are concatenated:
// one fused-kernel launch evaluates every centre of every cell (uneven cell
// sizes balance across the persistent grid), then one block per cell sums
// its per-atom energies and virials in a fixed order.  Energies (eV),
// forces (eV/A, per atom) and the virial per cell (LAMMPS order xx yy zz xy
// xz yz, -sum r_ij (x) f_ij) come back to the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/mlipg.h"

namespace {

__global__ void k_cell_sums(const int* __restrict__ off, const double* __restrict__ eatom,
                            const double* __restrict__ vatom, double* __restrict__ out7) {
  const int c = blockIdx.x;
  __shared__ double red[7][128];
  double s[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int i = off[c] + threadIdx.x; i < off[c + 1]; i += blockDim.x) {
    s[0] += eatom[i];
    for (int k = 0; k < 6; ++k) s[1 + k] += vatom[6 * (size_t)i + k];
  }
  for (int k = 0; k < 7; ++k) red[k][threadIdx.x] = s[k];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int k = 0; k < 7; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 7) out7[7 * (size_t)c + threadIdx.x] = red[threadIdx.x][0];
}

// Stream-ordered device buffer: allocated and freed on the batch's stream
// from the device's memory pool, so creating and retiring batches never
// synchronises the device (other streams keep running).
template <typename T>
struct Dev {
  T* p = nullptr;
  cudaStream_t s = nullptr;
  cudaError_t alloc(size_t n, cudaStream_t stream) {
    s = stream;
    return cudaMallocAsync(reinterpret_cast<void**>(&p), std::max<size_t>(n, 1) * sizeof(T), s);
  }
  ~Dev() {
    if (p) cudaFreeAsync(p, s);
  }
};

}  // namespace

struct mlipg_batch {
  mlipg_handle* h = nullptr;
  cudaStream_t s = nullptr;
  int ncells = 0;
  int natoms = 0;
  long long npairs = 0;
  int nb_cap = 0;
  std::vector<int> cell_off;
  Dev<double4> x4;
  Dev<int> centers, off, idx, img, ccell, d_cell_off;
  Dev<double> lat, f, eatom, vatom, out8, cell7;
  std::vector<double> h_cell7;
};

extern "C" int mlipg_batch_create(mlipg_handle* h, int ncells, const int* natoms,
                                  const double* lattices, const double* x, const int* elements,
                                  mlipg_batch** out) {
  if (!h || ncells <= 0 || !natoms || !lattices || !x || !elements || !out) return MLIPG_EINVAL;
  *out = nullptr;
  cudaStream_t s = static_cast<cudaStream_t>(mlipg_stream(h));
  if (!s) return MLIPG_ENOGPU;
  const double rc = mlipg_cutoff(h);
  std::vector<int> aoff(ncells + 1, 0);
  for (int c = 0; c < ncells; ++c) {
    if (natoms[c] <= 0) return MLIPG_EINVAL;
    aoff[c + 1] = aoff[c] + natoms[c];
  }
  const int N = aoff[ncells];
  // per-cell neighbour lists (image-coded, owner indices), built in parallel
  std::vector<std::vector<int>> c_off(ncells), c_idx(ncells), c_img(ncells);
  std::vector<std::vector<double>> c_x(ncells);
  int err = MLIPG_OK;
#pragma omp parallel for schedule(dynamic, 4)
  for (int c = 0; c < ncells; ++c) {
    mlipg_nlist* nl = nullptr;
    const int n = natoms[c];
    if (mlipg_nlist_build(lattices + 9 * (size_t)c, n, x + 3 * (size_t)aoff[c],
                          elements + aoff[c], rc, &nl) != MLIPG_OK) {
      err = MLIPG_EINVAL;
      continue;
    }
    int nall = 0;
    long long np = 0;
    mlipg_nlist_sizes(nl, &nall, &np);
    std::vector<double> xa((size_t)nall * 3);
    std::vector<int> owner(nall), image(nall);
    c_off[c].resize(n + 1);
    c_idx[c].resize((size_t)np);
    mlipg_nlist_copy(nl, xa.data(), nullptr, owner.data(), image.data(), c_off[c].data(),
                     c_idx[c].data());
    mlipg_nlist_destroy(nl);
    c_img[c].resize((size_t)np);
    for (long long p = 0; p < np; ++p) {
      const int j = c_idx[c][p];
      c_img[c][p] = image[j];
      c_idx[c][p] = owner[j] + aoff[c];
    }
    xa.resize((size_t)n * 3);
    c_x[c] = std::move(xa);
  }
  if (err != MLIPG_OK) return err;
  {
    // keep freed batch memory in the pool (a serving loop reuses it at once)
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      unsigned long long keep = ~0ULL;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  mlipg_batch* b = new mlipg_batch();
  b->h = h;
  b->s = s;
  b->ncells = ncells;
  b->natoms = N;
  b->cell_off = aoff;
  std::vector<long long> poff(ncells + 1, 0);
  for (int c = 0; c < ncells; ++c) poff[c + 1] = poff[c] + (long long)c_idx[c].size();
  b->npairs = poff[ncells];
  if (b->npairs > 2147483647LL) {
    delete b;
    return MLIPG_EINVAL;
  }
  std::vector<double4> hx4(N);
  std::vector<int> hcent(N), hoff(N + 1), hcc(N), hidx((size_t)b->npairs), himg((size_t)b->npairs);
  int maxn = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(max : maxn)
  for (int c = 0; c < ncells; ++c) {
    for (int i = 0; i < natoms[c]; ++i) {
      const int g = aoff[c] + i;
      hx4[g] = double4{c_x[c][3 * i], c_x[c][3 * i + 1], c_x[c][3 * i + 2],
                       (double)elements[g]};
      hcent[g] = g;
      hcc[g] = c;
      hoff[g] = (int)(poff[c] + c_off[c][i]);
      maxn = std::max(maxn, c_off[c][i + 1] - c_off[c][i]);
    }
    std::memcpy(hidx.data() + poff[c], c_idx[c].data(), c_idx[c].size() * sizeof(int));
    std::memcpy(himg.data() + poff[c], c_img[c].data(), c_img[c].size() * sizeof(int));
  }
  hoff[N] = (int)b->npairs;
  b->nb_cap = maxn;
  bool ok = b->x4.alloc(N, s) == cudaSuccess && b->centers.alloc(N, s) == cudaSuccess &&
            b->off.alloc(N + 1, s) == cudaSuccess && b->idx.alloc(b->npairs, s) == cudaSuccess &&
            b->img.alloc(b->npairs, s) == cudaSuccess && b->ccell.alloc(N, s) == cudaSuccess &&
            b->d_cell_off.alloc(ncells + 1, s) == cudaSuccess &&
            b->lat.alloc(9 * (size_t)ncells, s) == cudaSuccess &&
            b->f.alloc(3 * (size_t)N, s) == cudaSuccess && b->eatom.alloc(N, s) == cudaSuccess &&
            b->vatom.alloc(6 * (size_t)N, s) == cudaSuccess &&
            b->out8.alloc(8, s) == cudaSuccess &&
            b->cell7.alloc(7 * (size_t)ncells, s) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    delete b;
    return MLIPG_ENOMEM;
  }
  cudaMemcpyAsync(b->x4.p, hx4.data(), N * sizeof(double4), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(b->centers.p, hcent.data(), N * sizeof(int), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(b->off.p, hoff.data(), (N + 1) * sizeof(int), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(b->idx.p, hidx.data(), hidx.size() * sizeof(int), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(b->img.p, himg.data(), himg.size() * sizeof(int), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(b->ccell.p, hcc.data(), N * sizeof(int), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(b->d_cell_off.p, aoff.data(), (ncells + 1) * sizeof(int),
                  cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(b->lat.p, lattices, 9 * (size_t)ncells * sizeof(double),
                  cudaMemcpyHostToDevice, s);
  // Copies from pageable memory are staged before cudaMemcpyAsync returns,
  // so the host vectors may go; the batch's work stays queued on the stream
  // behind whatever the stream already holds.
  if (cudaGetLastError() != cudaSuccess) {
    delete b;
    return MLIPG_ECUDA;
  }
  b->h_cell7.resize(7 * (size_t)ncells);
  *out = b;
  return MLIPG_OK;
}

extern "C" int mlipg_batch_launch(mlipg_batch* b) {
  if (!b) return MLIPG_EINVAL;
  if (cudaMemsetAsync(b->f.p, 0, 3 * (size_t)b->natoms * sizeof(double), b->s) != cudaSuccess)
    return MLIPG_ECUDA;
  int rc = mlipg_compute_device(b->h, b->natoms, b->x4.p, b->centers.p, b->off.p, b->idx.p,
                                b->img.p, b->lat.p, b->ccell.p, nullptr, b->nb_cap, b->f.p,
                                b->eatom.p, b->vatom.p, b->out8.p);
  if (rc != MLIPG_OK) return rc;
  k_cell_sums<<<b->ncells, 128, 0, b->s>>>(b->d_cell_off.p, b->eatom.p, b->vatom.p, b->cell7.p);
  return cudaGetLastError() == cudaSuccess ? MLIPG_OK : MLIPG_ECUDA;
}

extern "C" int mlipg_batch_results(mlipg_batch* b, double* energies, double* forces,
                                   double* virials);

extern "C" int mlipg_batch_compute(mlipg_batch* b, double* energies, double* forces,
                                   double* virials) {
  int rc = mlipg_batch_launch(b);
  if (rc != MLIPG_OK) return rc;
  return mlipg_batch_results(b, energies, forces, virials);
}

// Copies the results of a finished (or queued) launch back to the host.
extern "C" int mlipg_batch_results(mlipg_batch* b, double* energies, double* forces,
                                   double* virials) {
  if (!b) return MLIPG_EINVAL;
  if (forces &&
      cudaMemcpyAsync(forces, b->f.p, 3 * (size_t)b->natoms * sizeof(double),
                      cudaMemcpyDeviceToHost, b->s) != cudaSuccess)
    return MLIPG_ECUDA;
  if (cudaMemcpyAsync(b->h_cell7.data(), b->cell7.p, b->h_cell7.size() * sizeof(double),
                      cudaMemcpyDeviceToHost, b->s) != cudaSuccess ||
      cudaStreamSynchronize(b->s) != cudaSuccess)
    return MLIPG_ECUDA;
  for (int c = 0; c < b->ncells; ++c) {
    if (energies) energies[c] = b->h_cell7[7 * (size_t)c];
    if (virials)
      for (int k = 0; k < 6; ++k) virials[6 * (size_t)c + k] = b->h_cell7[7 * (size_t)c + 1 + k];
  }
  return MLIPG_OK;
}

extern "C" int mlipg_batch_autotune(mlipg_batch* b, int max_report, double* report,
                                    int* nreport) {
  if (!b) return MLIPG_EINVAL;
  return mlipg_autotune(b->h, b->natoms, b->x4.p, b->centers.p, b->off.p, b->idx.p, b->img.p,
                        b->lat.p, b->ccell.p, b->nb_cap, b->f.p, b->out8.p, max_report, report,
                        nreport);
}

extern "C" size_t mlipg_batch_device_bytes(const mlipg_batch* b) {
  if (!b) return 0;
  return (size_t)b->natoms * (sizeof(double4) + 4 + 4 + 4 + 24 + 8 + 48) +
         (size_t)b->ncells * (9 * 8 + 4 + 56) + (size_t)b->npairs * 8;
}

extern "C" int mlipg_batch_sizes(const mlipg_batch* b, int* natoms, long long* npairs) {
  if (!b) return MLIPG_EINVAL;
  if (natoms) *natoms = b->natoms;
  if (npairs) *npairs = b->npairs;
  return MLIPG_OK;
}

extern "C" void mlipg_batch_destroy(mlipg_batch* b) { delete b; }
