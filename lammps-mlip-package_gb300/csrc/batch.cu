// Many independent periodic cells evaluated in one persistent launch.
//
// The cells' atoms are uploaded once (positions + element as double4, the
// lattices) and the device neighbour builder wraps them into their cells and
// writes full lists of owned atoms whose entries carry packed periodic image
// codes (no ghost atoms; small cells see their own images).  The lists are
// built on the batch's own stream, so building one batch never waits for
// the evaluations queued on the handle's stream.  One fused-kernel launch
// evaluates every centre of every cell (uneven cell sizes balance across
// the persistent grid), then one block per cell sums its per-atom energies
// and virials in a fixed order.  Energies (eV), forces (eV/A, per atom) and
// the virial per cell (LAMMPS order xx yy zz xy xz yz, -sum r_ij (x) f_ij)
// come back to the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/mlipg.h"

// Maps the fused kernel's status bits (d_out8[7]) to a C-ABI status code and
// sets the handle's message.
int mlipg_internal_status_fail(mlipg_handle* h, int bits);

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

__global__ void k_iota(int n, int* __restrict__ v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = i;
}

// Stream-ordered device buffer: allocated and freed on the batch's build
// stream from the device's memory pool, so creating and retiring batches
// never synchronises the device (other streams keep running).
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
  cudaStream_t s = nullptr;    // the handle's stream: evaluations
  cudaStream_t bs = nullptr;   // this batch's stream: upload, lists, buffer lifetime
  cudaEvent_t built = nullptr, done = nullptr;
  int ncells = 0;
  int natoms = 0;
  long long npairs = 0;
  int nb_cap = 0;
  mlipg_dnlist* nl = nullptr;
  Dev<double4> x4;
  Dev<int> centers, d_cell_off;
  Dev<double> f, eatom, vatom, out8, cell7;
  std::vector<double> h_cell7;
  double h_status = 0;   // d_out8[7] of the last launch: the kernel's status bits
  ~mlipg_batch() {
    // buffers are freed on bs once every evaluation queued on s has finished
    if (done && s && bs && cudaEventRecord(done, s) == cudaSuccess) cudaStreamWaitEvent(bs, done, 0);
    mlipg_dnlist_destroy(nl);
    if (built) cudaEventDestroy(built);
    if (done) cudaEventDestroy(done);
  }
};

static void keep_pool_memory() {
  // keep freed batch memory in the pool (a serving loop reuses it at once)
  int dev = 0;
  cudaMemPool_t pool;
  if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    unsigned long long keep = ~0ULL;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
}

extern "C" int mlipg_batch_create(mlipg_handle* h, int ncells, const int* natoms,
                                  const double* lattices, const double* x, const int* elements,
                                  mlipg_batch** out) {
  if (!h || ncells <= 0 || !natoms || !lattices || !x || !elements || !out) return MLIPG_EINVAL;
  *out = nullptr;
  cudaStream_t s = static_cast<cudaStream_t>(mlipg_stream(h));
  if (!s) return MLIPG_ENOGPU;
  const int ne = mlipg_num_elements(h);
  std::vector<int> aoff(ncells + 1, 0);
  for (int c = 0; c < ncells; ++c) {
    if (natoms[c] <= 0 || aoff[c] > (1 << 30) - natoms[c]) return MLIPG_EINVAL;
    aoff[c + 1] = aoff[c] + natoms[c];
  }
  const int N = aoff[ncells];
  std::vector<double4> hx4(N);
  for (int i = 0; i < N; ++i) {
    if (elements[i] < 0 || elements[i] >= ne) return MLIPG_EINVAL;
    hx4[i] = double4{x[3 * (size_t)i], x[3 * (size_t)i + 1], x[3 * (size_t)i + 2],
                     (double)elements[i]};
  }
  keep_pool_memory();
  mlipg_batch* b = new mlipg_batch();
  b->h = h;
  b->s = s;
  b->ncells = ncells;
  b->natoms = N;
  if (cudaStreamCreateWithFlags(&b->bs, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->built, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    mlipg_batch_destroy(b);
    return MLIPG_ECUDA;
  }
  cudaStream_t bs = b->bs;
  const bool ok = b->x4.alloc(N, bs) == cudaSuccess && b->centers.alloc(N, bs) == cudaSuccess &&
                  b->d_cell_off.alloc(ncells + 1, bs) == cudaSuccess &&
                  b->f.alloc(3 * (size_t)N, bs) == cudaSuccess &&
                  b->eatom.alloc(N, bs) == cudaSuccess &&
                  b->vatom.alloc(6 * (size_t)N, bs) == cudaSuccess &&
                  b->out8.alloc(8, bs) == cudaSuccess &&
                  b->cell7.alloc(7 * (size_t)ncells, bs) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    mlipg_batch_destroy(b);
    return MLIPG_ENOMEM;
  }
  // copies from pageable memory are staged before cudaMemcpyAsync returns
  if (cudaMemcpyAsync(b->x4.p, hx4.data(), N * sizeof(double4), cudaMemcpyHostToDevice, bs) !=
          cudaSuccess ||
      cudaMemcpyAsync(b->d_cell_off.p, aoff.data(), (ncells + 1) * sizeof(int),
                      cudaMemcpyHostToDevice, bs) != cudaSuccess) {
    cudaGetLastError();
    mlipg_batch_destroy(b);
    return MLIPG_ECUDA;
  }
  k_iota<<<(N + 255) / 256, 256, 0, bs>>>(N, b->centers.p);
  int rc = mlipg_dnlist_create(bs, &b->nl);
  if (rc == MLIPG_OK) rc = mlipg_dnlist_build(b->nl, ncells, natoms, lattices, b->x4.p,
                                              mlipg_cutoff(h), 0);
  if (rc == MLIPG_OK) {
    int maxn = 0;
    mlipg_dnlist_arrays(b->nl, nullptr, nullptr, nullptr, nullptr, nullptr, &b->npairs, &maxn,
                        nullptr);
    b->nb_cap = maxn;
    if (cudaEventRecord(b->built, bs) != cudaSuccess) rc = MLIPG_ECUDA;
  }
  if (rc != MLIPG_OK) {
    cudaGetLastError();
    mlipg_batch_destroy(b);
    return rc;
  }
  b->h_cell7.resize(7 * (size_t)ncells);
  *out = b;
  return MLIPG_OK;
}

extern "C" int mlipg_batch_launch(mlipg_batch* b) {
  if (!b) return MLIPG_EINVAL;
  const int *off = nullptr, *idx = nullptr, *img = nullptr, *ccell = nullptr;
  const double* lat = nullptr;
  mlipg_dnlist_arrays(b->nl, &off, &idx, &img, &ccell, &lat, nullptr, nullptr, nullptr);
  if (cudaStreamWaitEvent(b->s, b->built, 0) != cudaSuccess ||
      cudaMemsetAsync(b->f.p, 0, 3 * (size_t)b->natoms * sizeof(double), b->s) != cudaSuccess)
    return MLIPG_ECUDA;
  int rc = mlipg_compute_device(b->h, b->natoms, b->x4.p, b->centers.p, off, idx, img, lat,
                                ccell, nullptr, b->nb_cap, b->f.p, b->eatom.p, b->vatom.p,
                                b->out8.p);
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
      cudaMemcpyAsync(&b->h_status, b->out8.p + 7, sizeof(double), cudaMemcpyDeviceToHost,
                      b->s) != cudaSuccess ||
      cudaStreamSynchronize(b->s) != cudaSuccess)
    return MLIPG_ECUDA;
  // a status bit (neighbour capacity, element index, adjoint range) means
  // some centre's energy and forces are missing: fail the whole batch
  if (b->h_status != 0.0) return mlipg_internal_status_fail(b->h, (int)b->h_status);
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
  const int *off = nullptr, *idx = nullptr, *img = nullptr, *ccell = nullptr;
  const double* lat = nullptr;
  mlipg_dnlist_arrays(b->nl, &off, &idx, &img, &ccell, &lat, nullptr, nullptr, nullptr);
  if (cudaStreamWaitEvent(b->s, b->built, 0) != cudaSuccess) return MLIPG_ECUDA;
  return mlipg_autotune(b->h, b->natoms, b->x4.p, b->centers.p, off, idx, img, lat, ccell,
                        b->nb_cap, b->f.p, b->out8.p, max_report, report, nreport);
}

extern "C" size_t mlipg_batch_device_bytes(const mlipg_batch* b) {
  if (!b) return 0;
  // batch buffers + builder (cell, bin, count, offset per atom; bins; pairs)
  return (size_t)b->natoms * (sizeof(double4) + 4 + 24 + 8 + 48 + 5 * 4) +
         (size_t)b->ncells * (9 * 8 + 4 + 56 + 192) + (size_t)b->npairs * 8;
}

extern "C" int mlipg_batch_sizes(const mlipg_batch* b, int* natoms, long long* npairs) {
  if (!b) return MLIPG_EINVAL;
  if (natoms) *natoms = b->natoms;
  if (npairs) *npairs = b->npairs;
  return MLIPG_OK;
}

extern "C" void mlipg_batch_destroy(mlipg_batch* b) {
  if (!b) return;
  cudaStream_t bs = b->bs;
  delete b;   // frees are queued on bs behind the last evaluation
  if (bs) cudaStreamDestroy(bs);
}
