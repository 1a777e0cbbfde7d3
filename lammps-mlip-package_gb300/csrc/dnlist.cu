// Device neighbour-list builder for one or many periodic cells.
//
// Full lists of owned atoms with packed periodic image codes, no ghost atoms
// (the form the fused kernel reads for batched cells and MD): entry (j, code)
// of atom i means x_j + n1 a1 + n2 a2 + n3 a3 lies within rlist of x_i, with
// code = (n1+512) | (n2+512) << 10 | (n3+512) << 20, or 0 when n = 0.
//
// Every cell gets its own bin grid in fractional coordinates: nb_k =
// floor(w_k / rlist) bins along axis k (w_k the perpendicular width, at
// least 1 bin) and a stencil of st_k = floor(rlist nb_k / w_k) + 1 bins on
// each side, walked with periodic wrap; a bin reached through the boundary
// carries the image shift, so cells narrower than 2 rlist see their own
// images without ghost copies.  The reference's standalone builder
// (src/USER-MLIP/mlipkk_cell.cpp:218-307) enumerates the same image shifts on
// the host and returns a half list of displacements.
//
// Steps (all on the builder's stream): wrap positions into their cell and
// bin them; counting sort into bins, each bin sorted by atom index (so the
// list order is deterministic); count neighbours per atom; exclusive scan to
// CSR offsets; read back the pair total and the longest list (8 bytes); grow
// the pair arrays if needed; write the lists.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/mlipg.h"

namespace {

struct CellParam {
  double lat[9];   // rows a1, a2, a3
  double inv[9];   // frac_k = sum_m x_m inv[3m + k]
  int nb[3];
  int st[3];
  int bin0;        // first bin of this cell in the global bin array
  int atom0;
  int natoms;
  int pad;
};

// Grow-only buffer from the stream-ordered pool of the builder's stream
// (allocating or freeing never synchronises the device).
template <typename T>
struct Buf {
  T* p = nullptr;
  size_t cap = 0;
  cudaStream_t s = nullptr;
  bool grow(size_t n, cudaStream_t stream, bool* moved = nullptr) {
    if (n <= cap && p) return true;
    if (p) cudaFreeAsync(p, s);
    s = stream;
    p = nullptr;
    cap = 0;
    const size_t want = std::max<size_t>(n, 16);
    if (cudaMallocAsync(reinterpret_cast<void**>(&p), want * sizeof(T), s) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    cap = want;
    if (moved) *moved = true;
    return true;
  }
  ~Buf() {
    if (p) cudaFreeAsync(p, s);
  }
};

__device__ __forceinline__ int floordiv(int a, int b) {
  const int q = a / b;
  return (a % b != 0 && ((a < 0) != (b < 0))) ? q - 1 : q;
}

__global__ void k_wrap_bin(int n, int ncells, const int* __restrict__ cell_off,
                           const CellParam* __restrict__ cp, double4* __restrict__ x4,
                           int* __restrict__ ccell, int* __restrict__ bin_of,
                           int* __restrict__ bin_cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int lo = 0, hi = ncells - 1;   // cell of atom i: cell_off[c] <= i < cell_off[c+1]
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(cell_off + mid) <= i) lo = mid;
    else hi = mid - 1;
  }
  const CellParam& P = cp[lo];
  double4 x = x4[i];
  double f[3];
  int b[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double v = x.x * P.inv[k] + x.y * P.inv[3 + k] + x.z * P.inv[6 + k];
    v -= floor(v);
    if (v >= 1.0) v = 0.0;
    f[k] = v;
    b[k] = min(P.nb[k] - 1, (int)(v * P.nb[k]));
  }
  x.x = f[0] * P.lat[0] + f[1] * P.lat[3] + f[2] * P.lat[6];
  x.y = f[0] * P.lat[1] + f[1] * P.lat[4] + f[2] * P.lat[7];
  x.z = f[0] * P.lat[2] + f[1] * P.lat[5] + f[2] * P.lat[8];
  x4[i] = x;
  ccell[i] = lo;
  const int g = P.bin0 + (b[2] * P.nb[1] + b[1]) * P.nb[0] + b[0];
  bin_of[i] = g;
  atomicAdd(bin_cnt + g, 1);
}

__global__ void k_bin_fill(int n, const int* __restrict__ bin_of, const int* __restrict__ start,
                           int* __restrict__ fill, int* __restrict__ atoms) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int g = bin_of[i];
  atoms[start[g] + atomicAdd(fill + g, 1)] = i;
}

// insertion sort of each bin by atom index (bins are short)
__global__ void k_bin_sort(int nbins, const int* __restrict__ start, int* __restrict__ atoms) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nbins) return;
  const int s = start[g], e = start[g + 1];
  for (int p = s + 1; p < e; ++p) {
    const int v = atoms[p];
    int q = p - 1;
    while (q >= s && atoms[q] > v) {
      atoms[q + 1] = atoms[q];
      --q;
    }
    atoms[q + 1] = v;
  }
}

// WRITE = false: count per atom (+ total and maximum); true: write the list.
template <bool WRITE>
__global__ void k_pairs(int n, const CellParam* __restrict__ cp, const double4* __restrict__ x4,
                        const int* __restrict__ ccell, const int* __restrict__ bin_of,
                        const int* __restrict__ start, const int* __restrict__ atoms, double r2,
                        int* __restrict__ cnt, unsigned long long* __restrict__ total,
                        int* __restrict__ maxn, const int* __restrict__ off,
                        int* __restrict__ idx, int* __restrict__ img) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int c = 0;
  if (i < n) {
    const CellParam& P = cp[ccell[i]];
    const double4 xi = x4[i];
    const int lb = bin_of[i] - P.bin0;
    const int bx = lb % P.nb[0], by = (lb / P.nb[0]) % P.nb[1], bz = lb / (P.nb[0] * P.nb[1]);
    int* oi = WRITE ? idx + off[i] : nullptr;
    int* mi = WRITE ? img + off[i] : nullptr;
    for (int dz = -P.st[2]; dz <= P.st[2]; ++dz) {
      const int uz = bz + dz, n3 = floordiv(uz, P.nb[2]), wz = uz - n3 * P.nb[2];
      for (int dy = -P.st[1]; dy <= P.st[1]; ++dy) {
        const int uy = by + dy, n2 = floordiv(uy, P.nb[1]), wy = uy - n2 * P.nb[1];
        for (int dx = -P.st[0]; dx <= P.st[0]; ++dx) {
          const int ux = bx + dx, n1 = floordiv(ux, P.nb[0]), wx = ux - n1 * P.nb[0];
          const double sx = n1 * P.lat[0] + n2 * P.lat[3] + n3 * P.lat[6];
          const double sy = n1 * P.lat[1] + n2 * P.lat[4] + n3 * P.lat[7];
          const double sz = n1 * P.lat[2] + n2 * P.lat[5] + n3 * P.lat[8];
          const bool zero = (n1 | n2 | n3) == 0;
          const int code = zero ? 0 : (n1 + 512) | ((n2 + 512) << 10) | ((n3 + 512) << 20);
          const int g = P.bin0 + (wz * P.nb[1] + wy) * P.nb[0] + wx;
          const int e = start[g + 1];
          for (int p = start[g]; p < e; ++p) {
            const int j = atoms[p];
            if (zero && j == i) continue;
            const double4 xj = x4[j];
            const double ddx = xj.x + sx - xi.x, ddy = xj.y + sy - xi.y, ddz = xj.z + sz - xi.z;
            if (ddx * ddx + ddy * ddy + ddz * ddz < r2) {
              if (WRITE) {
                oi[c] = j;
                mi[c] = code;
              }
              ++c;
            }
          }
        }
      }
    }
    if (!WRITE) cnt[i] = c;
  }
  if (!WRITE) {
    // block totals, then one atomic per block
    __shared__ unsigned long long s_tot;
    __shared__ int s_max;
    if (threadIdx.x == 0) {
      s_tot = 0;
      s_max = 0;
    }
    __syncthreads();
    if (i < n) {
      atomicAdd(&s_tot, (unsigned long long)c);
      atomicMax(&s_max, c);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      atomicAdd(total, s_tot);
      atomicMax(maxn, s_max);
    }
  }
}

// ---- exclusive scan of int (three phases, 1024 elements per block)
constexpr int kScanB = 1024;

__device__ __forceinline__ int block_incl_scan(int v, int* warp_sums) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  if (lane == 31) warp_sums[w] = v;
  __syncthreads();
  if (w == 0) {
    int s = warp_sums[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += t;
    }
    warp_sums[lane] = s;
  }
  __syncthreads();
  return v + (w > 0 ? warp_sums[w - 1] : 0);
}

__global__ void k_scan_tiles(int n, const int* __restrict__ in, int* __restrict__ out,
                             int* __restrict__ tile_sums) {
  __shared__ int ws[32];
  const int i = blockIdx.x * kScanB + threadIdx.x;
  const int v = i < n ? in[i] : 0;
  const int inc = block_incl_scan(v, ws);
  if (i < n) out[i] = inc - v;
  if (threadIdx.x == kScanB - 1) tile_sums[blockIdx.x] = inc;
}

__global__ void k_scan_sums(int ntiles, int* __restrict__ tile_sums) {
  __shared__ int ws[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int b = 0; b < ntiles; b += kScanB) {
    const int i = b + threadIdx.x;
    const int v = i < ntiles ? tile_sums[i] : 0;
    const int inc = block_incl_scan(v, ws);
    const int base = carry;
    if (i < ntiles) tile_sums[i] = base + inc - v;
    __syncthreads();
    if (threadIdx.x == kScanB - 1) carry = base + inc;
    __syncthreads();
  }
}

__global__ void k_scan_add(int n, int* __restrict__ out, const int* __restrict__ tile_sums) {
  const int i = blockIdx.x * kScanB + threadIdx.x;
  if (i < n && blockIdx.x > 0) out[i] += tile_sums[blockIdx.x];
}

}  // namespace

struct mlipg_dnlist {
  cudaStream_t s = nullptr;
  int ncells = 0, natoms = 0, nbins = 0, maxn = 0;
  long long npairs = 0;
  int generation = 0;
  std::vector<CellParam> hcp;
  std::vector<int> hcell_off;
  Buf<CellParam> cp;
  Buf<double> lat;
  Buf<int> cell_off, ccell, bin_of, bin_cnt, bin_start, bin_atoms, cnt, off, tiles, idx, img, maxn_d;
  Buf<unsigned long long> total_d;
  unsigned long long* h_total = nullptr;
  int* h_maxn = nullptr;
};

static int scan(mlipg_dnlist* L, const int* in, int* out, int n) {
  const int tiles = (n + kScanB - 1) / kScanB;
  if (!L->tiles.grow(tiles, L->s)) return MLIPG_ENOMEM;
  k_scan_tiles<<<tiles, kScanB, 0, L->s>>>(n, in, out, L->tiles.p);
  k_scan_sums<<<1, kScanB, 0, L->s>>>(tiles, L->tiles.p);
  k_scan_add<<<tiles, kScanB, 0, L->s>>>(n, out, L->tiles.p);
  return cudaGetLastError() == cudaSuccess ? MLIPG_OK : MLIPG_ECUDA;
}

extern "C" int mlipg_dnlist_create(void* stream, mlipg_dnlist** out) {
  if (!out) return MLIPG_EINVAL;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return MLIPG_ENOGPU;
  }
  mlipg_dnlist* L = new mlipg_dnlist();
  L->s = static_cast<cudaStream_t>(stream);
  if (cudaHostAlloc(&L->h_total, sizeof(unsigned long long), cudaHostAllocDefault) !=
          cudaSuccess ||
      cudaHostAlloc(&L->h_maxn, sizeof(int), cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    mlipg_dnlist_destroy(L);
    return MLIPG_ENOMEM;
  }
  *out = L;
  return MLIPG_OK;
}

extern "C" int mlipg_dnlist_build(mlipg_dnlist* L, int ncells, const int* natoms,
                                  const double* lattices, void* d_x4, double rlist,
                                  int headroom_pct) {
  if (!L || ncells <= 0 || !natoms || !lattices || !d_x4 || !(rlist > 0) || headroom_pct < 0)
    return MLIPG_EINVAL;
  // per-cell bin grids
  L->hcp.assign(ncells, CellParam{});
  L->hcell_off.assign(ncells + 1, 0);
  long long nbins = 0;
  for (int c = 0; c < ncells; ++c) {
    if (natoms[c] <= 0) return MLIPG_EINVAL;
    L->hcell_off[c + 1] = L->hcell_off[c] + natoms[c];
    CellParam& P = L->hcp[c];
    const double* a = lattices + 9 * (size_t)c;
    std::memcpy(P.lat, a, sizeof P.lat);
    const double det = a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
                       a[2] * (a[3] * a[7] - a[4] * a[6]);
    if (!(std::fabs(det) > 0)) return MLIPG_EINVAL;
    double* o = P.inv;
    o[0] = (a[4] * a[8] - a[5] * a[7]) / det;
    o[1] = (a[2] * a[7] - a[1] * a[8]) / det;
    o[2] = (a[1] * a[5] - a[2] * a[4]) / det;
    o[3] = (a[5] * a[6] - a[3] * a[8]) / det;
    o[4] = (a[0] * a[8] - a[2] * a[6]) / det;
    o[5] = (a[2] * a[3] - a[0] * a[5]) / det;
    o[6] = (a[3] * a[7] - a[4] * a[6]) / det;
    o[7] = (a[1] * a[6] - a[0] * a[7]) / det;
    o[8] = (a[0] * a[4] - a[1] * a[3]) / det;
    for (int k = 0; k < 3; ++k) {
      const double* u = a + 3 * ((k + 1) % 3);
      const double* v = a + 3 * ((k + 2) % 3);
      const double c0 = u[1] * v[2] - u[2] * v[1], c1 = u[2] * v[0] - u[0] * v[2],
                   c2 = u[0] * v[1] - u[1] * v[0];
      const double w = std::fabs(det) / std::sqrt(c0 * c0 + c1 * c1 + c2 * c2);
      P.nb[k] = std::max(1, std::min(1024, (int)(w / rlist)));
      P.st[k] = (int)(rlist * P.nb[k] / w) + 1;
      if (P.st[k] > 500) return MLIPG_ENOTSUP;   // image codes hold |n| < 512
    }
    P.bin0 = (int)nbins;
    P.atom0 = L->hcell_off[c];
    P.natoms = natoms[c];
    nbins += (long long)P.nb[0] * P.nb[1] * P.nb[2];
    if (nbins > (1LL << 30)) return MLIPG_ENOTSUP;
  }
  const long long N64 = L->hcell_off[ncells];
  if (N64 > (1LL << 30)) return MLIPG_ENOTSUP;
  const int N = (int)N64, NB = (int)nbins;
  L->ncells = ncells;
  L->natoms = N;
  L->nbins = NB;
  bool moved = false;
  cudaStream_t s = L->s;
  if (!L->cp.grow(ncells, s) || !L->lat.grow(9 * (size_t)ncells, s, &moved) ||
      !L->cell_off.grow(ncells + 1, s) || !L->ccell.grow(N, s, &moved) ||
      !L->bin_of.grow(N, s) || !L->bin_cnt.grow((size_t)NB + 1, s) ||
      !L->bin_start.grow((size_t)NB + 1, s) || !L->bin_atoms.grow(N, s) ||
      !L->cnt.grow((size_t)N + 1, s) || !L->off.grow((size_t)N + 1, s, &moved) ||
      !L->maxn_d.grow(1, s) || !L->total_d.grow(1, s))
    return MLIPG_ENOMEM;
  double4* x4 = static_cast<double4*>(d_x4);
  std::vector<double> hl((size_t)9 * ncells);
  for (int c = 0; c < ncells; ++c) std::memcpy(&hl[9 * (size_t)c], L->hcp[c].lat, 9 * sizeof(double));
  const int B = 256, G = (N + B - 1) / B, GB = (NB + B - 1) / B;
  if (cudaMemcpyAsync(L->cp.p, L->hcp.data(), ncells * sizeof(CellParam), cudaMemcpyHostToDevice,
                      s) != cudaSuccess ||
      cudaMemcpyAsync(L->lat.p, hl.data(), hl.size() * sizeof(double), cudaMemcpyHostToDevice,
                      s) != cudaSuccess ||
      cudaMemcpyAsync(L->cell_off.p, L->hcell_off.data(), (ncells + 1) * sizeof(int),
                      cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemsetAsync(L->bin_cnt.p, 0, ((size_t)NB + 1) * sizeof(int), s) != cudaSuccess ||
      cudaMemsetAsync(L->cnt.p + N, 0, sizeof(int), s) != cudaSuccess ||
      cudaMemsetAsync(L->maxn_d.p, 0, sizeof(int), s) != cudaSuccess ||
      cudaMemsetAsync(L->total_d.p, 0, sizeof(unsigned long long), s) != cudaSuccess)
    return MLIPG_ECUDA;
  k_wrap_bin<<<G, B, 0, s>>>(N, ncells, L->cell_off.p, L->cp.p, x4, L->ccell.p, L->bin_of.p,
                             L->bin_cnt.p);
  int rc = scan(L, L->bin_cnt.p, L->bin_start.p, NB + 1);
  if (rc != MLIPG_OK) return rc;
  if (cudaMemsetAsync(L->bin_cnt.p, 0, ((size_t)NB + 1) * sizeof(int), s) != cudaSuccess)
    return MLIPG_ECUDA;
  k_bin_fill<<<G, B, 0, s>>>(N, L->bin_of.p, L->bin_start.p, L->bin_cnt.p, L->bin_atoms.p);
  k_bin_sort<<<GB, B, 0, s>>>(NB, L->bin_start.p, L->bin_atoms.p);
  const double r2 = rlist * rlist;
  k_pairs<false><<<G, B, 0, s>>>(N, L->cp.p, x4, L->ccell.p, L->bin_of.p, L->bin_start.p,
                                 L->bin_atoms.p, r2, L->cnt.p, L->total_d.p, L->maxn_d.p, nullptr,
                                 nullptr, nullptr);
  rc = scan(L, L->cnt.p, L->off.p, N + 1);
  if (rc != MLIPG_OK) return rc;
  if (cudaMemcpyAsync(L->h_total, L->total_d.p, sizeof(unsigned long long),
                      cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(L->h_maxn, L->maxn_d.p, sizeof(int), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    return MLIPG_ECUDA;
  }
  const unsigned long long P = *L->h_total;
  if (P > 2147483647ULL) return MLIPG_ECAPACITY;   // CSR offsets are int
  L->npairs = (long long)P;
  L->maxn = *L->h_maxn;
  if (L->idx.cap < P || !L->idx.p) {
    // grow with headroom so that later rebuilds keep the addresses
    const size_t want = std::max<size_t>((size_t)P + (size_t)P * headroom_pct / 100, 1);
    if (!L->idx.grow(want, s, &moved) || !L->img.grow(want, s, &moved)) return MLIPG_ENOMEM;
  }
  k_pairs<true><<<G, B, 0, s>>>(N, L->cp.p, x4, L->ccell.p, L->bin_of.p, L->bin_start.p,
                                L->bin_atoms.p, r2, nullptr, nullptr, nullptr, L->off.p,
                                L->idx.p, L->img.p);
  if (cudaGetLastError() != cudaSuccess) return MLIPG_ECUDA;
  if (moved) L->generation++;
  return MLIPG_OK;
}

extern "C" int mlipg_dnlist_arrays(const mlipg_dnlist* L, const int** d_off, const int** d_idx,
                                   const int** d_img, const int** d_center_cell,
                                   const double** d_cells, long long* npairs, int* max_neigh,
                                   int* generation) {
  if (!L) return MLIPG_EINVAL;
  if (d_off) *d_off = L->off.p;
  if (d_idx) *d_idx = L->idx.p;
  if (d_img) *d_img = L->img.p;
  if (d_center_cell) *d_center_cell = L->ccell.p;
  if (d_cells) *d_cells = L->lat.p;
  if (npairs) *npairs = L->npairs;
  if (max_neigh) *max_neigh = L->maxn;
  if (generation) *generation = L->generation;
  return MLIPG_OK;
}

extern "C" int mlipg_dnlist_copy(const mlipg_dnlist* L, int* off, int* idx, int* img) {
  if (!L) return MLIPG_EINVAL;
  cudaStream_t s = L->s;
  if ((off && cudaMemcpyAsync(off, L->off.p, ((size_t)L->natoms + 1) * sizeof(int),
                              cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
      (idx && L->npairs &&
       cudaMemcpyAsync(idx, L->idx.p, (size_t)L->npairs * sizeof(int), cudaMemcpyDeviceToHost,
                       s) != cudaSuccess) ||
      (img && L->npairs &&
       cudaMemcpyAsync(img, L->img.p, (size_t)L->npairs * sizeof(int), cudaMemcpyDeviceToHost,
                       s) != cudaSuccess) ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    return MLIPG_ECUDA;
  }
  return MLIPG_OK;
}

extern "C" void mlipg_dnlist_destroy(mlipg_dnlist* L) {
  if (!L) return;
  if (L->h_total) cudaFreeHost(L->h_total);
  if (L->h_maxn) cudaFreeHost(L->h_maxn);
  delete L;
}
