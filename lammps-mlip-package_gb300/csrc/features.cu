// Training features of a structure on the GPU, in FP64: the quantities a
// potential is fitted to.  The energy, forces and stress of the linearized
// MLIP are linear in its regression coefficients w:
//   E = sum_i P_i . w,   F_k = FF_k . w,   stress = SF . w,
// with P_i,p = prod_{f in p} d_i,f the polynomial features of atom i (d the
// structural features), FF the force features and SF the stress features.
// This replaces the reference's MLIPModel::prepare_features and its getters
// (src/USER-MLIP/mlipkk.cpp:461-470, 609-666, 992-1281, 1322-1381).
//
// Four kernels on the handle's stream, one periodic cell with an
// image-coded full list built on the device (no ghost atoms):
//   feat_order_params  one CTA per centre: a[t][n][lm] for all m (m > 0 from
//                      a_{l,-m} = (-1)^m conj(a_{l,m})), mlipkk.cpp:538-607
//   feat_structural    one thread per (centre, feature): d = sum_terms
//                      Re(c prod a), mlipkk.cpp:628-663
//   feat_polynomial    one thread per (centre, coefficient): P = prod d,
//                      mlipkk.cpp:1167-1179
//   feat_pairs         one CTA per centre, its neighbours in turn: Y_lm and
//                      dY_lm of the pair, the derivative of every feature of
//                      the centre with respect to the pair displacement
//                      (the reference's dirj, mlipkk.cpp:1054-1150), then per
//                      coefficient dP/dr_ij = sum_nu dirj(f_nu) prod_{nu'}
//                      d(f_nu'), scattered as FF[i] += , FF[j] -= and
//                      SF -= r_ij (x) dP/dr_ij (mlipkk.cpp:1217-1273).
// The owner-computes form (each centre handles its own half of every pair)
// sums to the reference's half-list result.  Uses the raw (unfolded)
// coupling table, so every term follows the reference's conventions
// directly; the training path is not the throughput path.
#define MLIPG_REAL double
#define MLIPG_TAG feat
#define MLIPG_NO_FUSED
#include "kernel_impl.cuh"

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mlipg.h"

namespace mlipg {
namespace feat {
namespace {

struct FeatTerm {        // 24 bytes
  double c;
  uint16_t lm[kMaxOrder];   // LMIdx l^2 + l + m of each slot
  uint16_t pad[2];
};
struct FeatItc {         // 24 bytes
  int irreps, q, term0, nterm;
  uint8_t tc[kMaxOrder];
  uint8_t inter;         // bit t: the feature exists for a centre of element t
  uint8_t pad;
};
struct FeatPoly {        // 20 bytes
  int f[kMaxPoly];       // feature indices (n * n_itc + itc), -1 past the order
  int order;
};

struct FeatArgs {
  const double4* x4;
  const int* off;
  const int* idx;
  const int* img;
  const double* cell;
  int n;                 // centres (= atoms of the cell)
  const FeatItc* itc;
  const FeatTerm* terms;
  const FeatPoly* poly;
  const int* other_type;  // [TC][T]
  const int* type_pairs;  // [T][T]
  const double* radial;
  int T, F, L, Lh, La, n_itc, D, C;
  double rc;
  double2* a;            // [n][T][16][La]
  double* d;             // [n][D]
  double* p;             // [n][C]
  double* ff;            // [n][C][3], accumulated
  double* sf;            // [C][6], accumulated
  double* dirj;          // [grid][D][3] scratch
  int* status;
};

__device__ __forceinline__ bool disp(const FeatArgs& A, int k, const double4& xi,
                                     const double4& xj, double& dx, double& dy, double& dz) {
  dx = xj.x - xi.x;
  dy = xj.y - xi.y;
  dz = xj.z - xi.z;
  const int code = A.img[k];
  if (code != 0) {
    const double n1 = (double)((code & 1023) - 512);
    const double n2 = (double)(((code >> 10) & 1023) - 512);
    const double n3 = (double)(((code >> 20) & 1023) - 512);
    const double* L = A.cell;
    dx += n1 * L[0] + n2 * L[3] + n3 * L[6];
    dy += n1 * L[1] + n2 * L[4] + n3 * L[7];
    dz += n1 * L[2] + n2 * L[5] + n3 * L[8];
  }
  const double r2 = dx * dx + dy * dy + dz * dz;
  return r2 > 0.0 && r2 <= A.rc * A.rc;
}

struct YStage {            // Y_lm of one neighbour into ys[lmh * kChunk + slot]
  double2* ys;
  int slot;
  __device__ __forceinline__ void operator()(int lmh, int, double yre, double yim, double,
                                             double, double, double, double, double) {
    ys[lmh * kChunk + slot] = double2{yre, yim};
  }
};

struct YdStage {           // Y_lm and its gradient of one pair
  double2 *y, *dx, *dy, *dz;
  __device__ __forceinline__ void operator()(int lmh, int, double yre, double yim, double xre,
                                             double xim, double yyre, double yyim, double zre,
                                             double zim) {
    y[lmh] = double2{yre, yim};
    dx[lmh] = double2{xre, xim};
    dy[lmh] = double2{yyre, yyim};
    dz[lmh] = double2{zre, zim};
  }
};

// a[t][n][lm] of every centre (FP64 sums over its neighbours of element t)
template <int LCAP>
__global__ void __launch_bounds__(kBlock) feat_order_params(const __grid_constant__ FeatArgs A) {
  constexpr int LS = (LCAP + 1) * (LCAP + 2) / 2;
  extern __shared__ __align__(16) unsigned char smem[];
  double2* ys = reinterpret_cast<double2*>(smem);                 // [LS][kChunk]
  double* fs = reinterpret_cast<double*>(ys + LS * kChunk);       // [kChunk][16]
  int* ej = reinterpret_cast<int*>(fs + kChunk * kNPad);          // [kChunk]
  double2* acc = reinterpret_cast<double2*>(ej + kChunk);         // [T][16][Lh]
  const int tid = threadIdx.x, T = A.T, Lh = A.Lh;
  const int nent = T * kNPad * Lh;
  for (int c = blockIdx.x; c < A.n; c += gridDim.x) {
    const double4 xi = A.x4[c];
    for (int e = tid; e < nent; e += kBlock) acc[e] = double2{0.0, 0.0};
    const int o0 = A.off[c], o1 = A.off[c + 1];
    __syncthreads();
    for (int cb = o0; cb < o1; cb += kChunk) {
      const int csz = min(kChunk, o1 - cb);
      if (tid < csz) {
        const int k = cb + tid;
        const int j = A.idx[k];
        const double4 xj = A.x4[j];
        double dx, dy, dz;
        const int tj = (int)xj.w;
        int e = -1;
        if (disp(A, k, xi, xj, dx, dy, dz)) {
          if (tj >= 0 && tj < T) {
            e = tj;
            const double r = sqrt(dx * dx + dy * dy + dz * dz);
            double f[kNPad], fd[kNPad];
            radial(A.radial, A.F, r, A.rc, f, fd, false);
#pragma unroll
            for (int q = 0; q < kNPad; ++q) fs[tid * kNPad + q] = f[q];
            YStage v{ys, tid};
            sh_visit<LCAP, false>(dx, dy, dz, r, A.L, v);
          } else if (tj >= T) {
            atomicOr(A.status, kStatusBadType);
          }
        }
        ej[tid] = e;
      }
      __syncthreads();
      for (int e = tid; e < nent; e += kBlock) {
        const int t = e / (kNPad * Lh), rem = e % (kNPad * Lh);
        const int n = rem / Lh, lmh = rem % Lh;
        double2 s = acc[e];
        for (int jj = 0; jj < csz; ++jj) {
          if (ej[jj] != t) continue;
          const double fv = fs[jj * kNPad + n];
          const double2 y = ys[lmh * kChunk + jj];
          s.x = fma(fv, y.x, s.x);
          s.y = fma(-fv, y.y, s.y);
        }
        acc[e] = s;
      }
      __syncthreads();
    }
    // all m: a_{l,m} for m <= 0 from the sums, a_{l,-m} = (-1)^m conj(a_{l,m})
    double2* out = A.a + (size_t)c * T * kNPad * A.La;
    for (int e = tid; e < T * kNPad * A.La; e += kBlock) {
      const int tn = e / A.La, lm = e % A.La;
      int l = 0;
      while ((l + 1) * (l + 1) <= lm) ++l;
      const int m = lm - l * l - l;
      const int lmh = l * (l + 1) / 2 + l - (m < 0 ? -m : m);
      const double2 v = acc[tn * Lh + lmh];
      if (m <= 0) out[e] = v;
      else out[e] = (m & 1) ? double2{-v.x, v.y} : double2{v.x, -v.y};
    }
    __syncthreads();
  }
}

// d[c][f] = sum_terms Re(c_term prod_p a[c][other(tc_p, t_c)][n][lm_p])
__global__ void __launch_bounds__(kBlock) feat_structural(const __grid_constant__ FeatArgs A) {
  const int c = blockIdx.y;
  const int f = blockIdx.x * kBlock + threadIdx.x;
  if (f >= A.D) return;
  const int ti = (int)A.x4[c].w;
  double v = 0.0;
  const int itc = f % A.n_itc, n = f / A.n_itc;
  const FeatItc it = A.itc[itc];
  if (ti >= 0 && ti < A.T && ((it.inter >> ti) & 1)) {
    const double2* a = A.a + (size_t)c * A.T * kNPad * A.La;
    int sl[kMaxOrder];
    for (int p = 0; p < it.q; ++p) sl[p] = (A.other_type[it.tc[p] * A.T + ti] * kNPad + n) * A.La;
    for (int k = it.term0; k < it.term0 + it.nterm; ++k) {
      const FeatTerm tm = A.terms[k];
      double pr = tm.c, pi = 0.0;
      for (int p = 0; p < it.q; ++p) {
        const double2 x = a[sl[p] + tm.lm[p]];
        const double tr = pr * x.x - pi * x.y;
        pi = pr * x.y + pi * x.x;
        pr = tr;
      }
      v += pr;
    }
  }
  A.d[(size_t)c * A.D + f] = v;
}

// P[c][p] = prod_{f in p} d[c][f]
__global__ void __launch_bounds__(kBlock) feat_polynomial(const __grid_constant__ FeatArgs A) {
  const int c = blockIdx.y;
  const int p = blockIdx.x * kBlock + threadIdx.x;
  if (p >= A.C) return;
  const FeatPoly pl = A.poly[p];
  double v = 1.0;
  for (int q = 0; q < pl.order; ++q) v *= A.d[(size_t)c * A.D + pl.f[q]];
  A.p[(size_t)c * A.C + p] = v;
}

// For each centre and each of its neighbours: dirj of every feature, then the
// force and stress features of every coefficient.
template <int LCAP>
__global__ void __launch_bounds__(kBlock) feat_pairs(const __grid_constant__ FeatArgs A) {
  constexpr int LS = (LCAP + 1) * (LCAP + 2) / 2;
  __shared__ double2 sy[LS], sdx[LS], sdy[LS], sdz[LS];
  __shared__ double sf_[kNPad], sfd[kNPad], sr[4];
  __shared__ int sj, stc;
  const int tid = threadIdx.x, T = A.T;
  double* dirj = A.dirj + (size_t)blockIdx.x * A.D * 3;
  for (int c = blockIdx.x; c < A.n; c += gridDim.x) {
    const double4 xi = A.x4[c];
    const int ti = (int)xi.w;
    if (ti < 0 || ti >= T) continue;
    const double* dc = A.d + (size_t)c * A.D;
    const double2* ac = A.a + (size_t)c * T * kNPad * A.La;
    for (int k = A.off[c]; k < A.off[c + 1]; ++k) {
      if (tid == 0) {
        const int j = A.idx[k];
        const double4 xj = A.x4[j];
        const int tj = (int)xj.w;
        double dx, dy, dz;
        const bool ok = disp(A, k, xi, xj, dx, dy, dz) && tj >= 0 && tj < T;
        sj = ok ? j : -1;
        if (ok) {
          const double r = sqrt(dx * dx + dy * dy + dz * dz);
          sr[0] = dx; sr[1] = dy; sr[2] = dz; sr[3] = r;
          stc = A.type_pairs[ti * T + tj];
          double f[kNPad], fd[kNPad];
          radial(A.radial, A.F, r, A.rc, f, fd, true);
          for (int q = 0; q < kNPad; ++q) { sf_[q] = f[q]; sfd[q] = fd[q]; }
          YdStage v{sy, sdx, sdy, sdz};
          sh_visit<LCAP, true>(dx, dy, dz, r, A.L, v);
        }
      }
      __syncthreads();
      if (sj < 0) {
        __syncthreads();   // every thread has read sj before thread 0 rewrites it
        continue;
      }
      const double dx = sr[0], dy = sr[1], dz = sr[2], invr = 1.0 / sr[3];
      const int tcij = stc;
      // dirj of every feature of the centre (mlipkk.cpp:1054-1150)
      for (int f = tid; f < A.D; f += kBlock) {
        const int itc = f % A.n_itc, n = f / A.n_itc;
        const FeatItc it = A.itc[itc];
        double g0 = 0.0, g1 = 0.0, g2 = 0.0;
        if ((it.inter >> ti) & 1) {
          for (int kk = it.term0; kk < it.term0 + it.nterm; ++kk) {
            const FeatTerm tm = A.terms[kk];
            for (int mu = 0; mu < it.q; ++mu) {
              if (it.tc[mu] != tcij) continue;
              double pr = tm.c, pi = 0.0;
              for (int mu2 = 0; mu2 < it.q; ++mu2) {
                if (mu2 == mu) continue;
                const int t2 = A.other_type[it.tc[mu2] * T + ti];
                const double2 x = ac[(t2 * kNPad + n) * A.La + tm.lm[mu2]];
                const double tr = pr * x.x - pi * x.y;
                pi = pr * x.y + pi * x.x;
                pr = tr;
              }
              const int lm = tm.lm[mu];
              int l = 0;
              while ((l + 1) * (l + 1) <= lm) ++l;
              const int m = lm - l * l - l;
              const int lmh = l * (l + 1) / 2 + l - (m < 0 ? -m : m);
              double2 y = sy[lmh], yx = sdx[lmh], yy = sdy[lmh], yz = sdz[lmh];
              if (m > 0) {   // (l, m) from (l, -m): (-1)^m conj
                const double sm = (m & 1) ? -1.0 : 1.0;
                y = double2{sm * y.x, -sm * y.y};
                yx = double2{sm * yx.x, -sm * yx.y};
                yy = double2{sm * yy.x, -sm * yy.y};
                yz = double2{sm * yz.x, -sm * yz.y};
              }
              const double f1r = sfd[n] * y.x, f1i = sfd[n] * y.y, fn = sf_[n];
              // conj(f' Y r_hat + f dY), then Re(tmp * that)
              const double bxr = f1r * dx * invr + fn * yx.x, bxi = -(f1i * dx * invr + fn * yx.y);
              const double byr = f1r * dy * invr + fn * yy.x, byi = -(f1i * dy * invr + fn * yy.y);
              const double bzr = f1r * dz * invr + fn * yz.x, bzi = -(f1i * dz * invr + fn * yz.y);
              g0 += pr * bxr - pi * bxi;
              g1 += pr * byr - pi * byi;
              g2 += pr * bzr - pi * bzi;
            }
          }
        }
        dirj[(size_t)f * 3] = g0;
        dirj[(size_t)f * 3 + 1] = g1;
        dirj[(size_t)f * 3 + 2] = g2;
      }
      __syncthreads();
      // force and stress features (mlipkk.cpp:1217-1273)
      const int j = sj;
      for (int p = tid; p < A.C; p += kBlock) {
        const FeatPoly pl = A.poly[p];
        double t0 = 0.0, t1 = 0.0, t2 = 0.0;
        for (int nu = 0; nu < pl.order; ++nu) {
          double prod = 1.0;
          for (int nu2 = 0; nu2 < pl.order; ++nu2)
            if (nu2 != nu) prod *= dc[pl.f[nu2]];
          const double* g = dirj + (size_t)pl.f[nu] * 3;
          t0 += g[0] * prod;
          t1 += g[1] * prod;
          t2 += g[2] * prod;
        }
        if (t0 == 0.0 && t1 == 0.0 && t2 == 0.0) continue;
        if (A.ff) {
          double* fi = A.ff + ((size_t)c * A.C + p) * 3;
          double* fj = A.ff + ((size_t)j * A.C + p) * 3;
          atomicAdd(fi, t0); atomicAdd(fi + 1, t1); atomicAdd(fi + 2, t2);
          atomicAdd(fj, -t0); atomicAdd(fj + 1, -t1); atomicAdd(fj + 2, -t2);
        }
        if (A.sf) {
          double* s = A.sf + (size_t)p * 6;
          atomicAdd(s, -dx * t0); atomicAdd(s + 1, -dy * t1); atomicAdd(s + 2, -dz * t2);
          atomicAdd(s + 3, -dy * t2); atomicAdd(s + 4, -dz * t0); atomicAdd(s + 5, -dx * t1);
        }
      }
      __syncthreads();
    }
  }
}

size_t order_params_smem(int L, int T) {
  const int lcap = L <= 6 ? 6 : (L <= 12 ? 12 : (L <= 16 ? 16 : 20));
  const size_t LS = (size_t)(lcap + 1) * (lcap + 2) / 2;
  return LS * kChunk * sizeof(double2) + kChunk * kNPad * sizeof(double) +
         kChunk * sizeof(int) + (size_t)T * kNPad * LS * sizeof(double2);
}

template <int LCAP>
cudaError_t launch_lcap(const FeatArgs& A, int grid, bool pairs, cudaStream_t s) {
  const size_t smem = order_params_smem(LCAP, A.T);
  cudaError_t e = cudaFuncSetAttribute(feat_order_params<LCAP>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  feat_order_params<LCAP><<<grid, kBlock, smem, s>>>(A);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  feat_structural<<<dim3((A.D + kBlock - 1) / kBlock, A.n), kBlock, 0, s>>>(A);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (A.p) {
    feat_polynomial<<<dim3((A.C + kBlock - 1) / kBlock, A.n), kBlock, 0, s>>>(A);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (pairs) {
    feat_pairs<LCAP><<<grid, kBlock, 0, s>>>(A);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

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

// model tables of the feature path, built once per handle
struct Tables {
  Dev<FeatTerm> terms;
  Dev<FeatItc> itc;
  Dev<FeatPoly> poly;
  Dev<int> other_type, type_pairs;
  Dev<double> radial;
};

std::mutex g_mu;
std::map<const mlipg_handle*, Tables*> g_tables;
bool g_constants[64] = {};

}  // namespace
}  // namespace feat
}  // namespace mlipg

using namespace mlipg;

const Model* mlipg_internal_model(const mlipg_handle* h);
int mlipg_internal_num_sms(const mlipg_handle* h);
int mlipg_internal_handle_device(const mlipg_handle* h);
int mlipg_internal_fail(mlipg_handle* h, int code, const char* msg);
int mlipg_internal_status_fail(mlipg_handle* h, int bits);

// Called by mlipg_destroy: the feature tables of the handle.
void mlipg_internal_features_release(const mlipg_handle* h) {
  std::lock_guard<std::mutex> lock(feat::g_mu);
  auto it = feat::g_tables.find(h);
  if (it == feat::g_tables.end()) return;
  delete it->second;
  feat::g_tables.erase(it);
}

static feat::Tables* feature_tables(mlipg_handle* h, cudaStream_t s, int* rc) {
  std::lock_guard<std::mutex> lock(feat::g_mu);
  auto it = feat::g_tables.find(h);
  if (it != feat::g_tables.end()) return it->second;
  const Model& M = *mlipg_internal_model(h);
  const int dev = mlipg_internal_handle_device(h);
  if (dev >= 0 && dev < 64 && !feat::g_constants[dev]) {
    if (feat::init_constants() != cudaSuccess) {
      *rc = MLIPG_ECUDA;
      return nullptr;
    }
    feat::g_constants[dev] = true;
  }
  std::vector<feat::FeatTerm> terms(M.term_c.size());
  for (size_t k = 0; k < terms.size(); ++k) {
    terms[k] = feat::FeatTerm{};
    terms[k].c = M.term_c[k];
    for (size_t p = 0; p < M.term_lm[k].size(); ++p) terms[k].lm[p] = (uint16_t)M.term_lm[k][p];
  }
  std::vector<feat::FeatItc> itc(M.n_itc);
  for (int i = 0; i < M.n_itc; ++i) {
    const ITC& x = M.itc[i];
    itc[i] = feat::FeatItc{};
    itc[i].irreps = x.irreps;
    itc[i].q = (int)x.type_combs.size();
    itc[i].term0 = M.irr_first[x.irreps];
    itc[i].nterm = M.irr_nterms[x.irreps];
    for (int p = 0; p < itc[i].q; ++p) itc[i].tc[p] = (uint8_t)x.type_combs[p];
    for (int t = 0; t < M.T; ++t)
      if (x.inter[t]) itc[i].inter |= (uint8_t)(1u << t);
  }
  std::vector<feat::FeatPoly> poly(M.poly.size());
  for (size_t p = 0; p < poly.size(); ++p) {
    for (int q = 0; q < kMaxPoly; ++q) poly[p].f[q] = -1;
    poly[p].order = (int)M.poly[p].size();
    for (int q = 0; q < poly[p].order; ++q) poly[p].f[q] = M.poly[p][q];
  }
  std::vector<double> radial;
  for (auto& pr : M.pot.params) {
    radial.push_back(pr.first);
    radial.push_back(pr.second);
  }
  feat::Tables* t = new feat::Tables();
  bool ok = t->terms.alloc(terms.size(), s) == cudaSuccess &&
            t->itc.alloc(itc.size(), s) == cudaSuccess &&
            t->poly.alloc(poly.size(), s) == cudaSuccess &&
            t->other_type.alloc(M.other_type.size(), s) == cudaSuccess &&
            t->type_pairs.alloc(M.type_pairs.size(), s) == cudaSuccess &&
            t->radial.alloc(radial.size(), s) == cudaSuccess;
  const auto up = [&](void* d, const void* src, size_t bytes) {
    if (ok && bytes) ok = cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, s) == cudaSuccess;
  };
  up(t->terms.p, terms.data(), terms.size() * sizeof(feat::FeatTerm));
  up(t->itc.p, itc.data(), itc.size() * sizeof(feat::FeatItc));
  up(t->poly.p, poly.data(), poly.size() * sizeof(feat::FeatPoly));
  up(t->other_type.p, M.other_type.data(), M.other_type.size() * sizeof(int));
  up(t->type_pairs.p, M.type_pairs.data(), M.type_pairs.size() * sizeof(int));
  up(t->radial.p, radial.data(), radial.size() * sizeof(double));
  if (ok) ok = cudaStreamSynchronize(s) == cudaSuccess;   // the host vectors die here
  if (!ok) {
    cudaGetLastError();
    delete t;
    *rc = MLIPG_ECUDA;
    return nullptr;
  }
  feat::g_tables[h] = t;
  return t;
}

extern "C" int mlipg_feature_sizes(const mlipg_handle* h, long long* n_structural,
                                   long long* n_polynomial) {
  if (!h || !n_structural || !n_polynomial) return MLIPG_EINVAL;
  const Model& M = *mlipg_internal_model(h);
  *n_structural = M.D;
  *n_polynomial = (long long)M.poly.size();
  return MLIPG_OK;
}

extern "C" int mlipg_features(mlipg_handle* h, int natoms, const double* lattice9,
                              const double* x, const int* elements, double* structural,
                              double* polynomial, double* force, double* stress) {
  if (!h) return MLIPG_EINVAL;
  if (natoms <= 0 || !lattice9 || !x || !elements)
    return mlipg_internal_fail(h, MLIPG_EINVAL, "mlipg_features: invalid arguments");
  cudaStream_t s = static_cast<cudaStream_t>(mlipg_stream(h));
  if (!s) return mlipg_internal_fail(h, MLIPG_ENOGPU, "no CUDA device is available");
  const Model& M = *mlipg_internal_model(h);
  if (M.pot.pair)
    return mlipg_internal_fail(h, MLIPG_ENOTSUP,
                               "mlipg_features: training features are defined for invariant "
                               "(gtinv) potentials");
  for (int i = 0; i < natoms; ++i)
    if (elements[i] < 0 || elements[i] >= M.T)
      return mlipg_internal_fail(h, MLIPG_EINVAL, "mlipg_features: element index out of range");
  if (feat::order_params_smem(M.L, M.T) > 227 * 1024)
    return mlipg_internal_fail(h, MLIPG_ENOTSUP,
                               "mlipg_features: order parameters of this model exceed shared "
                               "memory (fewer elements or a lower max_l)");
  int rc = MLIPG_OK;
  feat::Tables* tab = feature_tables(h, s, &rc);
  if (!tab) return mlipg_internal_fail(h, rc, "mlipg_features: table upload failed");
  const int C = (int)M.poly.size(), D = M.D, La = (M.L + 1) * (M.L + 1);
  const bool pairs = force || stress;
  const int grid = std::max(1, std::min(natoms, 2 * mlipg_internal_num_sms(h)));
  feat::Dev<double4> x4;
  feat::Dev<double2> a;
  feat::Dev<double> d, p, ff, sf, dirj;
  feat::Dev<int> status;
  bool ok = x4.alloc(natoms, s) == cudaSuccess &&
            a.alloc((size_t)natoms * M.T * kNPad * La, s) == cudaSuccess &&
            d.alloc((size_t)natoms * D, s) == cudaSuccess &&
            status.alloc(1, s) == cudaSuccess;
  if (ok && polynomial) ok = p.alloc((size_t)natoms * C, s) == cudaSuccess;
  if (ok && force) ok = ff.alloc((size_t)natoms * C * 3, s) == cudaSuccess;
  if (ok && stress) ok = sf.alloc((size_t)C * 6, s) == cudaSuccess;
  if (ok && pairs) ok = dirj.alloc((size_t)grid * D * 3, s) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    return mlipg_internal_fail(h, MLIPG_ENOMEM, "mlipg_features: device allocation failed");
  }
  std::vector<double4> hx4(natoms);
  for (int i = 0; i < natoms; ++i)
    hx4[i] = double4{x[3 * (size_t)i], x[3 * (size_t)i + 1], x[3 * (size_t)i + 2],
                     (double)elements[i]};
  ok = cudaMemcpyAsync(x4.p, hx4.data(), natoms * sizeof(double4), cudaMemcpyHostToDevice, s) ==
           cudaSuccess &&
       cudaMemsetAsync(status.p, 0, sizeof(int), s) == cudaSuccess &&
       (!force || cudaMemsetAsync(ff.p, 0, (size_t)natoms * C * 3 * sizeof(double), s) ==
                      cudaSuccess) &&
       (!stress || cudaMemsetAsync(sf.p, 0, (size_t)C * 6 * sizeof(double), s) == cudaSuccess);
  if (!ok) {
    cudaGetLastError();
    return mlipg_internal_fail(h, MLIPG_ECUDA, "mlipg_features: upload failed");
  }
  mlipg_dnlist* nl = nullptr;
  rc = mlipg_dnlist_create(s, &nl);
  if (rc == MLIPG_OK) rc = mlipg_dnlist_build(nl, 1, &natoms, lattice9, x4.p, M.pot.cutoff, 0);
  if (rc != MLIPG_OK) {
    mlipg_dnlist_destroy(nl);
    return mlipg_internal_fail(h, rc, "mlipg_features: neighbour list build failed");
  }
  feat::FeatArgs A{};
  mlipg_dnlist_arrays(nl, &A.off, &A.idx, &A.img, nullptr, &A.cell, nullptr, nullptr, nullptr);
  A.x4 = x4.p;
  A.n = natoms;
  A.itc = tab->itc.p;
  A.terms = tab->terms.p;
  A.poly = tab->poly.p;
  A.other_type = tab->other_type.p;
  A.type_pairs = tab->type_pairs.p;
  A.radial = tab->radial.p;
  A.T = M.T;
  A.F = M.F;
  A.L = M.L;
  A.Lh = M.Lh;
  A.La = La;
  A.n_itc = M.n_itc;
  A.D = D;
  A.C = C;
  A.rc = M.pot.cutoff;
  A.a = a.p;
  A.d = d.p;
  A.p = polynomial ? p.p : nullptr;
  A.ff = force ? ff.p : nullptr;
  A.sf = stress ? sf.p : nullptr;
  A.dirj = dirj.p;
  A.status = status.p;
  cudaError_t e;
  if (M.L <= 6) e = feat::launch_lcap<6>(A, grid, pairs, s);
  else if (M.L <= 12) e = feat::launch_lcap<12>(A, grid, pairs, s);
  else if (M.L <= 16) e = feat::launch_lcap<16>(A, grid, pairs, s);
  else e = feat::launch_lcap<20>(A, grid, pairs, s);
  int st = 0;
  if (e == cudaSuccess && structural)
    e = cudaMemcpyAsync(structural, d.p, (size_t)natoms * D * sizeof(double),
                        cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && polynomial)
    e = cudaMemcpyAsync(polynomial, p.p, (size_t)natoms * C * sizeof(double),
                        cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && force)
    e = cudaMemcpyAsync(force, ff.p, (size_t)natoms * C * 3 * sizeof(double),
                        cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && stress)
    e = cudaMemcpyAsync(stress, sf.p, (size_t)C * 6 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&st, status.p, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  mlipg_dnlist_destroy(nl);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return mlipg_internal_fail(h, MLIPG_ECUDA, cudaGetErrorString(e));
  }
  if (st) return mlipg_internal_status_fail(h, st);
  return MLIPG_OK;
}
