// C-ABI boundary of the GB300 MLIP path (declared in include/mlipg.h).
//
// The LAMMPS-facing call mlipg_compute mirrors the reference pair style's
// compute (pair_mlip_gtinv_kokkos_impl.h:272-406): it packs positions and
// element indices, flattens the full neighbour list into CSR (4 bytes per
// pair instead of the reference's 36-byte per-pair records,
// :411-599), runs the fused kernel and returns forces for owned and ghost
// atoms, the energy and the virial in LAMMPS order (mlipkk_lmp.h:942-955).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mlipg.h"
#include "kernels.cuh"
#include "model.hpp"

using namespace mlipg;

struct mlipg_handle;
void mlipg_internal_features_release(const mlipg_handle* h);   // features.cu

namespace {

thread_local std::string g_last_error;

constexpr int kNeighMask = 0x3FFFFFFF;  // LAMMPS NEIGHMASK (SBBITS = 30)
constexpr int kNbCapMax = 2048;

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t reserve(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    const size_t want = std::max<size_t>(bytes + bytes / 4, 256);
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <typename T> T* as() const { return static_cast<T*>(p); }
};

struct HostBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t reserve(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    const size_t want = std::max<size_t>(bytes + bytes / 4, 256);
    cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocDefault);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
  }
  template <typename T> T* as() const { return static_cast<T*>(p); }
};

}  // namespace

struct mlipg_handle {
  Model model;
  int precision = MLIPG_PREC_FP64;
  std::string err;
  std::vector<int> type_map;   // LAMMPS type -> element, index 0 unused, -1 = NULL
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  // model tables on the device
  DevBuf d_terms, d_units, d_unit_off, d_nl, d_nl_off, d_poly, d_poly_off, d_wlin, d_radial;
  DevBuf d_terms_f;   // the same terms with the coefficient as FP32 (mixed path)
  DevBuf d_terms_df;  // ... as a (high, low) FP32 pair (double-float path)
  DevBuf d_iunits, d_iunit_off, d_tuples, d_wlin_f, d_phase, d_adj_base, d_adj_off, d_adj;
  DevBuf d_wlin_df;
  DevBuf d_radial_rec;   // FP64 radial recurrence constants (common beta), or empty
  DevBuf d_pair_terms, d_pair_term_off, d_pair_adj, d_pair_adj_off, d_type_pairs;
  double rec_q = 0.0;
  // per-call buffers (grow only)
  DevBuf d_x4, d_centers, d_off, d_idx, d_f, d_eatom, d_vatom, d_partials, d_status, d_out8;
  DevBuf d_gexp;   // [2][kMaxTypes] adapted fixed-point exponents (mixed, double-float)
  HostBuf h_x4, h_centers, h_off, h_idx, h_f, h_eatom, h_out;
  int last_status = 0;
  const int* last_status_dev = nullptr;   // status word of the last launch (device)
  int tiling_gen = 0;   // bumped whenever the schedules on the device change
  // per-launch timing of the fused kernel (measurement support)
  bool profiling = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pending;
  std::vector<cudaEvent_t> ev_pool;
};

static int fail(mlipg_handle* h, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (h) h->err = buf;
  g_last_error = buf;
  return code;
}

static int cuda_fail(mlipg_handle* h, cudaError_t e, const char* what) {
  return fail(h, e == cudaErrorMemoryAllocation ? MLIPG_ENOMEM : MLIPG_ECUDA, "%s: %s", what,
              cudaGetErrorString(e));
}

#define CK(call, what)                                  \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, what); \
  } while (0)

// FP64 -> FP32 with IEEE overflow to +-inf (a plain cast of a value beyond
// the FP32 range is undefined in C++)
static float to_f32(double v) {
  if (std::fabs(v) > 3.4028234663852886e38) return v > 0 ? INFINITY : -INFINITY;
  return (float)v;
}

template <typename T>
static cudaError_t upload(DevBuf& b, const std::vector<T>& v, cudaStream_t s) {
  cudaError_t e = b.reserve(std::max<size_t>(v.size() * sizeof(T), 16));
  if (e != cudaSuccess || v.empty()) return e;
  return cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

static int upload_model(mlipg_handle* h) {
  const Model& M = h->model;
  std::vector<DeviceUnit> units, nl;
  std::vector<DevicePoly> poly;
  std::vector<DeviceIrrUnit> iunits;
  std::vector<DeviceTuple> tuples;
  std::vector<int> uoff(M.T + 1, 0), noff(M.T + 1, 0), poff(M.T + 1, 0), ioff(M.T + 1, 0);
  std::vector<int> abase(M.T + 1, 0), adj_off;
  std::vector<DeviceAdj> adj;
  for (int t = 0; t < M.T; ++t) {
    const Schedule& S = M.sched[t];
    ioff[t] = (int)iunits.size();
    const int tbase = (int)tuples.size();
    for (DeviceIrrUnit iu : S.iunits) {
      iu.tup += tbase;
      iunits.push_back(iu);
    }
    tuples.insert(tuples.end(), S.tuples.begin(), S.tuples.end());
    uoff[t] = (int)units.size();
    noff[t] = (int)nl.size();
    poff[t] = (int)poly.size();
    units.insert(units.end(), S.units.begin(), S.units.end());
    nl.insert(nl.end(), S.nl_units.begin(), S.nl_units.end());
    poly.insert(poly.end(), S.poly.begin(), S.poly.end());
    abase[t] = (int)adj_off.size();
    for (int v : S.adj_off) adj_off.push_back((int)adj.size() + v);
    for (int v : S.adj) {
      const DevicePoly& dp = S.poly[v >> 2];
      DeviceAdj a{};
      a.w = dp.w;
      int o = 0;
      for (int q = 0; q < dp.order; ++q)
        if (q != (v & 3)) a.other[o++] = dp.k[q];
      for (; o < kMaxPoly - 1; ++o) a.other[o] = -1;
      adj.push_back(a);
    }
  }
  ioff[M.T] = (int)iunits.size();
  uoff[M.T] = (int)units.size();
  noff[M.T] = (int)nl.size();
  poff[M.T] = (int)poly.size();
  std::vector<double> radial;
  for (auto& pr : M.pot.params) {
    radial.push_back(pr.first);
    radial.push_back(pr.second);
  }
  cudaStream_t s = h->stream;
  CK(upload(h->d_terms, M.cterms, s), "upload terms");
  {
    // FP32 coefficients for the mixed path, times Y_00^q: its spherical
    // harmonics are normalised by Y_00 = 1/(2 sqrt(pi)) (exact start of the
    // FP32 recursion), so an order-q product of its order parameters is
    // Y_00^-q times the true one
    std::vector<DeviceTerm> tf(M.cterms);
    const double y00 = 0.28209479177387814347;
    for (size_t k = 0; k < M.irr_l.size(); ++k) {
      const double sc = std::pow(y00, (double)M.irr_l[k].size());
      for (int i = M.irr_cfirst[k]; i < M.irr_cfirst[k] + M.irr_cnterms[k]; ++i) {
        const float cf = to_f32(tf[i].c * sc);
        tf[i].c = 0.0;
        std::memcpy(&tf[i].c, &cf, sizeof cf);   // low word of the 8-byte field
      }
    }
    CK(upload(h->d_terms_f, tf, s), "upload FP32 terms");
    // double-float coefficients: high word = FP32 rounding, low word = the
    // FP32 rounding of the rest (the 8-byte field's two 4-byte halves)
    std::vector<DeviceTerm> td(M.cterms);
    for (auto& t : td) {
      const float hi = to_f32(t.c), lo = to_f32(t.c - (double)hi);
      std::memcpy(reinterpret_cast<char*>(&t.c), &hi, sizeof hi);
      std::memcpy(reinterpret_cast<char*>(&t.c) + 4, &lo, sizeof lo);
    }
    CK(upload(h->d_terms_df, td, s), "upload double-float terms");
  }
  CK(upload(h->d_units, units, s), "upload units");
  CK(upload(h->d_iunits, iunits, s), "upload batched units");
  CK(upload(h->d_iunit_off, ioff, s), "upload batched unit offsets");
  CK(upload(h->d_tuples, tuples, s), "upload tuples");
  CK(upload(h->d_unit_off, uoff, s), "upload unit offsets");
  CK(upload(h->d_nl, nl, s), "upload nonlinear units");
  CK(upload(h->d_nl_off, noff, s), "upload nonlinear offsets");
  CK(upload(h->d_poly, poly, s), "upload polynomial");
  CK(upload(h->d_poly_off, poff, s), "upload polynomial offsets");
  CK(upload(h->d_adj_base, abase, s), "upload adjoint gather bases");
  CK(upload(h->d_adj_off, adj_off, s), "upload adjoint gather offsets");
  CK(upload(h->d_adj, adj, s), "upload adjoint gather lists");
  CK(upload(h->d_wlin, M.w_lin, s), "upload linear weights");
  {
    std::vector<float> wf(M.w_lin.size());
    for (size_t k = 0; k < wf.size(); ++k) wf[k] = to_f32(M.w_lin[k]);
    CK(upload(h->d_wlin_f, wf, s), "upload linear weights (FP32)");
    std::vector<float> wd(2 * M.w_lin.size());
    for (size_t k = 0; k < M.w_lin.size(); ++k) {
      wd[2 * k] = to_f32(M.w_lin[k]);
      wd[2 * k + 1] = to_f32(M.w_lin[k] - (double)wd[2 * k]);
    }
    CK(upload(h->d_wlin_df, wd, s), "upload linear weights (double-float)");
  }
  CK(upload(h->d_radial, radial, s), "upload radial parameters");
  CK(upload(h->d_gexp, std::vector<int>(2 * kMaxTypes, 0), s), "upload scale exponents");
  if (M.pot.pair) {
    CK(upload(h->d_pair_terms, M.pair_terms, s), "upload pair terms");
    CK(upload(h->d_pair_term_off, M.pair_term_off, s), "upload pair term offsets");
    CK(upload(h->d_pair_adj, M.pair_adj, s), "upload pair adjoint records");
    CK(upload(h->d_pair_adj_off, M.pair_adj_off, s), "upload pair adjoint offsets");
    CK(upload(h->d_type_pairs, M.type_pairs, s), "upload type pairs");
  }
  {
    // Common beta: f_{n+1} = f_n exp(-beta (mu_{n+1} - mu_n)(mu_{n+1} + mu_n - 2r)),
    // written with the mean spacing d as exp(2 beta d r) * K_n * exp(eps_n r),
    // eps_n = 2 beta (mu_{n+1} - mu_n - d); kept when every |eps_n| rc is so
    // small that exp(eps_n r) = 1 + eps_n r to FP64 precision.
    const auto& pr = M.pot.params;
    const int F = (int)pr.size();
    bool common = F >= 2;
    for (int n = 1; n < F && common; ++n) common = pr[n].first == pr[0].first;
    std::vector<double> rec;
    if (common) {
      const double beta = pr[0].first;
      const double d = (pr[F - 1].second - pr[0].second) / (F - 1);
      for (int n = 0; n + 1 < F; ++n) {
        const double dn = pr[n + 1].second - pr[n].second;
        const double eps = 2.0 * beta * (dn - d);
        if (std::fabs(eps) * M.pot.cutoff > 1e-9) common = false;
        rec.push_back(std::exp(-beta * dn * (pr[n + 1].second + pr[n].second)));
        rec.push_back(eps);
      }
      h->rec_q = 2.0 * beta * d;
    }
    if (!common) rec.clear();
    CK(upload(h->d_radial_rec, rec, s), "upload radial recurrence");
    if (rec.empty()) h->d_radial_rec.release();
  }
  CK(cudaStreamSynchronize(s), "model upload");
  return MLIPG_OK;
}

extern "C" {

const char* mlipg_last_error(const mlipg_handle* h) {
  if (h && !h->err.empty()) return h->err.c_str();
  return g_last_error.c_str();
}

int mlipg_create(const char* path, int precision, mlipg_handle** out) {
  if (!out || !path) return fail(nullptr, MLIPG_EINVAL, "mlipg_create: null argument");
  *out = nullptr;
  if (precision < MLIPG_PREC_FP64 || precision > MLIPG_PREC_FP64_NATIVE)
    return fail(nullptr, MLIPG_EINVAL, "unknown precision %d", precision);
  mlipg_handle* h = new mlipg_handle();
  h->precision = precision;
  std::string err;
  if (!read_potential(path, h->model.pot, err)) {
    g_last_error = err;
    delete h;
    return MLIPG_EIO;
  }
  if (!build_model(h->model, err)) {
    g_last_error = err;
    delete h;
    return MLIPG_ENOTSUP;
  }
  // default type map: LAMMPS type k -> element k-1
  h->type_map.assign(h->model.T + 1, -1);
  for (int k = 1; k <= h->model.T; ++k) h->type_map[k] = k - 1;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    // host-only handle: the model is parsed and queryable; every compute
    // call fails with MLIPG_ENOGPU
    cudaGetLastError();
    h->device = -1;
    *out = h;
    return MLIPG_OK;
  }
  cudaGetDevice(&h->device);
  cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = init_device_constants();
  if (e != cudaSuccess) {
    g_last_error = std::string("CUDA initialisation failed: ") + cudaGetErrorString(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return MLIPG_ECUDA;
  }
  int rc = upload_model(h);
  if (rc != MLIPG_OK) {
    g_last_error = h->err;
    mlipg_destroy(h);
    return rc;
  }
  *out = h;
  return MLIPG_OK;
}

int mlipg_destroy(mlipg_handle* h) {
  if (!h) return MLIPG_OK;
  if (h->device < 0) {
    delete h;
    return MLIPG_OK;
  }
  mlipg_internal_features_release(h);
  DevBuf* bufs[] = {&h->d_adj_base, &h->d_adj_off, &h->d_adj,
                    &h->d_iunits, &h->d_iunit_off, &h->d_tuples, &h->d_wlin_f, &h->d_phase,
                    &h->d_terms, &h->d_terms_f, &h->d_terms_df, &h->d_wlin_df,
                    &h->d_units, &h->d_unit_off, &h->d_nl,
                    &h->d_nl_off,
                    &h->d_poly, &h->d_poly_off, &h->d_wlin, &h->d_radial, &h->d_radial_rec,
                    &h->d_pair_terms, &h->d_pair_term_off, &h->d_pair_adj, &h->d_pair_adj_off,
                    &h->d_type_pairs,
                    &h->d_x4,
                    &h->d_centers, &h->d_off, &h->d_idx, &h->d_f, &h->d_eatom, &h->d_vatom, &h->d_partials,
                    &h->d_status, &h->d_out8, &h->d_gexp};
  for (DevBuf* b : bufs) b->release();
  for (auto& pr : h->ev_pending) h->ev_pool.insert(h->ev_pool.end(), {pr.first, pr.second});
  for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
  HostBuf* hb[] = {&h->h_x4, &h->h_centers, &h->h_off, &h->h_idx, &h->h_f, &h->h_eatom,
                   &h->h_out};
  for (HostBuf* b : hb) b->release();
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return MLIPG_OK;
}

int mlipg_set_precision(mlipg_handle* h, int precision) {
  if (!h) return fail(nullptr, MLIPG_EINVAL, "null handle");
  if (precision < MLIPG_PREC_FP64 || precision > MLIPG_PREC_FP64_NATIVE)
    return fail(h, MLIPG_EINVAL, "unknown precision %d", precision);
  h->precision = precision;
  return MLIPG_OK;
}

int mlipg_num_elements(const mlipg_handle* h) { return h ? h->model.T : 0; }

const char* mlipg_element_name(const mlipg_handle* h, int k) {
  if (!h || k < 0 || k >= h->model.T) return nullptr;
  return h->model.pot.elements[k].c_str();
}

double mlipg_element_mass(const mlipg_handle* h, int k) {
  if (!h || k < 0 || k >= h->model.T) return 0.0;
  return h->model.pot.masses[k];
}

double mlipg_cutoff(const mlipg_handle* h) { return h ? h->model.pot.cutoff : 0.0; }

int mlipg_set_type_map(mlipg_handle* h, int n, const char* const* names) {
  if (!h) return fail(nullptr, MLIPG_EINVAL, "null handle");
  if (n < 1 || !names) return fail(h, MLIPG_EINVAL, "Incorrect args for pair coefficients");
  std::vector<int> map(n + 1, -1);
  int count = 0;
  for (int k = 1; k <= n; ++k) {
    const char* s = names[k - 1];
    if (!s) return fail(h, MLIPG_EINVAL, "Incorrect args for pair coefficients");
    if (std::strcmp(s, "NULL") == 0) continue;
    int j = 0;
    for (; j < h->model.T; ++j)
      if (h->model.pot.elements[j] == s) break;
    if (j == h->model.T)
      return fail(h, MLIPG_EINVAL,
                  "No matching element in Machine Learning Interatomic Potential file");
    map[k] = j;
    ++count;
  }
  if (count == 0) return fail(h, MLIPG_EINVAL, "Incorrect args for pair coefficients");
  h->type_map = map;
  return MLIPG_OK;
}

void* mlipg_stream(mlipg_handle* h) { return h ? (void*)h->stream : nullptr; }

int mlipg_device_status(mlipg_handle* h, int* bits) {
  if (!h || !bits) return fail(h, MLIPG_EINVAL, "null argument");
  *bits = 0;
  if (h->device < 0 || !h->last_status_dev) return MLIPG_OK;
  CK(cudaStreamSynchronize(h->stream), "mlipg_device_status");
  int v = 0;
  CK(cudaMemcpy(&v, h->last_status_dev, sizeof(int), cudaMemcpyDeviceToHost), "read status");
  h->last_status = v;
  *bits = v;
  return MLIPG_OK;
}

}  // extern "C"

// Status bits of a launch -> C-ABI status code, with the handle's message.
static int status_fail(mlipg_handle* h, int bits, int nb_cap) {
  if (bits & kStatusNeighbourCapacity)
    return fail(h, MLIPG_ECAPACITY,
                "an atom has more than %d neighbours inside the cutoff (its energy and "
                "forces were skipped)",
                nb_cap);
  if (bits & kStatusBadType) return fail(h, MLIPG_EINVAL, "element index out of range");
  if (bits & kStatusAdjointRange)
    return fail(h, MLIPG_ENOTSUP, "adjoint values outside the mixed path's fixed-point range");
  return MLIPG_OK;
}

// Used by the MD, batch and serving layers after reading d_out8[7].
int mlipg_internal_status_fail(mlipg_handle* h, int bits) {
  return status_fail(h, bits, 0);
}

static int effective_nb_cap(int nb_cap) {
  return std::max(32, std::min(kNbCapMax, (nb_cap + 31) / 32 * 32));
}

static bool is_mixed(int precision) {
  return precision == MLIPG_PREC_MIXED || precision == MLIPG_PREC_MIXED_A64;
}

// Kernel instantiation of the handle's precision: MLIPG_PREC_FP64 runs the
// double-float invariant/adjoint phase when its fixed-point bound exists and
// its shared memory fits, else the all-FP64 kernel.
static int kernel_variant(const mlipg_handle* h, int nb_cap) {
  const Model& M = h->model;
  if (is_mixed(h->precision)) return kVariantF32;
  if (h->precision == MLIPG_PREC_FP64 && M.g_bound_df > 0 &&
      fused_smem_bytes(kVariantF64DF, M.T, M.L, nb_cap, std::max(M.max_nl, 1), 0) <= 227 * 1024)
    return kVariantF64DF;
  return kVariantF64;
}

// Shared-memory bytes and resident CTAs per SM of the fused kernel for this
// handle's model, precision and neighbour capacity.
static int kernel_shape(mlipg_handle* h, int nb_cap, size_t* smem, int* bps) {
  const Model& M = h->model;
  if (M.pot.pair) {
    // the radial-only kernel: FP64 in every precision, no neighbour capacity
    *smem = pair_smem_bytes(M.F, M.D);
    *bps = pair_max_blocks(*smem);
    if (*bps < 1) return fail(h, MLIPG_ENOTSUP, "pair kernel cannot be resident (smem %zu)", *smem);
    return MLIPG_OK;
  }
  const int var = kernel_variant(h, nb_cap);
  *smem = fused_smem_bytes(var, M.T, M.L, nb_cap, std::max(M.max_nl, 1),
                           var == kVariantF32 ? M.lh64 : 0);
  if (*smem > 227 * 1024)
    return fail(h, MLIPG_ENOTSUP,
                "model needs %zu bytes of shared memory per CTA (limit 232448): "
                "reduce elements, max_l or radial functions",
                *smem);
  *bps = fused_max_blocks_per_sm(var, M.L, *smem);
  if (*bps < 1) return fail(h, MLIPG_ENOTSUP, "fused kernel cannot be resident (smem %zu)", *smem);
  if (M.tiling.ctas_per_sm > 0) *bps = std::min(*bps, M.tiling.ctas_per_sm);
  return MLIPG_OK;
}

// Grid of the persistent fused kernel for ncenters centres (the number of
// per-CTA partial-sum slots a launch needs).
static int launch_grid(mlipg_handle* h, int ncenters, int nb_cap, int* grid) {
  size_t smem = 0;
  int bps = 0;
  const int rc = kernel_shape(h, effective_nb_cap(nb_cap), &smem, &bps);
  if (rc != MLIPG_OK) return rc;
  *grid = std::max(1, std::min(ncenters, bps * h->num_sms));
  return MLIPG_OK;
}

// Launches the fused kernel and the partial-sum reduction on the handle's
// stream with the given scratch: per-CTA partial sums (partial_slots rows of
// 8 doubles) and the status word.  Allocates nothing; with `timed`, brackets
// the launch with pooled CUDA events (measurement support).
static int launch_eval(mlipg_handle* h, int ncenters, const double4* x4, const int* centers,
                       const int* off, const int* idx, const int* img, const double* cell,
                       const int* center_cell, const int* fold, int nb_cap, double* f,
                       double* eatom, double* vatom, double* out8, double* partials,
                       int partial_slots, int* status, bool timed) {
  const Model& M = h->model;
  nb_cap = effective_nb_cap(nb_cap);
  const int var = kernel_variant(h, nb_cap);
  size_t smem = 0;
  int bps = 0;
  int rc = kernel_shape(h, nb_cap, &smem, &bps);
  if (rc != MLIPG_OK) return rc;
  const int grid = std::max(1, std::min(ncenters, bps * h->num_sms));
  if (grid > partial_slots)
    return fail(h, MLIPG_ECAPACITY, "launch needs %d partial-sum slots; the scratch holds %d",
                grid, partial_slots);
  CK(cudaMemsetAsync(status, 0, sizeof(int), h->stream), "memset status");
  h->last_status_dev = status;
  KernelArgs a{};
  a.x4 = x4;
  a.centers = centers;
  a.nbr_off = off;
  a.nbr_idx = idx;
  a.img = img;
  a.cell = cell;
  a.center_cell = center_cell;
  a.fold = fold;
  a.ncenters = ncenters;
  a.terms = (var == kVariantF32 ? h->d_terms_f
                                 : (var == kVariantF64DF ? h->d_terms_df : h->d_terms))
                .as<DeviceTerm>();
  a.terms64 = h->d_terms.as<DeviceTerm>();
  a.units = h->d_units.as<DeviceUnit>();
  a.unit_off = h->d_unit_off.as<int>();
  a.iunits = h->d_iunits.as<DeviceIrrUnit>();
  a.iunit_off = h->d_iunit_off.as<int>();
  a.tuples = h->d_tuples.as<DeviceTuple>();
  a.nl_units = h->d_nl.as<DeviceUnit>();
  a.nl_off = h->d_nl_off.as<int>();
  a.poly = h->d_poly.as<DevicePoly>();
  a.poly_off = h->d_poly_off.as<int>();
  a.adj_base = h->d_adj_base.as<int>();
  a.adj_off = h->d_adj_off.as<int>();
  a.adj = h->d_adj.as<DeviceAdj>();
  a.w_lin = h->d_wlin.as<double>();
  a.w_lin_f = h->d_wlin_f.as<float>();
  a.w_lin_df = h->d_wlin_df.as<float2>();
  a.phase_clocks = h->profiling ? h->d_phase.as<unsigned long long>() : nullptr;
  a.radial = h->d_radial.as<double>();
  a.pair_terms = h->d_pair_terms.as<DevicePairTerm>();
  a.pair_term_off = h->d_pair_term_off.as<int>();
  a.pair_adj = h->d_pair_adj.as<DevicePairAdj>();
  a.pair_adj_off = h->d_pair_adj_off.as<int>();
  a.type_pairs = h->d_type_pairs.as<int>();
  a.pair_nd = M.pot.pair ? M.D : 0;
  a.radial_rec = h->d_radial_rec.as<double>();
  a.rec_q = h->rec_q;
  a.T = M.T;
  a.F = M.F;
  a.L = M.L;
  a.Lh = M.Lh;
  a.nb_cap = nb_cap;
  a.nl_cap = std::max(M.max_nl, 1);
  a.rc = M.pot.cutoff;
  a.g_bound = (float)(var == kVariantF64DF ? M.g_bound_df : M.g_bound);
  a.gexp_cache = var == kVariantF64 ? nullptr
                                    : h->d_gexp.as<int>() + (var == kVariantF64DF ? kMaxTypes : 0);
  a.unit_dyn = M.tiling.warp_order == 2 ? 1 : 0;
  a.sum64 = h->precision == MLIPG_PREC_MIXED_A64 ? 1 : 0;
  a.lh64 = var == kVariantF32 ? M.lh64 : 0;
  a.f = f;
  a.eatom = eatom;
  a.vatom = vatom;
  a.partials = partials;
  a.status = status;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  if (timed && h->profiling && ncenters > 0) {
    for (cudaEvent_t* ev : {&ev0, &ev1}) {
      if (!h->ev_pool.empty()) {
        *ev = h->ev_pool.back();
        h->ev_pool.pop_back();
      } else {
        CK(cudaEventCreate(ev), "event create");
      }
    }
    CK(cudaEventRecord(ev0, h->stream), "event record");
  }
  if (ncenters > 0 && M.pot.pair) {
    CK(launch_pair(a, grid, smem, h->stream), "pair kernel launch");
  } else if (ncenters > 0) {
    CK(launch_fused(var, M.L, a, grid, smem, h->stream), "fused kernel launch");
  } else {
    CK(cudaMemsetAsync(partials, 0, 8 * sizeof(double), h->stream), "memset partials");
  }
  if (ev0) {
    CK(cudaEventRecord(ev1, h->stream), "event record");
    h->ev_pending.push_back({ev0, ev1});
  }
  CK(launch_finalize(partials, ncenters > 0 ? grid : 1, status, out8, h->stream),
     "finalize launch");
  return MLIPG_OK;
}

// The handle's own scratch (grow-only partial sums and status word).
static int run_kernel(mlipg_handle* h, int ncenters, const double4* x4, const int* centers,
                      const int* off, const int* idx, const int* img, const double* cell,
                      const int* center_cell, const int* fold, int nb_cap, double* f,
                      double* eatom, double* vatom, double* out8) {
  int grid = 0;
  const int rc = launch_grid(h, ncenters, nb_cap, &grid);
  if (rc != MLIPG_OK) return rc;
  CK(h->d_partials.reserve((size_t)grid * 8 * sizeof(double)), "alloc partials");
  CK(h->d_status.reserve(sizeof(int)), "alloc status");
  return launch_eval(h, ncenters, x4, centers, off, idx, img, cell, center_cell, fold, nb_cap, f,
                     eatom, vatom, out8, h->d_partials.as<double>(), grid,
                     h->d_status.as<int>(), true);
}

extern "C" int mlipg_compute_device(mlipg_handle* h, int ncenters, const void* d_x4,
                                    const int* d_centers, const int* d_nbr_off,
                                    const int* d_nbr_idx, const int* d_img, const double* d_cell,
                                    const int* d_center_cell, const int* d_fold, int nb_cap,
                                    double* d_f, double* d_eatom, double* d_vatom,
                                    double* d_out8) {
  if (!h) return fail(nullptr, MLIPG_EINVAL, "null handle");
  if (h->device < 0) return fail(h, MLIPG_ENOGPU, "no CUDA device is available");
  if (ncenters < 0 || (ncenters > 0 && (!d_x4 || !d_centers || !d_nbr_off || !d_nbr_idx)) ||
      !d_f || !d_out8)
    return fail(h, MLIPG_EINVAL, "mlipg_compute_device: invalid arguments");
  if (d_img && (!d_cell || !d_center_cell))
    return fail(h, MLIPG_EINVAL, "image codes need the cell lattices and centre cell ids");
  return run_kernel(h, ncenters, static_cast<const double4*>(d_x4), d_centers, d_nbr_off,
                    d_nbr_idx, d_img, d_cell, d_center_cell, d_fold, nb_cap, d_f, d_eatom,
                    d_vatom, d_out8);
}

extern "C" int mlipg_compute(mlipg_handle* h, int nlocal, int nall, const double* x,
                             const int* type, int inum, const int* ilist, const int* numneigh,
                             const int* const* firstneigh, int eflag, int vflag, double* f,
                             double* energy, double* virial, double* eatom, double* vatom) {
  if (!h) return fail(nullptr, MLIPG_EINVAL, "null handle");
  if (h->device < 0) return fail(h, MLIPG_ENOGPU, "no CUDA device is available");
  if (nlocal < 0 || nall < nlocal || inum < 0 || (nall > 0 && (!x || !type)) ||
      (inum > 0 && (!ilist || !numneigh || !firstneigh)) || (nall > 0 && !f))
    return fail(h, MLIPG_EINVAL, "mlipg_compute: invalid arguments");
  if ((eflag && !energy) || (vflag && !virial))
    return fail(h, MLIPG_EINVAL, "mlipg_compute: eflag/vflag set without output pointer");
  const int ntypes = (int)h->type_map.size() - 1;
  // pack positions and element indices
  CK(h->h_x4.reserve((size_t)std::max(nall, 1) * sizeof(double4)), "pinned x4");
  double4* hx = h->h_x4.as<double4>();
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nall; ++i) {
    const int t = type[i];
    const int e = (t >= 1 && t <= ntypes) ? h->type_map[t] : -1;
    hx[i] = double4{x[3 * i], x[3 * i + 1], x[3 * i + 2], (double)e};
  }
  // centres = owned atoms of ilist; CSR of their full lists
  CK(h->h_centers.reserve((size_t)std::max(inum, 1) * sizeof(int)), "pinned centres");
  CK(h->h_off.reserve((size_t)(inum + 1) * sizeof(int)), "pinned offsets");
  int* hc = h->h_centers.as<int>();
  int* ho = h->h_off.as<int>();
  int nc = 0, maxn = 0;
  long long np = 0;
  ho[0] = 0;
  for (int ii = 0; ii < inum; ++ii) {
    const int i = ilist[ii];
    if (i < 0 || i >= nlocal) continue;
    hc[nc] = i;
    np += numneigh[i];
    maxn = std::max(maxn, numneigh[i]);
    if (np > 2147483647LL) return fail(h, MLIPG_EINVAL, "more than 2^31 neighbour pairs");
    ho[nc + 1] = (int)np;
    ++nc;
  }
  CK(h->h_idx.reserve((size_t)std::max<long long>(np, 1) * sizeof(int)), "pinned neighbours");
  int* hi = h->h_idx.as<int>();
  int bad = -1;
#pragma omp parallel for schedule(dynamic, 1024)
  for (int c = 0; c < nc; ++c) {
    const int i = hc[c];
    const int* jl = firstneigh[i];
    int* dst = hi + ho[c];
    for (int jj = 0; jj < numneigh[i]; ++jj) {
      const int j = jl[jj] & kNeighMask;
      if (j < 0 || j >= nall) bad = j;
      dst[jj] = j;
    }
  }
  if (bad != -1) return fail(h, MLIPG_EINVAL, "neighbour index %d outside nall", bad);
  // upload
  cudaStream_t s = h->stream;
  CK(h->d_x4.reserve((size_t)std::max(nall, 1) * sizeof(double4)), "alloc x4");
  CK(h->d_centers.reserve((size_t)std::max(nc, 1) * sizeof(int)), "alloc centres");
  CK(h->d_off.reserve((size_t)(nc + 1) * sizeof(int)), "alloc offsets");
  CK(h->d_idx.reserve((size_t)std::max<long long>(np, 1) * sizeof(int)), "alloc neighbours");
  CK(h->d_f.reserve((size_t)std::max(nall, 1) * 3 * sizeof(double)), "alloc forces");
  CK(h->d_eatom.reserve((size_t)std::max(nc, 1) * sizeof(double)), "alloc eatom");
  CK(h->d_vatom.reserve((size_t)std::max(nc, 1) * 6 * sizeof(double)), "alloc vatom");
  CK(h->d_out8.reserve(8 * sizeof(double)), "alloc out");
  CK(cudaMemcpyAsync(h->d_x4.p, hx, (size_t)nall * sizeof(double4), cudaMemcpyHostToDevice, s),
     "copy x4");
  CK(cudaMemcpyAsync(h->d_centers.p, hc, (size_t)nc * sizeof(int), cudaMemcpyHostToDevice, s),
     "copy centres");
  CK(cudaMemcpyAsync(h->d_off.p, ho, (size_t)(nc + 1) * sizeof(int), cudaMemcpyHostToDevice, s),
     "copy offsets");
  if (np > 0)
    CK(cudaMemcpyAsync(h->d_idx.p, hi, (size_t)np * sizeof(int), cudaMemcpyHostToDevice, s),
       "copy neighbours");
  CK(cudaMemsetAsync(h->d_f.p, 0, (size_t)nall * 3 * sizeof(double), s), "memset forces");
  int rc = run_kernel(h, nc, h->d_x4.as<double4>(), h->d_centers.as<int>(), h->d_off.as<int>(),
                      h->d_idx.as<int>(), nullptr, nullptr, nullptr, nullptr, maxn,
                      h->d_f.as<double>(), h->d_eatom.as<double>(),
                      vatom ? h->d_vatom.as<double>() : nullptr, h->d_out8.as<double>());
  if (rc != MLIPG_OK) return rc;
  // download
  CK(h->h_f.reserve((size_t)std::max(nall, 1) * 3 * sizeof(double)), "pinned forces");
  CK(h->h_eatom.reserve((size_t)std::max(nc, 1) * 7 * sizeof(double)), "pinned eatom");
  CK(h->h_out.reserve(16 * sizeof(double)), "pinned out");
  CK(cudaMemcpyAsync(h->h_f.p, h->d_f.p, (size_t)nall * 3 * sizeof(double),
                     cudaMemcpyDeviceToHost, s),
     "copy forces");
  if (eatom)
    CK(cudaMemcpyAsync(h->h_eatom.p, h->d_eatom.p, (size_t)nc * sizeof(double),
                       cudaMemcpyDeviceToHost, s),
       "copy eatom");
  if (vatom)
    CK(cudaMemcpyAsync(h->h_eatom.as<double>() + nc, h->d_vatom.p, (size_t)nc * 6 * sizeof(double),
                       cudaMemcpyDeviceToHost, s),
       "copy vatom");
  CK(cudaMemcpyAsync(h->h_out.p, h->d_out8.p, 8 * sizeof(double), cudaMemcpyDeviceToHost, s),
     "copy energy");
  CK(cudaMemcpyAsync(h->h_out.as<double>() + 8, h->d_status.p, sizeof(int),
                     cudaMemcpyDeviceToHost, s),
     "copy status");
  CK(cudaStreamSynchronize(s), "mlipg_compute");
  int status = 0;
  std::memcpy(&status, h->h_out.as<double>() + 8, sizeof(int));
  h->last_status = status;
  if (status) return status_fail(h, status, effective_nb_cap(maxn));
  const double* hf = h->h_f.as<double>();
  const long long nf = (long long)nall * 3;
#pragma omp parallel for schedule(static)
  for (long long k = 0; k < nf; ++k) f[k] += hf[k];
  const double* o = h->h_out.as<double>();
  if (eflag) *energy = o[0];
  if (vflag) {
    // kernel order xx yy zz yz zx xy -> LAMMPS xx yy zz xy xz yz
    virial[0] = o[1];
    virial[1] = o[2];
    virial[2] = o[3];
    virial[3] = o[6];
    virial[4] = o[5];
    virial[5] = o[4];
  }
  if (eatom) {
    const double* he = h->h_eatom.as<double>();
    for (int c = 0; c < nc; ++c) eatom[hc[c]] += he[c];
  }
  if (vatom) {
    const double* hv = h->h_eatom.as<double>() + nc;
    for (int c = 0; c < nc; ++c)
      for (int k = 0; k < 6; ++k) vatom[6 * (size_t)hc[c] + k] += hv[6 * (size_t)c + k];
  }
  return MLIPG_OK;
}

extern "C" int mlipg_set_profiling(mlipg_handle* h, int on) {
  if (!h) return fail(nullptr, MLIPG_EINVAL, "null handle");
  if (on && h->device >= 0) {
    CK(h->d_phase.reserve(8 * sizeof(unsigned long long)), "alloc phase clocks");
    CK(cudaMemset(h->d_phase.p, 0, 8 * sizeof(unsigned long long)), "memset phase clocks");
  }
  h->profiling = on != 0;
  return MLIPG_OK;
}

extern "C" int mlipg_phase_cycles(mlipg_handle* h, unsigned long long* out8) {
  if (!h || !out8) return fail(h, MLIPG_EINVAL, "null argument");
  for (int k = 0; k < 8; ++k) out8[k] = 0;
  if (h->device < 0 || !h->d_phase.p) return MLIPG_OK;
  CK(cudaStreamSynchronize(h->stream), "phase clocks");
  CK(cudaMemcpy(out8, h->d_phase.p, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost),
     "copy phase clocks");
  CK(cudaMemset(h->d_phase.p, 0, 8 * sizeof(unsigned long long)), "reset phase clocks");
  return MLIPG_OK;
}

extern "C" int mlipg_kernel_times(mlipg_handle* h, float* ms, int cap) {
  if (!h || (cap > 0 && !ms)) return -1;
  int n = 0;
  for (auto& pr : h->ev_pending) {
    if (n < cap) {
      if (cudaEventSynchronize(pr.second) != cudaSuccess ||
          cudaEventElapsedTime(ms + n, pr.first, pr.second) != cudaSuccess)
        ms[n] = -1.0f;
      ++n;
    }
    h->ev_pool.push_back(pr.first);
    h->ev_pool.push_back(pr.second);
  }
  h->ev_pending.clear();
  return n;
}

extern "C" int mlipg_count_coefficients(int n_types, int model_type, int maxp, int maxl,
                                        int gtinv_order, const int* gtinv_maxl,
                                        const int* gtinv_sym, int n_fn, long long* n_coeffs,
                                        long long* n_features) {
  if (!n_coeffs || !n_features || (gtinv_order > 1 && (!gtinv_maxl || !gtinv_sym)))
    return fail(nullptr, MLIPG_EINVAL, "mlipg_count_coefficients: null argument");
  std::string err;
  if (!count_coefficients(n_types, model_type, maxp, maxl, gtinv_order, gtinv_maxl, gtinv_sym,
                          n_fn, n_coeffs, n_features, err))
    return fail(nullptr, MLIPG_EINVAL, "%s", err.c_str());
  return MLIPG_OK;
}

extern "C" int mlipg_model_info(const mlipg_handle* h, long long* out) {
  if (!h || !out) return fail(nullptr, MLIPG_EINVAL, "null argument");
  const Model& M = h->model;
  long long v[13] = {M.T, M.F, M.L, M.Lh, (long long)M.irr_l.size(), (long long)M.term_c.size(),
                     (long long)M.cterms.size(), M.n_itc, M.D, (long long)M.poly.size(),
                     M.pot.model_type, M.pot.maxp, M.max_nl};
  std::memcpy(out, v, sizeof v);
  return MLIPG_OK;
}

extern "C" long mlipg_dump_itc(const mlipg_handle* h, int* out, long cap) {
  if (!h) return -1;
  long k = 0;
  for (auto& x : h->model.itc) {
    const long q = (long)x.type_combs.size();
    if (out && k + 2 + q <= cap) {
      out[k] = x.irreps;
      out[k + 1] = (int)q;
      for (long p = 0; p < q; ++p) out[k + 2 + p] = x.type_combs[p];
    }
    k += 2 + q;
  }
  return k;
}

extern "C" long mlipg_dump_poly(const mlipg_handle* h, int* out, long cap) {
  if (!h) return -1;
  long k = 0;
  for (auto& row : h->model.poly) {
    const long q = (long)row.size();
    if (out && k + 1 + q <= cap) {
      out[k] = (int)q;
      for (long p = 0; p < q; ++p) out[k + 1 + p] = row[p];
    }
    k += 1 + q;
  }
  return k;
}

extern "C" double mlipg_flops_per_atom_step(const mlipg_handle* h, int elem, double nbar) {
  if (!h || elem < 0 || elem >= h->model.T) return 0.0;
  return flops_per_atom_step(h->model, elem, nbar);
}

extern "C" double mlipg_flops_per_atom_step_executed(const mlipg_handle* h, int elem,
                                                     double nbar) {
  if (!h || elem < 0 || elem >= h->model.T) return 0.0;
  return flops_per_atom_step(h->model, elem, nbar, true);
}


// ------------------------------------------------------------------ tiling

int mlipg_internal_tiling_generation(const mlipg_handle* h) { return h ? h->tiling_gen : 0; }

extern "C" int mlipg_set_tiling(mlipg_handle* h, int irr_chunk, int warp_order,
                                int ctas_per_sm) {
  if (!h) return fail(nullptr, MLIPG_EINVAL, "null handle");
  Model& M = h->model;
  const Tiling old = M.tiling;
  M.tiling = Tiling{irr_chunk, warp_order, ctas_per_sm};
  std::string err;
  if (!build_schedules(M, err)) {
    M.tiling = old;
    std::string e2;
    build_schedules(M, e2);
    return fail(h, MLIPG_EINVAL, "mlipg_set_tiling(%d, %d, %d): %s", irr_chunk, warp_order,
                ctas_per_sm, err.c_str());
  }
  h->tiling_gen++;
  if (h->device < 0) return MLIPG_OK;
  // the previous schedules may still be read by queued launches
  CK(cudaStreamSynchronize(h->stream), "tiling: drain stream");
  return upload_model(h);
}

extern "C" int mlipg_get_tiling(const mlipg_handle* h, int* out3) {
  if (!h || !out3) return MLIPG_EINVAL;
  out3[0] = h->model.tiling.irr_chunk;
  out3[1] = h->model.tiling.warp_order;
  out3[2] = h->model.tiling.ctas_per_sm;
  return MLIPG_OK;
}

extern "C" int mlipg_autotune(mlipg_handle* h, int ncenters, const void* d_x4,
                              const int* d_centers, const int* d_nbr_off, const int* d_nbr_idx,
                              const int* d_img, const double* d_cell, const int* d_center_cell,
                              int nb_cap, double* d_f, double* d_out8, int max_report,
                              double* report, int* nreport) {
  if (!h) return fail(nullptr, MLIPG_EINVAL, "null handle");
  if (h->device < 0) return fail(h, MLIPG_ENOGPU, "no CUDA device is available");
  if (ncenters <= 0 || !d_x4 || !d_centers || !d_nbr_off || !d_nbr_idx || !d_f || !d_out8)
    return fail(h, MLIPG_EINVAL, "mlipg_autotune: invalid arguments");
  const Model& M = h->model;
  if (M.pot.pair) {   // the radial-only kernel has no tile shape to choose
    if (nreport) *nreport = 0;
    return MLIPG_OK;
  }
  const int cap = effective_nb_cap(nb_cap);
  const int var = kernel_variant(h, cap);
  const size_t smem = fused_smem_bytes(var, M.T, M.L, cap, std::max(M.max_nl, 1),
                                       var == kVariantF32 ? M.lh64 : 0);
  const int bps_max = std::max(1, fused_max_blocks_per_sm(var, M.L, smem));
  // a sample of 16 centres per resident CTA keeps each candidate short
  const int sample = std::min(ncenters, 16 * bps_max * h->num_sms);
  const Tiling start = M.tiling;
  struct Row { int chunk, order, cps; float ms; };
  std::vector<Row> rows;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0), "event create");
  CK(cudaEventCreate(&e1), "event create");
  int rc = MLIPG_OK;
  for (int chunk : {12, 24, 48, 96})
    for (int order : {0, 1, 2})
      for (int cps = 1; cps <= bps_max && rc == MLIPG_OK; ++cps) {
        rc = mlipg_set_tiling(h, chunk, order, cps);
        if (rc != MLIPG_OK) break;
        float best = 1e30f;
        for (int rep = 0; rep < 3 && rc == MLIPG_OK; ++rep) {
          cudaEventRecord(e0, h->stream);
          rc = run_kernel(h, sample, static_cast<const double4*>(d_x4), d_centers, d_nbr_off,
                          d_nbr_idx, d_img, d_cell, d_center_cell, nullptr, nb_cap, d_f,
                          nullptr, nullptr, d_out8);
          cudaEventRecord(e1, h->stream);
          if (rc == MLIPG_OK && cudaEventSynchronize(e1) != cudaSuccess) rc = MLIPG_ECUDA;
          float ms = 0;
          if (rc == MLIPG_OK && rep > 0 && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess)
            best = std::min(best, ms);
        }
        rows.push_back({chunk, order, cps, best});
      }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != MLIPG_OK) {
    mlipg_set_tiling(h, start.irr_chunk, start.warp_order, start.ctas_per_sm);
    return rc;
  }
  const Row* best = &rows[0];
  for (const Row& r : rows)
    if (r.ms < best->ms) best = &r;
  const Row pick = *best;
  if (report)
    for (int k = 0; k < (int)rows.size() && k < max_report; ++k) {
      report[4 * k + 0] = rows[k].chunk;
      report[4 * k + 1] = rows[k].order;
      report[4 * k + 2] = rows[k].cps;
      report[4 * k + 3] = rows[k].ms;
    }
  if (nreport) *nreport = (int)rows.size();
  return mlipg_set_tiling(h, pick.chunk, pick.order, pick.cps);
}

// Support of the allocation-free entry point (noalloc.cu): the same launch as
// mlipg_compute_device, with the partial-sum and status scratch supplied by
// the caller and without touching any grow-only buffer (nothing is
// allocated here; the launch is not bracketed by profiling events).
int mlipg_internal_fail(mlipg_handle* h, int code, const char* msg) {
  return fail(h, code, "%s", msg);
}

int mlipg_internal_handle_device(const mlipg_handle* h) { return h ? h->device : -1; }
const Model* mlipg_internal_model(const mlipg_handle* h) { return h ? &h->model : nullptr; }
int mlipg_internal_num_sms(const mlipg_handle* h) { return h ? std::max(h->num_sms, 1) : 1; }

int mlipg_internal_launch_scratch(mlipg_handle* h, int ncenters, const void* d_x4,
                                  const int* d_centers, const int* d_nbr_off,
                                  const int* d_nbr_idx, const int* d_img, const double* d_cell,
                                  const int* d_center_cell, const int* d_fold, int nb_cap,
                                  double* d_f, double* d_eatom, double* d_vatom, double* d_out8,
                                  double* partials, int partial_slots, int* status) {
  if (!h) return fail(nullptr, MLIPG_EINVAL, "null handle");
  if (h->device < 0) return fail(h, MLIPG_ENOGPU, "no CUDA device is available");
  if (ncenters < 0 || (ncenters > 0 && (!d_x4 || !d_centers || !d_nbr_off || !d_nbr_idx)) ||
      !d_f || !d_out8)
    return fail(h, MLIPG_EINVAL, "mlipg_compute_device_noalloc: invalid arguments");
  if (d_img && (!d_cell || !d_center_cell))
    return fail(h, MLIPG_EINVAL, "image codes need the cell lattices and centre cell ids");
  return launch_eval(h, ncenters, static_cast<const double4*>(d_x4), d_centers, d_nbr_off,
                     d_nbr_idx, d_img, d_cell, d_center_cell, d_fold, nb_cap, d_f, d_eatom,
                     d_vatom, d_out8, partials, partial_slots, status, false);
}
