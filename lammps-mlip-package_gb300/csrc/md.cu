// Device-resident NVE molecular dynamics around the MLIP force evaluation.
//
// Velocity Verlet exactly as LAMMPS `fix nve` integrates it (the integrator
// of the reference's regression runs, test/regression/*.in): per step
//   v += dtf f / m ; x += dt v ; F = F(x) ; v += dtf f / m,
// dtf = dt/2 * ftm2v, in LAMMPS metal units (A, ps, eV, g/mol).  Forces come
// from the fused kernel through mlipg_compute_device with a full neighbour
// list of owned atoms whose entries carry periodic image codes (no ghost
// atoms), built on the device with cutoff + skin and rebuilt there when an
// atom has moved more than skin/2 since the last build.  Each step is one CUDA graph launch
// (integrate, zero forces, fused kernel, reduction, integrate, displacement
// check) on the handle's stream.  Thermo (temperature, pressure tensor, total
// energy) follows LAMMPS's `thermo_temp` / `pressure` computes: dof = 3N-3.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/mlipg.h"

// Changes whenever the handle's work schedules are rebuilt (autotuning):
// a captured step holds their device addresses and launch shape.
int mlipg_internal_tiling_generation(const mlipg_handle* h);
// Maps the fused kernel's status bits (d_out8[7]) to a C-ABI status code and
// sets the handle's message.
int mlipg_internal_status_fail(mlipg_handle* h, int bits);

namespace {

constexpr double kFtm2v = 1.0 / 1.0364269e-4;  // metal units
constexpr double kMvv2e = 1.0364269e-4;
constexpr double kBoltz = 8.617343e-5;
constexpr double kNktv2p = 1.6021765e6;

__global__ void k_initial(int n, double4* x4, double* v, const double* f, const double* minv,
                          double dtf, double dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double s = dtf * minv[i];
  double4 p = x4[i];
  const double vx = v[3 * i] + s * f[3 * i];
  const double vy = v[3 * i + 1] + s * f[3 * i + 1];
  const double vz = v[3 * i + 2] + s * f[3 * i + 2];
  v[3 * i] = vx;
  v[3 * i + 1] = vy;
  v[3 * i + 2] = vz;
  p.x += dt * vx;
  p.y += dt * vy;
  p.z += dt * vz;
  x4[i] = p;
}

__global__ void k_final(int n, double* v, const double* f, const double* minv, double dtf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double s = dtf * minv[i];
  v[3 * i] += s * f[3 * i];
  v[3 * i + 1] += s * f[3 * i + 1];
  v[3 * i + 2] += s * f[3 * i + 2];
}

__global__ void k_disp_check(int n, const double4* x4, const double* xref, double thr2,
                             int* flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double dx = x4[i].x - xref[3 * i], dy = x4[i].y - xref[3 * i + 1],
               dz = x4[i].z - xref[3 * i + 2];
  if (dx * dx + dy * dy + dz * dz > thr2) atomicOr(flag, 1);
}

// kinetic tensor sum m v_a v_b (xx yy zz xy xz yz), one block, fixed order
__global__ void k_kinetic(int n, const double* v, const double* mass, double* out6) {
  __shared__ double red[6][256];
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double m = mass[i], vx = v[3 * i], vy = v[3 * i + 1], vz = v[3 * i + 2];
    s[0] += m * vx * vx; s[1] += m * vy * vy; s[2] += m * vz * vz;
    s[3] += m * vx * vy; s[4] += m * vx * vz; s[5] += m * vy * vz;
  }
  for (int k = 0; k < 6; ++k) red[k][threadIdx.x] = s[k];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int k = 0; k < 6; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 6) out6[threadIdx.x] = red[threadIdx.x][0];
}

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    if (count <= n) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) n = std::max<size_t>(count, 1);
    return e;
  }
  ~DBuf() {
    if (p) cudaFree(p);
  }
};

}  // namespace

struct mlipg_md {
  mlipg_handle* h = nullptr;
  cudaStream_t s = nullptr;
  int n = 0;
  double lat[9];
  double volume = 0;
  double skin = 0;
  double rc = 0;
  int nb_cap = 0;
  long long rebuilds = 0;
  std::vector<int> elem;
  std::vector<double> mass;
  DBuf<double4> x4;
  DBuf<double> v, f, minv, m, xref, out8, kin6;
  DBuf<int> centers, flag;
  mlipg_dnlist* nl = nullptr;   // device neighbour lists (image-coded, rc + skin)
  int nl_gen = -1;
  cudaGraphExec_t graph = nullptr;
  double graph_dt = 0;
  int graph_tiling = 0;   // schedule generation the graph was captured with
  int* hflag = nullptr;      // pinned: rebuild flag, then (at +8 bytes) the status of the step
  double* hstat = nullptr;
};

#define MCK(call)                                                               \
  do {                                                                          \
    if ((call) != cudaSuccess) {                                                \
      cudaGetLastError();                                                       \
      return MLIPG_ECUDA;                                                       \
    }                                                                           \
  } while (0)

__global__ void k_set_ref(int n, const double4* __restrict__ x4, double* __restrict__ xref) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double4 p = x4[i];
  xref[3 * i] = p.x;
  xref[3 * i + 1] = p.y;
  xref[3 * i + 2] = p.z;
}

static void md_drop_graph(mlipg_md* md) {
  if (md->graph) {
    cudaGraphExecDestroy(md->graph);
    md->graph = nullptr;
  }
}

// (Re)builds the image-coded full list on the device from the positions in
// x4 (uploaded from `x` first when given): wraps them into the cell and
// records them as the displacement reference.  A captured step stays valid
// unless a list array moved or the longest list outgrew the kernel's
// neighbour capacity.
static int md_build_list(mlipg_md* md, const double* x) {
  if (x) {
    std::vector<double4> x4(md->n);
    for (int i = 0; i < md->n; ++i)
      x4[i] = double4{x[3 * (size_t)i], x[3 * (size_t)i + 1], x[3 * (size_t)i + 2],
                      (double)md->elem[i]};
    MCK(md->x4.alloc(md->n));
    MCK(md->xref.alloc((size_t)md->n * 3));
    MCK(cudaMemcpyAsync(md->x4.p, x4.data(), md->n * sizeof(double4), cudaMemcpyHostToDevice,
                        md->s));
  }
  const int rc = mlipg_dnlist_build(md->nl, 1, &md->n, md->lat, md->x4.p, md->rc + md->skin, 20);
  if (rc != MLIPG_OK) return rc;
  k_set_ref<<<(md->n + 255) / 256, 256, 0, md->s>>>(md->n, md->x4.p, md->xref.p);
  MCK(cudaGetLastError());
  int maxn = 0, gen = 0;
  mlipg_dnlist_arrays(md->nl, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, &maxn, &gen);
  if (maxn > md->nb_cap) {
    md->nb_cap = maxn + maxn / 8;   // headroom: later rebuilds keep the captured step
    md_drop_graph(md);
  }
  if (gen != md->nl_gen) {
    md->nl_gen = gen;
    md_drop_graph(md);
  }
  return MLIPG_OK;
}

static int md_forces(mlipg_md* md) {
  MCK(cudaMemsetAsync(md->f.p, 0, (size_t)md->n * 3 * sizeof(double), md->s));
  const int *off = nullptr, *idx = nullptr, *img = nullptr, *ccell = nullptr;
  const double* cell = nullptr;
  mlipg_dnlist_arrays(md->nl, &off, &idx, &img, &ccell, &cell, nullptr, nullptr, nullptr);
  return mlipg_compute_device(md->h, md->n, md->x4.p, md->centers.p, off, idx, img, cell, ccell,
                              nullptr, md->nb_cap, md->f.p, nullptr, nullptr, md->out8.p);
}

// enqueues one velocity-Verlet step on the stream
static int md_enqueue_step(mlipg_md* md, double dt) {
  const int B = 256, G = (md->n + B - 1) / B;
  const double dtf = 0.5 * dt * kFtm2v;
  k_initial<<<G, B, 0, md->s>>>(md->n, md->x4.p, md->v.p, md->f.p, md->minv.p, dtf, dt);
  int rc = md_forces(md);
  if (rc != MLIPG_OK) return rc;
  k_final<<<G, B, 0, md->s>>>(md->n, md->v.p, md->f.p, md->minv.p, dtf);
  const double thr = 0.5 * md->skin;
  k_disp_check<<<G, B, 0, md->s>>>(md->n, md->x4.p, md->xref.p, thr * thr, md->flag.p);
  MCK(cudaGetLastError());
  return MLIPG_OK;
}

extern "C" int mlipg_md_create(mlipg_handle* h, const double* lattice9, int natoms,
                               const double* x, const double* v, const int* elements,
                               double skin, mlipg_md** out) {
  if (!h || !lattice9 || natoms <= 0 || !x || !elements || skin < 0 || !out) return MLIPG_EINVAL;
  *out = nullptr;
  mlipg_md* md = new mlipg_md();
  md->h = h;
  md->s = static_cast<cudaStream_t>(mlipg_stream(h));
  if (!md->s) {
    delete md;
    return MLIPG_ENOGPU;
  }
  md->n = natoms;
  std::memcpy(md->lat, lattice9, sizeof md->lat);
  const double* L = md->lat;
  md->volume = std::fabs(L[0] * (L[4] * L[8] - L[5] * L[7]) - L[1] * (L[3] * L[8] - L[5] * L[6]) +
                         L[2] * (L[3] * L[7] - L[4] * L[6]));
  md->skin = skin;
  md->rc = mlipg_cutoff(h);
  const int ne = mlipg_num_elements(h);
  md->elem.assign(elements, elements + natoms);
  md->mass.resize(natoms);
  std::vector<double> minv(natoms);
  for (int i = 0; i < natoms; ++i) {
    if (elements[i] < 0 || elements[i] >= ne) {
      delete md;
      return MLIPG_EINVAL;
    }
    md->mass[i] = mlipg_element_mass(h, elements[i]);
    minv[i] = 1.0 / md->mass[i];
  }
  std::vector<int> cent(natoms);
  for (int i = 0; i < natoms; ++i) cent[i] = i;
  std::vector<double> vv((size_t)natoms * 3, 0.0);
  if (v) std::memcpy(vv.data(), v, vv.size() * sizeof(double));
  if (md->v.alloc(vv.size()) != cudaSuccess || md->f.alloc(vv.size()) != cudaSuccess ||
      md->minv.alloc(natoms) != cudaSuccess || md->m.alloc(natoms) != cudaSuccess ||
      md->out8.alloc(8) != cudaSuccess || md->kin6.alloc(6) != cudaSuccess ||
      md->centers.alloc(natoms) != cudaSuccess || md->flag.alloc(1) != cudaSuccess ||
      mlipg_dnlist_create(md->s, &md->nl) != MLIPG_OK ||
      cudaHostAlloc(&md->hflag, 16, cudaHostAllocDefault) != cudaSuccess) {
    mlipg_md_destroy(md);
    return MLIPG_ENOMEM;
  }
  md->hstat = reinterpret_cast<double*>(reinterpret_cast<char*>(md->hflag) + 8);
  cudaMemcpyAsync(md->v.p, vv.data(), vv.size() * sizeof(double), cudaMemcpyHostToDevice, md->s);
  cudaMemcpyAsync(md->minv.p, minv.data(), natoms * sizeof(double), cudaMemcpyHostToDevice, md->s);
  cudaMemcpyAsync(md->m.p, md->mass.data(), natoms * sizeof(double), cudaMemcpyHostToDevice,
                  md->s);
  cudaMemcpyAsync(md->centers.p, cent.data(), natoms * sizeof(int), cudaMemcpyHostToDevice, md->s);
  cudaMemsetAsync(md->flag.p, 0, sizeof(int), md->s);
  int rc = md_build_list(md, x);
  if (rc == MLIPG_OK) rc = md_forces(md);
  if (rc == MLIPG_OK &&
      (cudaMemcpyAsync(md->hstat, md->out8.p + 7, sizeof(double), cudaMemcpyDeviceToHost,
                       md->s) != cudaSuccess ||
       cudaStreamSynchronize(md->s) != cudaSuccess))
    rc = MLIPG_ECUDA;
  if (rc == MLIPG_OK && *md->hstat != 0.0) rc = mlipg_internal_status_fail(h, (int)*md->hstat);
  if (rc != MLIPG_OK) {
    mlipg_md_destroy(md);
    return rc;
  }
  *out = md;
  return MLIPG_OK;
}

extern "C" int mlipg_md_run(mlipg_md* md, int nsteps, double dt, int use_graph) {
  if (!md || nsteps < 0 || !(dt > 0)) return MLIPG_EINVAL;
  if (md->graph &&
      (md->graph_dt != dt || md->graph_tiling != mlipg_internal_tiling_generation(md->h))) {
    cudaGraphExecDestroy(md->graph);
    md->graph = nullptr;
  }
  for (int step = 0; step < nsteps; ++step) {
    int rc;
    const bool eager = !(use_graph && md->graph);
    if (eager) {
      rc = md_enqueue_step(md, dt);
      if (rc != MLIPG_OK) return rc;
    } else {
      MCK(cudaGraphLaunch(md->graph, md->s));
    }
    MCK(cudaMemcpyAsync(md->hflag, md->flag.p, sizeof(int), cudaMemcpyDeviceToHost, md->s));
    MCK(cudaMemcpyAsync(md->hstat, md->out8.p + 7, sizeof(double), cudaMemcpyDeviceToHost,
                        md->s));
    MCK(cudaStreamSynchronize(md->s));
    // the force evaluation of this step raised a status bit (neighbour
    // capacity, element index, adjoint range): its forces are incomplete
    if (*md->hstat != 0.0) return mlipg_internal_status_fail(md->h, (int)*md->hstat);
    if (*md->hflag) {
      // an atom moved more than skin/2: rebuild on the device
      rc = md_build_list(md, nullptr);
      if (rc != MLIPG_OK) return rc;
      MCK(cudaMemsetAsync(md->flag.p, 0, sizeof(int), md->s));
      MCK(cudaStreamSynchronize(md->s));
      ++md->rebuilds;
    } else if (use_graph && !md->graph && step + 1 < nsteps) {
      // every buffer the launch path uses exists now: capture one step
      cudaGraph_t g = nullptr;
      MCK(cudaStreamBeginCapture(md->s, cudaStreamCaptureModeThreadLocal));
      rc = md_enqueue_step(md, dt);
      const cudaError_t ec = cudaStreamEndCapture(md->s, &g);
      if (rc != MLIPG_OK || ec != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return rc != MLIPG_OK ? rc : MLIPG_ECUDA;
      }
      const cudaError_t e = cudaGraphInstantiate(&md->graph, g, 0);
      cudaGraphDestroy(g);
      MCK(e);
      md->graph_dt = dt;
      md->graph_tiling = mlipg_internal_tiling_generation(md->h);
    }
  }
  MCK(cudaStreamSynchronize(md->s));
  return MLIPG_OK;
}

extern "C" int mlipg_md_state(mlipg_md* md, double* x, double* v, double* f) {
  if (!md) return MLIPG_EINVAL;
  MCK(cudaStreamSynchronize(md->s));
  if (x) {
    std::vector<double4> x4(md->n);
    MCK(cudaMemcpy(x4.data(), md->x4.p, md->n * sizeof(double4), cudaMemcpyDeviceToHost));
    for (int i = 0; i < md->n; ++i) {
      x[3 * i] = x4[i].x;
      x[3 * i + 1] = x4[i].y;
      x[3 * i + 2] = x4[i].z;
    }
  }
  if (v) MCK(cudaMemcpy(v, md->v.p, (size_t)md->n * 3 * sizeof(double), cudaMemcpyDeviceToHost));
  if (f) MCK(cudaMemcpy(f, md->f.p, (size_t)md->n * 3 * sizeof(double), cudaMemcpyDeviceToHost));
  return MLIPG_OK;
}

// Autotunes the handle's tile shape on this system, then recomputes the
// forces at the current positions (the tuning launches overwrite them).
extern "C" int mlipg_md_autotune(mlipg_md* md, int max_report, double* report, int* nreport) {
  if (!md) return MLIPG_EINVAL;
  const int *off = nullptr, *idx = nullptr, *img = nullptr, *ccell = nullptr;
  const double* cell = nullptr;
  mlipg_dnlist_arrays(md->nl, &off, &idx, &img, &ccell, &cell, nullptr, nullptr, nullptr);
  int rc = mlipg_autotune(md->h, md->n, md->x4.p, md->centers.p, off, idx, img, cell, ccell,
                          md->nb_cap, md->f.p, md->out8.p, max_report, report, nreport);
  if (rc != MLIPG_OK) return rc;
  rc = md_forces(md);
  if (rc != MLIPG_OK) return rc;
  MCK(cudaMemcpyAsync(md->hstat, md->out8.p + 7, sizeof(double), cudaMemcpyDeviceToHost, md->s));
  MCK(cudaStreamSynchronize(md->s));
  if (*md->hstat != 0.0) return mlipg_internal_status_fail(md->h, (int)*md->hstat);
  return MLIPG_OK;
}

// out[0..10]: potential energy, kinetic energy, temperature (K), total energy,
// pressure (bar), Pxx Pyy Pzz Pxy Pxz Pyz (bar), number of list rebuilds
extern "C" int mlipg_md_thermo(mlipg_md* md, double* out12) {
  if (!md || !out12) return MLIPG_EINVAL;
  k_kinetic<<<1, 256, 0, md->s>>>(md->n, md->v.p, md->m.p, md->kin6.p);
  double kin[6], o8[8];
  MCK(cudaMemcpyAsync(kin, md->kin6.p, 6 * sizeof(double), cudaMemcpyDeviceToHost, md->s));
  MCK(cudaMemcpyAsync(o8, md->out8.p, 8 * sizeof(double), cudaMemcpyDeviceToHost, md->s));
  MCK(cudaStreamSynchronize(md->s));
  const double ke = 0.5 * (kin[0] + kin[1] + kin[2]) * kMvv2e;
  const double dof = 3.0 * md->n - 3.0;
  const double temp = dof > 0 ? 2.0 * ke / (dof * kBoltz) : 0.0;
  // fused-kernel virial order xx yy zz yz zx xy -> LAMMPS xx yy zz xy xz yz
  const double w[6] = {o8[1], o8[2], o8[3], o8[6], o8[5], o8[4]};
  const double inv = 1.0 / md->volume;
  out12[0] = o8[0];
  out12[1] = ke;
  out12[2] = temp;
  out12[3] = o8[0] + ke;
  out12[4] = (dof * kBoltz * temp + w[0] + w[1] + w[2]) / 3.0 * inv * kNktv2p;
  for (int k = 0; k < 6; ++k) out12[5 + k] = (kin[k] * kMvv2e + w[k]) * inv * kNktv2p;
  out12[11] = (double)md->rebuilds;
  return MLIPG_OK;
}

extern "C" void mlipg_md_destroy(mlipg_md* md) {
  if (!md) return;
  if (md->graph) cudaGraphExecDestroy(md->graph);
  if (md->hflag) cudaFreeHost(md->hflag);
  mlipg_dnlist_destroy(md->nl);
  delete md;
}
