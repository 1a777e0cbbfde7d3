// Host neighbour-list builder: owned + ghost atoms and a full list.
//
// Produces what LAMMPS hands the reference pair style ("neigh full"): the
// owned atoms followed by ghost images within the ghost cutoff (selected in
// fractional coordinates, as LAMMPS does for a triclinic box), each ghost's
// owner, and a full neighbour list (distance < cutoff) of the owned atoms in
// CSR form.  Self images are ordinary ghosts.  The reference's standalone
// builder (src/USER-MLIP/mlipkk_cell.cpp:218-307) returns a half list of
// displacement vectors instead; this one keeps LAMMPS's layout so the same
// C ABI serves both.  Binning over the bounding box of owned + ghost atoms
// with bins >= cutoff; OpenMP over owned atoms in two passes (count, fill).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/mlipg.h"

struct mlipg_nlist {
  int nlocal = 0;
  std::vector<double> x;      // [nall*3]
  std::vector<int> type;      // [nall]
  std::vector<int> owner;     // [nall]
  std::vector<int> image;     // [nall] packed image code of each atom (0 for owned)
  std::vector<int> off;       // [nlocal+1]
  std::vector<int> idx;       // [npairs]
};

namespace {

void inv3(const double* a, double* o) {
  const double det = a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
                     a[2] * (a[3] * a[7] - a[4] * a[6]);
  o[0] = (a[4] * a[8] - a[5] * a[7]) / det;
  o[1] = (a[2] * a[7] - a[1] * a[8]) / det;
  o[2] = (a[1] * a[5] - a[2] * a[4]) / det;
  o[3] = (a[5] * a[6] - a[3] * a[8]) / det;
  o[4] = (a[0] * a[8] - a[2] * a[6]) / det;
  o[5] = (a[2] * a[3] - a[0] * a[5]) / det;
  o[6] = (a[3] * a[7] - a[4] * a[6]) / det;
  o[7] = (a[1] * a[6] - a[0] * a[7]) / det;
  o[8] = (a[0] * a[4] - a[1] * a[3]) / det;
}

}  // namespace

extern "C" int mlipg_nlist_build(const double* lat, int n, const double* xin, const int* tin,
                                 double rcut, mlipg_nlist** out) {
  if (!lat || n < 0 || (n > 0 && (!xin || !tin)) || !(rcut > 0) || !out) return MLIPG_EINVAL;
  *out = nullptr;
  const double det = lat[0] * (lat[4] * lat[8] - lat[5] * lat[7]) -
                     lat[1] * (lat[3] * lat[8] - lat[5] * lat[6]) +
                     lat[2] * (lat[3] * lat[7] - lat[4] * lat[6]);
  if (!(std::fabs(det) > 0)) return MLIPG_EINVAL;
  double inv[9];
  inv3(lat, inv);  // frac = x * inv (row vector times matrix)
  // perpendicular widths
  double w[3];
  for (int k = 0; k < 3; ++k) {
    const double* a = lat + 3 * ((k + 1) % 3);
    const double* b = lat + 3 * ((k + 2) % 3);
    const double c0 = a[1] * b[2] - a[2] * b[1], c1 = a[2] * b[0] - a[0] * b[2],
                 c2 = a[0] * b[1] - a[1] * b[0];
    w[k] = std::fabs(det) / std::sqrt(c0 * c0 + c1 * c1 + c2 * c2);
  }
  double delta[3];
  int nmax[3];
  for (int k = 0; k < 3; ++k) {
    delta[k] = rcut / w[k];
    nmax[k] = (int)std::ceil(delta[k]);
    if (nmax[k] > 500) return MLIPG_ENOTSUP;
  }
  mlipg_nlist* L = new mlipg_nlist();
  L->nlocal = n;
  std::vector<double> frac((size_t)3 * n);
  for (int i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) {
      double f = xin[3 * i] * inv[k] + xin[3 * i + 1] * inv[3 + k] + xin[3 * i + 2] * inv[6 + k];
      f -= std::floor(f);
      if (f >= 1.0) f = 0.0;
      frac[3 * i + k] = f;
    }
  }
  auto cart = [&](const double* f, double* x) {
    for (int k = 0; k < 3; ++k) x[k] = f[0] * lat[k] + f[1] * lat[3 + k] + f[2] * lat[6 + k];
  };
  L->x.resize((size_t)3 * n);
  L->type.assign(tin, tin + n);
  L->owner.resize(n);
  L->image.assign(n, 0);
  for (int i = 0; i < n; ++i) {
    cart(&frac[3 * i], &L->x[3 * i]);
    L->owner[i] = i;
  }
  for (int a = -nmax[0]; a <= nmax[0]; ++a)
    for (int b = -nmax[1]; b <= nmax[1]; ++b)
      for (int c = -nmax[2]; c <= nmax[2]; ++c) {
        if (!a && !b && !c) continue;
        const int code = (a + 512) | ((b + 512) << 10) | ((c + 512) << 20);
        for (int i = 0; i < n; ++i) {
          const double f[3] = {frac[3 * i] + a, frac[3 * i + 1] + b, frac[3 * i + 2] + c};
          if (f[0] < -delta[0] || f[0] >= 1.0 + delta[0] || f[1] < -delta[1] ||
              f[1] >= 1.0 + delta[1] || f[2] < -delta[2] || f[2] >= 1.0 + delta[2])
            continue;
          double x[3];
          cart(f, x);
          L->x.insert(L->x.end(), x, x + 3);
          L->type.push_back(tin[i]);
          L->owner.push_back(i);
          L->image.push_back(code);
        }
      }
  const int nall = (int)L->type.size();
  // bins over the bounding box
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int i = 0; i < nall; ++i)
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], L->x[3 * i + k]);
      hi[k] = std::max(hi[k], L->x[3 * i + k]);
    }
  int nb[3];
  double bs[3];
  for (int k = 0; k < 3; ++k) {
    const double ext = std::max(hi[k] - lo[k], 1e-9);
    nb[k] = std::max(1, std::min(1024, (int)(ext / rcut)));
    bs[k] = ext / nb[k] * (1.0 + 1e-12);
  }
  const long nbins = (long)nb[0] * nb[1] * nb[2];
  std::vector<int> bin_of(nall), head(nbins + 1, 0), list(nall);
  for (int i = 0; i < nall; ++i) {
    int c[3];
    for (int k = 0; k < 3; ++k)
      c[k] = std::min(nb[k] - 1, std::max(0, (int)((L->x[3 * i + k] - lo[k]) / bs[k])));
    bin_of[i] = (c[2] * nb[1] + c[1]) * nb[0] + c[0];
    head[bin_of[i] + 1]++;
  }
  for (long b = 0; b < nbins; ++b) head[b + 1] += head[b];
  {
    std::vector<int> cur(head.begin(), head.end() - 1);
    for (int i = 0; i < nall; ++i) list[cur[bin_of[i]]++] = i;
  }
  const double rc2 = rcut * rcut;
  std::vector<int> cnt(n + 1, 0);
  auto visit = [&](int i, auto&& fn) {
    const int b = bin_of[i];
    const int bx = b % nb[0], by = (b / nb[0]) % nb[1], bz = b / (nb[0] * nb[1]);
    for (int dz = -1; dz <= 1; ++dz) {
      const int z = bz + dz;
      if (z < 0 || z >= nb[2]) continue;
      for (int dy = -1; dy <= 1; ++dy) {
        const int y = by + dy;
        if (y < 0 || y >= nb[1]) continue;
        for (int dx = -1; dx <= 1; ++dx) {
          const int x = bx + dx;
          if (x < 0 || x >= nb[0]) continue;
          const int bb = (z * nb[1] + y) * nb[0] + x;
          for (int p = head[bb]; p < head[bb + 1]; ++p) {
            const int j = list[p];
            if (j == i) continue;
            const double ddx = L->x[3 * j] - L->x[3 * i], ddy = L->x[3 * j + 1] - L->x[3 * i + 1],
                         ddz = L->x[3 * j + 2] - L->x[3 * i + 2];
            if (ddx * ddx + ddy * ddy + ddz * ddz < rc2) fn(j);
          }
        }
      }
    }
  };
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; ++i) {
    int c = 0;
    visit(i, [&](int) { ++c; });
    cnt[i + 1] = c;
  }
  L->off.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) L->off[i + 1] = L->off[i] + cnt[i + 1];
  L->idx.resize((size_t)L->off[n]);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; ++i) {
    int* dst = L->idx.data() + L->off[i];
    int c = 0;
    visit(i, [&](int j) { dst[c++] = j; });
    std::sort(dst, dst + c);
  }
  *out = L;
  return MLIPG_OK;
}

extern "C" int mlipg_nlist_sizes(const mlipg_nlist* L, int* nall, long long* npairs) {
  if (!L || !nall || !npairs) return MLIPG_EINVAL;
  *nall = (int)L->type.size();
  *npairs = (long long)L->idx.size();
  return MLIPG_OK;
}

extern "C" int mlipg_nlist_copy(const mlipg_nlist* L, double* x, int* type, int* owner, int* image,
                                int* off, int* idx) {
  if (!L) return MLIPG_EINVAL;
  if (x) std::memcpy(x, L->x.data(), L->x.size() * sizeof(double));
  if (type) std::memcpy(type, L->type.data(), L->type.size() * sizeof(int));
  if (owner) std::memcpy(owner, L->owner.data(), L->owner.size() * sizeof(int));
  if (image) std::memcpy(image, L->image.data(), L->image.size() * sizeof(int));
  if (off) std::memcpy(off, L->off.data(), L->off.size() * sizeof(int));
  if (idx) std::memcpy(idx, L->idx.data(), L->idx.size() * sizeof(int));
  return MLIPG_OK;
}

extern "C" void mlipg_nlist_destroy(mlipg_nlist* L) { delete L; }
