// Probe of the reference package's own standalone-compilable sources.
//
// TEST INFRASTRUCTURE ONLY.  build_ref.sh compiles this file together with
// the reference's unmodified sources (parser, coupling table, irreps x
// typecomb enumeration, polynomial index, host spherical harmonics, neighbour
// builder) into oracle/_ref/libmlipref.so.  Tests use it to pin the model
// structure, spherical harmonics and neighbour counts of both the oracle
// and the product against the reference's own code, and to regenerate the
// golden fixtures.  The reference's Kokkos kernels themselves cannot be
// built here (no Kokkos / LAMMPS), so the compute stages are pinned through
// the oracle and the regression logs instead.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "mlipkk_cell.h"
#include "mlipkk_irreps_type.h"
#include "mlipkk_polynomial.h"
#include "mlipkk_potential_parser.h"
#include "mlipkk_spherical_harmonics.h"

using namespace MLIP_NS;

namespace {
struct Loaded {
  MLIPInput in;
  std::vector<std::string> ele;
  vector1d mass, coeffs;
  Readgtinv gt;
  std::vector<IrrepsTypePair> itp;
  MLIPPolynomial* poly = nullptr;
};
Loaded* g = nullptr;
}  // namespace

extern "C" {

// Loads a potential file with the reference's parser (mlipkk_potential_parser.cpp:14-105).
int ref_load(const char* path) {
  delete g;
  g = new Loaded();
  read_potential_file(path, g->ele, g->mass, &g->in, g->coeffs, g->gt);
  g->itp = get_unique_irreps_type_pairs(g->in.n_type, g->gt.get_l_comb());
  g->poly = new MLIPPolynomial(g->in.model_type, g->in.maxp, (int)g->in.params.size(),
                               g->in.n_type, g->itp);
  return 0;
}

// [n_irreps, n_terms, ITC, D, n_coeffs, n_type, n_fn]
void ref_info(int* out) {
  out[0] = (int)g->gt.get_l_comb().size();
  out[1] = (int)g->gt.get_flatten_lm_coeffs().size();
  out[2] = (int)g->itp.size();
  out[3] = g->poly->get_n_des();
  out[4] = g->poly->get_n_coeffs();
  out[5] = g->in.n_type;
  out[6] = (int)g->in.params.size();
}

long ref_dump_itc(int* out, long cap) {
  long k = 0;
  for (auto& x : g->itp) {
    if (out && k + 2 + (long)x.type_combs.size() <= cap) {
      out[k] = x.irreps_idx;
      out[k + 1] = (int)x.type_combs.size();
      for (size_t p = 0; p < x.type_combs.size(); ++p) out[k + 2 + p] = x.type_combs[p];
    }
    k += 2 + (long)x.type_combs.size();
  }
  return k;
}

long ref_dump_poly(int* out, long cap) {
  long k = 0;
  for (auto& row : g->poly->get_polynomial_index()) {
    if (out && k + 1 + (long)row.size() <= cap) {
      out[k] = (int)row.size();
      for (size_t p = 0; p < row.size(); ++p) out[k + 1 + p] = row[p];
    }
    k += 1 + (long)row.size();
  }
  return k;
}

// term table after screening: per term [c, lm_0..lm_{q-1}] flattened as doubles
long ref_dump_terms(double* out, long cap) {
  const auto& lm = g->gt.get_flatten_lm_seq();
  const auto& c = g->gt.get_flatten_lm_coeffs();
  long k = 0;
  for (size_t t = 0; t < c.size(); ++t) {
    if (out && k + 1 + (long)lm[t].size() <= cap) {
      out[k] = c[t];
      for (size_t p = 0; p < lm[t].size(); ++p) out[k + 1 + p] = lm[t][p];
    }
    k += 1 + (long)lm[t].size();
  }
  return k;
}

void ref_coeffs(double* out) {
  for (size_t i = 0; i < g->coeffs.size(); ++i) out[i] = g->coeffs[i];
}

// Host twin of the spherical harmonics (mlipkk_spherical_harmonics.cpp).
// Outputs complex pairs indexed by LMInfoIdx.
void ref_sph(int lmax, double x, double y, double z, double* ylm, double* dx, double* dy,
             double* dz) {
  SphericalHarmonics sph(lmax);
  const double r = std::sqrt(x * x + y * y + z * z);
  vector1dc a, b, c, d;
  sph.compute_ylm(z / r, std::atan2(y, x), a);
  sph.compute_ylm_der(z / r, std::atan2(y, x), r, b, c, d);
  for (size_t k = 0; k < a.size(); ++k) {
    ylm[2 * k] = a[k].real(); ylm[2 * k + 1] = a[k].imag();
    dx[2 * k] = b[k].real(); dx[2 * k + 1] = b[k].imag();
    dy[2 * k] = c[k].real(); dy[2 * k + 1] = c[k].imag();
    dz[2 * k] = d[k].real(); dz[2 * k + 1] = d[k].imag();
  }
}

// Half neighbour list with periodic images (mlipkk_cell.cpp:218-307):
// returns the number of (i, j-image) entries within the cutoff.
long ref_count_half_pairs(int n, const double* pos, const double* lat, double cutoff) {
  vector2d coords(n, vector1d(3));
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) coords[i][k] = pos[3 * i + k];
  vector2d lattice(3, vector1d(3));
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) lattice[i][k] = lat[3 * i + k];
  vector3d disp;
  vector2i nb;
  get_neighbors(coords, lattice, cutoff, disp, nb);
  long tot = 0;
  for (auto& v : nb) tot += (long)v.size();
  return tot;
}
}
