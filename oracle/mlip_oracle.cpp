// CPU oracle for the linearized-MLIP (gtinv) energy / force / virial path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: tests, the smoke
// check and the CPU-baseline leg of bench.py call it through ctypes to
// obtain reference results.  The product library never links or calls it.
//
// It restates, in plain serial/OpenMP FP64 C++, the algorithm of the
// reference package's Kokkos pair style on a LAMMPS full neighbour list
// with ghost atoms ("neigh full newton on"):
//   potential file      src/USER-MLIP/mlipkk_potential_parser.cpp:14-105
//   table screening     src/USER-MLIP/mlipkk_gtinv_data_reader.cpp:18-76
//   irreps x typecomb   src/USER-MLIP/mlipkk_irreps_type.cpp:48-100
//   polynomial index    src/USER-MLIP/mlipkk_polynomial.cpp:12-208
//   combinations        src/USER-MLIP/mlipkk_utils.cpp:5-98
//   spherical harm.     src/USER-MLIP/mlipkk_spherical_harmonics_kk.h:10-177
//   radial basis        src/USER-MLIP/mlipkk_features_kk.h:9-48
//   sph. coefficients   src/USER-MLIP/mlipkk.cpp:199-272
//   order parameters    src/USER-MLIP/mlipkk_lmp.h:314-387
//   invariants          src/USER-MLIP/mlipkk_lmp.h:407-469
//   energy              src/USER-MLIP/mlipkk_lmp.h:489-537
//   polynomial adjoint  src/USER-MLIP/mlipkk_lmp.h:557-625
//   basis adjoint       src/USER-MLIP/mlipkk_lmp.h:645-733
//   forces / stress     src/USER-MLIP/mlipkk_lmp.h:753-922
//   virial reorder      src/USER-MLIP/mlipkk_lmp.h:942-955
// with the same loop order and complex-product association, so results agree
// with the reference to rounding of the summation order.
//
// Potentials of the radial-only descriptor (des_type "pair", the reference's
// `pair_style mlip_pair`) follow the legacy pair style instead:
//   file reader          src/USER-MLIP/mlip_model.h:31-112 (coefficients x2/scale)
//   enumeration          src/USER-MLIP/mlip_model_params.cpp:26-81, 180-213
//   power terms          src/USER-MLIP/mlip_polynomial.cpp:33-43
//   energy and forces    src/USER-MLIP/pair_mlip_pair.cpp:56-264
// restated in the owner-computes form (orc_pair_compute).
//
// A second entry point, orc_compute_centers, evaluates the same physics for
// a subset of centre atoms in the owner-computes form (each centre scatters
// only its own adjoint onto its neighbours).  It is used to time the CPU
// baseline on a bounded sample of a large workload.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <queue>
#include <set>
#include <sstream>
#include <string>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct cplx {
  double re, im;
};
inline cplx cmul(cplx a, cplx b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
inline cplx cscale(cplx a, double s) { return {a.re * s, a.im * s}; }
// Re(lhs * rhs), mlipkk_lmp.h:962-966
inline double prod_real(cplx l, cplx r) { return l.re * r.re - l.im * r.im; }

using vi = std::vector<int>;
using vvi = std::vector<vi>;
using vd = std::vector<double>;

std::string g_err;

// ---------------------------------------------------------------- parser
struct Potential {
  bool pair = false;              // des_type "pair" (radial-only descriptor)
  std::vector<std::string> elements;
  double cutoff = 0;
  int model_type = 0, maxp = 0, maxl = 0, gtinv_order = 0;
  vi gtinv_maxl;
  std::vector<int> gtinv_sym;
  vd coeffs;                      // already divided by the scales
  std::vector<std::pair<double, double>> params;  // (beta, mu)
  vd masses;
};

bool next_line(std::ifstream& in, std::string& line) {
  if (!std::getline(in, line)) return false;
  return true;
}

// Each value line: the first tokens are parsed, trailing comments ignored
// (mlipkk_utils.h:25-54).
bool read_potential(const char* path, Potential& p) {
  std::ifstream in(path);
  if (!in) { g_err = std::string("cannot open potential file ") + path; return false; }
  std::string line;
  // line 1: element names, then a trailing "# element" comment
  if (!next_line(in, line)) { g_err = "empty potential file"; return false; }
  {
    std::stringstream ss(line);
    std::string tok;
    while (ss >> tok) {
      if (tok[0] == '#') break;
      p.elements.push_back(tok);
    }
  }
  auto get_line = [&](std::stringstream& ss) -> bool {
    std::string l;
    if (!next_line(in, l)) { g_err = "truncated potential file"; return false; }
    ss.str(l); ss.clear();
    return true;
  };
  std::stringstream ss;
  if (!get_line(ss)) return false;
  ss >> p.cutoff;
  std::string s;
  if (!get_line(ss)) return false;
  ss >> s;
  if (s != "gaussian") { g_err = "Unknown pair_type: " + s; return false; }
  if (!get_line(ss)) return false;
  ss >> s;
  if (s != "gtinv" && s != "pair") { g_err = "Unsupported des_type: " + s; return false; }
  p.pair = s == "pair";
  if (!get_line(ss)) return false;
  ss >> p.model_type;
  if (!get_line(ss)) return false;
  ss >> p.maxp;
  if (!get_line(ss)) return false;
  ss >> p.maxl;
  if (p.pair) {
    // the pair descriptor's file has no invariant lines (mlip_model.h:61-74)
    p.gtinv_order = 1;
  } else {
    if (!get_line(ss)) return false;
    ss >> p.gtinv_order;
    const int nm = p.gtinv_order - 1;
    if (!get_line(ss)) return false;
    p.gtinv_maxl.assign(nm, 0);
    for (int k = 0; k < nm; ++k) ss >> p.gtinv_maxl[k];
    if (!get_line(ss)) return false;
    p.gtinv_sym.assign(nm, 0);
    for (int k = 0; k < nm; ++k) ss >> p.gtinv_sym[k];
  }
  int nc = 0;
  if (!get_line(ss)) return false;
  ss >> nc;
  p.coeffs.assign(nc, 0.0);
  if (!get_line(ss)) return false;
  for (int k = 0; k < nc; ++k) ss >> p.coeffs[k];
  if (!get_line(ss)) return false;
  for (int k = 0; k < nc; ++k) {
    double sc = 1.0;
    ss >> sc;
    p.coeffs[k] /= sc;
  }
  int npar = 0;
  if (!get_line(ss)) return false;
  ss >> npar;
  for (int k = 0; k < npar; ++k) {
    if (!get_line(ss)) return false;
    double b = 0, m = 0;
    ss >> b >> m;
    p.params.push_back({b, m});
  }
  if (!get_line(ss)) return false;
  p.masses.assign(p.elements.size(), 0.0);
  for (auto& m : p.masses) ss >> m;
  return true;
}

// ---------------------------------------------------------------- table
struct Table {
  vvi l;
  std::vector<vvi> m;
  std::vector<vd> c;
};

bool read_table(const char* path, Table& t) {
  std::ifstream in(path);
  if (!in) { g_err = std::string("cannot open table ") + path; return false; }
  std::string line;
  std::vector<std::string> toks;
  std::string tok;
  // gather tokens skipping comment lines
  std::stringstream all;
  while (std::getline(in, line)) {
    if (!line.empty() && line[0] == '#') continue;
    all << line << '\n';
  }
  int n = 0;
  all >> n;
  t.l.resize(n); t.m.resize(n); t.c.resize(n);
  for (int i = 0; i < n; ++i) {
    int q = 0; all >> q;
    t.l[i].resize(q);
    for (int k = 0; k < q; ++k) all >> t.l[i][k];
    int nt = 0; all >> nt;
    t.m[i].assign(nt, vi(q));
    t.c[i].assign(nt, 0.0);
    for (int j = 0; j < nt; ++j) {
      all >> t.c[i][j];
      for (int k = 0; k < q; ++k) all >> t.m[i][j][k];
    }
  }
  if (!all) { g_err = "malformed coupling table"; return false; }
  return true;
}

// ---------------------------------------------------------------- model
struct ITC {
  int irreps;
  vi type_combs;
  std::vector<char> inter;   // inter[type]
};

struct Model {
  Potential pot;
  int T = 0, TC = 0, F = 0, L = 0, Lh = 0, La = 0;
  // screened irreps
  vvi irr_l;
  vi irr_first, irr_nterms;
  vvi term_lm;     // IrrepsTermIdx -> LMIdx per slot
  vd term_c;
  std::vector<ITC> itc;
  int ITC_n = 0, D = 0;
  vvi poly;        // PolynomialIdx -> FeatureIdx list
  vvi other_type;  // [tc][type]
  vvi type_pairs;  // [t1][t2] -> tc
  vd sphA, sphB;   // indexed by lm2i(l, m)
  vi lm_l, lm_m;   // LMIdx -> l, m
  vi lh_l, lh_m;   // LMInfoIdx -> l, m (m <= 0)
};

inline int lm2i(int l, int m) { return l * (l + 1) / 2 + m; }

// mlipkk_gtinv_data_reader.cpp:18-76
void screen(const Table& tab, const Potential& p, Model& M) {
  int count_terms = 0;
  for (size_t i = 0; i < tab.l.size(); ++i) {
    const vi& lc = tab.l[i];
    const int order = (int)lc.size();
    const int maxl = lc.back();
    bool req = true;
    if (order > 1) {
      if (order > p.gtinv_order || maxl > p.gtinv_maxl[order - 2]) req = false;
      else if (p.gtinv_sym[order - 2]) {
        int ne = (int)std::count(lc.begin(), lc.end(), lc[0]);
        if (ne != order) req = false;
      }
    }
    if (!req) continue;
    M.irr_l.push_back(lc);
    M.irr_first.push_back(count_terms);
    M.irr_nterms.push_back((int)tab.m[i].size());
    for (size_t j = 0; j < tab.m[i].size(); ++j) {
      vi lm(order);
      for (int k = 0; k < order; ++k) lm[k] = lc[k] * lc[k] + lc[k] + tab.m[i][j][k];
      M.term_lm.push_back(lm);
      M.term_c.push_back(tab.c[i][j]);
      ++count_terms;
    }
  }
}

std::vector<std::pair<int, int>> type_pairs_mapping(int T) {
  std::vector<std::pair<int, int>> v;
  for (int a = 0; a < T; ++a)
    for (int b = a; b < T; ++b) v.push_back({a, b});
  return v;
}

// mlipkk_irreps_type.cpp:21-35
std::vector<char> type_intersection(int T, const std::vector<std::pair<int, int>>& tpm,
                                    const vi& comb) {
  std::vector<char> inter(T, 1);
  for (int idx : comb) {
    auto p = tpm[idx];
    for (int t = 0; t < T; ++t)
      if (t != p.first && t != p.second) inter[t] = 0;
  }
  return inter;
}

// mlipkk_utils.cpp:33-58 (breadth-first, children appended in increasing order)
vvi comb_with_rep(int n, int r) {
  vvi ret;
  std::queue<vi> q;
  q.push(vi());
  while (!q.empty()) {
    vi c = q.front(); q.pop();
    if ((int)c.size() == r) { ret.push_back(c); continue; }
    int last = c.empty() ? 0 : c.back();
    for (int i = last; i < n; ++i) { vi nc(c); nc.push_back(i); q.push(nc); }
  }
  return ret;
}

// mlipkk_utils.cpp:64-98 ("historical" order used for polynomial indices)
vvi comb_with_rep_gtinv(int n, int r) {
  vvi ret;
  for (int first = 0; first < n; ++first) {
    std::queue<vi> q;
    q.push(vi{first});
    while (!q.empty()) {
      vi c = q.front(); q.pop();
      if ((int)c.size() == r) { ret.push_back(c); continue; }
      int last = c.back();
      for (int i = 0; i <= last; ++i) { vi nc(c); nc.push_back(i); q.push(nc); }
    }
  }
  return ret;
}

// mlipkk_irreps_type.cpp:48-100
void build_itc(Model& M) {
  const int T = M.T;
  const int ntc = T * (T + 1) / 2;
  auto tpm = type_pairs_mapping(T);
  int max_order = (int)M.irr_l.back().size();
  std::vector<vvi> uniq(max_order);
  for (int order = 1; order <= max_order; ++order) {
    for (auto& comb : comb_with_rep(ntc, order)) {
      auto inter = type_intersection(T, tpm, comb);
      if (std::any_of(inter.begin(), inter.end(), [](char e) { return e != 0; }))
        uniq[order - 1].push_back(comb);
    }
  }
  for (int i = 0; i < (int)M.irr_l.size(); ++i) {
    const vi& lc = M.irr_l[i];
    const int order = (int)lc.size();
    std::set<std::vector<std::pair<int, int>>> sets;
    for (auto sorted : uniq[order - 1]) {
      vi tcomb(sorted);
      do {
        std::vector<std::pair<int, int>> ms;
        for (int j = 0; j < order; ++j) ms.push_back({lc[j], tcomb[j]});
        std::sort(ms.begin(), ms.end());
        sets.insert(ms);
      } while (std::next_permutation(tcomb.begin(), tcomb.end()));
    }
    for (auto& ms : sets) {
      vi tc;
      for (auto& pr : ms) tc.push_back(pr.second);
      ITC x{i, tc, type_intersection(T, tpm, tc)};
      M.itc.push_back(x);
    }
  }
}

// mlipkk_polynomial.cpp:12-208
bool build_poly(Model& M) {
  const int D = M.D, ITCn = M.ITC_n, T = M.T;
  auto inter_of = [&](const vi& fcomb) {
    std::vector<char> in(T, 1);
    for (int f : fcomb) {
      const auto& x = M.itc[f % ITCn].inter;
      for (int t = 0; t < T; ++t) in[t] = in[t] && x[t];
    }
    return in;
  };
  auto any = [](const std::vector<char>& v) {
    return std::any_of(v.begin(), v.end(), [](char e) { return e != 0; });
  };
  const int mt = M.pot.model_type, maxp = M.pot.maxp;
  if (mt == 1) {
    for (int po = 1; po <= maxp; ++po)
      for (int f = 0; f < D; ++f) {
        vi fc(po, f);
        if (any(M.itc[f % ITCn].inter)) M.poly.push_back(fc);
      }
  } else if (mt == 2) {
    for (int po = 1; po <= maxp; ++po)
      for (auto& fc : comb_with_rep_gtinv(D, po))
        if (any(inter_of(fc))) M.poly.push_back(fc);
  } else if (mt == 3 || mt == 4) {
    vi lower;
    for (int f = 0; f < D; ++f) {
      int q = (int)M.itc[f % ITCn].type_combs.size();
      if ((mt == 3 && q == 1) || (mt == 4 && q <= 2)) lower.push_back(f);
    }
    for (int f = 0; f < D; ++f) M.poly.push_back(vi{f});
    for (int po = 2; po <= maxp; ++po)
      for (auto& ch : comb_with_rep_gtinv((int)lower.size(), po)) {
        vi fc;
        for (int k : ch) fc.push_back(lower[k]);
        if (any(inter_of(fc))) M.poly.push_back(fc);
      }
  } else {
    g_err = "Unknown model_type";
    return false;
  }
  return true;
}

bool build_model(Model& M, const char* pot_path, const char* table_path) {
  if (!read_potential(pot_path, M.pot)) return false;
  Table tab;
  if (!read_table(table_path, tab)) return false;
  M.T = (int)M.pot.elements.size();
  M.TC = M.T * (M.T + 1) / 2;
  M.F = (int)M.pot.params.size();
  M.L = M.pot.maxl;
  M.Lh = (M.L + 1) * (M.L + 2) / 2;
  M.La = (M.L + 1) * (M.L + 1);
  screen(tab, M.pot, M);
  build_itc(M);
  M.ITC_n = (int)M.itc.size();
  M.D = M.F * M.ITC_n;
  if (!build_poly(M)) return false;
  if ((int)M.poly.size() != (int)M.pot.coeffs.size()) {
    char b[256];
    snprintf(b, sizeof b, "coefficient count mismatch: file %zu, model %zu",
             M.pot.coeffs.size(), M.poly.size());
    g_err = b;
    return false;
  }
  // typecomb tables, mlipkk.cpp:160-196
  M.other_type.assign(M.TC, vi(M.T, -1));
  auto tpm = type_pairs_mapping(M.T);
  for (int tc = 0; tc < M.TC; ++tc) {
    M.other_type[tc][tpm[tc].first] = tpm[tc].second;
    M.other_type[tc][tpm[tc].second] = tpm[tc].first;
  }
  M.type_pairs.assign(M.T, vi(M.T, 0));
  int cnt = 0;
  for (int a = 0; a < M.T; ++a)
    for (int b = a; b < M.T; ++b) { M.type_pairs[a][b] = M.type_pairs[b][a] = cnt++; }
  // sph coefficients, mlipkk.cpp:247-272
  M.sphA.assign(M.Lh, 0.0);
  M.sphB.assign(M.Lh, 0.0);
  for (int l = 2; l <= M.L; ++l) {
    double ls = l * l, lm1s = (l - 1) * (l - 1);
    for (int m = 0; m <= l - 2; ++m) {
      double ms = m * m;
      M.sphA[lm2i(l, m)] = std::sqrt((4.0 * ls - 1.0) / (ls - ms));
      M.sphB[lm2i(l, m)] = -std::sqrt((lm1s - ms) / (4.0 * lm1s - 1.0));
    }
  }
  M.lh_l.assign(M.Lh, 0);
  M.lh_m.assign(M.Lh, 0);
  for (int l = 0; l <= M.L; ++l)
    for (int m = -l; m <= 0; ++m) {
      M.lh_l[l * (l + 1) / 2 + l + m] = l;
      M.lh_m[l * (l + 1) / 2 + l + m] = m;
    }
  M.lm_l.assign(M.La, 0);
  M.lm_m.assign(M.La, 0);
  for (int l = 0; l <= M.L; ++l)
    for (int m = -l; m <= l; ++m) { M.lm_l[l * l + l + m] = l; M.lm_m[l * l + l + m] = m; }
  return true;
}

// ------------------------------------------------- spherical harmonics
// mlipkk_spherical_harmonics_kk.h:18-177, arrays indexed by lm2i(l, m), m >= 0.
struct SHWork {
  vd alp, alps;
  std::vector<cplx> ylm, dx, dy, dz;  // indexed by LMInfoIdx (l, -mp)
};

void compute_sh(const Model& M, double costheta, double azimuthal, double r, bool der,
                SHWork& w) {
  const int maxl = M.L;
  w.alp.assign(M.Lh, 0.0);
  w.alps.assign(M.Lh, 0.0);
  w.ylm.assign(M.Lh, {0, 0});
  w.dx.assign(M.Lh, {0, 0});
  w.dy.assign(M.Lh, {0, 0});
  w.dz.assign(M.Lh, {0, 0});
  const double sintheta = std::sqrt(1.0 - costheta * costheta);
  // compute_alp
  {
    double tmp = 0.39894228040143267794;
    w.alp[lm2i(0, 0)] = tmp;
    if (maxl > 0) {
      const double SQRT3 = 1.7320508075688772935;
      w.alp[lm2i(1, 0)] = costheta * SQRT3 * tmp;
      const double SQRT3DIV2 = -1.2247448713915890491;
      tmp *= SQRT3DIV2 * sintheta;
      w.alp[lm2i(1, 1)] = tmp;
      for (int l = 2; l <= maxl; ++l) {
        for (int m = 0; m <= l - 2; ++m)
          w.alp[lm2i(l, m)] = M.sphA[lm2i(l, m)] *
              (costheta * w.alp[lm2i(l - 1, m)] + M.sphB[lm2i(l, m)] * w.alp[lm2i(l - 2, m)]);
        w.alp[lm2i(l, l - 1)] = costheta * std::sqrt(2.0 * (l - 1.0) + 3.0) * tmp;
        tmp *= -std::sqrt(1.0 + 0.5 / l) * sintheta;
        w.alp[lm2i(l, l)] = tmp;
      }
    }
  }
  // compute_ylm
  {
    for (int l = 0; l <= maxl; ++l)
      w.ylm[lm2i(l, l)] = {w.alp[lm2i(l, 0)] * 0.5 * M_SQRT2, 0.0};
    double c1 = 1.0, c2 = std::cos(azimuthal);
    double s1 = 0.0, s2 = -std::sin(azimuthal);
    const double tc = 2.0 * c2;
    double sign = -1;
    for (int mp = 1; mp <= maxl; ++mp) {
      const double s = tc * s1 - s2;
      const double c = tc * c1 - c2;
      c2 = c1; c1 = c; s2 = s1; s1 = s;
      for (int l = mp; l <= maxl; ++l) {
        const double t = sign * w.alp[lm2i(l, mp)] * 0.5 * M_SQRT2;
        w.ylm[lm2i(l, l - mp)] = {t * c, t * (-s)};
      }
      sign *= -1;
    }
  }
  if (!der || maxl == 0) return;
  // compute_alp_sintheta
  {
    double tmp = -0.48860251190291992263;
    w.alps[lm2i(1, 1)] = tmp;
    for (int l = 2; l <= maxl; ++l) {
      for (int m = 1; m <= l - 2; ++m)
        w.alps[lm2i(l, m)] = M.sphA[lm2i(l, m)] *
            (costheta * w.alps[lm2i(l - 1, m)] + M.sphB[lm2i(l, m)] * w.alps[lm2i(l - 2, m)]);
      w.alps[lm2i(l, l - 1)] = costheta * std::sqrt(2.0 * (l - 1.0) + 3.0) * tmp;
      tmp *= -std::sqrt(1.0 + 0.5 / l) * sintheta;
      w.alps[lm2i(l, l)] = tmp;
    }
  }
  // compute_ylm_der
  {
    const double cosphi = std::cos(azimuthal);
    const double sinphi = std::sin(azimuthal);
    double c1 = 1.0, c2 = cosphi;
    double s1 = 0.0, s2 = -sinphi;
    const double tc = 2.0 * c2;
    const double invr = 1.0 / r;
    for (int l = 1; l <= maxl; ++l) {
      const double common = w.alps[lm2i(l, 1)] * sintheta * invr * std::sqrt(0.5 * l * (l + 1));
      w.dx[lm2i(l, l)] = {common * costheta * cosphi, 0.0};
      w.dy[lm2i(l, l)] = {common * costheta * sinphi, 0.0};
      w.dz[lm2i(l, l)] = {-common * sintheta, 0.0};
    }
    double sign = -1.0;
    for (int mp = 1; mp <= maxl; ++mp) {
      const double s = tc * s1 - s2;
      const double c = tc * c1 - c2;
      c2 = c1; c1 = c; s2 = s1; s1 = s;
      for (int l = mp; l <= maxl; ++l) {
        // common = e^{i mp phi} * sqrt(2)/2 / r
        const cplx common = cscale(cscale({c, s}, 0.5 * M_SQRT2), invr);
        double dtheta = mp * costheta * w.alps[lm2i(l, mp)];
        if (mp != l)
          dtheta += std::sqrt(static_cast<double>(l - mp) * (l + mp + 1)) *
                    w.alps[lm2i(l, mp + 1)] * sintheta;
        const cplx dphi = {0.0, mp * w.alps[lm2i(l, mp)]};
        // x: conj(common * (dtheta cos cos - dphi sin))
        cplx ax = {dtheta * costheta * cosphi - dphi.re * sinphi, -dphi.im * sinphi};
        cplx ay = {dtheta * costheta * sinphi + dphi.re * cosphi, dphi.im * cosphi};
        cplx az = {-dtheta * sintheta, 0.0};
        cplx px = cmul(common, ax), py = cmul(common, ay), pz = cmul(common, az);
        w.dx[lm2i(l, l - mp)] = {sign * px.re, -sign * px.im};
        w.dy[lm2i(l, l - mp)] = {sign * py.re, -sign * py.im};
        w.dz[lm2i(l, l - mp)] = {sign * pz.re, -sign * pz.im};
      }
      sign *= -1.0;
    }
  }
}

// radial basis, mlipkk_features_kk.h:9-48
void compute_fn(const Model& M, double r, vd& fn, vd& fnd) {
  const double rc = M.pot.cutoff;
  double fc = 0.0, fcd = 0.0;
  if (r < rc) {
    fc = 0.5 * (std::cos(M_PI * r / rc) + 1.0);
    fcd = -0.5 * M_PI / rc * std::sin(M_PI * r / rc);
  }
  fn.resize(M.F);
  fnd.resize(M.F);
  for (int n = 0; n < M.F; ++n) {
    const double beta = M.pot.params[n].first, mu = M.pot.params[n].second;
    const double bf = std::exp(-beta * (r - mu) * (r - mu));
    const double bfd = -2.0 * beta * (r - mu) * bf;
    fn[n] = bf * fc;
    fnd[n] = bfd * fc + bf * fcd;
  }
}

// ------------------------------------------------------ per-atom stages
// a[type][n][LMIdx] for one centre atom, order parameters for all m.
struct AtomState {
  std::vector<cplx> a;   // [T][F][La]
  vd d;                  // [D]
  vd H;                  // [D]
  std::vector<cplx> G;   // [TC][F][Lh]
  double E = 0.0;
};

struct Geometry {
  int nlocal, nall;
  const double* x;
  const int* type;  // element index per atom (nall), -1 = not handled
  const int* off;   // neighbour CSR offsets, nlocal + 1
  const int* nbr;   // neighbour local indices (may include ghosts)
};

// mlipkk_lmp.h:314-387 restricted to one centre atom.
void atom_order_params(const Model& M, const Geometry& g, int i, AtomState& s, SHWork& w,
                       vd& fn, vd& fnd) {
  const int T = M.T, F = M.F, Lh = M.Lh, La = M.La;
  vd ar((size_t)T * F * Lh, 0.0), ai((size_t)T * F * Lh, 0.0);
  for (int p = g.off[i]; p < g.off[i + 1]; ++p) {
    const int j = g.nbr[p];
    const int tj = g.type[j];
    if (tj < 0) continue;
    const double dx = g.x[3 * j] - g.x[3 * i];
    const double dy = g.x[3 * j + 1] - g.x[3 * i + 1];
    const double dz = g.x[3 * j + 2] - g.x[3 * i + 2];
    const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
    if (r > M.pot.cutoff) continue;
    compute_sh(M, dz / r, std::atan2(dy, dx), r, false, w);
    compute_fn(M, r, fn, fnd);
    for (int n = 0; n < F; ++n)
      for (int lmi = 0; lmi < Lh; ++lmi) {
        const cplx val = cscale(w.ylm[lmi], fn[n]);
        ar[((size_t)tj * F + n) * Lh + lmi] += val.re;
        ai[((size_t)tj * F + n) * Lh + lmi] -= val.im;
      }
  }
  s.a.assign((size_t)T * F * La, {0, 0});
  for (int t = 0; t < T; ++t)
    for (int n = 0; n < F; ++n)
      for (int l = 0; l <= M.L; ++l)
        for (int m = -l; m <= 0; ++m) {
          const int lmi = l * (l + 1) / 2 + l + m;
          const int lm1 = l * l + l + m, lm2 = l * l + l - m;
          const size_t k = ((size_t)t * F + n) * Lh + lmi;
          const double cc = (m % 2) ? -1.0 : 1.0;
          s.a[((size_t)t * F + n) * La + lm1] = {ar[k], ai[k]};
          s.a[((size_t)t * F + n) * La + lm2] = {cc * ar[k], -cc * ai[k]};
        }
}

// invariants, energy, polynomial and basis adjoints for one centre atom
void atom_adjoints(const Model& M, int ti, AtomState& s) {
  const int F = M.F, La = M.La, Lh = M.Lh, ITCn = M.ITC_n;
  s.d.assign(M.D, 0.0);
  for (int f = 0; f < M.D; ++f) {
    const int itc = f % ITCn;
    if (!M.itc[itc].inter[ti]) continue;
    const int n = f / ITCn;
    const auto& tcs = M.itc[itc].type_combs;
    const int ir = M.itc[itc].irreps;
    double feat = 0.0;
    for (int term = 0; term < M.irr_nterms[ir]; ++term) {
      const int it = M.irr_first[ir] + term;
      cplx tmp = {M.term_c[it], 0.0};
      for (size_t p = 0; p < tcs.size(); ++p) {
        const int t2 = M.other_type[tcs[p]][ti];
        tmp = cmul(tmp, s.a[((size_t)t2 * F + n) * La + M.term_lm[it][p]]);
      }
      feat += tmp.re;
    }
    s.d[f] = feat;
  }
  // energy, mlipkk_lmp.h:506-518
  s.E = 0.0;
  for (size_t pi = 0; pi < M.poly.size(); ++pi) {
    double feat = 1.0;
    for (int f : M.poly[pi]) feat *= s.d[f];
    s.E += M.pot.coeffs[pi] * feat;
  }
  // polynomial adjoints, mlipkk_lmp.h:595-619
  s.H.assign(M.D, 0.0);
  for (size_t pi = 0; pi < M.poly.size(); ++pi) {
    const vi& row = M.poly[pi];
    const int po = (int)row.size();
    for (int p1 = 0; p1 < po; ++p1) {
      double adj = M.pot.coeffs[pi];
      for (int p2 = 0; p2 < po; ++p2) {
        if (p2 == p1) continue;
        adj *= s.d[row[p2]];
      }
      s.H[row[p1]] += adj;
    }
  }
  // basis function adjoints, mlipkk_lmp.h:680-728
  s.G.assign((size_t)M.TC * F * Lh, {0, 0});
  for (int itc = 0; itc < ITCn; ++itc) {
    if (!M.itc[itc].inter[ti]) continue;
    const auto& tcs = M.itc[itc].type_combs;
    const int ir = M.itc[itc].irreps;
    const int order = (int)tcs.size();
    for (int n = 0; n < F; ++n) {
      const int f = n * ITCn + itc;
      for (int term = 0; term < M.irr_nterms[ir]; ++term) {
        const int it = M.irr_first[ir] + term;
        const double cg = M.term_c[it];
        for (int mu = 0; mu < order; ++mu) {
          const int lm_mu = M.term_lm[it][mu];
          const int m_mu = M.lm_m[lm_mu];
          if (m_mu > 0) continue;
          const int l_mu = M.lm_l[lm_mu];
          const int lmi_mu = l_mu * (l_mu + 1) / 2 + l_mu + m_mu;
          cplx tmp = {cg * s.H[f], 0.0};
          for (int mu2 = 0; mu2 < order; ++mu2) {
            if (mu2 == mu) continue;
            const int t2 = M.other_type[tcs[mu2]][ti];
            tmp = cmul(tmp, s.a[((size_t)t2 * F + n) * La + M.term_lm[it][mu2]]);
          }
          cplx& gg = s.G[((size_t)tcs[mu] * F + n) * Lh + lmi_mu];
          gg.re += tmp.re;
          gg.im += tmp.im;
        }
      }
    }
  }
}

// pair force from one adjoint (G of atom `owner`), mlipkk_lmp.h:807-892
struct PairForce {
  double fx, fy, fz;
};

// ------------------------------------------------ radial-only descriptor
// Legacy pair model: features dn[tc * F + n] = sum_j f_n(r_ij) over the
// neighbours j with type pair tc = tc(t_i, t_j), and a polynomial in them.
struct PairModel {
  int T = 0, F = 0, TC = 0;
  vvi tc_types;            // [tc] -> {a, b}, a <= b (type_comb_pair order)
  vvi pair_tc;             // [t1][t2] -> tc
  vvi terms;               // coefficient index -> feature seqs (tc * F + n)
};

// mlip_model_params.cpp:29-71 (type_comb_pair: one entry per a <= b),
// 180-213 (combination2 / combination3), mlip_polynomial.cpp:33-43 (powers)
bool build_pair_model(const Potential& p, PairModel& P) {
  P.T = (int)p.elements.size();
  P.F = (int)p.params.size();
  if (P.T < 1 || P.T > 2) {
    g_err = "the pair descriptor supports one or two elements";
    return false;
  }
  for (int a = 0; a < P.T; ++a)
    for (int b = a; b < P.T; ++b) P.tc_types.push_back({a, b});
  P.TC = (int)P.tc_types.size();
  P.pair_tc.assign(P.T, vi(P.T, 0));
  for (int tc = 0; tc < P.TC; ++tc) {
    P.pair_tc[P.tc_types[tc][0]][P.tc_types[tc][1]] = tc;
    P.pair_tc[P.tc_types[tc][1]][P.tc_types[tc][0]] = tc;
  }
  const int nd = P.F * P.TC;
  const auto has = [&](int tc, int t) { return P.tc_types[tc][0] == t || P.tc_types[tc][1] == t; };
  const auto shared = [&](std::initializer_list<int> seqs) {
    for (int t = 0; t < P.T; ++t) {
      bool all = true;
      for (int q : seqs) all = all && has(q / P.F, t);
      if (all) return true;
    }
    return false;
  };
  for (int n = 0; n < nd; ++n) P.terms.push_back({n});
  if (p.model_type == 1) {
    if (p.maxp > 1) for (int n = 0; n < nd; ++n) P.terms.push_back({n, n});
    if (p.maxp > 2) for (int n = 0; n < nd; ++n) P.terms.push_back({n, n, n});
  } else if (p.model_type == 2) {
    if (p.maxp > 1)
      for (int i1 = 0; i1 < nd; ++i1)
        for (int i2 = 0; i2 <= i1; ++i2)
          if (shared({i1, i2})) P.terms.push_back({i2, i1});
    if (p.maxp > 2)
      for (int i1 = 0; i1 < nd; ++i1)
        for (int i2 = 0; i2 <= i1; ++i2)
          for (int i3 = 0; i3 <= i2; ++i3)
            if (shared({i1, i2, i3})) P.terms.push_back({i3, i2, i1});
  }
  if (P.terms.size() != p.coeffs.size()) {
    char b[200];
    snprintf(b, sizeof b, "coefficient count mismatch: file %zu, pair model %zu",
             p.coeffs.size(), P.terms.size());
    g_err = b;
    return false;
  }
  return true;
}

struct Oracle {
  Model M;
  PairModel P;
  int nthreads = 1;
};

}  // namespace

extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

void* orc_create(const char* pot_path, const char* table_path) {
  Oracle* o = new Oracle();
  Potential probe;
  if (!read_potential(pot_path, probe)) {
    delete o;
    return nullptr;
  }
  if (probe.pair) {
    o->M.pot = probe;
    o->M.T = (int)probe.elements.size();
    o->M.F = (int)probe.params.size();
    if (!build_pair_model(probe, o->P)) {
      delete o;
      return nullptr;
    }
    return o;
  }
  if (!build_model(o->M, pot_path, table_path)) {
    delete o;
    return nullptr;
  }
  return o;
}

int orc_is_pair(void* h) { return static_cast<Oracle*>(h)->M.pot.pair ? 1 : 0; }

// The radial-only descriptor (pair_mlip_pair.cpp:56-264) on a full list with
// ghost atoms, owner-computes: per owned atom i the features dn_i, its energy
// E_i = sum_f c_f dn_i,f + sum_p c_p prod dn_i (c = file coefficient / scale:
// the legacy reader doubles the coefficients, mlip_model.h:90, and its
// half-list pair sums count every term twice over), and for every neighbour
// j the force of E_i, f = dE_i/dr_ij = sum_n f_n'(r) dE_i/d dn_i[tc,n] r_hat,
// scattered as F_i += f, F_j -= f, virial -= r_ij (x) f.
int orc_pair_compute(void* h, int nlocal, int nall, const double* x, const int* type,
                     const int* off, const int* nbr, double* f, double* energy, double* virial,
                     double* eatom) {
  Oracle* o = static_cast<Oracle*>(h);
  const Potential& p = o->M.pot;
  const PairModel& P = o->P;
  const int F = P.F, nd = F * P.TC;
  std::fill(f, f + (size_t)3 * nall, 0.0);
  double E = 0.0, vir[6] = {0, 0, 0, 0, 0, 0};
  std::vector<double> dn(nd), H(nd), fn, fnd;
  Model Mr;
  Mr.pot = p;
  Mr.F = F;
  for (int i = 0; i < nlocal; ++i) {
    const int ti = type[i];
    if (ti < 0) {
      if (eatom) eatom[i] = 0.0;
      continue;
    }
    std::fill(dn.begin(), dn.end(), 0.0);
    for (int q = off[i]; q < off[i + 1]; ++q) {
      const int j = nbr[q];
      if (type[j] < 0) continue;
      const double dx = x[3 * j] - x[3 * i], dy = x[3 * j + 1] - x[3 * i + 1],
                   dz = x[3 * j + 2] - x[3 * i + 2];
      const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
      if (r >= p.cutoff) continue;
      compute_fn(Mr, r, fn, fnd);
      const int tc = P.pair_tc[ti][type[j]];
      for (int n = 0; n < F; ++n) dn[tc * F + n] += fn[n];
    }
    // energy and dE/d dn
    double Ei = 0.0;
    std::fill(H.begin(), H.end(), 0.0);
    for (size_t k = 0; k < P.terms.size(); ++k) {
      // (features of type pairs without t_i are zero, and so is every term
      // that contains one)
      const vi& row = P.terms[k];
      double prod = p.coeffs[k];
      for (int q : row) prod *= dn[q];
      Ei += prod;
      for (size_t a = 0; a < row.size(); ++a) {
        double g = p.coeffs[k];
        for (size_t b = 0; b < row.size(); ++b)
          if (b != a) g *= dn[row[b]];
        H[row[a]] += g;
      }
    }
    E += Ei;
    if (eatom) eatom[i] = Ei;
    for (int q = off[i]; q < off[i + 1]; ++q) {
      const int j = nbr[q];
      if (type[j] < 0) continue;
      const double dx = x[3 * j] - x[3 * i], dy = x[3 * j + 1] - x[3 * i + 1],
                   dz = x[3 * j + 2] - x[3 * i + 2];
      const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
      if (r >= p.cutoff) continue;
      compute_fn(Mr, r, fn, fnd);
      const int tc = P.pair_tc[ti][type[j]];
      double g = 0.0;
      for (int n = 0; n < F; ++n) g += fnd[n] * H[tc * F + n];
      const double fx = g * dx / r, fy = g * dy / r, fz = g * dz / r;
      f[3 * i] += fx; f[3 * i + 1] += fy; f[3 * i + 2] += fz;
      f[3 * j] -= fx; f[3 * j + 1] -= fy; f[3 * j + 2] -= fz;
      vir[0] -= dx * fx; vir[1] -= dy * fy; vir[2] -= dz * fz;
      vir[3] -= dx * fy; vir[4] -= dx * fz; vir[5] -= dy * fz;
    }
  }
  *energy = E;
  for (int k = 0; k < 6; ++k) virial[k] = vir[k];   // LAMMPS order xx yy zz xy xz yz
  return 0;
}

void orc_destroy(void* h) { delete static_cast<Oracle*>(h); }

void orc_set_threads(void* h, int n) { static_cast<Oracle*>(h)->nthreads = n > 0 ? n : 1; }

// Model sizes: [T, TC, F, L, Lh, La, n_irreps, n_terms, ITC, D, n_coeffs, model_type, maxp]
int orc_pair_compute(void* h, int nlocal, int nall, const double* x, const int* type,
                     const int* off, const int* nbr, double* f, double* energy, double* virial,
                     double* eatom);

void orc_info(void* h, int* out13, double* cutoff) {
  const Model& M = static_cast<Oracle*>(h)->M;
  if (M.pot.pair) {
    const PairModel& P = static_cast<Oracle*>(h)->P;
    int v[13] = {P.T, P.TC, P.F, 0, 1, 1, 0, 0, P.TC, P.F * P.TC, (int)P.terms.size(),
                 M.pot.model_type, M.pot.maxp};
    std::memcpy(out13, v, sizeof v);
    *cutoff = M.pot.cutoff;
    return;
  }
  int v[13] = {M.T, M.TC, M.F, M.L, M.Lh, M.La, (int)M.irr_l.size(), (int)M.term_c.size(),
               M.ITC_n, M.D, (int)M.poly.size(), M.pot.model_type, M.pot.maxp};
  std::memcpy(out13, v, sizeof v);
  *cutoff = M.pot.cutoff;
}

// regression coefficients (divided by their scales), [n_coeffs]
void orc_coeffs(void* h, double* out) {
  const Model& M = static_cast<Oracle*>(h)->M;
  std::copy(M.pot.coeffs.begin(), M.pot.coeffs.end(), out);
}

// flattened model structure for cross-checks: itc list and polynomial index
// itc_out: for each itc [irreps, q, tc_0..tc_{q-1}] concatenated; returns total ints
long orc_dump_itc(void* h, int* out, long cap) {
  const Model& M = static_cast<Oracle*>(h)->M;
  long k = 0;
  for (auto& x : M.itc) {
    if (out && k + 2 + (long)x.type_combs.size() <= cap) {
      out[k] = x.irreps;
      out[k + 1] = (int)x.type_combs.size();
      for (size_t p = 0; p < x.type_combs.size(); ++p) out[k + 2 + p] = x.type_combs[p];
    }
    k += 2 + (long)x.type_combs.size();
  }
  return k;
}

long orc_dump_poly(void* h, int* out, long cap) {
  const Model& M = static_cast<Oracle*>(h)->M;
  long k = 0;
  for (auto& row : M.poly) {
    if (out && k + 1 + (long)row.size() <= cap) {
      out[k] = (int)row.size();
      for (size_t p = 0; p < row.size(); ++p) out[k + 1 + p] = row[p];
    }
    k += 1 + (long)row.size();
  }
  return k;
}

// Spherical harmonics for one displacement: ylm, dx, dy, dz as complex pairs
// indexed by LMInfoIdx (Lh entries each).
void orc_sph(void* h, double x, double y, double z, double* ylm, double* dx, double* dy,
             double* dz) {
  const Model& M = static_cast<Oracle*>(h)->M;
  SHWork w;
  const double r = std::sqrt(x * x + y * y + z * z);
  compute_sh(M, z / r, std::atan2(y, x), r, true, w);
  for (int k = 0; k < M.Lh; ++k) {
    ylm[2 * k] = w.ylm[k].re; ylm[2 * k + 1] = w.ylm[k].im;
    dx[2 * k] = w.dx[k].re; dx[2 * k + 1] = w.dx[k].im;
    dy[2 * k] = w.dy[k].re; dy[2 * k + 1] = w.dy[k].im;
    dz[2 * k] = w.dz[k].re; dz[2 * k + 1] = w.dz[k].im;
  }
}

void orc_radial(void* h, double r, double* fn, double* fnd) {
  const Model& M = static_cast<Oracle*>(h)->M;
  vd a, b;
  compute_fn(M, r, a, b);
  for (int n = 0; n < M.F; ++n) { fn[n] = a[n]; fnd[n] = b[n]; }
}

// Full-list LAMMPS semantics (mlipkk_lmp.h, "neigh full newton on").
// x: [nall*3]; type: element index per atom (nall), -1 = unmapped.
// off/nbr: full neighbour CSR for the nlocal owned atoms.
// f: [nall*3] overwritten; eatom: [nlocal] (may be null);
// virial: LAMMPS order xx yy zz xy xz yz.
// anlm_out (optional): [nlocal][T][F][Lh] complex pairs (m <= 0 entries).
int orc_compute(void* h, int nlocal, int nall, const double* x, const int* type,
                const int* off, const int* nbr, double* f, double* energy, double* virial,
                double* eatom, double* anlm_out) {
  Oracle* o = static_cast<Oracle*>(h);
  if (o->M.pot.pair)
    return orc_pair_compute(h, nlocal, nall, x, type, off, nbr, f, energy, virial, eatom);
  const Model& M = o->M;
  const Geometry g{nlocal, nall, x, type, off, nbr};
  const int F = M.F, Lh = M.Lh, La = M.La, T = M.T;
  std::vector<AtomState> st(nlocal);
#ifdef _OPENMP
#pragma omp parallel num_threads(o->nthreads)
#endif
  {
    SHWork w;
    vd fn, fnd;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
    for (int i = 0; i < nlocal; ++i) {
      if (type[i] < 0) continue;
      atom_order_params(M, g, i, st[i], w, fn, fnd);
      atom_adjoints(M, type[i], st[i]);
      st[i].a.clear();
      st[i].a.shrink_to_fit();
      st[i].d.clear();
      st[i].d.shrink_to_fit();
      st[i].H.clear();
      st[i].H.shrink_to_fit();
    }
  }
  if (anlm_out) {
    // recompute order parameters for output (cheap relative to adjoints)
    SHWork w;
    vd fn, fnd;
    for (int i = 0; i < nlocal; ++i) {
      AtomState s;
      if (type[i] >= 0) atom_order_params(M, g, i, s, w, fn, fnd);
      for (int t = 0; t < T; ++t)
        for (int n = 0; n < F; ++n)
          for (int l = 0; l <= M.L; ++l)
            for (int m = -l; m <= 0; ++m) {
              const int lmi = l * (l + 1) / 2 + l + m;
              cplx v = {0, 0};
              if (type[i] >= 0) v = s.a[((size_t)t * F + n) * La + l * l + l + m];
              const size_t k = ((((size_t)i * T + t) * F + n) * Lh + lmi) * 2;
              anlm_out[k] = v.re;
              anlm_out[k + 1] = v.im;
            }
    }
  }
  // energy, mlipkk_lmp.h:526-534
  double E = 0.0;
  for (int i = 0; i < nlocal; ++i) {
    E += st[i].E;
    if (eatom) eatom[i] = st[i].E;
  }
  *energy = E;
  // forces and stress, mlipkk_lmp.h:779-916 (serial, reference order)
  std::fill(f, f + (size_t)3 * nall, 0.0);
  double sxx = 0, syy = 0, szz = 0, syz = 0, szx = 0, sxy = 0;
  SHWork w;
  vd fn, fnd;
  for (int i = 0; i < nlocal; ++i) {
    if (type[i] < 0) continue;
    for (int p = off[i]; p < off[i + 1]; ++p) {
      const int j = nbr[p];
      if (type[j] < 0) continue;
      const double dx = x[3 * j] - x[3 * i];
      const double dy = x[3 * j + 1] - x[3 * i + 1];
      const double dz = x[3 * j + 2] - x[3 * i + 2];
      const double dis = std::sqrt(dx * dx + dy * dy + dz * dz);
      if (dis > M.pot.cutoff) continue;
      const bool local_lower = (j < nlocal && j < i);
      const bool ghost = (j >= nlocal);
      if (!local_lower && !ghost) continue;
      const double invdis = 1.0 / dis;
      compute_sh(M, dz / dis, std::atan2(dy, dx), dis, true, w);
      compute_fn(M, dis, fn, fnd);
      const int tc = M.type_pairs[type[i]][type[j]];
      double fx = 0, fy = 0, fz = 0;
      for (int n = 0; n < F; ++n)
        for (int lmi = 0; lmi < Lh; ++lmi) {
          const int l = M.lh_l[lmi], m = M.lh_m[lmi];
          const double coeff = (m == 0) ? 1.0 : 2.0;
          const cplx f1 = cscale(w.ylm[lmi], fnd[n]);
          cplx bx = {f1.re * dx * invdis + fn[n] * w.dx[lmi].re,
                     f1.im * dx * invdis + fn[n] * w.dx[lmi].im};
          cplx by = {f1.re * dy * invdis + fn[n] * w.dy[lmi].re,
                     f1.im * dy * invdis + fn[n] * w.dy[lmi].im};
          cplx bz = {f1.re * dz * invdis + fn[n] * w.dz[lmi].re,
                     f1.im * dz * invdis + fn[n] * w.dz[lmi].im};
          bx.im *= -1; by.im *= -1; bz.im *= -1;
          const cplx gi = st[i].G[((size_t)tc * F + n) * Lh + lmi];
          fx += coeff * prod_real(gi, bx);
          fy += coeff * prod_real(gi, by);
          fz += coeff * prod_real(gi, bz);
          if (local_lower) {
            const double scale = (l % 2) ? -1.0 : 1.0;
            const cplx gj = st[j].G[((size_t)tc * F + n) * Lh + lmi];
            fx += coeff * scale * prod_real(gj, bx);
            fy += coeff * scale * prod_real(gj, by);
            fz += coeff * scale * prod_real(gj, bz);
          }
        }
      f[3 * i] += fx; f[3 * i + 1] += fy; f[3 * i + 2] += fz;
      f[3 * j] -= fx; f[3 * j + 1] -= fy; f[3 * j + 2] -= fz;
      sxx -= dx * fx; syy -= dy * fy; szz -= dz * fz;
      syz -= dy * fz; szx -= dz * fx; sxy -= dx * fy;
    }
  }
  // LAMMPS order xx yy zz xy xz yz, mlipkk_lmp.h:942-955
  virial[0] = sxx; virial[1] = syy; virial[2] = szz;
  virial[3] = sxy; virial[4] = szx; virial[5] = syz;
  return 0;
}

// Training features of one structure (the reference's prepare_features:
// mlipkk.cpp:461-470 with compute_structural_features :609-666,
// compute_polynomial_features :1167-1179, compute_dirj :1011-1154 and
// compute_force_and_stress_features :1181-1281), on a full neighbour list
// with ghost atoms in the owner-computes form: centre i's features d_i,
// its polynomial features P_i,p = prod_{f in p} d_i,f, and for every
// neighbour j the derivative of d_i with respect to the pair displacement
// r_j - r_i (the reference's dirj), contracted into the force features
// FF[i][p] += dP_i,p/dr_ij, FF[j][p] -= dP_i,p/dr_ij and the stress features
// SF[p] -= r_ij (x) dP_i,p/dr_ij (reference order xx yy zz yz zx xy).
// Summed over all centres this is the reference's half-list result, and
// E = sum_i P_i . w, F = FF . w, virial = SF . w for the coefficients w.
// d_out [nlocal][D], p_out [nlocal][C], ff_out [nall][C][3] (accumulated),
// sf_out [C][6] (accumulated); any may be null.  Test infrastructure.
int orc_features(void* h, int nlocal, int nall, const double* x, const int* type, const int* off,
                 const int* nbr, double* d_out, double* p_out, double* ff_out, double* sf_out) {
  Oracle* o = static_cast<Oracle*>(h);
  const Model& M = o->M;
  const Geometry g{nlocal, nall, x, type, off, nbr};
  const int F = M.F, La = M.La, ITCn = M.ITC_n, D = M.D;
  const int C = (int)M.poly.size();
  int nth = o->nthreads;
  std::vector<vd> ffb(nth), sfb(nth);
#ifdef _OPENMP
#pragma omp parallel num_threads(nth)
#endif
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    vd& ffl = ffb[tid];
    vd& sfl = sfb[tid];
    if (ff_out) ffl.assign((size_t)nall * C * 3, 0.0);
    if (sf_out) sfl.assign((size_t)C * 6, 0.0);
    SHWork w;
    vd fn, fnd;
    AtomState s;
    vd dirj((size_t)D * 3);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
    for (int i = 0; i < nlocal; ++i) {
      const int ti = type[i];
      if (ti < 0) continue;
      atom_order_params(M, g, i, s, w, fn, fnd);
      // structural features, mlipkk.cpp:628-663
      vd d(D, 0.0);
      for (int f = 0; f < D; ++f) {
        const int itc = f % ITCn;
        if (!M.itc[itc].inter[ti]) continue;
        const int n = f / ITCn;
        const auto& tcs = M.itc[itc].type_combs;
        const int ir = M.itc[itc].irreps;
        double feat = 0.0;
        for (int term = 0; term < M.irr_nterms[ir]; ++term) {
          const int it = M.irr_first[ir] + term;
          cplx tmp = {M.term_c[it], 0.0};
          for (size_t p = 0; p < tcs.size(); ++p) {
            const int t2 = M.other_type[tcs[p]][ti];
            tmp = cmul(tmp, s.a[((size_t)t2 * F + n) * La + M.term_lm[it][p]]);
          }
          feat += tmp.re;
        }
        d[f] = feat;
      }
      if (d_out) std::copy(d.begin(), d.end(), d_out + (size_t)i * D);
      // polynomial features, mlipkk.cpp:1167-1179
      if (p_out)
        for (int pi = 0; pi < C; ++pi) {
          double v = 1.0;
          for (int f : M.poly[pi]) v *= d[f];
          p_out[(size_t)i * C + pi] = v;
        }
      if (!ff_out && !sf_out) continue;
      for (int q = off[i]; q < off[i + 1]; ++q) {
        const int j = nbr[q];
        const int tj = type[j];
        if (tj < 0) continue;
        const double dx = x[3 * j] - x[3 * i];
        const double dy = x[3 * j + 1] - x[3 * i + 1];
        const double dz = x[3 * j + 2] - x[3 * i + 2];
        const double dis = std::sqrt(dx * dx + dy * dy + dz * dz);
        if (dis > M.pot.cutoff) continue;
        const double invdis = 1.0 / dis;
        compute_sh(M, dz / dis, std::atan2(dy, dx), dis, true, w);
        compute_fn(M, dis, fn, fnd);
        const int tc_ij = M.type_pairs[ti][tj];
        // dirj, mlipkk.cpp:1054-1150 (the centre's half of each pair)
        std::fill(dirj.begin(), dirj.end(), 0.0);
        for (int f = 0; f < D; ++f) {
          const int itc = f % ITCn;
          if (!M.itc[itc].inter[ti]) continue;
          const int n = f / ITCn;
          const auto& tcs = M.itc[itc].type_combs;
          const int ir = M.itc[itc].irreps;
          const int order = (int)tcs.size();
          for (int term = 0; term < M.irr_nterms[ir]; ++term) {
            const int it = M.irr_first[ir] + term;
            for (int mu = 0; mu < order; ++mu) {
              if (tcs[mu] != tc_ij) continue;
              cplx tmp = {M.term_c[it], 0.0};
              for (int mu2 = 0; mu2 < order; ++mu2) {
                if (mu2 == mu) continue;
                const int t2 = M.other_type[tcs[mu2]][ti];
                tmp = cmul(tmp, s.a[((size_t)t2 * F + n) * La + M.term_lm[it][mu2]]);
              }
              const int lm_mu = M.term_lm[it][mu];
              const int l_mu = M.lm_l[lm_mu], m_mu = M.lm_m[lm_mu];
              cplx ylm, ydx, ydy, ydz;
              if (m_mu > 0) {
                const int lmi = l_mu * (l_mu + 1) / 2 + l_mu - m_mu;   // (l, -m)
                const double sm = (m_mu % 2) ? -1.0 : 1.0;
                ylm = {sm * w.ylm[lmi].re, -sm * w.ylm[lmi].im};
                ydx = {sm * w.dx[lmi].re, -sm * w.dx[lmi].im};
                ydy = {sm * w.dy[lmi].re, -sm * w.dy[lmi].im};
                ydz = {sm * w.dz[lmi].re, -sm * w.dz[lmi].im};
              } else {
                const int lmi = l_mu * (l_mu + 1) / 2 + l_mu + m_mu;
                ylm = w.ylm[lmi];
                ydx = w.dx[lmi];
                ydy = w.dy[lmi];
                ydz = w.dz[lmi];
              }
              const cplx f1 = cscale(ylm, fnd[n]);
              cplx bx = {f1.re * dx * invdis + fn[n] * ydx.re, f1.im * dx * invdis + fn[n] * ydx.im};
              cplx by = {f1.re * dy * invdis + fn[n] * ydy.re, f1.im * dy * invdis + fn[n] * ydy.im};
              cplx bz = {f1.re * dz * invdis + fn[n] * ydz.re, f1.im * dz * invdis + fn[n] * ydz.im};
              bx.im *= -1;
              by.im *= -1;
              bz.im *= -1;
              dirj[(size_t)f * 3] += prod_real(tmp, bx);
              dirj[(size_t)f * 3 + 1] += prod_real(tmp, by);
              dirj[(size_t)f * 3 + 2] += prod_real(tmp, bz);
            }
          }
        }
        // force and stress features, mlipkk.cpp:1217-1273
        for (int pi = 0; pi < C; ++pi) {
          const vi& row = M.poly[pi];
          double t3[3] = {0, 0, 0};
          for (size_t nu = 0; nu < row.size(); ++nu) {
            double prod = 1.0;
            for (size_t nu2 = 0; nu2 < row.size(); ++nu2)
              if (nu2 != nu) prod *= d[row[nu2]];
            for (int k = 0; k < 3; ++k) t3[k] += dirj[(size_t)row[nu] * 3 + k] * prod;
          }
          if (ff_out) {
            for (int k = 0; k < 3; ++k) {
              ffl[((size_t)i * C + pi) * 3 + k] += t3[k];
              ffl[((size_t)j * C + pi) * 3 + k] -= t3[k];
            }
          }
          if (sf_out) {
            double* sp = &sfl[(size_t)pi * 6];
            sp[0] -= dx * t3[0]; sp[1] -= dy * t3[1]; sp[2] -= dz * t3[2];
            sp[3] -= dy * t3[2]; sp[4] -= dz * t3[0]; sp[5] -= dx * t3[1];
          }
        }
      }
    }
  }
  for (int t = 0; t < nth; ++t) {
    if (ff_out && !ffb[t].empty())
      for (size_t k = 0; k < ffb[t].size(); ++k) ff_out[k] += ffb[t][k];
    if (sf_out && !sfb[t].empty())
      for (size_t k = 0; k < sfb[t].size(); ++k) sf_out[k] += sfb[t][k];
  }
  return 0;
}

// Conditioning of the linear energy terms, for the error bound of an
// evaluation with FP32 products: per owned atom, the sum over the features
// that enter no polynomial term of order >= 2 ("linear-only" features) of
// |w_f| * sum_terms |c| prod |a|.  An evaluation whose products and inputs
// carry a relative error eps errs by at most a small multiple of eps times
// this sum in those terms.  (The polynomial's input features are not
// counted: their energy is evaluated in FP64 by the mixed GPU path.)
// out[nlocal]; 0 for unhandled atoms.  Test infrastructure.
int orc_linear_conditioning(void* h, int nlocal, int nall, const double* x, const int* type,
                            const int* off, const int* nbr, double* out) {
  Oracle* o = static_cast<Oracle*>(h);
  const Model& M = o->M;
  const Geometry g{nlocal, nall, x, type, off, nbr};
  const int F = M.F, La = M.La, ITCn = M.ITC_n;
  std::vector<char> nl(ITCn, 0);
  vd w(M.D, 0.0);
  for (size_t pi = 0; pi < M.poly.size(); ++pi) {
    if (M.poly[pi].size() >= 2)
      for (int f : M.poly[pi]) nl[f % ITCn] = 1;
    else
      w[M.poly[pi][0]] += M.pot.coeffs[pi];
  }
#ifdef _OPENMP
#pragma omp parallel num_threads(o->nthreads)
#endif
  {
    SHWork sw;
    vd fn, fnd;
    AtomState s;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
    for (int i = 0; i < nlocal; ++i) {
      out[i] = 0.0;
      const int ti = type[i];
      if (ti < 0) continue;
      atom_order_params(M, g, i, s, sw, fn, fnd);
      double acc = 0.0;
      for (int f = 0; f < M.D; ++f) {
        const int itc = f % ITCn;
        if (nl[itc] || !M.itc[itc].inter[ti] || w[f] == 0.0) continue;
        const int n = f / ITCn;
        const auto& tcs = M.itc[itc].type_combs;
        const int ir = M.itc[itc].irreps;
        double D = 0.0;
        for (int term = 0; term < M.irr_nterms[ir]; ++term) {
          const int it = M.irr_first[ir] + term;
          double prod = std::fabs(M.term_c[it]);
          for (size_t p = 0; p < tcs.size(); ++p) {
            const int t2 = M.other_type[tcs[p]][ti];
            const cplx v = s.a[((size_t)t2 * F + n) * La + M.term_lm[it][p]];
            prod *= std::sqrt(v.re * v.re + v.im * v.im);
          }
          D += prod;
        }
        acc += std::fabs(w[f]) * D;
      }
      out[i] = acc;
    }
  }
  return 0;
}

// Owner-computes evaluation for a list of centre atoms: each centre's energy,
// and the forces/virial generated by its own adjoint only (the other half of
// every pair comes from the neighbour's own centre evaluation).  Summed over
// all atoms this equals orc_compute; on a subset it is the per-atom cost
// sample used for the CPU baseline.  f accumulates into [nall*3].
int orc_compute_centers(void* h, int ncenters, const int* centers, int nall, const double* x,
                        const int* type, const int* off, const int* nbr, double* f,
                        double* energy, double* virial, double* eatom) {
  Oracle* o = static_cast<Oracle*>(h);
  const Model& M = o->M;
  const Geometry g{0, nall, x, type, off, nbr};
  const int F = M.F, Lh = M.Lh;
  double E = 0.0;
  double vir[6] = {0, 0, 0, 0, 0, 0};
  int nth = o->nthreads;
  std::vector<vd> fbuf(nth);
#ifdef _OPENMP
#pragma omp parallel num_threads(nth) reduction(+ : E)
#endif
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    vd& fl = fbuf[tid];
    fl.assign((size_t)3 * nall, 0.0);
    double vl[6] = {0, 0, 0, 0, 0, 0};
    SHWork w;
    vd fn, fnd;
    AtomState s;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
    for (int c = 0; c < ncenters; ++c) {
      const int i = centers[c];
      if (type[i] < 0) continue;
      atom_order_params(M, g, i, s, w, fn, fnd);
      atom_adjoints(M, type[i], s);
      E += s.E;
      if (eatom) eatom[c] = s.E;
      for (int p = off[i]; p < off[i + 1]; ++p) {
        const int j = nbr[p];
        if (type[j] < 0) continue;
        const double dx = x[3 * j] - x[3 * i];
        const double dy = x[3 * j + 1] - x[3 * i + 1];
        const double dz = x[3 * j + 2] - x[3 * i + 2];
        const double dis = std::sqrt(dx * dx + dy * dy + dz * dz);
        if (dis > M.pot.cutoff) continue;
        const double invdis = 1.0 / dis;
        compute_sh(M, dz / dis, std::atan2(dy, dx), dis, true, w);
        compute_fn(M, dis, fn, fnd);
        const int tc = M.type_pairs[type[i]][type[j]];
        double fx = 0, fy = 0, fz = 0;
        int lmi = 0;
        for (int l = 0; l <= M.L; ++l)
          for (int m = -l; m <= 0; ++m, ++lmi) {
            const double coeff = (m == 0) ? 1.0 : 2.0;
            for (int n = 0; n < F; ++n) {
              const cplx f1 = cscale(w.ylm[lmi], fnd[n]);
              cplx bx = {f1.re * dx * invdis + fn[n] * w.dx[lmi].re,
                         -(f1.im * dx * invdis + fn[n] * w.dx[lmi].im)};
              cplx by = {f1.re * dy * invdis + fn[n] * w.dy[lmi].re,
                         -(f1.im * dy * invdis + fn[n] * w.dy[lmi].im)};
              cplx bz = {f1.re * dz * invdis + fn[n] * w.dz[lmi].re,
                         -(f1.im * dz * invdis + fn[n] * w.dz[lmi].im)};
              const cplx gi = s.G[((size_t)tc * F + n) * Lh + lmi];
              fx += coeff * prod_real(gi, bx);
              fy += coeff * prod_real(gi, by);
              fz += coeff * prod_real(gi, bz);
            }
          }
        fl[3 * i] += fx; fl[3 * i + 1] += fy; fl[3 * i + 2] += fz;
        fl[3 * j] -= fx; fl[3 * j + 1] -= fy; fl[3 * j + 2] -= fz;
        vl[0] -= dx * fx; vl[1] -= dy * fy; vl[2] -= dz * fz;
        vl[3] -= dx * fy; vl[4] -= dz * fx; vl[5] -= dy * fz;
      }
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    for (int k = 0; k < 6; ++k) vir[k] += vl[k];
  }
  for (int t = 0; t < nth; ++t)
    if (!fbuf[t].empty())
      for (size_t k = 0; k < (size_t)3 * nall; ++k) f[k] += fbuf[t][k];
  *energy = E;
  for (int k = 0; k < 6; ++k) virial[k] = vir[k];
  return 0;
}

}  // extern "C"
