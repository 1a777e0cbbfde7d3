// Host-side model: parser, coupling table, enumeration and device schedules.
// See model.hpp for the reference functions restated here.
#include "model.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <map>
#include <queue>
#include <set>
#include <sstream>

namespace mlipg {

namespace {

#include "gtinv_table.inc"  // defines kGtinvTableText (generated from data/gtinv_table.txt)

struct Table {
  std::vector<std::vector<int>> l;
  std::vector<std::vector<std::vector<int>>> m;
  std::vector<std::vector<double>> c;
};

const Table& table() {
  static Table t = [] {
    Table tab;
    std::stringstream all;
    std::stringstream src(kGtinvTableText);
    std::string line;
    while (std::getline(src, line)) {
      if (!line.empty() && line[0] == '#') continue;
      all << line << '\n';
    }
    int n = 0;
    all >> n;
    tab.l.resize(n);
    tab.m.resize(n);
    tab.c.resize(n);
    for (int i = 0; i < n; ++i) {
      int q = 0;
      all >> q;
      tab.l[i].resize(q);
      for (int k = 0; k < q; ++k) all >> tab.l[i][k];
      int nt = 0;
      all >> nt;
      tab.m[i].assign(nt, std::vector<int>(q));
      tab.c[i].assign(nt, 0.0);
      for (int j = 0; j < nt; ++j) {
        all >> tab.c[i][j];
        for (int k = 0; k < q; ++k) all >> tab.m[i][j][k];
      }
    }
    return tab;
  }();
  return t;
}

bool getline_ss(std::ifstream& in, std::stringstream& ss, std::string& err) {
  std::string l;
  if (!std::getline(in, l)) {
    err = "potential file is truncated";
    return false;
  }
  ss.str(l);
  ss.clear();
  return true;
}

std::vector<std::pair<int, int>> type_pairs_mapping(int T) {
  std::vector<std::pair<int, int>> v;
  for (int a = 0; a < T; ++a)
    for (int b = a; b < T; ++b) v.push_back({a, b});
  return v;
}

std::vector<char> intersection_of(int T, const std::vector<std::pair<int, int>>& tpm,
                                  const std::vector<int>& comb) {
  std::vector<char> in(T, 1);
  for (int idx : comb)
    for (int t = 0; t < T; ++t)
      if (t != tpm[idx].first && t != tpm[idx].second) in[t] = 0;
  return in;
}

bool any_of(const std::vector<char>& v) {
  return std::any_of(v.begin(), v.end(), [](char e) { return e != 0; });
}

// Multisets of size r over {0..n-1} in lexicographic order (the breadth-first
// generation of mlipkk_utils.cpp:33-58 visits them in this order).
void multisets_lex(int n, int r, std::vector<std::vector<int>>& out) {
  std::vector<int> c(r, 0);
  if (r == 0) return;
  while (true) {
    out.push_back(c);
    int k = r - 1;
    while (k >= 0 && c[k] == n - 1) --k;
    if (k < 0) break;
    int v = c[k] + 1;
    for (int j = k; j < r; ++j) c[j] = v;
  }
}

// Non-increasing sequences of length r with first element ascending, then
// lexicographic: the "historical" order of mlipkk_utils.cpp:64-98.
void sequences_gtinv(int n, int r, std::vector<std::vector<int>>& out) {
  std::vector<int> c(r, 0);
  for (int first = 0; first < n; ++first) {
    c[0] = first;
    for (int j = 1; j < r; ++j) c[j] = 0;
    while (true) {
      out.push_back(c);
      int k = r - 1;
      while (k >= 1 && c[k] == c[k - 1]) --k;
      if (k < 1) break;
      ++c[k];
      for (int j = k + 1; j < r; ++j) c[j] = 0;
    }
  }
}

void screen(const Potential& p, Model& M) {
  const Table& tab = table();
  int count = 0;
  for (size_t i = 0; i < tab.l.size(); ++i) {
    const auto& lc = tab.l[i];
    const int order = (int)lc.size();
    bool req = true;
    if (order > 1) {
      if (order > p.gtinv_order || lc.back() > p.gtinv_maxl[order - 2]) req = false;
      else if (p.gtinv_sym[order - 2] &&
               (int)std::count(lc.begin(), lc.end(), lc[0]) != order)
        req = false;
    }
    if (!req) continue;
    M.irr_l.push_back(lc);
    M.irr_first.push_back(count);
    M.irr_nterms.push_back((int)tab.m[i].size());
    for (size_t j = 0; j < tab.m[i].size(); ++j) {
      std::vector<int> lm(order);
      for (int k = 0; k < order; ++k) lm[k] = lc[k] * lc[k] + lc[k] + tab.m[i][j][k];
      M.term_lm.push_back(lm);
      M.term_c.push_back(tab.c[i][j]);
      ++count;
    }
  }
}

void build_itc(Model& M) {
  const int T = M.T, ntc = T * (T + 1) / 2;
  auto tpm = type_pairs_mapping(T);
  const int max_order = (int)M.irr_l.back().size();
  std::vector<std::vector<std::vector<int>>> uniq(max_order);
  for (int order = 1; order <= max_order; ++order) {
    std::vector<std::vector<int>> all;
    multisets_lex(ntc, order, all);
    for (auto& c : all)
      if (any_of(intersection_of(T, tpm, c))) uniq[order - 1].push_back(c);
  }
  for (int i = 0; i < (int)M.irr_l.size(); ++i) {
    const auto& lc = M.irr_l[i];
    const int order = (int)lc.size();
    std::set<std::vector<std::pair<int, int>>> sets;
    for (auto tcomb : uniq[order - 1]) {
      do {
        std::vector<std::pair<int, int>> ms(order);
        for (int j = 0; j < order; ++j) ms[j] = {lc[j], tcomb[j]};
        std::sort(ms.begin(), ms.end());
        sets.insert(ms);
      } while (std::next_permutation(tcomb.begin(), tcomb.end()));
    }
    for (auto& ms : sets) {
      ITC x;
      x.irreps = i;
      for (auto& pr : ms) x.type_combs.push_back(pr.second);
      x.inter = intersection_of(T, tpm, x.type_combs);
      M.itc.push_back(x);
    }
  }
}

std::vector<char> poly_intersection(const Model& M, const std::vector<int>& fc) {
  std::vector<char> in(M.T, 1);
  for (int f : fc) {
    const auto& x = M.itc[f % M.n_itc].inter;
    for (int t = 0; t < M.T; ++t) in[t] = in[t] && x[t];
  }
  return in;
}

bool build_poly(Model& M, std::string& err) {
  const int D = M.D, mt = M.pot.model_type, maxp = M.pot.maxp;
  const size_t limit = 200000000;  // entries; larger models are not representable
  auto check = [&](size_t n) {
    if (n > limit) {
      err = "polynomial index too large for this model_type";
      return false;
    }
    return true;
  };
  if (mt == 1) {
    for (int po = 1; po <= maxp; ++po)
      for (int f = 0; f < D; ++f)
        if (any_of(M.itc[f % M.n_itc].inter)) M.poly.push_back(std::vector<int>(po, f));
  } else if (mt == 2) {
    for (int po = 1; po <= maxp; ++po) {
      double est = 1;
      for (int k = 0; k < po; ++k) est = est * (D + k) / (k + 1);
      if (!check((size_t)est * po)) return false;
      std::vector<std::vector<int>> all;
      sequences_gtinv(D, po, all);
      for (auto& fc : all)
        if (any_of(poly_intersection(M, fc))) M.poly.push_back(fc);
    }
  } else if (mt == 3 || mt == 4) {
    std::vector<int> lower;
    for (int f = 0; f < D; ++f) {
      const int q = (int)M.itc[f % M.n_itc].type_combs.size();
      if ((mt == 3 && q == 1) || (mt == 4 && q <= 2)) lower.push_back(f);
    }
    for (int f = 0; f < D; ++f) M.poly.push_back({f});
    for (int po = 2; po <= maxp; ++po) {
      std::vector<std::vector<int>> all;
      sequences_gtinv((int)lower.size(), po, all);
      for (auto& ch : all) {
        std::vector<int> fc(po);
        for (int k = 0; k < po; ++k) fc[k] = lower[ch[k]];
        if (any_of(poly_intersection(M, fc))) M.poly.push_back(fc);
      }
    }
  } else {
    err = "Unknown model_type: " + std::to_string(mt);
    return false;
  }
  return true;
}

// Folds each conjugate pair of raw terms into one canonical DeviceTerm.
bool fold_terms(Model& M, std::string& err) {
  for (size_t k = 0; k < M.irr_l.size(); ++k) {
    const auto& lc = M.irr_l[k];
    const int q = (int)lc.size();
    M.irr_cfirst.push_back((int)M.cterms.size());
    std::map<std::vector<int>, double> byM;
    for (int j = 0; j < M.irr_nterms[k]; ++j) {
      const int t = M.irr_first[k] + j;
      std::vector<int> mv(q);
      for (int p = 0; p < q; ++p) mv[p] = M.term_lm[t][p] - lc[p] * lc[p] - lc[p];
      byM[mv] = M.term_c[t];
    }
    int n = 0;
    for (int j = 0; j < M.irr_nterms[k]; ++j) {
      const int t = M.irr_first[k] + j;
      std::vector<int> mv(q), neg(q);
      for (int p = 0; p < q; ++p) {
        mv[p] = M.term_lm[t][p] - lc[p] * lc[p] - lc[p];
        neg[p] = -mv[p];
      }
      int first_nz = 0;
      for (int p = 0; p < q; ++p)
        if (mv[p] != 0) { first_nz = mv[p]; break; }
      const bool self = (first_nz == 0);
      if (first_nz > 0) {
        if (!byM.count(neg)) {
          err = "coupling table is not closed under m -> -m";
          return false;
        }
        continue;  // represented by its partner
      }
      if (!self && !byM.count(neg)) {
        err = "coupling table is not closed under m -> -m";
        return false;
      }
      DeviceTerm d{};
      double c = M.term_c[t];
      uint16_t code = 0;
      for (int p = 0; p < q; ++p) {
        const int l = lc[p], m = mv[p];
        d.lmh[p] = (uint8_t)(l * (l + 1) / 2 + l - std::abs(m));
        int sc;
        if (m > 0) {
          if (m % 2) c = -c;
          sc = kSlotConj;
        } else if (m < 0) {
          sc = kSlotNormal;
        } else {
          sc = self ? kSlotSelf : kSlotMZero;
        }
        code |= (uint16_t)(sc << (2 * p));
      }
      if (self) code |= (uint16_t)(1u << 12);
      d.c = c;
      d.code = code;
      M.cterms.push_back(d);
      ++n;
    }
    M.irr_cnterms.push_back(n);
  }
  return true;
}

// Deals cost-sorted work items to kCtaWarps lists, each item onto the
// least-loaded list (longest processing time first), and interleaves the
// lists so that the kernel's round-robin `for (u = warp; ...; u += kCtaWarps)`
// walks exactly list `warp`; short lists are padded with `pad`.
template <typename U, typename Cost>
std::vector<U> deal_longest_first(std::vector<U> v, Cost cost, double* load, const U& pad) {
  std::stable_sort(v.begin(), v.end(), [&](const U& a, const U& b) { return cost(a) > cost(b); });
  std::vector<std::vector<U>> lists(kCtaWarps);
  for (const U& x : v) {
    int w = 0;
    for (int k = 1; k < kCtaWarps; ++k)
      if (load[k] < load[w]) w = k;
    lists[w].push_back(x);
    load[w] += cost(x);
  }
  size_t rounds = 0;
  for (auto& l : lists) rounds = std::max(rounds, l.size());
  std::vector<U> out(rounds * kCtaWarps, pad);
  for (int w = 0; w < kCtaWarps; ++w)
    for (size_t r = 0; r < lists[w].size(); ++r) out[r * kCtaWarps + w] = lists[w][r];
  return out;
}

// Upper bound of the adjoint flushes one order-parameter row lm of a centre
// of element t receives: every term of every unit flushes each slot at most
// once (counted per lm over all elements of the slot, which over-counts).
int max_flushes_per_entry(const Model& M, int t) {
  const Schedule& S = M.sched[t];
  std::vector<int> cnt(std::max(M.Lh, 1), 0);
  const auto add_terms = [&](int term0, int nterm, int q) {
    for (int k = term0; k < term0 + nterm; ++k)
      for (int p = 0; p < q; ++p) cnt[M.cterms[k].lmh[p]]++;
  };
  for (const DeviceIrrUnit& u : S.iunits)
    if (u.nterm > 0) add_terms(u.term0, u.nterm, u.q);
  for (const DeviceUnit& u : S.units)
    if (u.nterm > 0) add_terms(u.term0, u.nterm, u.q);
  return *std::max_element(cnt.begin(), cnt.end());
}

void set_adjoint_bound(Model& M) {
  int cmax = 1;
  for (int t = 0; t < M.T; ++t) cmax = std::max(cmax, max_flushes_per_entry(M, t));
  // high parts are multiples of 2^16 (at most bound / 2^16 each): their int32
  // sum stays below 2^31; the high-part rounding is exact below 2^38; low
  // parts (|.| <= 2^15) cannot overflow for fewer than 2^16 flushes
  double b = 274877906944.0;   // 2^38
  while ((b / 65536.0) * (cmax + 1) >= 2147483648.0 && b > 65536.0) b *= 0.5;
  M.g_bound = cmax < 65535 ? b : 0.0;   // 0: no fixed-point accumulation possible
  // double-float path: four words, multiples of 2^48 (at most bound / 2^48
  // each, int32 sum below 2^31), of 2^32, 2^16 and 1 (at most 2^16 + 2 per
  // flush: fewer than 2^15 - 2 flushes cannot overflow); the split's
  // magic-number roundings are exact below 2^70
  double bd = 1180591620717411303424.0;   // 2^70
  while ((bd / 281474976710656.0) * (cmax + 1) >= 2147483648.0 && bd > 65536.0) bd *= 0.5;
  M.g_bound_df = cmax < 32765 ? bd : 0.0;
  // the double-float path has FP32's exponent range: potentials whose
  // coefficients come near it (|.| > 1e30) run the all-FP64 kernel instead
  double cmaxabs = 0.0;
  for (double v : M.pot.coeffs) cmaxabs = std::max(cmaxabs, std::fabs(v));
  for (const DeviceTerm& t : M.cterms) cmaxabs = std::max(cmaxabs, std::fabs(t.c));
  if (!(cmaxabs <= 1e30)) M.g_bound_df = 0.0;
}

bool schedules_for_tiling(Model& M, std::string& err) {
  const int T = M.T, F = M.F;
  // nonlinear itc: appear in any polynomial term of order >= 2
  std::vector<char> is_nl(M.n_itc, 0);
  for (auto& row : M.poly)
    if (row.size() >= 2)
      for (int f : row) is_nl[f % M.n_itc] = 1;
  M.w_lin.assign((size_t)M.n_itc * kNPad, 0.0);
  for (size_t pi = 0; pi < M.poly.size(); ++pi)
    if (M.poly[pi].size() == 1) {
      const int f = M.poly[pi][0];
      M.w_lin[(size_t)(f % M.n_itc) * kNPad + f / M.n_itc] += M.pot.coeffs[pi];
    }
  M.sched.assign(T, Schedule());
  M.max_nl = 0;
  M.lh64 = 0;
  for (int t = 0; t < T; ++t) {
    Schedule& S = M.sched[t];
    std::vector<int> slot(M.n_itc, -1);
    // nonlinear slots first (independent of how the itc is evaluated)
    for (int i = 0; i < M.n_itc; ++i) {
      if (!M.itc[i].inter[t] || !is_nl[i]) continue;
      const int k = M.itc[i].irreps;
      DeviceUnit u{};
      u.itc = i;
      u.term0 = M.irr_cfirst[k];
      u.nterm = M.irr_cnterms[k];
      u.q = (uint8_t)M.irr_l[k].size();
      for (int p = 0; p < u.q; ++p) u.s[p] = (uint8_t)M.other_type[M.itc[i].type_combs[p] * T + t];
      u.nl_slot = (int)S.nl_units.size();
      slot[i] = u.nl_slot;
      S.nl_units.push_back(u);
    }
    // batched-tuple units for orders <= 4 when T <= 3
    std::vector<char> covered(M.n_itc, 0);
    if (T <= 3) {
      std::map<std::pair<int, std::vector<int>>, int> itc_of;
      for (int i = 0; i < M.n_itc; ++i) itc_of[{M.itc[i].irreps, M.itc[i].type_combs}] = i;
      for (int k = 0; k < (int)M.irr_l.size(); ++k) {
        const auto& lc = M.irr_l[k];
        const int q = (int)lc.size();
        if (q > 4) continue;
        int nt = 1;
        for (int p = 0; p < q; ++p) nt *= T;
        const int tup0 = (int)S.tuples.size();
        for (int j = 0; j < nt; ++j) {
          std::vector<int> sv(q), tc(q);
          int r = j;
          for (int p = q - 1; p >= 0; --p) { sv[p] = r % T; r /= T; }
          bool canon = true;
          for (int p = 1; p < q; ++p)
            if (lc[p] == lc[p - 1] && sv[p] < sv[p - 1]) canon = false;
          DeviceTuple d{-1, -1};
          if (canon) {
            for (int p = 0; p < q; ++p) tc[p] = M.type_pairs[t * T + sv[p]];
            auto it = itc_of.find({k, tc});
            if (it != itc_of.end() && M.itc[it->second].inter[t]) {
              d.itc = it->second;
              d.nl_slot = slot[it->second];
              covered[it->second] = 1;
            }
          }
          S.tuples.push_back(d);
        }
        // order 4: one unit per element of slot 0, each over the T^3 tuples
        // of the other slots; lower orders: one unit over all T^q tuples;
        // blocks without any feature are skipped
        const int nsub = q == 4 ? T : 1;
        const int block = q == 1 ? T : (q == 2 ? T * T : T * T * T);
        for (int f = 0; f < nsub; ++f) {
          bool any = false;
          for (int j = 0; j < block; ++j) any = any || S.tuples[tup0 + f * block + j].itc >= 0;
          if (!any) continue;
          for (int c0 = 0; c0 < M.irr_cnterms[k]; c0 += M.tiling.irr_chunk) {
            DeviceIrrUnit iu{};
            iu.term0 = M.irr_cfirst[k] + c0;
            iu.nterm = std::min(M.tiling.irr_chunk, M.irr_cnterms[k] - c0);
            iu.tup = tup0 + f * block;
            iu.q = (uint8_t)q;
            iu.s0 = (uint8_t)f;
            S.iunits.push_back(iu);
          }
        }
      }
      std::stable_sort(S.iunits.begin(), S.iunits.end(),
                       [](const DeviceIrrUnit& a, const DeviceIrrUnit& b) {
                         if (a.nterm * a.q != b.nterm * b.q) return a.nterm * a.q > b.nterm * b.q;
                         return a.q > b.q;
                       });
    }
    for (int i = 0; i < M.n_itc; ++i) {
      if (!M.itc[i].inter[t] || covered[i]) continue;
      const int k = M.itc[i].irreps;
      DeviceUnit u{};
      u.itc = i;
      u.term0 = M.irr_cfirst[k];
      u.nterm = M.irr_cnterms[k];
      u.q = (uint8_t)M.irr_l[k].size();
      for (int p = 0; p < u.q; ++p) u.s[p] = (uint8_t)M.other_type[M.itc[i].type_combs[p] * T + t];
      u.nl_slot = slot[i];
      S.units.push_back(u);
    }
    // longest units first, grouped by order
    std::stable_sort(S.units.begin(), S.units.end(), [](const DeviceUnit& a, const DeviceUnit& b) {
      if (a.q != b.q) return a.q > b.q;
      return a.nterm > b.nterm;
    });
    M.max_nl = std::max(M.max_nl, (int)S.nl_units.size());
    for (const DeviceUnit& u : S.nl_units) {
      const auto& lc = M.irr_l[M.itc[u.itc].irreps];
      const int lmax = *std::max_element(lc.begin(), lc.end());
      M.lh64 = std::max(M.lh64, (lmax + 1) * (lmax + 2) / 2);
    }
    for (size_t pi = 0; pi < M.poly.size(); ++pi) {
      const auto& row = M.poly[pi];
      if (row.size() < 2) continue;
      bool ok = true;
      for (int f : row) ok = ok && M.itc[f % M.n_itc].inter[t];
      if (!ok) continue;
      DevicePoly dp{};
      dp.w = M.pot.coeffs[pi];
      dp.order = (int)row.size();
      for (int p = 0; p < dp.order; ++p)
        dp.k[p] = slot[row[p] % M.n_itc] * kNPad + row[p] / M.n_itc;
      S.poly.push_back(dp);
    }
    {
      const size_t ne = S.nl_units.size() * kNPad;
      std::vector<std::vector<int>> lists(ne);
      for (size_t pi = 0; pi < S.poly.size(); ++pi)
        for (int q = 0; q < S.poly[pi].order; ++q)
          lists[S.poly[pi].k[q]].push_back((int)pi * 4 + q);
      S.adj_off.assign(ne + 1, 0);
      S.adj.clear();
      for (size_t e = 0; e < ne; ++e) {
        S.adj.insert(S.adj.end(), lists[e].begin(), lists[e].end());
        S.adj_off[e + 1] = (int)S.adj.size();
      }
    }
    (void)F;
    // a batched unit is all polynomial inputs or all linear-only features
    // (nonlinearity is a property of the irreps' order for every model type)
    for (DeviceIrrUnit& iu : S.iunits) {
      int nl = -1;
      const int nt = iu.q == 1 ? T : (iu.q == 2 ? T * T : T * T * T);
      for (int j = 0; j < nt; ++j) {
        const DeviceTuple& d = S.tuples[iu.tup + j];
        if (d.itc < 0) continue;
        const int v = d.nl_slot >= 0 ? 1 : 0;
        if (nl >= 0 && nl != v) {
          err = "internal error: a work unit mixes polynomial and linear-only features";
          return false;
        }
        nl = v;
      }
      iu.nl = (uint8_t)(nl > 0 ? 1 : 0);
    }
    // every feature valid for this element is evaluated exactly once
    std::vector<int> seen(M.n_itc, 0);
    for (const DeviceTuple& d : S.tuples)
      if (d.itc >= 0) seen[d.itc]++;
    for (const DeviceUnit& u : S.units) seen[u.itc]++;
    for (int i = 0; i < M.n_itc; ++i)
      if (seen[i] != (M.itc[i].inter[t] ? 1 : 0)) {
        err = "internal error: work schedule does not cover every feature once";
        return false;
      }
    if (M.tiling.warp_order == 2) {
      // taken by the warps from a shared counter in this order: one coupling
      // order at a time (same code path), longest units first
      std::stable_sort(S.iunits.begin(), S.iunits.end(),
                       [](const DeviceIrrUnit& a, const DeviceIrrUnit& b) {
                         if (a.q != b.q) return a.q > b.q;
                         return a.nterm > b.nterm;
                       });
    }
    if (M.tiling.warp_order == 1) {
      // per-warp cost ~ terms x tuples x order (products and adjoint products)
      // batched unit per term: products over the tuple block, one atomic
      // pair per (slot, element)
      const auto icost = [&](const DeviceIrrUnit& u) {
        const double nz = u.q >= 3 ? T : 1;
        return (double)u.nterm * (u.q == 1 ? 2.0 * T : nz * 8.0 * T * T + 12.0 * T * (u.q - 1));
      };
      const auto ucost = [](const DeviceUnit& u) { return (double)u.nterm * u.q; };
      double load[kCtaWarps] = {};
      DeviceIrrUnit ipad{};
      ipad.tup = S.iunits.empty() ? 0 : S.iunits[0].tup;
      DeviceUnit upad{};
      upad.itc = -1;
      upad.nl_slot = -1;
      // dealt one order at a time (highest first), so that the warps run the
      // same unit variant at the same time (one code path in the
      // instruction cache); balance carries over between the groups
      std::vector<DeviceIrrUnit> dealt;
      for (int q = kMaxOrder; q >= 1; --q) {
        std::vector<DeviceIrrUnit> grp;
        for (const DeviceIrrUnit& u : S.iunits)
          if (u.q == q) grp.push_back(u);
        if (grp.empty()) continue;
        grp = deal_longest_first(grp, icost, load, ipad);
        dealt.insert(dealt.end(), grp.begin(), grp.end());
      }
      S.iunits = dealt;
      S.units = deal_longest_first(S.units, ucost, load, upad);
    }
  }
  return true;
}

}  // namespace

bool build_schedules(Model& M, std::string& err) {
  if (M.pot.pair) return true;   // the radial-only kernel has no tile shape
  if (M.tiling.irr_chunk < 2 || M.tiling.irr_chunk > 4096 || M.tiling.irr_chunk % 2 ||
      M.tiling.warp_order < 0 || M.tiling.warp_order > 2 || M.tiling.ctas_per_sm < 0) {
    err = "invalid tiling";
    return false;
  }
  if (!schedules_for_tiling(M, err)) return false;
  set_adjoint_bound(M);
  return true;
}

bool read_potential(const std::string& path, Potential& p, std::string& err) {
  std::ifstream in(path);
  if (!in) {
    err = "Could not open mlip file: " + path;
    return false;
  }
  std::string line;
  if (!std::getline(in, line)) {
    err = "potential file is empty";
    return false;
  }
  {
    // line 1: element names, then a "# element" comment
    std::stringstream ss(line);
    std::string tok;
    while (ss >> tok) {
      if (tok[0] == '#') break;
      p.elements.push_back(tok);
    }
  }
  if (p.elements.empty()) {
    err = "no element names on the first line of the potential file";
    return false;
  }
  std::stringstream ss;
  std::string s;
  if (!getline_ss(in, ss, err)) return false;
  ss >> p.cutoff;
  if (!getline_ss(in, ss, err)) return false;
  ss >> s;
  if (s != "gaussian") {
    err = "Unknown pair_type: " + s;
    return false;
  }
  if (!getline_ss(in, ss, err)) return false;
  ss >> s;
  if (s != "gtinv" && s != "pair") {
    err = "Unknown des_type: " + s;
    return false;
  }
  p.pair = s == "pair";
  if (!getline_ss(in, ss, err)) return false;
  ss >> p.model_type;
  if (!getline_ss(in, ss, err)) return false;
  ss >> p.maxp;
  if (!getline_ss(in, ss, err)) return false;
  ss >> p.maxl;
  if (p.pair) {
    // the radial-only descriptor's file has no invariant lines
    // (src/USER-MLIP/mlip_model.h:61-74)
    p.gtinv_order = 1;
  } else {
    if (!getline_ss(in, ss, err)) return false;
    ss >> p.gtinv_order;
    const int nm = p.gtinv_order - 1;
    if (nm < 0 || nm > kMaxOrder - 1) {
      err = "gtinv_order out of range";
      return false;
    }
    if (!getline_ss(in, ss, err)) return false;
    p.gtinv_maxl.assign(nm, 0);
    for (auto& v : p.gtinv_maxl) ss >> v;
    if (!getline_ss(in, ss, err)) return false;
    p.gtinv_sym.assign(nm, 0);
    for (auto& v : p.gtinv_sym) ss >> v;
  }
  long nc = 0;
  if (!getline_ss(in, ss, err)) return false;
  ss >> nc;
  if (nc < 0) {
    err = "negative number of regression coefficients";
    return false;
  }
  p.coeffs.assign(nc, 0.0);
  if (!getline_ss(in, ss, err)) return false;
  for (auto& v : p.coeffs) ss >> v;
  if (!ss && nc > 0) {
    err = "too few regression coefficients";
    return false;
  }
  if (!getline_ss(in, ss, err)) return false;
  for (long k = 0; k < nc; ++k) {
    double sc = 1.0;
    ss >> sc;
    p.coeffs[k] /= sc;
  }
  int npar = 0;
  if (!getline_ss(in, ss, err)) return false;
  ss >> npar;
  for (int k = 0; k < npar; ++k) {
    if (!getline_ss(in, ss, err)) return false;
    double b = 0, m = 0;
    ss >> b >> m;
    p.params.push_back({b, m});
  }
  if (!getline_ss(in, ss, err)) return false;
  p.masses.assign(p.elements.size(), 0.0);
  for (auto& m : p.masses) ss >> m;
  return true;
}

// Radial-only descriptor of the legacy `pair_style mlip_pair`: feature
// index tc * F + n, with the type pairs tc ordered (a, b), a <= b
// (src/USER-MLIP/mlip_model_params.cpp:29-34); coefficient order: the linear
// terms, then the second- and third-order terms -- every feature squared and
// cubed for model_type 1 (mlip_polynomial.cpp:33-38), for model_type 2 the
// multisets of features whose type pairs share an element, enumerated
// i1 >= i2 (>= i3) (mlip_model_params.cpp:180-213); model_types 3 and 4 are
// linear for this descriptor (mlip_model_params.cpp:42-66).  The legacy
// reader doubles the coefficients (mlip_model.h:90) and its half-list pair
// sums count each term twice, so the per-atom energy is the plain polynomial
// of dn with coefficient / scale.
bool build_pair_model(Model& M, std::string& err) {
  const Potential& p = M.pot;
  const int T = M.T, F = M.F;
  if (T < 1 || T > 2) {
    err = "the pair descriptor supports one or two elements";
    return false;
  }
  if (F < 1 || F > kPairMaxF) {
    err = "number of radial functions of a pair potential must be in [1, 64]";
    return false;
  }
  M.TC = T * (T + 1) / 2;
  std::vector<std::pair<int, int>> tcs;
  for (int a = 0; a < T; ++a)
    for (int b = a; b < T; ++b) tcs.push_back({a, b});
  M.type_pairs.assign(T * T, 0);
  for (int tc = 0; tc < M.TC; ++tc) {
    M.type_pairs[tcs[tc].first * T + tcs[tc].second] = tc;
    M.type_pairs[tcs[tc].second * T + tcs[tc].first] = tc;
  }
  const int nd = F * M.TC;
  const auto has = [&](int seq, int t) {
    return tcs[seq / F].first == t || tcs[seq / F].second == t;
  };
  const auto shared = [&](const std::vector<int>& seqs) {
    for (int t = 0; t < T; ++t) {
      bool all = true;
      for (int q : seqs) all = all && has(q, t);
      if (all) return true;
    }
    return false;
  };
  M.poly.clear();
  for (int n = 0; n < nd; ++n) M.poly.push_back({n});
  if (p.model_type == 1) {
    if (p.maxp > 1) for (int n = 0; n < nd; ++n) M.poly.push_back({n, n});
    if (p.maxp > 2) for (int n = 0; n < nd; ++n) M.poly.push_back({n, n, n});
  } else if (p.model_type == 2) {
    if (p.maxp > 1)
      for (int i1 = 0; i1 < nd; ++i1)
        for (int i2 = 0; i2 <= i1; ++i2)
          if (shared({i1, i2})) M.poly.push_back({i2, i1});
    if (p.maxp > 2)
      for (int i1 = 0; i1 < nd; ++i1)
        for (int i2 = 0; i2 <= i1; ++i2)
          for (int i3 = 0; i3 <= i2; ++i3)
            if (shared({i1, i2, i3})) M.poly.push_back({i3, i2, i1});
  } else if (p.model_type < 1 || p.model_type > 4) {
    err = "Unknown model_type: " + std::to_string(p.model_type);
    return false;
  }
  if (M.poly.size() != p.coeffs.size()) {
    char b[200];
    snprintf(b, sizeof b, "number of regression coefficients %zu does not match the model (%zu)",
             p.coeffs.size(), M.poly.size());
    err = b;
    return false;
  }
  M.D = nd;
  // per centre element: the terms whose type pairs all contain it (the
  // others multiply a feature that is zero for it), and the adjoint records
  M.pair_terms.clear();
  M.pair_term_off.assign(T + 1, 0);
  M.pair_adj.clear();
  M.pair_adj_off.assign((size_t)T * nd + 1, 0);
  for (int t = 0; t < T; ++t) {
    M.pair_term_off[t] = (int)M.pair_terms.size();
    std::vector<std::vector<DevicePairAdj>> adj(nd);
    for (size_t k = 0; k < M.poly.size(); ++k) {
      const auto& row = M.poly[k];
      bool ok = true;
      for (int q : row) ok = ok && has(q, t);
      if (!ok) continue;
      DevicePairTerm dt{};
      dt.c = p.coeffs[k];
      dt.order = (int)row.size();
      for (int q = 0; q < 3; ++q) dt.f[q] = q < dt.order ? row[q] : -1;
      M.pair_terms.push_back(dt);
      for (int a = 0; a < dt.order; ++a) {
        DevicePairAdj r{};
        r.c = dt.c;
        int o = 0;
        for (int b = 0; b < dt.order; ++b)
          if (b != a) r.other[o++] = row[b];
        for (; o < 2; ++o) r.other[o] = -1;
        adj[row[a]].push_back(r);
      }
    }
    for (int f = 0; f < nd; ++f) {
      M.pair_adj.insert(M.pair_adj.end(), adj[f].begin(), adj[f].end());
      M.pair_adj_off[(size_t)t * nd + f + 1] = (int)M.pair_adj.size();
    }
  }
  M.pair_term_off[T] = (int)M.pair_terms.size();
  if (nd > kBlockThreads) {
    err = "too many pair features for the kernel";
    return false;
  }
  return true;
}

bool build_model(Model& M, std::string& err) {
  const Potential& p = M.pot;
  M.T = (int)p.elements.size();
  if (p.pair) {
    M.F = (int)p.params.size();
    M.L = 0;
    M.Lh = 1;
    if (p.cutoff <= 0) {
      err = "cutoff must be positive";
      return false;
    }
    M.sched.assign(M.T, Schedule());   // no tile schedules: one empty per element
    return build_pair_model(M, err);
  }
  if (M.T > kMaxTypes) {
    err = "more than 8 elements are not supported";
    return false;
  }
  M.TC = M.T * (M.T + 1) / 2;
  M.F = (int)p.params.size();
  M.L = p.maxl;
  if (M.F < 1 || M.F > kNPad) {
    err = "number of radial functions must be in [1, 16]";
    return false;
  }
  if (M.L < 0 || M.L > kMaxL) {
    err = "max_l must be in [0, 20]";
    return false;
  }
  if (p.cutoff <= 0) {
    err = "cutoff must be positive";
    return false;
  }
  M.Lh = (M.L + 1) * (M.L + 2) / 2;
  screen(p, M);
  // every screened term must reference l <= max_l
  for (auto& lc : M.irr_l)
    if (lc.back() > M.L) {
      err = "gtinv_maxl exceeds max_l";
      return false;
    }
  build_itc(M);
  M.n_itc = (int)M.itc.size();
  M.D = M.F * M.n_itc;
  if (!build_poly(M, err)) return false;
  if (M.poly.size() != p.coeffs.size()) {
    char b[200];
    snprintf(b, sizeof b, "number of regression coefficients %zu does not match the model (%zu)",
             p.coeffs.size(), M.poly.size());
    err = b;
    return false;
  }
  for (auto& row : M.poly)
    if ((int)row.size() > kMaxPoly) {
      err = "polynomial order above 4 is not supported";
      return false;
    }
  M.type_pairs.assign(M.T * M.T, 0);
  int cnt = 0;
  for (int a = 0; a < M.T; ++a)
    for (int b = a; b < M.T; ++b) M.type_pairs[a * M.T + b] = M.type_pairs[b * M.T + a] = cnt++;
  M.other_type.assign(M.TC * M.T, -1);
  auto tpm = type_pairs_mapping(M.T);
  for (int tc = 0; tc < M.TC; ++tc) {
    M.other_type[tc * M.T + tpm[tc].first] = tpm[tc].second;
    M.other_type[tc * M.T + tpm[tc].second] = tpm[tc].first;
  }
  if (!fold_terms(M, err)) return false;
  if (!schedules_for_tiling(M, err)) return false;
  set_adjoint_bound(M);
  return true;
}

bool count_coefficients(int n_types, int model_type, int maxp, int maxl, int gtinv_order,
                        const int* gtinv_maxl, const int* gtinv_sym, int n_fn,
                        long long* n_coeffs, long long* n_features, std::string& err) {
  Model M;
  M.pot.elements.assign(n_types, "X");
  M.pot.model_type = model_type;
  M.pot.maxp = maxp;
  M.pot.maxl = maxl;
  M.pot.gtinv_order = gtinv_order;
  M.pot.gtinv_maxl.assign(gtinv_maxl, gtinv_maxl + gtinv_order - 1);
  M.pot.gtinv_sym.assign(gtinv_sym, gtinv_sym + gtinv_order - 1);
  M.T = n_types;
  M.F = n_fn;
  if (n_types < 1 || n_types > kMaxTypes || gtinv_order < 1 || gtinv_order > kMaxOrder) {
    err = "invalid model specification";
    return false;
  }
  screen(M.pot, M);
  build_itc(M);
  M.n_itc = (int)M.itc.size();
  const long long D = (long long)n_fn * M.n_itc;
  *n_features = D;
  // polynomial count by inclusion-exclusion over element subsets: number of
  // multisets of size p whose features share at least one element
  auto mask_of = [&](long long f) {
    int m = 0;
    for (int t = 0; t < n_types; ++t)
      if (M.itc[f % M.n_itc].inter[t]) m |= 1 << t;
    return m;
  };
  auto multichoose = [](long long n, int p) {
    long double v = 1;
    for (int k = 0; k < p; ++k) v = v * (n + k) / (k + 1);
    return (long long)(v + 0.5);
  };
  auto count_from = [&](const std::vector<long long>& feats, int p) {
    std::vector<long long> by_mask(1 << n_types, 0);
    for (long long f : feats) by_mask[mask_of(f)]++;
    long long tot = 0;
    for (int S = 1; S < (1 << n_types); ++S) {
      long long nS = 0;
      for (int m = 0; m < (1 << n_types); ++m)
        if ((m & S) == S) nS += by_mask[m];
      const int bits = __builtin_popcount(S);
      tot += ((bits % 2) ? 1 : -1) * multichoose(nS, p);
    }
    return tot;
  };
  std::vector<long long> all, lower;
  for (long long f = 0; f < D; ++f) {
    all.push_back(f);
    const int q = (int)M.itc[f % M.n_itc].type_combs.size();
    if ((model_type == 3 && q == 1) || (model_type == 4 && q <= 2)) lower.push_back(f);
  }
  long long n = 0;
  if (model_type == 1) {
    long long valid = 0;
    for (long long f : all) valid += mask_of(f) != 0;
    n = valid * maxp;
  } else if (model_type == 2) {
    for (int p = 1; p <= maxp; ++p) n += count_from(all, p);
  } else if (model_type == 3 || model_type == 4) {
    n = D;
    for (int p = 2; p <= maxp; ++p) n += count_from(lower, p);
  } else {
    err = "Unknown model_type";
    return false;
  }
  *n_coeffs = n;
  return true;
}

double flops_per_atom_step(const Model& M, int t, double nbar, bool folded) {
  if (M.pot.pair) {
    // radial-only descriptor: per neighbour and radial function the feature
    // sum (1) and the force contraction (2 + 3); the polynomial and its
    // adjoint per valid term
    double f = nbar * M.F * 6.0;
    for (int k = M.pair_term_off[t]; k < M.pair_term_off[t + 1]; ++k) {
      const double p = M.pair_terms[k].order;
      f += 2.0 * p + 2.0 * p * (p - 1.0);
    }
    return f;
  }
  double f = nbar * M.F * M.Lh * (4.0 + 30.0);
  for (int i = 0; i < M.n_itc; ++i) {
    if (!M.itc[i].inter[t]) continue;
    const int k = M.itc[i].irreps;
    const double Ti = folded ? M.irr_cnterms[k] : M.irr_nterms[k];
    const int q = (int)M.irr_l[k].size();
    f += M.F * Ti * (6.0 * (q - 1) + 3.0);
    f += M.F * Ti * q * (6.0 * std::max(q - 2, 0) + 4.0);
  }
  for (size_t pi = 0; pi < M.poly.size(); ++pi) {
    bool ok = true;
    for (int ff : M.poly[pi]) ok = ok && M.itc[ff % M.n_itc].inter[t];
    if (!ok) continue;
    const double p = (double)M.poly[pi].size();
    f += 2.0 * p + 2.0 * p * (p - 1.0);
  }
  return f;
}

}  // namespace mlipg
