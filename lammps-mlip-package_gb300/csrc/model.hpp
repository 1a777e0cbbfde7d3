// Host-side model for the GB300 MLIP (gtinv) path: potential-file parser,
// coupling table, model structure and the per-element work schedules that
// the device kernel consumes.
//
// Reference interfaces restated here (same meaning, same ordering):
//   potential file        src/USER-MLIP/mlipkk_potential_parser.cpp:14-105
//   table screening       src/USER-MLIP/mlipkk_gtinv_data_reader.cpp:18-76
//   irreps x typecomb     src/USER-MLIP/mlipkk_irreps_type.cpp:48-100
//   polynomial index      src/USER-MLIP/mlipkk_polynomial.cpp:12-208
//   feature index         fidx = n * n_itc + itc (mlipkk_polynomial.cpp:48-51)
#pragma once

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

namespace mlipg {

constexpr int kNPad = 16;      // radial index n is padded to 16 lanes
constexpr int kMaxOrder = 6;   // coupling table orders 1..6
constexpr int kMaxPoly = 4;    // polynomial terms of order <= 4
constexpr int kMaxL = 20;      // coupling table angular momenta <= 20
constexpr int kMaxTypes = 8;

struct Potential {
  bool pair = false;       // des_type "pair": the radial-only descriptor
  std::vector<std::string> elements;
  std::vector<double> masses;
  double cutoff = 0;
  int model_type = 0, maxp = 0, maxl = 0, gtinv_order = 0;
  std::vector<int> gtinv_maxl, gtinv_sym;
  std::vector<double> coeffs;                       // divided by the scales
  std::vector<std::pair<double, double>> params;    // (beta, mu) per radial function
};

// Canonical member of a conjugate pair of coupling terms, sign-folded.
// The table is closed under m -> -m with equal coefficients, and
// a_{l,-m} = (-1)^m conj(a_{l,m}); so the pair (m, -m) contributes
// 2 Re(c' prod a~) to the invariant, where a~ are the stored m <= 0 order
// parameters (conjugated for slots with m > 0) and c' carries the signs.
// Self-conjugate terms (all m = 0) contribute c' prod a~ once.
struct DeviceTerm {       // 16 bytes, read warp-uniformly
  double c;               // folded coefficient c'
  uint8_t lmh[kMaxOrder]; // LMInfoIdx l(l+1)/2 + l - |m| of each slot
  uint16_t code;          // 2 bits per slot (see SlotCode) + bit 12 = self-conjugate
};
enum SlotCode : int { kSlotNormal = 0, kSlotConj = 1, kSlotMZero = 2, kSlotSelf = 3 };

// One (irreps, element tuple) for a given centre element: the invariant
// d(n) = sum over its canonical terms, for all n at once (16 lanes).
struct DeviceUnit {       // 32 bytes
  int itc;                // irreps-typecomb index (feature fidx = n*ITC + itc)
  int term0;              // first canonical term
  int nterm;              // number of canonical terms
  int nl_slot;            // slot of this itc among nonlinear features, -1 if linear only
  uint8_t s[kMaxOrder];   // neighbour element of each slot
  uint8_t q;              // order
  uint8_t pad;
  int pad2[2];
};

// Polynomial term of order >= 2 valid for a centre element.
struct DevicePoly {       // 32 bytes
  double w;
  int k[kMaxPoly];        // index into the nonlinear-feature array: slot*16 + n
  int order;
  int pad;
};

// One (polynomial term, factor) pair of the adjoint gather, flattened so that
// the kernel reads one record per pair: dE/dd_k += w * prod(d[other])
struct DeviceAdj {        // 32 bytes
  double w;               // the term's weight
  int other[kMaxPoly - 1];  // the term's other factors (slot*16 + n), -1 past its order
  int pad[3];
};

// Element tuples of one irreps (orders 1..4, up to 3 elements) over a chunk
// of its canonical terms.  Order-4 units fix the element of slot 0 (s0) and
// cover the T^3 tuples of the other slots; lower orders cover all T^q tuples;
// one set of order-parameter loads per term.  Tuples are ordered
// lexicographically over T^q; the DeviceTuple block at `tup` maps each of
// the unit's tuples to its itc (or -1 for orderings that are not the
// canonical multiset order).
struct DeviceIrrUnit {    // 16 bytes
  int term0;
  int nterm;
  int tup;                // first DeviceTuple of this unit's block
  uint8_t q;
  uint8_t s0;             // fixed element of slot 0 (order 4)
  uint8_t nl;             // 1: the unit's features are polynomial inputs (their
                          // energy is taken from the polynomial phase)
  uint8_t pad;
};
struct DeviceTuple {      // 8 bytes
  int itc;                // -1: not a feature (non-canonical ordering)
  int nl_slot;            // slot among nonlinear features, -1 if linear only
};
constexpr int kIrrChunk = 24;  // default canonical terms per batched unit
constexpr int kCtaWarps = 8;   // warps of the fused kernel's CTA (units are dealt to them)

// Tile shape of the fused kernel's invariant/adjoint phase, chosen by the
// autotuner: terms per batched unit, the order in which units are dealt to
// the CTA's warps (0 = cost-sorted round robin, 1 = longest-first onto the
// least-loaded warp, padded with empty units, 2 = taken dynamically from a
// shared counter), and CTAs per SM of the
// persistent grid (0 = as many as are resident).
struct Tiling {
  int irr_chunk = kIrrChunk;
  int warp_order = 0;
  int ctas_per_sm = 0;
};

// Radial-only descriptor ("pair" potentials): features
// dn[tc * F + n] = sum_j f_n(r_ij) over neighbours j with type pair
// tc = tc(t_i, t_j), energy E_i = sum_k c_k prod_{f in term k} dn[f].
constexpr int kPairMaxF = 64;     // radial functions of a pair potential
constexpr int kBlockThreads = 256;  // threads of the pair kernel's CTA (one per feature)
struct DevicePairTerm {   // 32 bytes: one polynomial term valid for a centre element
  double c;
  int f[3];               // feature indices, -1 past the order
  int order;
  int pad[2];
};
struct DevicePairAdj {    // 16 bytes: dE/d dn[f] += c * prod dn[other]
  double c;
  int other[2];           // -1 past the term's order - 1
};

struct ITC {
  int irreps;
  std::vector<int> type_combs;
  std::vector<char> inter;
};

struct Schedule {         // per centre element
  std::vector<DeviceIrrUnit> iunits; // batched-tuple units (T <= 3, order <= 3)
  std::vector<DeviceTuple> tuples;   // tuple -> itc tables of the batched units
  std::vector<DeviceUnit> units;     // remaining valid itc, sorted by cost
  std::vector<DeviceUnit> nl_units;  // nonlinear itc, nl_slot = position
  std::vector<DevicePoly> poly;      // order >= 2 polynomial terms
  // polynomial adjoint gather: entry e = slot*16 + n of the nonlinear
  // features lists the (poly term, factor) pairs it receives, as p*4 + q
  std::vector<int> adj_off;          // [nl_units.size()*16 + 1]
  std::vector<int> adj;
};

struct Model {
  Potential pot;
  int T = 0, TC = 0, F = 0, L = 0, Lh = 0;
  // screened irreps
  std::vector<std::vector<int>> irr_l;
  std::vector<int> irr_first, irr_nterms;     // raw (unfolded) terms
  std::vector<std::vector<int>> term_lm;      // raw term -> LMIdx per slot
  std::vector<double> term_c;
  std::vector<int> irr_cfirst, irr_cnterms;   // canonical folded terms
  std::vector<DeviceTerm> cterms;
  std::vector<ITC> itc;
  int n_itc = 0, D = 0;
  std::vector<std::vector<int>> poly;         // PolynomialIdx -> FeatureIdx list
  std::vector<double> w_lin;                  // [n_itc][kNPad], order-1 weights
  std::vector<int> type_pairs;                // [T*T] -> tc
  std::vector<int> other_type;                // [TC*T]
  std::vector<Schedule> sched;                // [T]
  Tiling tiling;
  int max_nl = 0;                             // max nonlinear itc over elements
  // rows (l, m <= 0 entries, l <= the largest l of any nonlinear feature) of
  // order parameters the mixed path evaluates in FP64 for the polynomial's
  // input features; 0 when the model has no polynomial terms of order >= 2
  int lh64 = 0;
  // radial-only descriptor: per centre element, its valid terms and, per
  // feature, the (weight, other factors) records of dE/d dn (CSR over
  // element * n_features + feature)
  std::vector<DevicePairTerm> pair_terms;
  std::vector<int> pair_term_off;        // [T + 1]
  std::vector<DevicePairAdj> pair_adj;
  std::vector<int> pair_adj_off;         // [T * TC * F + 1]
  // Largest scaled adjoint flush allowed in the mixed path's fixed-point
  // adjoint accumulation (high parts in multiples of 2^16): a power of two with
  // (flushes per entry) x bound / 2^16 < 2^31, so no integer sum overflows.
  double g_bound = 274877906944.0;
  double g_bound_df = 1180591620717411303424.0;   // double-float path's bound (2^70 at most)
};

// Parses a potential file; returns false with `err` set on failure.
bool read_potential(const std::string& path, Potential& p, std::string& err);

// Builds the complete model (table screening, enumeration, schedules).
bool build_model(Model& m, std::string& err);

// Rebuilds the per-element work schedules for m.tiling.
bool build_schedules(Model& m, std::string& err);

// Counts coefficients and features for a model specification.
bool count_coefficients(int n_types, int model_type, int maxp, int maxl, int gtinv_order,
                        const int* gtinv_maxl, const int* gtinv_sym, int n_fn,
                        long long* n_coeffs, long long* n_features, std::string& err);

// Algorithmic flop count per atom step for a centre element with nbar
// neighbours inside the cutoff (counting rule: complex*complex 6,
// real*complex 2, complex add 2, real fma 2; transcendentals and
// recomputation excluded).
// folded: count the invariant/adjoint work on the folded table (each
// conjugate pair of terms once, as the kernels run it) instead of the raw one
double flops_per_atom_step(const Model& m, int elem, double nbar, bool folded = false);

}  // namespace mlipg
