// Fused per-atom MLIP kernel, included once per arithmetic precision.
//
// One CTA evaluates one centre atom at a time (persistent grid-stride loop
// over centres); every intermediate of the reference's seven stages stays in
// shared memory:
//   P1  neighbour compaction: keep r <= rc, stable-sort by element (all
//       warps, per-warp counts and a prefix keep the list order)
//   P2  order parameters a[s][lm][n] = sum_j f_n(r) conj(Y_lm): f_n and Y_lm
//       evaluated in REAL; FP64 kernels (and the mixed precision that asks
//       for FP64 sums): staged as FP64 by four warps that split the
//       harmonic columns, summed with FP64 FMAs; mixed path: FP32 products
//       summed with Kahan compensation (mlipkk_lmp.h:314-387,
//       mlipkk_features_kk.h:9-48, mlipkk_spherical_harmonics_kk.h:18-81)
//   P2b mixed path: the order parameters that the polynomial's input
//       features read, in FP64 (FP64 radial functions, Y_lm and sums; the
//       l = 0 rows inside P2's windows)
//   P3  the polynomial's input features ("nonlinear" features, in FP64) and
//       their whole energy: linear terms and polynomial terms of order >= 2,
//       and H = dE/dd for them (mlipkk_lmp.h:489-625)
//   P5  invariants d over the folded coupling table, the linear energy
//       sum w_f d_f of the other features, and G = dE/da via H
//       (mlipkk_lmp.h:407-469, 645-733)
//   P6  per-pair forces f_ij = sum coeff Re(G . dphi*) with the centre's own
//       adjoint, scattered as F_i += f, F_j -= f; virial -= r_ij (x) f
//       (mlipkk_lmp.h:753-922, spherical-harmonic derivatives :117-177);
//       FP64 kernels split the harmonic columns over four warps, the mixed
//       path the 16 radial channels over four threads per neighbour
// The "owner computes" force form: a pair's other half comes from the
// neighbour's own evaluation (identical to the reference's j<i / ghost
// split up to summation order).
//
// Required macros: MLIPG_REAL (float|double), MLIPG_TAG (f32|f64|f64df);
// MLIPG_DF (with MLIPG_REAL double) runs P5's products in double-float
// arithmetic (dfloat.cuh) on the FP32 pipe, with the adjoint accumulated in
// exact four-word fixed point; every other phase stays FP64.  With
// MLIPG_NO_FUSED defined, only the device helpers (spherical harmonics,
// radial basis, displacements) and init_constants are compiled.

#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "dfloat.cuh"
#include "kernels.cuh"

#define MLIPG_CAT2(a, b) a##b
#define MLIPG_CAT(a, b) MLIPG_CAT2(a, b)

namespace mlipg {
namespace MLIPG_TAG {

using R = MLIPG_REAL;
template <typename T> struct Cx;
template <> struct Cx<float> { using type = float2; };
template <> struct Cx<double> { using type = double2; };
template <> struct Cx<DF> { using type = DFc; };
using Rc = Cx<R>::type;
#ifdef MLIPG_DF
constexpr bool kDF = true;
#else
constexpr bool kDF = false;
#endif
// P5's arithmetic type, its complex type and the adjoint's storage word:
// FP32 (fixed point in int32 pairs), FP64 (FP64 atomics) or double-float
// (fixed point in four int32 words)
using P = std::conditional_t<kDF, DF, R>;
using Pc = Cx<P>::type;
using PG = std::conditional_t<kDF, int, R>;
// the adjoint is accumulated in fixed point (and range-checked)
constexpr bool kFixG = sizeof(R) == 4 || kDF;
// 4-byte words of adjoint storage per complex entry
constexpr int kGWords = kDF ? 8 : 4;
// resident CTAs per SM the register allocation targets: two for FP32
// products (shared memory allows two), one for FP64 (its shared memory
// allows only one, so registers are not capped)
constexpr int kMinBlocks = sizeof(R) == 4 ? 2 : 1;

namespace {

// spherical-harmonic recursion constants (mlipkk.cpp:247-272 and
// mlipkk_spherical_harmonics_kk.h), indexed by lm2i(l, m) = l(l+1)/2 + m
__constant__ R cA[kLhMax];
__constant__ R cB[kLhMax];
__constant__ R cLM[kLhMax];        // sqrt((l-m)(l+m+1))
__constant__ R cDiag[kMaxL + 2];   // -sqrt(1 + 0.5/m), m >= 1
__constant__ R cOff[kMaxL + 2];    // sqrt(2m + 3)
__constant__ R cLL[kMaxL + 1];     // sqrt(0.5 l (l+1)) (FP32: sqrt(l (l+1)), see sh_visit)

// the same recursion constants in FP64 for the mixed path's FP64 order
// parameters of the polynomial's input features
__constant__ double cA64[kLhMax];
__constant__ double cB64[kLhMax];
__constant__ double cDiag64[kMaxL + 2];
__constant__ double cOff64[kMaxL + 2];

__device__ __forceinline__ int lm2i(int l, int m) { return l * (l + 1) / 2 + m; }

// Y_{l,m} (m <= 0, l <= lmax) of one displacement in FP64, by the column
// recursion of sh_visit below, stored at ys[lmh * stride + slot]
// (lmh = l(l+1)/2 + l - |m|).
__device__ __forceinline__ void sh_values64(double dx, double dy, double dz, double r, int lmax,
                                         double2* ys, int stride, int slot) {
  const double invr = 1.0 / r;
  const double ct = dz * invr;
  const double st = sqrt(fmax(0.0, 1.0 - ct * ct));
  const double rho2 = dx * dx + dy * dy;
  double cp = 1.0, sp = 0.0;
  if (rho2 > 0.0) {
    const double ir = 1.0 / sqrt(rho2);
    cp = dx * ir;
    sp = dy * ir;
  }
  const double h = 0.70710678118654752440;
  double pdiag = 0.39894228040143267794;
  double cm = 1.0, sm = 0.0, cprev = cp, sprev = -sp;
  const double tc = 2.0 * cp;
  double sgn = 1.0;
  for (int mp = 0; mp <= lmax; ++mp) {
    if (mp > 0) {
      const double sn = tc * sm - sprev;
      const double cn = tc * cm - cprev;
      cprev = cm; cm = cn; sprev = sm; sm = sn;
      pdiag = pdiag * (cDiag64[mp] * st);
      sgn = -sgn;
    }
    double p1 = 0.0, p2 = 0.0;
    for (int l = mp; l <= lmax; ++l) {
      double P;
      if (l == mp) P = pdiag;
      else if (l == mp + 1) P = (ct * cOff64[mp]) * p1;
      else P = cA64[lm2i(l, mp)] * (ct * p1 + cB64[lm2i(l, mp)] * p2);
      p2 = p1;
      p1 = P;
      double yre, yim;
      if (mp == 0) {
        yre = P * h;
        yim = 0.0;
      } else {
        const double t = sgn * P * h;
        yre = t * cm;
        yim = -(t * sm);
      }
      ys[(l * (l + 1) / 2 + l - mp) * stride + slot] = double2{yre, yim};
    }
  }
}


__device__ __forceinline__ float rsqrt_r(float v) { return rsqrtf(v); }
__device__ __forceinline__ double rsqrt_r(double v) { return 1.0 / sqrt(v); }

__device__ __forceinline__ R exp_r(R v) { return exp(v); }
__device__ __forceinline__ void sincospi_r(R v, R* s, R* c) { sincospi(v, s, c); }

// Visits every (l, m <= 0) with Y_{l,m} and, if DERIV, dY/dx, dY/dy, dY/dz,
// in the order m = 0, -1, ..., -L (outer) and l = |m|..L (inner).  The
// associated-Legendre columns are advanced in registers: the recursion of
// the reference (DLMF 14.10.3 / 14.7.15 with normalised P and Q = P/sin) is
// the same, evaluated column by column.
// The FP32 instantiation returns Y / Y_00 (Y_00 = 1/(2 sqrt(pi))): its
// recursion starts from P = 1, exact, instead of the FP32-rounded
// normalisation, whose rounding (0.87 ulp) would scale every order parameter
// alike and bias each order-q invariant by q times that error.  The FP32
// coupling coefficients carry the factor Y_00^q instead (rounded once per
// term), and the forces are unchanged: G' dY' = (Y_00 G) (dY / Y_00).
template <int LCAP, bool DERIV, typename V>
__device__ __forceinline__ void sh_visit(R dx, R dy, R dz, R r, int L, V& vis) {
  const R invr = R(1) / r;
  const R ct = dz * invr;
  const R st = sqrt(fmax(R(0), R(1) - ct * ct));
  const R rho2 = dx * dx + dy * dy;
  R cp = R(1), sp = R(0);
  if (rho2 > R(0)) {
    const R ir = rsqrt_r(rho2);
    cp = dx * ir;
    sp = dy * ir;
  }
  constexpr bool kUnit = sizeof(R) == 4;   // FP32: Y / Y_00 (see above)
  const R h = kUnit ? R(1) : R(0.70710678118654752440);  // 0.5 * sqrt(2)
  R Qc[LCAP + 2];
#pragma unroll
  for (int l = 0; l < LCAP + 2; ++l) Qc[l] = R(0);
  R pdiag = kUnit ? R(1) : R(0.39894228040143267794);    // P_0^0 = sqrt(1/(2 pi))
  R cm = R(1), sm = R(0), cprev = cp, sprev = -sp;
  const R tc = R(2) * cp;
  R sgn = R(1);
#pragma unroll
  for (int mp = 0; mp <= LCAP; ++mp) {
    if (mp > L) break;
    if (mp > 0) {
      const R s = tc * sm - sprev;
      const R c = tc * cm - cprev;
      cprev = cm; cm = c; sprev = sm; sm = s;
      pdiag = pdiag * (cDiag[mp] * st);
      sgn = -sgn;
    }
    // next Q column (m = mp + 1): diagonal start
    R qn_diag = R(0);
    if (DERIV) {
      // Q_1^1 = P_0^0 cDiag[1]
      qn_diag = (mp == 0) ? (kUnit ? cDiag[1] : R(-0.48860251190291992263))
                          : Qc[mp] * (cDiag[mp + 1] * st);
    }
    R p1 = R(0), p2 = R(0), qn1 = R(0), qn2 = R(0);
#pragma unroll
    for (int l = mp; l <= LCAP; ++l) {
      if (l > L) break;
      R P;
      if (l == mp) P = pdiag;
      else if (l == mp + 1) P = (ct * cOff[mp]) * p1;
      else P = cA[lm2i(l, mp)] * (ct * p1 + cB[lm2i(l, mp)] * p2);
      p2 = p1;
      p1 = P;
      R Qn = R(0);
      if (DERIV) {
        if (l == mp + 1) Qn = qn_diag;
        else if (l == mp + 2) Qn = (ct * cOff[mp + 1]) * qn1;
        else if (l >= mp + 3) Qn = cA[lm2i(l, mp + 1)] * (ct * qn1 + cB[lm2i(l, mp + 1)] * qn2);
        if (l >= mp + 1) { qn2 = qn1; qn1 = Qn; }
      }
      R yre, yim;
      if (mp == 0) {
        yre = P * h;
        yim = R(0);
      } else {
        const R t = sgn * P * h;
        yre = t * cm;
        yim = -(t * sm);
      }
      const int lmh = l * (l + 1) / 2 + l - mp;
      if (DERIV) {
        R xre = 0, xim = 0, yyre = 0, yyim = 0, zre = 0, zim = 0;
        if (mp == 0) {
          if (l >= 1) {
            const R common = Qn * st * invr * cLL[l];
            xre = common * ct * cp;
            yyre = common * ct * sp;
            zre = -common * st;
          }
        } else {
          const R qc = Qc[l];
          R dth = R(mp) * ct * qc;
          if (l != mp) dth += cLM[lm2i(l, mp)] * Qn * st;
          const R dph = R(mp) * qc;
          const R ere = cm * h * invr, eim = sm * h * invr;
          // v = (dth ct cp) + i(-dph sp), (dth ct sp) + i(dph cp), (-dth st)
          const R vxr = dth * ct * cp, vxi = -dph * sp;
          const R vyr = dth * ct * sp, vyi = dph * cp;
          const R vzr = -dth * st;
          xre = sgn * (ere * vxr - eim * vxi);
          xim = -sgn * (ere * vxi + eim * vxr);
          yyre = sgn * (ere * vyr - eim * vyi);
          yyim = -sgn * (ere * vyi + eim * vyr);
          zre = sgn * (ere * vzr);
          zim = -sgn * (eim * vzr);
        }
        vis(lmh, mp, yre, yim, xre, xim, yyre, yyim, zre, zim);
        if (l >= mp + 1) Qc[l] = Qn;
      } else {
        vis(lmh, mp, yre, yim, R(0), R(0), R(0), R(0), R(0), R(0));
      }
    }
  }
}

// radial basis: f_n = exp(-beta (r-mu)^2) fc(r), fc = (cos(pi r/rc) + 1)/2
__device__ __forceinline__ void radial(const double* __restrict__ prm, int F, R r, R rc, R* f,
                                       R* fd, bool deriv) {
  R sn, cs;
  sincospi_r(r / rc, &sn, &cs);
  const bool in = r < rc;
  const R fc = in ? R(0.5) * (cs + R(1)) : R(0);
  const R fcd = in ? R(-0.5) * R(3.14159265358979323846) / rc * sn : R(0);
#pragma unroll
  for (int n = 0; n < kNPad; ++n) {
    if (n < F) {
      const R beta = (R)__ldg(prm + 2 * n), mu = (R)__ldg(prm + 2 * n + 1);
      const R dr = r - mu;
      const R bf = exp_r(-beta * dr * dr);
      f[n] = bf * fc;
      if (deriv) fd[n] = (R(-2) * beta * dr * bf) * fc + bf * fcd;
    } else {
      f[n] = R(0);
      if (deriv) fd[n] = R(0);
    }
  }
}

// radial basis for the 4 channels n0..n0+3 (P6: 4 threads per neighbour)
__device__ __forceinline__ void radial4(const double* __restrict__ prm, int F, int n0, R r, R rc,
                                        R* f, R* fd) {
  R sn, cs;
  sincospi_r(r / rc, &sn, &cs);
  const bool in = r < rc;
  const R fc = in ? R(0.5) * (cs + R(1)) : R(0);
  const R fcd = in ? R(-0.5) * R(3.14159265358979323846) / rc * sn : R(0);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int n = n0 + q;
    if (n < F) {
      const R beta = (R)__ldg(prm + 2 * n), mu = (R)__ldg(prm + 2 * n + 1);
      const R dr = r - mu;
      const R bf = exp_r(-beta * dr * dr);
      f[q] = bf * fc;
      fd[q] = (R(-2) * beta * dr * bf) * fc + bf * fcd;
    } else {
      f[q] = R(0);
      fd[q] = R(0);
    }
  }
}

// Stages Y_lm of one neighbour as FP64 (exact conversion of the REAL value)
// for the FP64 order-parameter sums.
struct StageVis {
  double2* ys;
  int slot;
  __device__ __forceinline__ void operator()(int lmh, int, R yre, R yim, R, R, R, R, R, R) {
    ys[lmh * kChunk + slot] = double2{(double)yre, (double)yim};
  }
};

// Stages Y_lm of one neighbour as FP32 pairs for the mixed path's
// compensated FP32 order-parameter sums (rows of 2 * kChunk neighbours).
struct StageVisW {
  float2* ys;
  int slot;
  __device__ __forceinline__ void operator()(int lmh, int, R yre, R yim, R, R, R, R, R, R) {
    ys[lmh * (2 * kChunk) + slot] = float2{(float)yre, (float)yim};
  }
};

// s + c += p with Knuth's TwoSum: s keeps the rounded running sum, c gathers
// every addition's exact rounding error (explicit _rn intrinsics, so nothing
// is contracted or reassociated).
__device__ __forceinline__ void two_sum_acc(float& s, float& c, float p) {
  const float t = __fadd_rn(s, p);
  const float bp = __fsub_rn(t, s);
  const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  c = __fadd_rn(c, e);
  s = t;
}

// s - c += a * b with Kahan's compensated summation, the product fused into
// the compensating FMA (c holds the negated part that the last addition lost;
// the value of the pair is s - c).
__device__ __forceinline__ void kahan_fma_acc(float& s, float& c, float a, float b) {
  const float y = __fmaf_rn(a, b, -c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

// Per-thread energy sum of the batched units.  FP64 path: a double.  Mixed
// path: a TwoSum pair in FP32 (running sum, gathered rounding errors), folded
// into the centre's FP64 energy once per centre.
struct ESumF {
  float s = 0.f, c = 0.f;
};
__device__ __forceinline__ void eadd(double& e, double v) { e += v; }
__device__ __forceinline__ void eadd(ESumF& e, float v) { two_sum_acc(e.s, e.c, v); }

// Adds one statically dealt unit's energy to the thread's sum: the mixed
// path's TwoSum pair, or the FP64 path's double.
__device__ __forceinline__ void merge_unit_energy(ESumF& es, double&, const ESumF& u) {
  two_sum_acc(es.s, es.c, u.s);
}
__device__ __forceinline__ void merge_unit_energy(ESumF&, double& ed, double u) { ed += u; }
// double-float path: a double-float sum per unit, added to the FP64 energy
__device__ __forceinline__ void eadd(DF& e, DF v) { e += v; }
__device__ __forceinline__ void merge_unit_energy(ESumF&, double& ed, const DF& u) {
  ed += df_to_double(u);
}

// Sum over the warp's lanes of one unit's energy, identical on every lane.
// FP64: a butterfly of FP64 adds.  Mixed: a butterfly of TwoSum steps in FP32
// (each step's rounding error is exact and the pair's sum is commutative, so
// partners agree bit for bit), returned as the FP64 value of sum + error.
__device__ __forceinline__ double warp_energy(double e) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  return e;
}
__device__ __forceinline__ double warp_energy(ESumF e) {
  float s = e.s, c = e.c;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float so = __shfl_xor_sync(0xffffffffu, s, o);
    const float co = __shfl_xor_sync(0xffffffffu, c, o);
    const float t = __fadd_rn(s, so);
    const float bp = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(so, bp));
    c = __fadd_rn(__fadd_rn(c, co), err);
    s = t;
  }
  return (double)s + (double)c;
}
__device__ __forceinline__ double warp_energy(DF e) { return warp_energy(df_to_double(e)); }

// sum of the two half-warps' partial invariants of one unit at channel n
__device__ __forceinline__ double half_pair_sum(float v) {
  v += __shfl_xor_sync(0xffffffffu, v, 16);
  return (double)v;
}
__device__ __forceinline__ double half_pair_sum(double v) {
  return v + __shfl_xor_sync(0xffffffffu, v, 16);
}
__device__ __forceinline__ double half_pair_sum(DF v) { return half_pair_sum(df_to_double(v)); }

// a statically dealt unit's energy accumulator
using EU = std::conditional_t<sizeof(R) == 4, ESumF, std::conditional_t<kDF, DF, double>>;
// an FP64 weight in P5's arithmetic type
__device__ __forceinline__ float to_p_as(double v, float*) { return (float)v; }
__device__ __forceinline__ double to_p_as(double v, double*) { return v; }
__device__ __forceinline__ DF to_p_as(double v, DF*) { return df_from_double(v); }
__device__ __forceinline__ P to_p(double v) { return to_p_as(v, (P*)nullptr); }

// four consecutive values from 16-byte aligned shared memory
__device__ __forceinline__ void load4(const float* p, float* v) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void load4(const double* p, double* v) {
  const double2 a = reinterpret_cast<const double2*>(p)[0];
  const double2 b = reinterpret_cast<const double2*>(p)[1];
  v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}

struct ForceVis {
  const R* g;    // Re G of the neighbour's element slot at channel n0: [Lh][16]; Im at g + gim
  int gim;
  const R* f;    // f_n, f'_n of channels n0..n0+3
  const R* fd;
  R ux, uy, uz;
  R fx, fy, fz;
  __device__ __forceinline__ void operator()(int lmh, int mp, R yre, R yim, R xre, R xim, R yyre,
                                             R yyim, R zre, R zim) {
    R gr[4], gi[4];
    load4(g + lmh * kNPad, gr);
    load4(g + gim + lmh * kNPad, gi);
    R g0r = 0, g0i = 0, g1r = 0, g1i = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      g0r += f[q] * gr[q];
      g0i += f[q] * gi[q];
      g1r += fd[q] * gr[q];
      g1i += fd[q] * gi[q];
    }
    const R coeff = (mp == 0) ? R(1) : R(2);
    const R ry = yre * g1r + yim * g1i;
    fx += coeff * (ry * ux + (xre * g0r + xim * g0i));
    fy += coeff * (ry * uy + (yyre * g0r + yyim * g0i));
    fz += coeff * (ry * uz + (zre * g0r + zim * g0i));
  }
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// displacement x_j - x_i (+ periodic image shift for batched cells)
__device__ __forceinline__ void pair_disp(const KernelArgs& A, int c, int k, const double4& xi,
                                          const double4& xj, double& dx, double& dy, double& dz) {
  dx = xj.x - xi.x;
  dy = xj.y - xi.y;
  dz = xj.z - xi.z;
  if (A.img != nullptr) {
    const int code = __ldg(A.img + k);
    if (code != 0) {
      const double n1 = (double)((code & 1023) - 512);
      const double n2 = (double)(((code >> 10) & 1023) - 512);
      const double n3 = (double)(((code >> 20) & 1023) - 512);
      const double* L = A.cell + 9 * __ldg(A.center_cell + c);
      dx += n1 * L[0] + n2 * L[3] + n3 * L[6];
      dy += n1 * L[1] + n2 * L[4] + n3 * L[7];
      dz += n1 * L[2] + n2 * L[5] + n3 * L[8];
    }
  }
}

// Coupling coefficient of a term record: FP64 in the FP64 path's table; the
// mixed path's table holds it as FP32 in the low word, the double-float
// table as (high, low) FP32 words (no conversion per term).
template <class V> __device__ __forceinline__ V term_coeff(const int4& raw);
template <> __device__ __forceinline__ float term_coeff<float>(const int4& raw) {
  return __int_as_float(raw.x);
}
template <> __device__ __forceinline__ double term_coeff<double>(const int4& raw) {
  return __hiloint2double(raw.y, raw.x);
}
template <> __device__ __forceinline__ DF term_coeff<DF>(const int4& raw) {
  return DF(__int_as_float(raw.x), __int_as_float(raw.y));
}

// Sum of the batched units' energies taken from a shared counter: the two
// 64-bit integer parts (2^-20 eV and 2^-60 eV) kept at misc[24..27].
__device__ __forceinline__ double unit_energy(const int* misc) {
  const unsigned long long* e = reinterpret_cast<const unsigned long long*>(misc + 24);
  return (double)(long long)e[0] * 0x1p-20 + (double)(long long)e[1] * 0x1p-60;
}

// Adjoint accumulation into shared memory.  FP64: double atomics.  Mixed
// path: exact 64-bit fixed point with native 32-bit integer atomics (a
// shared-memory FP32 atomic add is a compare-and-swap loop, six times slower).
// Each flush is scaled by 2^e (e adapted per centre element) and split
// exactly into a high part, a multiple of 2^16, and a low part of at most
// 2^15 (both rounded by the exact magic-number add), which go to two int32
// arrays (the low-part array follows the high parts of re and im); no
// carries are needed because the host bounds the flushes per entry.
// Double-float path: four words, multiples of 2^48, 2^32, 2^16 and 1.
// Sums are exact and order independent; the centre's largest |scaled flush|
// is tracked so that out-of-range flushes are detected (the invariant phase
// is then redone at a smaller scale).
template <class V> struct GFixT {
  V scale;     // 2^e (1 in FP64)
  V vmax;      // largest |scaled flush| of this thread
};
template <> struct GFixT<DF> {
  float scale;
  float vmax;
};
__device__ __forceinline__ float gscale(float c, const GFixT<float>& g) { return c * g.scale; }
__device__ __forceinline__ double gscale(double c, const GFixT<double>& g) { return c * g.scale; }
__device__ __forceinline__ DF gscale(DF c, const GFixT<DF>& g) { return df_scale(c, g.scale); }

// y: the flush already multiplied by g.scale; lo: word offset of the next
// lower word array (2 x the imaginary offset)
__device__ __forceinline__ void gput(float* p, float y, GFixT<float>& g, int lo) {
  g.vmax = fmaxf(g.vmax, fabsf(y));
  const float th = fmaf(y, 1.0f / 65536.0f, 12582912.0f);   // rint(y / 2^16) + 1.5 * 2^23
  const float yl = fmaf(-(th - 12582912.0f), 65536.0f, y);  // y - hi * 2^16, exact
  atomicAdd(reinterpret_cast<int*>(p), __float_as_int(th) - 0x4B400000);
  atomicAdd(reinterpret_cast<int*>(p) + lo, __float2int_rn(yl));   // |yl| <= 2^15 + 1/2
}
__device__ __forceinline__ void gput(double* p, double y, GFixT<double>&, int) {
  atomicAdd(p, y);
}
// Double-float flush y = yh + yl (|yh| below the host's bound, at most 2^70):
// yh = t3 2^48 + t2 2^32 + t1 2^16 + r0 and yl = u2 2^32 + u1 2^16 + q0
// exactly (magic-number roundings; every remainder is representable), then
// the words t3, t2 + u2, t1 + u1 and rint(r0 + q0) (|.| <= 2^16 + 1) are
// added: 64 bits below the largest flush, so an entry 2^16 times smaller
// than the centre's largest flush still keeps 48 bits.
__device__ __forceinline__ int magic_int(float t) { return __float_as_int(t) - 0x4B400000; }
__device__ __forceinline__ void gput(int* p, DF y, GFixT<DF>& g, int lo) {
  constexpr float kMagic = 12582912.0f;   // 1.5 * 2^23
  g.vmax = fmaxf(g.vmax, fabsf(y.h));
  const float th3 = __fmaf_rn(y.h, 0x1p-48f, kMagic);
  const float r2 = __fmaf_rn(-__fsub_rn(th3, kMagic), 0x1p48f, y.h);   // |r2| <= 2^47
  const float th2 = __fmaf_rn(r2, 0x1p-32f, kMagic);
  const float r1 = __fmaf_rn(-__fsub_rn(th2, kMagic), 0x1p32f, r2);    // |r1| <= 2^31
  const float th1 = __fmaf_rn(r1, 0x1p-16f, kMagic);
  const float r0 = __fmaf_rn(-__fsub_rn(th1, kMagic), 65536.0f, r1);   // |r0| <= 2^15
  const float sh2 = __fmaf_rn(y.l, 0x1p-32f, kMagic);
  const float q1 = __fmaf_rn(-__fsub_rn(sh2, kMagic), 0x1p32f, y.l);   // |q1| <= 2^31
  const float sh1 = __fmaf_rn(q1, 0x1p-16f, kMagic);
  const float q0 = __fmaf_rn(-__fsub_rn(sh1, kMagic), 65536.0f, q1);   // |q0| <= 2^15
  const float t0 = __fadd_rn(__fadd_rn(r0, q0), kMagic);
  atomicAdd(p, magic_int(th3));
  atomicAdd(p + lo, magic_int(th2) + magic_int(sh2));
  atomicAdd(p + 2 * lo, magic_int(th1) + magic_int(sh1));
  atomicAdd(p + 3 * lo, magic_int(t0));
}

template <class V, int Q, bool WITH_G, int Lh, class GT>
__device__ __forceinline__ void run_unit(const DeviceUnit& u, const DeviceTerm* __restrict__ terms,
                                         const typename Cx<V>::type* sa, GT* sg, int gim,
                                         GFixT<V>& gf, int n, int half, bool act, V H, V& dsum) {
  using Vc = typename Cx<V>::type;
  int off[Q];
#pragma unroll
  for (int p = 0; p < Q; ++p) off[p] = (int)u.s[p] * Lh * kNPad + n;
  const int kend = u.term0 + u.nterm;
  for (int k = u.term0 + half; k < kend; k += 2) {
    const int4 raw = __ldg(reinterpret_cast<const int4*>(terms + k));
    const V c = term_coeff<V>(raw);
    const unsigned lw = (unsigned)raw.z, hw = (unsigned)raw.w;
    const unsigned code = hw >> 16;
    int lmh[Q];
    V ar[Q], ai[Q];
#pragma unroll
    for (int p = 0; p < Q; ++p) {
      lmh[p] = p < 4 ? (int)((lw >> (8 * p)) & 255u) : (int)((hw >> (8 * (p - 4))) & 255u);
      const Vc v = sa[off[p] + lmh[p] * kNPad];
      const unsigned cd = (code >> (2 * p)) & 3u;
      ar[p] = v.x;
      ai[p] = (cd == (unsigned)kSlotConj) ? -v.y : v.y;
    }
    const bool self = (code >> 12) & 1u;
    // prefix products pr[p] = prod_{p' < p} a~, suffix su[p] = prod_{p' > p} a~
    V prr[Q], pri[Q], sur[Q], sui[Q];
    prr[0] = V(1); pri[0] = V(0);
#pragma unroll
    for (int p = 1; p < Q; ++p) {
      if (p == 1) { prr[1] = ar[0]; pri[1] = ai[0]; }
      else {
        prr[p] = prr[p - 1] * ar[p - 1] - pri[p - 1] * ai[p - 1];
        pri[p] = prr[p - 1] * ai[p - 1] + pri[p - 1] * ar[p - 1];
      }
    }
    sur[Q - 1] = V(1); sui[Q - 1] = V(0);
#pragma unroll
    for (int p = Q - 2; p >= 0; --p) {
      if (p == Q - 2) { sur[p] = ar[Q - 1]; sui[p] = ai[Q - 1]; }
      else {
        sur[p] = sur[p + 1] * ar[p + 1] - sui[p + 1] * ai[p + 1];
        sui[p] = sur[p + 1] * ai[p + 1] + sui[p + 1] * ar[p + 1];
      }
    }
    // full product real part
    const V full = prr[Q - 1] * ar[Q - 1] - pri[Q - 1] * ai[Q - 1];
    dsum += (self ? c : V(2) * c) * full;
    if (WITH_G) {
      const V cc = c * H;
#pragma unroll
      for (int p = 0; p < Q; ++p) {
        V Pr, Pi;
        if (p == 0) { Pr = sur[0]; Pi = sui[0]; }
        else if (p == Q - 1) { Pr = prr[Q - 1]; Pi = pri[Q - 1]; }
        else {
          Pr = prr[p] * sur[p] - pri[p] * sui[p];
          Pi = prr[p] * sui[p] + pri[p] * sur[p];
        }
        const unsigned cd = (code >> (2 * p)) & 3u;
        const V kr = (cd == (unsigned)kSlotMZero) ? V(2) : V(1);
        const V ki = (cd == 0u) ? V(1) : (cd == 1u ? V(-1) : V(0));
        // unconditional: lanes n >= F and unused imaginary parts add exact
        // zeros (to padding entries / entries nothing reads), which keeps the
        // flush free of divergent branches
        GT* gp = sg + off[p] + lmh[p] * kNPad;
        const V cs = gscale(cc, gf);
        gput(gp, cs * kr * Pr, gf, 2 * gim);
        gput(gp + gim, cs * ki * Pi, gf, 2 * gim);
      }
    }
  }
}

// linear weights in P5's arithmetic type
__device__ __forceinline__ const float* wlin_pick(const KernelArgs& A, float*) { return A.w_lin_f; }
__device__ __forceinline__ const double* wlin_pick(const KernelArgs& A, double*) { return A.w_lin; }
__device__ __forceinline__ const DF* wlin_pick(const KernelArgs& A, DF*) {
  return reinterpret_cast<const DF*>(A.w_lin_df);
}
__device__ __forceinline__ const P* wlin_table(const KernelArgs& A) {
  return wlin_pick(A, (P*)nullptr);
}
__device__ __forceinline__ float ldg_v(const float* p) { return __ldg(p); }
__device__ __forceinline__ double ldg_v(const double* p) { return __ldg(p); }
__device__ __forceinline__ DF ldg_v(const DF* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return DF(v.x, v.y);
}

// Direct form for up to two elements and orders <= 3: every tuple of the
// unit (TT^Q of them, all elements of every slot) is formed from shared
// leave-one-out products, with adjoint partials per (slot, element) in
// registers flushed once per term; the unit's energy comes from the last
// slot's partials (sum_j H_j Pi_j = sum_s g_last[s] a_last[s]).  Shorter
// dependency chains than the factorized form, which pays off only with
// three elements.
// Weight H = w + dE_poly/dd of one tuple at channel n (0 for a non-feature
// tuple or an idle lane).  Both loads are issued unconditionally from clamped
// rows (row 0 always exists; the nonlinear row n < 16 lies inside shared
// memory) so the unrolled setup of a unit issues all its loads at once.
template <class V>
__device__ __forceinline__ V tuple_weight(int2 e, const V* __restrict__ wlin, const V* hnl, int n,
                                          bool act) {
  const V w = ldg_v(wlin + (size_t)max(e.x, 0) * kNPad + n);
  const V hn = hnl[max(e.y, 0) * kNPad + n];
  const V h = e.y >= 0 ? w + hn : w;
  return (act && e.x >= 0) ? h : V(0);
}

template <class V, int Q, int TT, int Lh, class EA, class GT>
__device__ __forceinline__ void run_irr_direct(const DeviceIrrUnit& u, const DeviceTuple* __restrict__ tups,
                                        const DeviceTerm* __restrict__ terms,
                                        const V* __restrict__ wlin, const V* hnl,
                                        const typename Cx<V>::type* sa, GT* sg, int gim,
                                        GFixT<V>& gf, int n, int half, bool act, EA& eacc) {
  using Vc = typename Cx<V>::type;
  constexpr int N0 = TT;                                  // elements of slot 0
  constexpr int NT = (Q == 1) ? N0 : (Q == 2 ? N0 * TT : N0 * TT * TT);
  constexpr int s0base = 0;
  V H[NT];
#pragma unroll
  for (int j = 0; j < NT; ++j) {
    const int2 e = __ldg(reinterpret_cast<const int2*>(tups + u.tup + j));
    H[j] = tuple_weight(e, wlin, hnl, n, act);
  }
  // Energy: sum_j H_j d_j of this unit's tuples, formed per term from the
  // last slot's adjoint partial (sum_j H_j Pi_j = sum_s g_last[s] a_last[s]);
  // the nonlinear part sum hnl d of H is subtracted once per centre.
  V eu = V(0);
  constexpr int es = Lh * kNPad;   // element stride in the a / G arrays
  constexpr int kIm = TT * es, kLo = 2 * kIm;   // imaginary / low-part offsets (T == TT)
  const int kend = u.term0 + u.nterm;
  for (int k = u.term0 + half; k < kend; k += 2) {
    const int4 raw = __ldg(reinterpret_cast<const int4*>(terms + k));
    const V c = term_coeff<V>(raw);
    const unsigned lw = (unsigned)raw.z, code = ((unsigned)raw.w) >> 16;
    const bool self = (code >> 12) & 1u;
    const V ce = self ? c : V(2) * c;
    int lo[Q];
    V ar0[N0], ai0[N0];
    V ar[Q][TT], ai[Q][TT];    // slots >= 1 (slot 0 uses ar0 / ai0)
#pragma unroll
    for (int p = 0; p < Q; ++p) {
      lo[p] = (int)((lw >> (8 * p)) & 255u) * kNPad + n;
      const bool cj = ((code >> (2 * p)) & 3u) == (unsigned)kSlotConj;
      if (p == 0) {
#pragma unroll
        for (int s = 0; s < N0; ++s) {
          const Vc v = sa[(s0base + s) * es + lo[0]];
          ar0[s] = v.x;
          ai0[s] = cj ? -v.y : v.y;
        }
      } else {
#pragma unroll
        for (int s = 0; s < TT; ++s) {
          const Vc v = sa[s * es + lo[p]];
          ar[p][s] = v.x;
          ai[p][s] = cj ? -v.y : v.y;
        }
      }
    }
    V g0r[N0], g0i[N0], gr[Q][TT], gi[Q][TT];
#pragma unroll
    for (int s = 0; s < N0; ++s) { g0r[s] = V(0); g0i[s] = V(0); }
#pragma unroll
    for (int p = 0; p < Q; ++p)
#pragma unroll
      for (int s = 0; s < TT; ++s) { gr[p][s] = V(0); gi[p][s] = V(0); }
    if (Q == 1) {
      V et = V(0);
#pragma unroll
      for (int s0 = 0; s0 < N0; ++s0) {
        g0r[s0] += H[s0];
        et += H[s0] * ar0[s0];
      }
      eu += ce * et;
    } else if (Q == 2) {
#pragma unroll
      for (int s0 = 0; s0 < N0; ++s0)
#pragma unroll
        for (int s1 = 0; s1 < TT; ++s1) {
          const int j = s0 * TT + s1;
          const V h = H[j];
          g0r[s0] += h * ar[1][s1]; g0i[s0] += h * ai[1][s1];
          gr[1][s1] += h * ar0[s0]; gi[1][s1] += h * ai0[s0];
        }
      V et = V(0);
#pragma unroll
      for (int s1 = 0; s1 < TT; ++s1) et += gr[1][s1] * ar[1][s1] - gi[1][s1] * ai[1][s1];
      eu += ce * et;
    } else {
      // b12[s1][s2] = a1 a2 (adjoint of slot 0)
      V b12r[TT][TT], b12i[TT][TT];
#pragma unroll
      for (int x = 0; x < TT; ++x)
#pragma unroll
        for (int y = 0; y < TT; ++y) {
          b12r[x][y] = ar[1][x] * ar[2][y] - ai[1][x] * ai[2][y];
          b12i[x][y] = ar[1][x] * ai[2][y] + ai[1][x] * ar[2][y];
        }
#pragma unroll
      for (int s0 = 0; s0 < N0; ++s0) {
        V b02r[TT], b02i[TT];   // a0 a2 (adjoint of slot 1)
#pragma unroll
        for (int y = 0; y < TT; ++y) {
          b02r[y] = ar0[s0] * ar[2][y] - ai0[s0] * ai[2][y];
          b02i[y] = ar0[s0] * ai[2][y] + ai0[s0] * ar[2][y];
        }
#pragma unroll
        for (int s1 = 0; s1 < TT; ++s1) {
          const V pr = ar0[s0] * ar[1][s1] - ai0[s0] * ai[1][s1];   // a0 a1 (slot 2)
          const V pi = ar0[s0] * ai[1][s1] + ai0[s0] * ar[1][s1];
#pragma unroll
          for (int s2 = 0; s2 < TT; ++s2) {
            const int j = (s0 * TT + s1) * TT + s2;
            const V h = H[j];
            g0r[s0] += h * b12r[s1][s2]; g0i[s0] += h * b12i[s1][s2];
            gr[1][s1] += h * b02r[s2];   gi[1][s1] += h * b02i[s2];
            gr[2][s2] += h * pr;         gi[2][s2] += h * pi;
          }
        }
      }
      V et = V(0);
#pragma unroll
      for (int s2 = 0; s2 < TT; ++s2) et += gr[2][s2] * ar[2][s2] - gi[2][s2] * ai[2][s2];
      eu += ce * et;
    }
    // unconditional flush (zeros from lanes n >= F and unused imaginary parts)
#pragma unroll
    for (int p = 0; p < Q; ++p) {
      const unsigned cd = (code >> (2 * p)) & 3u;
      const V cs = gscale(c, gf);
      const V kr = (cd == (unsigned)kSlotMZero) ? V(2) * cs : cs;
      const V ki = (cd == 0u) ? cs : (cd == 1u ? -cs : V(0));
      if (p == 0) {
#pragma unroll
        for (int s = 0; s < N0; ++s) {
          GT* gp = sg + (s0base + s) * es + lo[0];
          gput(gp, kr * g0r[s], gf, kLo);
          gput(gp + kIm, ki * g0i[s], gf, kLo);
        }
      } else {
#pragma unroll
        for (int s = 0; s < TT; ++s) {
          GT* gp = sg + s * es + lo[p];
          gput(gp, kr * gr[p][s], gf, kLo);
          gput(gp + kIm, ki * gi[p][s], gf, kLo);
        }
      }
    }
  }
  // this half-warp's terms, in REAL, into the thread's energy sum (zero on
  // lanes n >= F)
  eadd(eacc, eu);
}

// acc += a * b (complex) as two fused multiply-add chains
template <class V>
__device__ __forceinline__ void cmac(V& accr, V& acci, V ar, V ai, V br, V bi) {
  accr = vfma(ar, br, accr);
  accr = vfma(-ai, bi, accr);
  acci = vfma(ar, bi, acci);
  acci = vfma(ai, br, acci);
}

// Element tuples of one irreps (order Q <= 4, TT elements) over a chunk of
// canonical terms.  Order 4 fixes the element of slot 0 per unit (u.s0; its
// order parameter is the prefix A); the last three slots z, x, y (the last
// two, x and y, for Q = 2; slot 0 alone for Q = 1) run over all elements.
// With H[z][x][y] the features' adjoint weights and a, b, c the order
// parameters of slots z, x, y, per term and per element z:
//   m[x] = sum_y H c[y],  w[y] = sum_x H b[x],  S_z = sum_x b[x] m[x],
//   G_z[z] += A S_z,  G_x[x] += A a[z] m[x],  G_y[y] += A a[z] w[y],
// and with S = sum_z a[z] S_z:  G_0 += S (order 4), energy += Re(A S)
// (= the sum over tuples of H times the tuple's invariant term).  One set of
// order-parameter loads per term; the adjoint partials of x and y are summed
// over z in registers and flushed with one shared-memory atomic per (slot,
// element).
template <class V, int Q, int TT, int Lh, class EA, class GT>
__device__ __forceinline__ void run_irr(const DeviceIrrUnit& u, const DeviceTuple* __restrict__ tups,
                                        const DeviceTerm* __restrict__ terms,
                                        const V* __restrict__ wlin, const V* hnl,
                                        const typename Cx<V>::type* sa, GT* sg, int gim,
                                        GFixT<V>& gf, int n, int half, bool act, EA& eacc) {
  using Vc = typename Cx<V>::type;
  constexpr int NZ = (Q >= 3) ? TT : 1;      // elements of slot z
  constexpr int NX = TT;                     // elements of slot x (slot 0 for Q = 1)
  constexpr int NY = (Q == 1) ? 1 : TT;      // elements of slot y
  constexpr int PZ = Q - 3;                  // slot indices (PZ, PY unused when absent)
  constexpr int PX = (Q == 1) ? 0 : Q - 2;
  constexpr int PY = Q - 1;
  V H[NZ][NX][NY];
#pragma unroll
  for (int z = 0; z < NZ; ++z)
#pragma unroll
    for (int x = 0; x < NX; ++x)
#pragma unroll
      for (int y = 0; y < NY; ++y) {
        const int2 e =
            __ldg(reinterpret_cast<const int2*>(tups + u.tup + (z * NX + x) * NY + y));
        H[z][x][y] = tuple_weight(e, wlin, hnl, n, act);
      }
  const int s0 = (int)u.s0;
  constexpr int es = Lh * kNPad;   // element stride in the a / G arrays
  constexpr int kIm = TT * es, kLo = 2 * kIm;   // imaginary / low-part offsets (T == TT)
  V eu = V(0);
  // the two half-warps take alternate terms; the adjoints of slot z (and of
  // the fixed slot 0 of order 4) are kept in registers while a half-warp's
  // consecutive terms address the same order parameter (runs of the table's
  // outer m loops) and flushed when its next term moves on
  const int ke = u.term0 + u.nterm, kb = u.term0 + half;
  V azr[NZ], azi[NZ], a0r = V(0), a0i = V(0);
#pragma unroll
  for (int z = 0; z < NZ; ++z) { azr[z] = V(0); azi[z] = V(0); }
  int4 nxt = kb < ke ? __ldg(reinterpret_cast<const int4*>(terms + kb)) : make_int4(0, 0, 0, 0);
  for (int k = kb; k < ke; k += 2) {
    const int4 raw = nxt;
    if (k + 2 < ke) nxt = __ldg(reinterpret_cast<const int4*>(terms + k + 2));
    const bool last = k + 2 >= ke;
    const V c = term_coeff<V>(raw);
    const unsigned lw = (unsigned)raw.z, code = ((unsigned)raw.w) >> 16;
    const bool self = (code >> 12) & 1u;
    const V ce = self ? c : V(2) * c;
    int lo[Q];
#pragma unroll
    for (int p = 0; p < Q; ++p) lo[p] = (int)((lw >> (8 * p)) & 255u) * kNPad + n;
    const auto conj_of = [&](int p) { return ((code >> (2 * p)) & 3u) == (unsigned)kSlotConj; };
    V Ar = V(1), Ai = V(0);   // fixed slot 0 of order 4
    if (Q == 4) {
      const Vc v = sa[s0 * es + lo[0]];
      Ar = v.x;
      Ai = conj_of(0) ? -v.y : v.y;
    }
    V zr[NZ], zi[NZ], br[NX], bi[NX], cr[NY], ci[NY];
    if (Q >= 3) {
      const bool cj = conj_of(PZ);
#pragma unroll
      for (int z = 0; z < NZ; ++z) {
        const Vc v = sa[z * es + lo[PZ]];
        zr[z] = v.x;
        zi[z] = cj ? -v.y : v.y;
      }
    } else {
      zr[0] = V(1);
      zi[0] = V(0);
    }
    {
      const bool cj = conj_of(PX);
#pragma unroll
      for (int x = 0; x < NX; ++x) {
        const Vc v = sa[x * es + lo[PX]];
        br[x] = v.x;
        bi[x] = cj ? -v.y : v.y;
      }
    }
    if (Q > 1) {
      const bool cj = conj_of(PY);
#pragma unroll
      for (int y = 0; y < NY; ++y) {
        const Vc v = sa[y * es + lo[PY]];
        cr[y] = v.x;
        ci[y] = cj ? -v.y : v.y;
      }
    }
    // adjoint partials summed over z: x and y (before the prefix A), and S
    V gxr[NX], gxi[NX], gyr[NY], gyi[NY], gzr[NZ], gzi[NZ];
    V Sr = V(0), Si = V(0);
#pragma unroll
    for (int x = 0; x < NX; ++x) { gxr[x] = V(0); gxi[x] = V(0); }
#pragma unroll
    for (int y = 0; y < NY; ++y) { gyr[y] = V(0); gyi[y] = V(0); }
#pragma unroll
    for (int z = 0; z < NZ; ++z) {
      V mr[NX], mi[NX];
#pragma unroll
      for (int x = 0; x < NX; ++x) {
        if (Q == 1) {
          mr[x] = H[0][x][0];
          mi[x] = V(0);
        } else {
          V tr = V(0), ti = V(0);
#pragma unroll
          for (int y = 0; y < NY; ++y) {
            tr = vfma(H[z][x][y], cr[y], tr);
            ti = vfma(H[z][x][y], ci[y], ti);
          }
          mr[x] = tr;
          mi[x] = ti;
        }
      }
      V szr = V(0), szi = V(0);
#pragma unroll
      for (int x = 0; x < NX; ++x) {
        cmac(szr, szi, br[x], bi[x], mr[x], mi[x]);
      }
      gzr[z] = szr;
      gzi[z] = szi;
      cmac(Sr, Si, zr[z], zi[z], szr, szi);
#pragma unroll
      for (int x = 0; x < NX; ++x) {
        cmac(gxr[x], gxi[x], zr[z], zi[z], mr[x], mi[x]);
      }
      if (Q > 1) {
#pragma unroll
        for (int y = 0; y < NY; ++y) {
          V tr = V(0), ti = V(0);
#pragma unroll
          for (int x = 0; x < NX; ++x) {
            tr = vfma(H[z][x][y], br[x], tr);
            ti = vfma(H[z][x][y], bi[x], ti);
          }
          cmac(gyr[y], gyi[y], zr[z], zi[z], tr, ti);
        }
      }
    }
    eu += ce * (Ar * Sr - Ai * Si);
    {
      // adjoint of slot p: A * partial, scaled by (kr, ki) from its storage
      // code; unconditional (lanes n >= F and unused imaginary parts add
      // exact zeros), so the flush has no divergent branches
      const V cs = gscale(c, gf);
      const auto flush = [&](int p, int e, V vr, V vi) {
        const unsigned cd = (code >> (2 * p)) & 3u;
        const V kr = (cd == (unsigned)kSlotMZero) ? V(2) * cs : cs;
        const V ki = (cd == 0u) ? cs : (cd == 1u ? -cs : V(0));
        GT* gp = sg + e * es + lo[p];
        gput(gp, kr * (Ar * vr - Ai * vi), gf, kLo);
        gput(gp + kIm, ki * (Ar * vi + Ai * vr), gf, kLo);
      };
#pragma unroll
      for (int x = 0; x < NX; ++x) flush(PX, x, gxr[x], gxi[x]);
      if (Q > 1) {
#pragma unroll
        for (int y = 0; y < NY; ++y) flush(PY, y, gyr[y], gyi[y]);
      }
    }
    if (Q >= 3) {   // slot z: A S_z, accumulated over the run
      const unsigned cd = (code >> (2 * PZ)) & 3u;
      const V cs = gscale(c, gf);
      const V kr = (cd == (unsigned)kSlotMZero) ? V(2) * cs : cs;
      const V ki = (cd == 0u) ? cs : (cd == 1u ? -cs : V(0));
#pragma unroll
      for (int z = 0; z < NZ; ++z) {
        azr[z] += kr * (Ar * gzr[z] - Ai * gzi[z]);
        azi[z] += ki * (Ar * gzi[z] + Ai * gzr[z]);
      }
      // flush when this half-warp's next term moves on; voted so that both
      // halves take the (then uniform) branch together
      const bool need = last || ((((unsigned)nxt.z ^ lw) >> (8 * PZ)) & 255u) != 0u;
      if (__any_sync(__activemask(), need)) {
#pragma unroll
        for (int z = 0; z < NZ; ++z) {
          GT* gp = sg + z * es + lo[PZ];
          gput(gp, azr[z], gf, kLo);
          gput(gp + kIm, azi[z], gf, kLo);
        }
#pragma unroll
        for (int z = 0; z < NZ; ++z) { azr[z] = V(0); azi[z] = V(0); }
      }
    }
    if (Q == 4) {   // slot 0: S, without the prefix A (it is slot 0's own factor)
      const unsigned cd = code & 3u;
      const V cs = gscale(c, gf);
      a0r += ((cd == (unsigned)kSlotMZero) ? V(2) * cs : cs) * Sr;
      a0i += ((cd == 0u) ? cs : (cd == 1u ? -cs : V(0))) * Si;
      const bool need0 = last || (((unsigned)nxt.z ^ lw) & 255u) != 0u;
      if (__any_sync(__activemask(), need0)) {
        GT* gp = sg + s0 * es + lo[0];
        gput(gp, a0r, gf, kLo);
        gput(gp + kIm, a0i, gf, kLo);
        a0r = V(0);
        a0i = V(0);
      }
    }
  }
  // this half-warp's terms, in REAL, into the thread's energy sum (zero on
  // lanes n >= F)
  eadd(eacc, eu);
}

// pick of entry z (a runtime index below N) of a register array by selects
// (no local-memory indexing)
template <int N>
__device__ __forceinline__ DF pick(int z, const DF (&v)[N]) {
  DF r = v[0];
#pragma unroll
  for (int k = 1; k < N; ++k) r = (z == k) ? v[k] : r;
  return r;
}

template <int N>
__device__ __forceinline__ void put_acc(int i, DFA (&v)[N], const DFA& x) {
#pragma unroll
  for (int k = 0; k < N; ++k) {
    v[k].s = (i == k) ? x.s : v[k].s;
    v[k].c = (i == k) ? x.c : v[k].c;
  }
}

// Double-float form of run_irr (same sums, same flushes).  The loop over
// the z elements is kept rolled (the weights and order parameters of the
// current z are picked from registers by selects): fully unrolled, the
// double-float body of one term outgrows the instruction cache and the
// warps wait on instruction fetch (rolling the (z, x) pairs as well shrinks
// the body further but its selects cost 13 % more time).  Sums go through
// DFA accumulators (one FP32 add of dependency per accumulation);
// accumulated values that are multiplied again are renormalised once.
template <int Q, int TT, int Lh, class EA>
__device__ __forceinline__ void run_irr_df(const DeviceIrrUnit& u, const DeviceTuple* __restrict__ tups,
                                           const DeviceTerm* __restrict__ terms,
                                           const DF* __restrict__ wlin, const DF* hnl,
                                           const DFc* sa, int* sg, int gim, GFixT<DF>& gf, int n,
                                           int half, bool act, EA& eacc) {
  constexpr int NZ = (Q >= 3) ? TT : 1;      // elements of slot z
  constexpr int NX = TT;                     // elements of slot x (slot 0 for Q = 1)
  constexpr int NY = (Q == 1) ? 1 : TT;      // elements of slot y
  constexpr int PZ = (Q >= 3) ? Q - 3 : 0;   // slot indices
  constexpr int PX = (Q == 1) ? 0 : Q - 2;
  constexpr int PY = Q - 1;
  DF H[NZ * NX][NY];   // weights of the tuple (z, x, y) at H[z NX + x][y]
#pragma unroll
  for (int zx = 0; zx < NZ * NX; ++zx)
#pragma unroll
    for (int y = 0; y < NY; ++y) {
      const int2 e = __ldg(reinterpret_cast<const int2*>(tups + u.tup + zx * NY + y));
      H[zx][y] = tuple_weight(e, wlin, hnl, n, act);
    }
  const int s0 = (int)u.s0;
  constexpr int es = Lh * kNPad;                // element stride in the a / G arrays
  constexpr int kIm = TT * es, kLo = 2 * kIm;   // imaginary / next-word offsets (T == TT)
  DF eu = DF(0.0f);
  const int ke = u.term0 + u.nterm, kb = u.term0 + half;
  DF azr[NZ], azi[NZ], a0r = DF(0.0f), a0i = DF(0.0f);
#pragma unroll
  for (int z = 0; z < NZ; ++z) { azr[z] = DF(0.0f); azi[z] = DF(0.0f); }
  int4 nxt = kb < ke ? __ldg(reinterpret_cast<const int4*>(terms + kb)) : make_int4(0, 0, 0, 0);
  for (int k = kb; k < ke; k += 2) {
    const int4 raw = nxt;
    if (k + 2 < ke) nxt = __ldg(reinterpret_cast<const int4*>(terms + k + 2));
    const bool last = k + 2 >= ke;
    const DF c = term_coeff<DF>(raw);
    const unsigned lw = (unsigned)raw.z, code = ((unsigned)raw.w) >> 16;
    const bool self = (code >> 12) & 1u;
    int lo[Q];
#pragma unroll
    for (int p = 0; p < Q; ++p) lo[p] = (int)((lw >> (8 * p)) & 255u) * kNPad + n;
    const auto conj_of = [&](int p) { return ((code >> (2 * p)) & 3u) == (unsigned)kSlotConj; };
    DF Ar = DF(1.0f), Ai = DF(0.0f);   // fixed slot 0 of order 4
    if (Q == 4) {
      const DFc v = sa[s0 * es + lo[0]];
      Ar = v.x;
      Ai = conj_of(0) ? -v.y : v.y;
    }
    DF zr[NZ], zi[NZ], br[NX], bi[NX], cr[NY], ci[NY];
    if (Q >= 3) {
      const bool cj = conj_of(PZ);
#pragma unroll
      for (int z = 0; z < NZ; ++z) {
        const DFc v = sa[z * es + lo[PZ]];
        zr[z] = v.x;
        zi[z] = cj ? -v.y : v.y;
      }
    } else {
      zr[0] = DF(1.0f);
      zi[0] = DF(0.0f);
    }
    {
      const bool cj = conj_of(PX);
#pragma unroll
      for (int x = 0; x < NX; ++x) {
        const DFc v = sa[x * es + lo[PX]];
        br[x] = v.x;
        bi[x] = cj ? -v.y : v.y;
      }
    }
    if (Q > 1) {
      const bool cj = conj_of(PY);
#pragma unroll
      for (int y = 0; y < NY; ++y) {
        const DFc v = sa[y * es + lo[PY]];
        cr[y] = v.x;
        ci[y] = cj ? -v.y : v.y;
      }
    } else {
      cr[0] = DF(1.0f);
      ci[0] = DF(0.0f);
    }
    DFA gzr[NZ], gzi[NZ], gxr[NX], gxi[NX], gyr[NY], gyi[NY];
    // Rolled loop over the z elements (x and y unrolled inside), with
    // m[x] = sum_y H c_y:  S_z = sum_x b_x m[x],  G_x += a_z m[x],
    // G_y += a_z sum_x H b_x; the weights of the current z are picked from
    // registers by selects.
#pragma unroll 1
    for (int z = 0; z < NZ; ++z) {
      DF Hc[NX][NY];
#pragma unroll
      for (int x = 0; x < NX; ++x)
#pragma unroll
        for (int y = 0; y < NY; ++y) {
          Hc[x][y] = H[x][y];
#pragma unroll
          for (int q = 1; q < NZ; ++q) Hc[x][y] = (z == q) ? H[q * NX + x][y] : Hc[x][y];
        }
      const DF ar = pick(z, zr), ai = pick(z, zi);
      DFA szr, szi;
#pragma unroll
      for (int x = 0; x < NX; ++x) {
        DF mr, mi;
        if (Q == 1) {
          mr = Hc[x][0];
          mi = DF(0.0f);
        } else {
          DFA tr, ti;
#pragma unroll
          for (int y = 0; y < NY; ++y) {
            acc_fma(tr, Hc[x][y], cr[y]);
            acc_fma(ti, Hc[x][y], ci[y]);
          }
          mr = acc_val(tr);
          mi = acc_val(ti);
        }
        cacc(szr, szi, br[x], bi[x], mr, mi);
        if (Q >= 3) {
          cacc(gxr[x], gxi[x], ar, ai, mr, mi);
        } else {
          acc_add(gxr[x], mr);
          acc_add(gxi[x], mi);
        }
      }
      put_acc(z, gzr, szr);
      put_acc(z, gzi, szi);
      if (Q > 1) {
#pragma unroll
        for (int y = 0; y < NY; ++y) {
          DFA tr, ti;
#pragma unroll
          for (int x = 0; x < NX; ++x) {
            acc_fma(tr, Hc[x][y], br[x]);
            acc_fma(ti, Hc[x][y], bi[x]);
          }
          if (Q >= 3) {
            cacc(gyr[y], gyi[y], ar, ai, acc_val(tr), acc_val(ti));
          } else {
            gyr[y] = tr;
            gyi[y] = ti;
          }
        }
      }
    }
    DF gzv_r[NZ], gzv_i[NZ];
    DFA Sr, Si;
#pragma unroll
    for (int z = 0; z < NZ; ++z) {
      gzv_r[z] = acc_val(gzr[z]);
      gzv_i[z] = acc_val(gzi[z]);
      if (Q >= 3) cacc(Sr, Si, zr[z], zi[z], gzv_r[z], gzv_i[z]);
      else { acc_add(Sr, gzv_r[z]); acc_add(Si, gzv_i[z]); }
    }
    const DF Sv = acc_val(Sr), Siv = acc_val(Si);
    const DF ce = self ? c : DF(2.0f) * c;
    eu += ce * (Q == 4 ? Ar * Sv - Ai * Siv : Sv);
    {
      // adjoint of slot p: A * partial, scaled by (kr, ki) from its storage
      // code; unconditional (lanes n >= F and unused imaginary parts add
      // exact zeros)
      const DF cs = gscale(c, gf);
      const auto flush = [&](int p, int lop, int e, DF vr, DF vi) {
        const unsigned cd = (code >> (2 * p)) & 3u;
        const DF kr = (cd == (unsigned)kSlotMZero) ? DF(2.0f) * cs : cs;
        const DF ki = (cd == 0u) ? cs : (cd == 1u ? -cs : DF(0.0f));
        int* gp = sg + e * es + lop;
        if (Q == 4) {
          gput(gp, kr * (Ar * vr - Ai * vi), gf, kLo);
          gput(gp + kIm, ki * (Ar * vi + Ai * vr), gf, kLo);
        } else {
          gput(gp, kr * vr, gf, kLo);
          gput(gp + kIm, ki * vi, gf, kLo);
        }
      };
      // one rolled loop over the (slot, element) pairs of x and y, the
      // values picked by selects (code size: see above)
      constexpr int NW = NX + (Q > 1 ? NY : 0);
      DF wr[NW], wi[NW];
#pragma unroll
      for (int x = 0; x < NX; ++x) { wr[x] = acc_val(gxr[x]); wi[x] = acc_val(gxi[x]); }
      if (Q > 1) {
#pragma unroll
        for (int y = 0; y < NY; ++y) { wr[NX + y] = acc_val(gyr[y]); wi[NX + y] = acc_val(gyi[y]); }
      }
#pragma unroll 1
      for (int w = 0; w < NW; ++w) {
        const bool isx = w < NX;
        flush(isx ? PX : PY, isx ? lo[PX] : lo[PY], isx ? w : w - NX, pick(w, wr), pick(w, wi));
      }
    }
    if (Q >= 3) {   // slot z: A S_z, accumulated over the run
      const unsigned cd = (code >> (2 * PZ)) & 3u;
      const DF cs = gscale(c, gf);
      const DF kr = (cd == (unsigned)kSlotMZero) ? DF(2.0f) * cs : cs;
      const DF ki = (cd == 0u) ? cs : (cd == 1u ? -cs : DF(0.0f));
#pragma unroll
      for (int z = 0; z < NZ; ++z) {
        if (Q == 4) {
          azr[z] += kr * (Ar * gzv_r[z] - Ai * gzv_i[z]);
          azi[z] += ki * (Ar * gzv_i[z] + Ai * gzv_r[z]);
        } else {
          azr[z] += kr * gzv_r[z];
          azi[z] += ki * gzv_i[z];
        }
      }
      const bool need = last || ((((unsigned)nxt.z ^ lw) >> (8 * PZ)) & 255u) != 0u;
      if (__any_sync(__activemask(), need)) {
#pragma unroll
        for (int z = 0; z < NZ; ++z) {
          int* gp = sg + z * es + lo[PZ];
          gput(gp, azr[z], gf, kLo);
          gput(gp + kIm, azi[z], gf, kLo);
        }
#pragma unroll
        for (int z = 0; z < NZ; ++z) { azr[z] = DF(0.0f); azi[z] = DF(0.0f); }
      }
    }
    if (Q == 4) {   // slot 0: S, without the prefix A (it is slot 0's own factor)
      const unsigned cd = code & 3u;
      const DF cs = gscale(c, gf);
      a0r += ((cd == (unsigned)kSlotMZero) ? DF(2.0f) * cs : cs) * Sv;
      a0i += ((cd == 0u) ? cs : (cd == 1u ? -cs : DF(0.0f))) * Siv;
      const bool need0 = last || (((unsigned)nxt.z ^ lw) & 255u) != 0u;
      if (__any_sync(__activemask(), need0)) {
        int* gp = sg + s0 * es + lo[0];
        gput(gp, a0r, gf, kLo);
        gput(gp + kIm, a0i, gf, kLo);
        a0r = DF(0.0f);
        a0i = DF(0.0f);
      }
    }
  }
  // this half-warp's terms into the thread's energy sum (zero on lanes n >= F)
  eadd(eacc, eu);
}

template <class V, int TT, int Lh, class EA, class GT>
__device__ __forceinline__ void dispatch_irr(const DeviceIrrUnit& u, const DeviceTuple* tups,
                                             const DeviceTerm* terms, const V* wlin,
                                             const V* hnl, const typename Cx<V>::type* sa,
                                             GT* sg, int gim, GFixT<V>& gf, int n, int half,
                                             bool act, EA& eacc) {
  if constexpr (std::is_same_v<V, DF>) {
    switch (u.q) {
      case 1: run_irr_df<1, TT, Lh>(u, tups, terms, wlin, hnl, sa, sg, gim, gf, n, half, act, eacc); break;
      case 2: run_irr_df<2, TT, Lh>(u, tups, terms, wlin, hnl, sa, sg, gim, gf, n, half, act, eacc); break;
      case 3: run_irr_df<3, TT, Lh>(u, tups, terms, wlin, hnl, sa, sg, gim, gf, n, half, act, eacc); break;
      default: run_irr_df<4, TT, Lh>(u, tups, terms, wlin, hnl, sa, sg, gim, gf, n, half, act, eacc); break;
    }
    return;
  } else {
  if (TT <= 2 && u.q <= 3) {
    switch (u.q) {
      case 1: run_irr_direct<V, 1, TT, Lh>(u, tups, terms, wlin, hnl, sa, sg, gim, gf, n, half, act, eacc); break;
      case 2: run_irr_direct<V, 2, TT, Lh>(u, tups, terms, wlin, hnl, sa, sg, gim, gf, n, half, act, eacc); break;
      default: run_irr_direct<V, 3, TT, Lh>(u, tups, terms, wlin, hnl, sa, sg, gim, gf, n, half, act, eacc); break;
    }
    return;
  }
  switch (u.q) {
    case 1: run_irr<V, 1, TT, Lh>(u, tups, terms, wlin, hnl, sa, sg, gim, gf, n, half, act, eacc); break;
    case 2: run_irr<V, 2, TT, Lh>(u, tups, terms, wlin, hnl, sa, sg, gim, gf, n, half, act, eacc); break;
    case 3: run_irr<V, 3, TT, Lh>(u, tups, terms, wlin, hnl, sa, sg, gim, gf, n, half, act, eacc); break;
    default: run_irr<V, 4, TT, Lh>(u, tups, terms, wlin, hnl, sa, sg, gim, gf, n, half, act, eacc); break;
  }
  }
}

template <class V, bool WITH_G, int Lh, class GT>
__device__ __forceinline__ void dispatch_unit(const DeviceUnit& u, const DeviceTerm* terms,
                                              const typename Cx<V>::type* sa, GT* sg, int gim,
                                              GFixT<V>& gf, int n, int half, bool act, V H,
                                              V& dsum) {
  switch (u.q) {
    case 1: run_unit<V, 1, WITH_G, Lh>(u, terms, sa, sg, gim, gf, n, half, act, H, dsum); break;
    case 2: run_unit<V, 2, WITH_G, Lh>(u, terms, sa, sg, gim, gf, n, half, act, H, dsum); break;
    case 3: run_unit<V, 3, WITH_G, Lh>(u, terms, sa, sg, gim, gf, n, half, act, H, dsum); break;
    case 4: run_unit<V, 4, WITH_G, Lh>(u, terms, sa, sg, gim, gf, n, half, act, H, dsum); break;
    case 5: run_unit<V, 5, WITH_G, Lh>(u, terms, sa, sg, gim, gf, n, half, act, H, dsum); break;
    default: run_unit<V, 6, WITH_G, Lh>(u, terms, sa, sg, gim, gf, n, half, act, H, dsum); break;
  }
}

// FP64 radial functions f_n(r), n < F (0 for the padding lanes): with a
// common beta, by the multiplicative recurrence of radial_rec (two exps per
// neighbour; every step multiplies, so the relative error stays at a few
// FP64 ulps), else one exp per function.
__device__ __forceinline__ void radial64(const KernelArgs& A, double r, double* f) {
  double sn, cs;
  sincospi(r / A.rc, &sn, &cs);
  const double fc = r < A.rc ? 0.5 * (cs + 1.0) : 0.0;
  const int F = A.F;
  if (A.radial_rec) {
    const double beta = __ldg(A.radial), mu0 = __ldg(A.radial + 1);
    const double q = exp(A.rec_q * r);
    double g = exp(-beta * (r - mu0) * (r - mu0));
#pragma unroll
    for (int n = 0; n < kNPad; ++n) {
      f[n] = n < F ? g * fc : 0.0;
      if (n + 1 < F) {
        const double2 ke = __ldg(reinterpret_cast<const double2*>(A.radial_rec) + n);
        g = g * q * ke.x * fma(ke.y, r, 1.0);
      }
    }
  } else {
#pragma unroll
    for (int n = 0; n < kNPad; ++n) {
      double fv = 0.0;
      if (n < F) {
        const double beta = __ldg(A.radial + 2 * n), mu = __ldg(A.radial + 2 * n + 1);
        const double dr = r - mu;
        fv = exp(-beta * dr * dr) * fc;
      }
      f[n] = fv;
    }
  }
}

// FP64 radial functions and their derivatives for all 16 channels (P6 of
// the FP64 kernels): the Gaussians g_n by the recurrence of radial64 when
// beta is common, f_n = g_n fc, f'_n = -2 beta (r - mu_n) g_n fc + g_n fc'.
__device__ __forceinline__ void radial64d(const KernelArgs& A, double r, double* f, double* fd) {
  double sn, cs;
  sincospi(r / A.rc, &sn, &cs);
  const bool in = r < A.rc;
  const double fc = in ? 0.5 * (cs + 1.0) : 0.0;
  const double fcd = in ? -0.5 * 3.14159265358979323846 / A.rc * sn : 0.0;
  const int F = A.F;
  if (A.radial_rec) {
    const double beta = __ldg(A.radial), mu0 = __ldg(A.radial + 1);
    const double q = exp(A.rec_q * r);
    double g = exp(-beta * (r - mu0) * (r - mu0));
#pragma unroll
    for (int n = 0; n < kNPad; ++n) {
      const double mu = n < F ? __ldg(A.radial + 2 * n + 1) : 0.0;
      f[n] = n < F ? g * fc : 0.0;
      fd[n] = n < F ? (-2.0 * beta * (r - mu) * g) * fc + g * fcd : 0.0;
      if (n + 1 < F) {
        const double2 ke = __ldg(reinterpret_cast<const double2*>(A.radial_rec) + n);
        g = g * q * ke.x * fma(ke.y, r, 1.0);
      }
    }
  } else {
#pragma unroll
    for (int n = 0; n < kNPad; ++n) {
      f[n] = 0.0;
      fd[n] = 0.0;
      if (n < F) {
        const double beta = __ldg(A.radial + 2 * n), dr = r - __ldg(A.radial + 2 * n + 1);
        const double g = exp(-beta * dr * dr);
        f[n] = g * fc;
        fd[n] = (-2.0 * beta * dr * g) * fc + g * fcd;
      }
    }
  }
}

// Force contributions of one neighbour at one (l, m <= 0) for all 16
// channels (P6 of the FP64 kernels): with G of the neighbour's element row,
// g0 = sum_n f_n G_n, g1 = sum_n f'_n G_n, and the same force expression as
// ForceVis.
struct ForceVis16 {
  const R* g;   // Re G of the neighbour's element slot, channel 0: [Lh][16]; Im at g + gim
  int gim;
  const R* f;
  const R* fd;
  R ux, uy, uz;
  R fx, fy, fz;
  __device__ __forceinline__ void operator()(int lmh, int mp, R yre, R yim, R xre, R xim,
                                             R yyre, R yyim, R zre, R zim) {
    R g0r = 0, g0i = 0, g1r = 0, g1i = 0;
#pragma unroll
    for (int q = 0; q < kNPad; q += 4) {
      R gr[4], gi[4];
      load4(g + lmh * kNPad + q, gr);
      load4(g + gim + lmh * kNPad + q, gi);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        g0r = fma(f[q + k], gr[k], g0r);
        g0i = fma(f[q + k], gi[k], g0i);
        g1r = fma(fd[q + k], gr[k], g1r);
        g1i = fma(fd[q + k], gi[k], g1i);
      }
    }
    const R coeff = (mp == 0) ? R(1) : R(2);
    const R ry = yre * g1r + yim * g1i;
    fx += coeff * (ry * ux + (xre * g0r + xim * g0i));
    fy += coeff * (ry * uy + (yyre * g0r + yyim * g0i));
    fz += coeff * (ry * uz + (zre * g0r + zim * g0i));
  }
};

// Column set of the force phase: column m goes to part
// (0 1 2 3 3 2 1 0 0 1 ...)[m] of the four, which balances the columns'
// lengths (L - m + 1 entries each).
__device__ __forceinline__ int column_part(int mp) {
  const int s = mp & 7;
  return s < 4 ? s : 7 - s;
}

// sh_visit restricted to the columns m of one part: every column still
// advances the angle recursions and (with DERIV) the cheap Q recursion that
// the next column's derivatives read; P, Y, dY and the visitor run for the
// part's own columns only.  `part` is uniform across the warp.
template <int LCAP, typename V, bool DERIV = true>
__device__ __forceinline__ void sh_visit_part(R dx, R dy, R dz, R r, int L,
                                              int part, V& vis) {
  const R invr = R(1) / r;
  const R ct = dz * invr;
  const R st = sqrt(fmax(R(0), R(1) - ct * ct));
  const R rho2 = dx * dx + dy * dy;
  R cp = R(1), sp = R(0);
  if (rho2 > R(0)) {
    const R ir = rsqrt_r(rho2);
    cp = dx * ir;
    sp = dy * ir;
  }
  constexpr bool kUnit = sizeof(R) == 4;   // FP32: Y / Y_00 (see sh_visit)
  const R h = kUnit ? R(1) : R(0.70710678118654752440);   // 0.5 * sqrt(2)
  R Qc[LCAP + 2];
#pragma unroll
  for (int l = 0; l < LCAP + 2; ++l) Qc[l] = R(0);
  R pdiag = kUnit ? R(1) : R(0.39894228040143267794);      // P_0^0 = sqrt(1/(2 pi))
  R cm = R(1), sm = R(0), cprev = cp, sprev = -sp;
  const R tc = R(2) * cp;
  R sgn = R(1);
#pragma unroll
  for (int mp = 0; mp <= LCAP; ++mp) {
    if (mp > L) break;
    if (mp > 0) {
      const R s = tc * sm - sprev;
      const R c = tc * cm - cprev;
      cprev = cm; cm = c; sprev = sm; sm = s;
      pdiag = pdiag * (cDiag[mp] * st);
      sgn = -sgn;
    }
    const bool mine = column_part(mp) == part;
    // Q_1^1 = P_0^0 cDiag[1]
    const R qn_diag = !DERIV ? R(0)
                      : (mp == 0) ? (kUnit ? cDiag[1] : R(-0.48860251190291992263))
                                  : Qc[mp] * (cDiag[mp + 1] * st);
    R p1 = R(0), p2 = R(0), qn1 = R(0), qn2 = R(0);
#pragma unroll
    for (int l = mp; l <= LCAP; ++l) {
      if (l > L) break;
      R Qn = R(0);
      if (DERIV) {
        if (l == mp + 1) Qn = qn_diag;
        else if (l == mp + 2) Qn = (ct * cOff[mp + 1]) * qn1;
        else if (l >= mp + 3) Qn = cA[lm2i(l, mp + 1)] * (ct * qn1 + cB[lm2i(l, mp + 1)] * qn2);
        if (l >= mp + 1) { qn2 = qn1; qn1 = Qn; }
      }
      if (mine) {
        R P;
        if (l == mp) P = pdiag;
        else if (l == mp + 1) P = (ct * cOff[mp]) * p1;
        else P = cA[lm2i(l, mp)] * (ct * p1 + cB[lm2i(l, mp)] * p2);
        p2 = p1;
        p1 = P;
        R yre, yim;
        if (mp == 0) {
          yre = P * h;
          yim = R(0);
        } else {
          const R t = sgn * P * h;
          yre = t * cm;
          yim = -(t * sm);
        }
        const int lmh = l * (l + 1) / 2 + l - mp;
        R xre = 0, xim = 0, yyre = 0, yyim = 0, zre = 0, zim = 0;
        if (!DERIV) {
          vis(lmh, mp, yre, yim, xre, xim, yyre, yyim, zre, zim);
          continue;
        }
        if (mp == 0) {
          if (l >= 1) {
            const R common = Qn * st * invr * cLL[l];
            xre = common * ct * cp;
            yyre = common * ct * sp;
            zre = -common * st;
          }
        } else {
          const R qc = Qc[l];
          R dth = R(mp) * ct * qc;
          if (l != mp) dth += cLM[lm2i(l, mp)] * Qn * st;
          const R dph = R(mp) * qc;
          const R ere = cm * h * invr, eim = sm * h * invr;
          const R vxr = dth * ct * cp, vxi = -dph * sp;
          const R vyr = dth * ct * sp, vyi = dph * cp;
          const R vzr = -dth * st;
          xre = sgn * (ere * vxr - eim * vxi);
          xim = -sgn * (ere * vxi + eim * vxr);
          yyre = sgn * (ere * vyr - eim * vyi);
          yyim = -sgn * (ere * vyi + eim * vyr);
          zre = sgn * (ere * vzr);
          zim = -sgn * (eim * vzr);
        }
        vis(lmh, mp, yre, yim, xre, xim, yyre, yyim, zre, zim);
      }
      if (DERIV && l >= mp + 1) Qc[l] = Qn;
    }
  }
}

// P2b of the mixed path (see fused_kernel): FP64 order parameters
// a64[element][lmh < lh64][n] of the rows the polynomial's input features
// read, from FP64 radial functions and Y_lm of the centre's compacted
// neighbours (misc[t]..misc[t+1] of nbk per element), staged in `stage`
// (the G space).  With l = 0 alone (model_type 3), a = Y_00 sum_j f_n(r_j):
// windows of 64 neighbours across elements, one radial evaluation per
// neighbour and thread.  Not inlined: it runs once per centre and its FP64
// registers would otherwise weigh on the hot phases.
__device__ __noinline__ void order_params64(const KernelArgs& A, int c, double4 xi, const int* misc,
                                            const int* nbk, double2* stage, double2* a64) {
  const int T = A.T, tid = threadIdx.x;
  const int lh64 = A.lh64;
  const int nkeep = misc[T];
  if (lh64 == 1) {
    constexpr int kWin = 2 * kChunk;
    double* fs64 = reinterpret_cast<double*>(stage);   // [kWin][16]
    const int t = tid >> 4, nn = tid & 15;
    double acc = 0.0;
    for (int w0 = 0; w0 < nkeep; w0 += kWin) {
      const int wsz = min(kWin, nkeep - w0);
      if (tid < wsz) {
        const int k = nbk[w0 + tid];
        const int j = __ldg(A.nbr_idx + k);
        double dx, dy, dz;
        pair_disp(A, c, k, xi, A.x4[j], dx, dy, dz);
        double f64[kNPad];
        radial64(A, sqrt(dx * dx + dy * dy + dz * dz), f64);
#pragma unroll
        for (int q = 0; q < kNPad; ++q) fs64[tid * kNPad + q] = f64[q];
      }
      __syncthreads();
      if (t < T) {
        const int j0 = max(misc[t], w0), j1 = min(misc[t + 1], w0 + wsz);
        for (int jj = j0 - w0; jj < j1 - w0; ++jj) acc += fs64[jj * kNPad + nn];
      }
      __syncthreads();
    }
    // Y_00 = sqrt(1 / (4 pi)), real
    if (t < T) a64[t * kNPad + nn] = double2{0.28209479177387814347 * acc, 0.0};
    __syncthreads();
    return;
  }
  int l64 = 0;
  while ((l64 + 1) * (l64 + 2) / 2 < lh64) ++l64;
  double2* ys64 = stage;                                                    // [lh64][kChunk]
  double* fs64 = reinterpret_cast<double*>(ys64 + (size_t)lh64 * kChunk);  // [kChunk][16]
  const int nent = lh64 * kNPad;
  // passes of 2 x 256 entries (one pass up to l = 6), two FP64 accumulator
  // pairs per thread
  for (int t = 0; t < T; ++t) {
    for (int e0 = 0; e0 < nent; e0 += 2 * kBlock) {
      double ar0 = 0.0, ai0 = 0.0, ar1 = 0.0, ai1 = 0.0;
      const int i0 = e0 + tid, i1 = e0 + kBlock + tid;
      const int b0 = misc[t], b1 = misc[t + 1];
      for (int cb = b0; cb < b1; cb += kChunk) {
        const int csz = min(kChunk, b1 - cb);
        if (tid < csz) {
          const int k = nbk[cb + tid];
          const int j = __ldg(A.nbr_idx + k);
          double dx, dy, dz;
          pair_disp(A, c, k, xi, A.x4[j], dx, dy, dz);
          const double r = sqrt(dx * dx + dy * dy + dz * dz);
          double f64[kNPad];
          radial64(A, r, f64);
#pragma unroll
          for (int q = 0; q < kNPad; ++q) fs64[tid * kNPad + q] = f64[q];
          sh_values64(dx, dy, dz, r, l64, ys64, kChunk, tid);
        }
        __syncthreads();
        if (i0 < nent) {
          const int lmh = i0 >> 4, nn = i0 & 15;
          for (int jj = 0; jj < csz; ++jj) {
            const double fv = fs64[jj * kNPad + nn];
            const double2 y = ys64[lmh * kChunk + jj];
            ar0 = fma(fv, y.x, ar0);
            ai0 = fma(-fv, y.y, ai0);
          }
        }
        if (i1 < nent) {
          const int lmh = i1 >> 4, nn = i1 & 15;
          for (int jj = 0; jj < csz; ++jj) {
            const double fv = fs64[jj * kNPad + nn];
            const double2 y = ys64[lmh * kChunk + jj];
            ar1 = fma(fv, y.x, ar1);
            ai1 = fma(-fv, y.y, ai1);
          }
        }
        __syncthreads();
      }
      if (i0 < nent) a64[(size_t)t * nent + i0] = double2{ar0, ai0};
      if (i1 < nent) a64[(size_t)t * nent + i1] = double2{ar1, ai1};
    }
  }
  __syncthreads();
}

// Invariant d(n) of one (irreps, element tuple) in FP64 from FP64 order
// parameters a64[element][lmh < lh64][n] (this half-warp's terms; the two
// halves take alternate terms).  Mixed path, polynomial input features.
__device__ __forceinline__ double nl_forward64(const DeviceUnit& u,
                                               const DeviceTerm* __restrict__ terms64,
                                               const double2* a64, int lh64, int n, int half) {
  double dsum = 0.0;
  const int kend = u.term0 + u.nterm;
  for (int k = u.term0 + half; k < kend; k += 2) {
    const int4 raw = __ldg(reinterpret_cast<const int4*>(terms64 + k));
    const double c = __hiloint2double(raw.y, raw.x);
    const unsigned lw = (unsigned)raw.z, hw = (unsigned)raw.w;
    const unsigned code = hw >> 16;
    double pr = 1.0, pi = 0.0;
    for (int p = 0; p < (int)u.q; ++p) {
      const int lmh = p < 4 ? (int)((lw >> (8 * p)) & 255u) : (int)((hw >> (8 * (p - 4))) & 255u);
      const double2 v = a64[((int)u.s[p] * lh64 + lmh) * kNPad + n];
      const double vi = ((code >> (2 * p)) & 3u) == (unsigned)kSlotConj ? -v.y : v.y;
      const double tr = pr * v.x - pi * vi;
      pi = pr * vi + pi * v.x;
      pr = tr;
    }
    const bool self = (code >> 12) & 1u;
    dsum += (self ? c : 2.0 * c) * pr;
  }
  return dsum;
}

}  // namespace

__host__ __device__ inline size_t align16(size_t v) { return (v + 15) & ~size_t(15); }

// the FP64 force phase's partial forces (64 neighbours x 4 parts x 3 doubles)
// fit the space of a of the smallest FP64 model (one element, l <= 6)
static_assert(sizeof(R) == 4 || 28 * kNPad * sizeof(Rc) >= 64 * 4 * 3 * sizeof(double),
              "force-phase scratch");

struct SmemLayout {
  size_t a, g, dnl, hnl, nbk, misc, red, a64, total;
};

__host__ __device__ inline SmemLayout smem_layout(int T, int Lh, int nb_cap, int nl_cap,
                                                  int lh64) {
  SmemLayout s;
  const size_t an = (size_t)T * Lh * kNPad * sizeof(Rc);
  // adjoint: FP64 re/im, the mixed path's int32 high + low parts of re/im,
  // or the double-float path's four int32 words of re/im
  const size_t gn = (size_t)T * Lh * kNPad * (4 * kGWords);
  // neighbour staging; with FP64 l = 0 inputs (lh64 == 1) the mixed
  // path's window also stages their FP64 radial functions (64 x 16 doubles)
  const size_t stage = (size_t)Lh * kChunk * sizeof(double2) + (size_t)kChunk * kNPad * sizeof(double) +
                       (lh64 == 1 ? (size_t)2 * kChunk * kNPad * sizeof(double) : 0);
  s.a = 0;
  s.g = align16(an);
  s.dnl = s.g + align16(gn > stage ? gn : stage);
  s.hnl = s.dnl + align16((size_t)nl_cap * kNPad * sizeof(double));
  s.nbk = s.hnl + align16((size_t)nl_cap * kNPad * sizeof(double));
  s.misc = s.nbk + align16((size_t)nb_cap * sizeof(int));
  s.red = s.misc + align16(32 * sizeof(int));
  s.a64 = s.red + align16(16 * (kBlock / 32) * sizeof(double));
  s.total = s.a64 + align16((size_t)T * lh64 * kNPad * sizeof(double2));
  return s;
}

#ifndef MLIPG_NO_FUSED   // units that only want the device helpers above
template <int LCAP>
__global__ void __launch_bounds__(kBlock, kMinBlocks) fused_kernel(const __grid_constant__ KernelArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int T = A.T, F = A.F, Lh = A.Lh, L = A.L;
  // rows of the a / G arrays per element: the instantiation's capacity, so
  // that element strides are compile-time constants (rows >= Lh are unused)
  constexpr int LS = (LCAP + 1) * (LCAP + 2) / 2;
  const SmemLayout lay = smem_layout(T, LS, A.nb_cap, A.nl_cap, sizeof(R) == 4 ? A.lh64 : 0);
  Rc* sa = reinterpret_cast<Rc*>(smem + lay.a);
  R* sg = reinterpret_cast<R*>(smem + lay.g);   // G: Re [T][Lh][16], then Im at sg + gim
  const int gim = T * LS * kNPad;
  double2* ys = reinterpret_cast<double2*>(sg);                     // P2 staging (FP64)
  double* fs = reinterpret_cast<double*>(smem + lay.g + (size_t)Lh * kChunk * sizeof(double2));
  double* dnl = reinterpret_cast<double*>(smem + lay.dnl);
  double* hnl = reinterpret_cast<double*>(smem + lay.hnl);
  int* nbk = reinterpret_cast<int*>(smem + lay.nbk);
  int* misc = reinterpret_cast<int*>(smem + lay.misc);   // [0..8] type offsets, [9] skip, [10] ctr
  double* red = reinterpret_cast<double*>(smem + lay.red);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const R rc = (R)A.rc;
  const double rc2 = A.rc * A.rc;
  constexpr int kLhCap = (LCAP + 1) * (LCAP + 2) / 2;
  constexpr int kEPT = (kLhCap * kNPad + kBlock - 1) / kBlock;

  double vir[6] = {0, 0, 0, 0, 0, 0};
  double ecta = 0.0;
  unsigned long long ph[6] = {0, 0, 0, 0, 0, 0};   // thread 0: cycles per phase
  long long tstamp = 0;
  const bool prof = A.phase_clocks != nullptr;
#define MLIPG_STAMP(k)                          \
  if (prof && tid == 0) {                       \
    const long long t_ = clock64();             \
    ph[k] += (unsigned long long)(t_ - tstamp); \
    tstamp = t_;                                \
  }

  // fixed-point paths: exponent of the adjoint's scale per centre element,
  // adapted from centre to centre (a centre whose flushes leave the range,
  // or use too little of it, is redone at the adapted scale); it starts from
  // the handle's cache of the values a previous launch ended with, so short
  // launches (small cells, MD steps) do not pay the adaptation again
  if (tid < kMaxTypes) misc[16 + tid] = A.gexp_cache ? A.gexp_cache[tid] : 0;
  __syncthreads();
  for (int c = blockIdx.x; c < A.ncenters; c += gridDim.x) {
    const int i = __ldg(A.centers + c);
    const double4 xi = A.x4[i];
    const int ti = (int)xi.w;
    if (ti < 0 || ti >= T) {
      if (tid == 0) {
        if (A.eatom) A.eatom[c] = 0.0;
        if (ti >= T) atomicOr(A.status, kStatusBadType);
      }
      continue;
    }
    const int o0 = __ldg(A.nbr_off + c), o1 = __ldg(A.nbr_off + c + 1);
    if (prof && tid == 0) tstamp = clock64();
    // ---------------------------------------------------------------- P1
    // Neighbour compaction.  Each warp classifies a contiguous range of
    // 32-entry chunks of the list (inside the cutoff, element); the per-(warp,
    // element) counts meet in shared memory (the block-reduction space, free
    // until the end of the centre) and each warp scatters its entries after
    // the elements before and the warps before it, which gives the serial
    // order: element-major, list order within an element.
    {
      const auto classify = [&](int k) {
        int t = -1;
        if (k < o1) {
          const int j = __ldg(A.nbr_idx + k);
          const double4 xj = A.x4[j];
          double dx, dy, dz;
          pair_disp(A, c, k, xi, xj, dx, dy, dz);
          const double r2 = dx * dx + dy * dy + dz * dz;
          t = (int)xj.w;
          if (!(t >= 0 && t < T && r2 <= rc2 && r2 > 0.0)) t = -1;
        }
        return t;
      };
      int* wcnt = reinterpret_cast<int*>(red);   // [warp][kMaxTypes]
      const int nch = (o1 - o0 + 31) >> 5;
      const int cpw = (nch + kBlock / 32 - 1) / (kBlock / 32);
      const int ch0 = warp * cpw, ch1 = min(nch, ch0 + cpw);
      int t0 = -1;   // class of this lane's entry in the warp's first chunk
      {
        int cnt[kMaxTypes];
#pragma unroll
        for (int t = 0; t < kMaxTypes; ++t) cnt[t] = 0;
        for (int ch = ch0; ch < ch1; ++ch) {
          const int t = classify(o0 + 32 * ch + lane);
          if (ch == ch0) t0 = t;
#pragma unroll
          for (int tt = 0; tt < kMaxTypes; ++tt)
            if (tt < T) cnt[tt] += __popc(__ballot_sync(0xffffffffu, t == tt));
        }
#pragma unroll
        for (int tt = 0; tt < kMaxTypes; ++tt)
          if (lane == tt) wcnt[warp * kMaxTypes + tt] = cnt[tt];
      }
      __syncthreads();
      if (ch0 < ch1 || warp == 0) {
        int tot = 0, toff[kMaxTypes + 1], cur[kMaxTypes];
#pragma unroll
        for (int tt = 0; tt < kMaxTypes; ++tt) {
          toff[tt] = tot;
          cur[tt] = tot;
          if (tt < T) {
            for (int w = 0; w < kBlock / 32; ++w) {
              const int v = wcnt[w * kMaxTypes + tt];
              if (w < warp) cur[tt] += v;
              tot += v;
            }
          }
        }
        toff[kMaxTypes] = tot;
        const bool over = tot > A.nb_cap;
        if (!over) {
          const unsigned lt = (1u << lane) - 1u;
          for (int ch = ch0; ch < ch1; ++ch) {
            const int k = o0 + 32 * ch + lane;
            const int t = ch == ch0 ? t0 : classify(k);
#pragma unroll
            for (int tt = 0; tt < kMaxTypes; ++tt) {
              if (tt < T) {
                const unsigned b = __ballot_sync(0xffffffffu, t == tt);
                if (t == tt) nbk[cur[tt] + __popc(b & lt)] = k;
                cur[tt] += __popc(b);
              }
            }
          }
        }
        if (tid == 0) {
#pragma unroll
          for (int tt = 0; tt <= kMaxTypes; ++tt) misc[tt] = tt < T ? toff[tt] : tot;
          misc[9] = over ? 1 : 0;
          misc[10] = 0;
          if (over) atomicOr(A.status, kStatusNeighbourCapacity);
        }
      }
    }
    __syncthreads();
    if (misc[9]) {
      if (tid == 0 && A.eatom) A.eatom[c] = 0.0;
      __syncthreads();
      continue;
    }
    const int nkeep = misc[T];
    MLIPG_STAMP(0)
    // ---------------------------------------------------------------- P2
    if (sizeof(R) == 4 && LCAP <= 16 && !A.sum64) {
      // Mixed path: FP32 products summed with Kahan compensation (sum and
      // compensation term per entry), rounded once to FP32 at the end; the FP32
      // pipe is some sixty times wider than the FP64 pipe on this GPU.  (At
      // l <= 20 the four accumulators per entry no longer fit in registers
      // beside the rest, so that instantiation keeps the FP64 sums, as does
      // the precision that asks for them.)
      // Neighbours are staged in windows of 64 (the FP32 stage takes half the
      // bytes of the FP64 one), across element boundaries, so one window
      // usually holds the whole neighbourhood; an element that spans windows
      // carries its rounded sum from the previous window.
      // With the polynomial's FP64 inputs at l = 0 alone (lh64 == 1, the
      // model_type 3 case), their FP64 order parameters a64[t][n] =
      // Y_00 sum_j f_n(r_j) are made in the same windows: the staging thread
      // also evaluates the FP64 radial functions and T x 16 threads sum them
      // (the order and the sums of order_params64, without its second pass
      // over the neighbours).
      constexpr int kWin = 2 * kChunk;
      float2* ysf = reinterpret_cast<float2*>(sg);
      float* fsf = reinterpret_cast<float*>(smem + lay.g + (size_t)LS * kWin * sizeof(float2));
      double* fs64 = reinterpret_cast<double*>(smem + lay.g + (size_t)LS * kWin * sizeof(float2) +
                                               (size_t)kWin * kNPad * sizeof(float));
      const bool fuse64 = A.lh64 == 1 && __ldg(A.nl_off + ti + 1) > __ldg(A.nl_off + ti);
      double acc64 = 0.0;   // thread t * 16 + n: element t, channel n
      const int n = tid & 15;
      for (int w0 = 0; w0 < nkeep; w0 += kWin) {
        const int wsz = min(kWin, nkeep - w0);
        if (tid < wsz) {
          const int k = nbk[w0 + tid];
          const int j = __ldg(A.nbr_idx + k);
          double dx, dy, dz;
          pair_disp(A, c, k, xi, A.x4[j], dx, dy, dz);
          const double r = sqrt(dx * dx + dy * dy + dz * dz);
          if (fuse64) {
            double f64[kNPad];
            radial64(A, r, f64);
#pragma unroll
            for (int q = 0; q < kNPad; ++q) fs64[tid * kNPad + q] = f64[q];
          }
          R f[kNPad], fdum[kNPad];
          radial(A.radial, F, (R)r, rc, f, fdum, false);
#pragma unroll
          for (int q = 0; q < kNPad; ++q) fsf[tid * kNPad + q] = (float)f[q];
          StageVisW v{ysf, tid};
          sh_visit<LCAP, false>((R)dx, (R)dy, (R)dz, (R)r, L, v);
        }
        __syncthreads();
        if (fuse64 && tid < T * kNPad) {
          const int t64 = tid >> 4;
          const int j0 = max(misc[t64], w0), j1 = min(misc[t64 + 1], w0 + wsz);
          for (int jj = j0 - w0; jj < j1 - w0; ++jj) acc64 += fs64[jj * kNPad + n];
        }
        for (int t = 0; t < T; ++t) {
          const int j0 = max(misc[t], w0), j1 = min(misc[t + 1], w0 + wsz);
          if (j0 >= j1) continue;
          const bool cont = misc[t] < w0;
#pragma unroll
          for (int e = 0; e < kEPT; ++e) {
            const int idx = tid + e * kBlock;
            const int lmh = idx >> 4;
            Rc* dst = sa + (t * LS + lmh) * kNPad + (idx & 15);
            float sr = 0.f, cr = 0.f, si = 0.f, ci = 0.f;
            if (cont && lmh < Lh) { sr = dst->x; si = dst->y; }
            // rows past Lh read a staged row and are never stored
            const float2* yrow = ysf + min(lmh, Lh - 1) * kWin;
#pragma unroll 4
            for (int jj = j0 - w0; jj < j1 - w0; ++jj) {
              const float fv = fsf[jj * kNPad + n];
              const float2 y = yrow[jj];
              kahan_fma_acc(sr, cr, fv, y.x);
              kahan_fma_acc(si, ci, -fv, y.y);
            }
            if (lmh < Lh) *dst = Rc{(R)__fsub_rn(sr, cr), (R)__fsub_rn(si, ci)};
          }
        }
        __syncthreads();
      }
      for (int t = 0; t < T; ++t)   // elements without neighbours
        if (misc[t] == misc[t + 1])
          for (int idx = tid; idx < Lh * kNPad; idx += kBlock) sa[t * LS * kNPad + idx] = Rc{R(0), R(0)};
      if (fuse64 && tid < T * kNPad)   // Y_00 = sqrt(1 / (4 pi)), real
        reinterpret_cast<double2*>(smem + lay.a64)[tid] = double2{0.28209479177387814347 * acc64, 0.0};
    } else
    for (int t = 0; t < T; ++t) {
      double accr[kEPT], acci[kEPT];
#pragma unroll
      for (int e = 0; e < kEPT; ++e) { accr[e] = 0.0; acci[e] = 0.0; }
      const int b0 = misc[t], b1 = misc[t + 1];
      for (int cb = b0; cb < b1; cb += kChunk) {
        const int csz = min(kChunk, b1 - cb);
        // staging by four warps: neighbour = lane, the warps split the
        // harmonic columns (warp 0 also the radial functions)
        const int slot = tid & 31, part = tid >> 5;
        if (part < 4 && slot < csz) {
          const int k = nbk[cb + slot];
          const int j = __ldg(A.nbr_idx + k);
          double dx, dy, dz;
          pair_disp(A, c, k, xi, A.x4[j], dx, dy, dz);
          const double r = sqrt(dx * dx + dy * dy + dz * dz);
          if (part == 0) {
            if constexpr (sizeof(R) == 8) {
              double f64[kNPad];
              radial64(A, r, f64);
#pragma unroll
              for (int n = 0; n < kNPad; ++n) fs[slot * kNPad + n] = f64[n];
            } else {   // mixed path with FP64 sums: FP32 radial functions
              R f[kNPad], fdum[kNPad];
              radial(A.radial, F, (R)r, rc, f, fdum, false);
#pragma unroll
              for (int n = 0; n < kNPad; ++n) fs[slot * kNPad + n] = (double)f[n];
            }
          }
          StageVis v{ys, slot};
          sh_visit_part<LCAP, StageVis, false>((R)dx, (R)dy, (R)dz, (R)r, L, part, v);
        }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < kEPT; ++e) {
          const int idx = tid + e * kBlock;
          const int lmh = idx >> 4, n = idx & 15;
          if (lmh < Lh && n < F) {
            for (int jj = 0; jj < csz; ++jj) {
              const double fv = fs[jj * kNPad + n];
              const double2 y = ys[lmh * kChunk + jj];
              accr[e] = fma(fv, y.x, accr[e]);
              acci[e] = fma(-fv, y.y, acci[e]);
            }
          }
        }
        __syncthreads();
      }
#pragma unroll
      for (int e = 0; e < kEPT; ++e) {
        const int idx = tid + e * kBlock;
        const int lmh = idx >> 4;
        if (lmh < Lh) sa[(t * LS + lmh) * kNPad + (idx & 15)] = Rc{(R)accr[e], (R)acci[e]};
      }
    }
    MLIPG_STAMP(1)
    const int nl0 = __ldg(A.nl_off + ti), nNL = __ldg(A.nl_off + ti + 1) - nl0;
    double2* a64 = reinterpret_cast<double2*>(smem + lay.a64);
    // ---------------------------------------------------------------- P2b
    // Mixed path: the order parameters that the polynomial's input features
    // read (l up to the largest l among them), in FP64 from FP64 radial
    // functions and spherical harmonics.  In fitted potentials the
    // polynomial's terms are thousands of times larger than the energy they
    // sum to, so their inputs must carry FP64 accuracy; for model_type 3
    // these are the l = 0 entries alone.
    if constexpr (sizeof(R) == 4) {
      // (made in P2's windows when lh64 == 1 and P2 summed in FP32)
      const bool in_p2 = LCAP <= 16 && !A.sum64 && A.lh64 == 1;
      if (A.lh64 > 0 && nNL > 0 && !in_p2) {
        __syncthreads();   // the staging of P2 (same space) is no longer read
        order_params64(A, c, xi, misc, nbk, reinterpret_cast<double2*>(sg), a64);
      }
    }
    // ---------------------------------------------------------------- P3
    // The polynomial's input features and their whole energy: linear terms
    // w_f d_f and the polynomial terms of order >= 2, in FP64.  (The
    // invariant phase computes no energy for these features, so no large
    // FP32 partial sums cancel against FP64 ones.)
    double eacc = 0.0;
    const int n = lane & 15, half = lane >> 4;
    const bool act = n < F;
    if (nNL > 0) {
      __syncthreads();  // a[] (and a64) complete
      for (int u = warp; u < nNL; u += kBlock / 32) {
        const DeviceUnit un = A.nl_units[nl0 + u];
        double dd;
        if (sizeof(R) == 4 && A.lh64 > 0) {
          dd = nl_forward64(un, A.terms64, a64, A.lh64, n, half);
        } else {
          // (the double-float path's FP64 table is terms64)
          R dsum = R(0);
          GFixT<R> gnone{R(1), R(0)};
          dispatch_unit<R, false, LS>(un, kDF ? A.terms64 : A.terms, sa, sg, gim, gnone, n, half,
                                      act, R(0), dsum);
          dd = (double)dsum;
        }
        dd += __shfl_xor_sync(0xffffffffu, dd, 16);
        if (half == 0) dnl[u * kNPad + n] = act ? dd : 0.0;
      }
      __syncthreads();
      for (int e = tid; e < nNL * kNPad; e += kBlock) {
        const int itc = __ldg(&A.nl_units[nl0 + (e >> 4)].itc);
        eacc += __ldg(A.w_lin + (size_t)itc * kNPad + (e & 15)) * dnl[e];
      }
      const int p0 = __ldg(A.poly_off + ti), np = __ldg(A.poly_off + ti + 1) - p0;
#pragma unroll 4
      for (int pt = tid; pt < np; pt += kBlock) {
        const DevicePoly dp = A.poly[p0 + pt];
        double v[kMaxPoly];
        double prod = 1.0;
#pragma unroll
        for (int q = 0; q < kMaxPoly; ++q) {
          v[q] = q < dp.order ? dnl[dp.k[q]] : 1.0;
          prod *= v[q];
        }
        eacc += dp.w * prod;
      }
      // dE_poly/dd per nonlinear entry, gathered in a fixed order (no atomics,
      // so the energies that weigh products with H stay reproducible).  With
      // few entries each one's list is cut into S contiguous slices summed by
      // S threads (partials in the G space, free until the adjoint phase) and
      // the slices are added in slice order.
      const int ab = __ldg(A.adj_base + ti);
      const int ne = nNL * kNPad;
      const int S = ne >= kBlock ? 1 : kBlock / ne;
      double* part = reinterpret_cast<double*>(sg);
      for (int w = tid; w < ne * S; w += kBlock) {
        const int e = w % ne, sl = w / ne;
        const int x0 = __ldg(A.adj_off + ab + e), len = __ldg(A.adj_off + ab + e + 1) - x0;
        const int xs = x0 + (len * sl) / S, xe = x0 + (len * (sl + 1)) / S;
        double h = 0.0;
#pragma unroll 4
        for (int x = xs; x < xe; ++x) {
          const DeviceAdj a = A.adj[x];
          double o = a.w;
#pragma unroll
          for (int q2 = 0; q2 < kMaxPoly - 1; ++q2)
            if (a.other[q2] >= 0) o *= dnl[a.other[q2]];
          h += o;
        }
        if (S == 1) hnl[e] = h;
        else part[w] = h;
      }
      if (S > 1) {
        __syncthreads();
        for (int e = tid; e < ne; e += kBlock) {
          double h = 0.0;
          for (int sl = 0; sl < S; ++sl) h += part[sl * ne + e];
          hnl[e] = h;
        }
        __syncthreads();   // partials read before the adjoint phase clears G
      }
    }
    // ---------------------------------------------------------------- P4
    // the batched units add hnl to the FP32 weights of every tuple: the mixed
    // path reads an FP32 copy (in the space of dnl, which is no longer read)
    const P* hnlR = reinterpret_cast<const P*>(hnl);
    if constexpr (sizeof(R) == 4) {
      __syncthreads();   // every thread's reads of dnl are done
      float* hf = reinterpret_cast<float*>(dnl);
      for (int e = tid; e < nNL * kNPad; e += kBlock) hf[e] = (float)hnl[e];
      hnlR = reinterpret_cast<const P*>(hf);   // visible after the barrier below
    }
    if constexpr (kDF) {
      // double-float path: hnl and the order parameters split into (high,
      // low) FP32 pairs, the latter in place (16 bytes per complex entry
      // either way; each thread converts the entries it reads)
      __syncthreads();   // every thread's reads of dnl and of a (P3) are done
      DF* hd = reinterpret_cast<DF*>(dnl);
      for (int e = tid; e < nNL * kNPad; e += kBlock) hd[e] = df_from_double(hnl[e]);
      hnlR = reinterpret_cast<const P*>(hd);
      for (int e = tid; e < T * LS * kNPad; e += kBlock) {
        const double2 v = reinterpret_cast<const double2*>(sa)[e];
        reinterpret_cast<DFc*>(sa)[e] = DFc{df_from_double(v.x), df_from_double(v.y)};
      }
    }
    const Pc* sp = reinterpret_cast<const Pc*>(sa);
    PG* sgp = reinterpret_cast<PG*>(sg);
    MLIPG_STAMP(2)
    // ---------------------------------------------------------------- P5
    // (mixed path: redone once at the measured scale if a flush left the
    // fixed-point range; the energy of the failed attempt is discarded)
    const double eacc0 = eacc;
    int gexp = 0;
    for (int attempt = 0;; ++attempt) {
    for (int e = tid; e < kGWords * gim; e += kBlock) reinterpret_cast<int*>(sg)[e] = 0;
    gexp = misc[16 + ti];
    if (tid == 0) {
      misc[12] = 0;
      misc[13] = 0;   // unit counter
      reinterpret_cast<unsigned long long*>(misc + 24)[0] = 0ull;   // unit energies
      reinterpret_cast<unsigned long long*>(misc + 24)[1] = 0ull;
    }
    __syncthreads();   // G zeroed; everyone has read this attempt's scale
    GFixT<P> gf;
    if constexpr (kFixG) gf = GFixT<P>{ldexpf(1.0f, gexp), 0.0f};
    else gf = GFixT<P>{P(1), P(0)};
    ESumF esum;   // mixed path: this thread's energy of the statically dealt units
    {
      const int u0 = __ldg(A.unit_off + ti), nU = __ldg(A.unit_off + ti + 1) - u0;
      const int i0 = __ldg(A.iunit_off + ti), nI = __ldg(A.iunit_off + ti + 1) - i0;
      // warp orders 0 and 1 deal the units to the warps statically (each
      // thread's energy sum has a fixed order, so energies are reproducible);
      // order 2 hands them out from a shared counter (below)
      const P* wl = wlin_table(A);
      const auto run_iu = [&](const DeviceIrrUnit& iu, auto& e) {
        if (T == 3)
          dispatch_irr<P, 3, LS>(iu, A.tuples, A.terms, wl, hnlR, sp, sgp, gim, gf, n, half, act, e);
        else if (T == 2)
          dispatch_irr<P, 2, LS>(iu, A.tuples, A.terms, wl, hnlR, sp, sgp, gim, gf, n, half, act, e);
        else
          dispatch_irr<P, 1, LS>(iu, A.tuples, A.terms, wl, hnlR, sp, sgp, gim, gf, n, half, act, e);
      };
      if (A.unit_dyn) {
        // warps take units from a shared counter (no end-of-phase imbalance);
        // each unit's energy is split exactly into 2^-20 eV and 2^-60 eV
        // integer parts and added to two 64-bit sums, so the total does not
        // depend on which warp ran which unit
        unsigned long long* efix = reinterpret_cast<unsigned long long*>(misc + 24);
        // the next unit is taken before the current one runs, and its
        // descriptor copied asynchronously (cp.async, no registers held) into
        // this warp's slot of the block-reduction space, unused until the end
        // of the centre
        DeviceIrrUnit* slot = reinterpret_cast<DeviceIrrUnit*>(red) + 2 * warp;
        const auto take = [&]() {
          int v = 0;
          if (lane == 0) v = atomicAdd(misc + 13, 1);
          return __shfl_sync(0xffffffffu, v, 0);
        };
        const auto fetch = [&](int v) {
          if (lane == 0 && v < nI) {
            const unsigned sa_ = (unsigned)__cvta_generic_to_shared(slot);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n\tcp.async.commit_group;" ::"r"(sa_),
                         "l"(A.iunits + i0 + v) : "memory");
          }
        };
        int u = take();
        fetch(u);
        while (u < nI) {
          if (lane == 0) asm volatile("cp.async.wait_all;" ::: "memory");
          __syncwarp();
          const DeviceIrrUnit cur = *slot;
          __syncwarp();   // every lane has read the slot before it is refilled
          const int un = take();
          fetch(un);
          EU eu{};
          run_iu(cur, eu);
          const double e = warp_energy(eu);
          // units of the polynomial's input features: energy taken in P3
          if (lane == 0 && !cur.nl) {
            const double sc = e * 0x1p20, hi = rint(sc);
            atomicAdd(efix, (unsigned long long)(long long)hi);
            atomicAdd(efix + 1, (unsigned long long)__double2ll_rn((sc - hi) * 0x1p40));
          }
          u = un;
        }
      } else {
        for (int u = warp; u < nI; u += kBlock / 32) {
          const DeviceIrrUnit iu = A.iunits[i0 + u];
          if (iu.nterm == 0) continue;   // padding of a balanced schedule
          EU eu{};
          run_iu(iu, eu);
          // units of the polynomial's input features: energy taken in P3
          if (!iu.nl) merge_unit_energy(esum, eacc, eu);
        }
      }
      MLIPG_STAMP(3)   // warp 0's batched units (the warps' shares are balanced)
      for (int u = warp; u < nU; u += kBlock / 32) {
        const DeviceUnit un = A.units[u0 + u];
        if (un.nterm == 0) continue;
        double hv = 0.0;
        if (act) {
          hv = __ldg(A.w_lin + (size_t)un.itc * kNPad + n);
          if (un.nl_slot >= 0) hv += hnl[un.nl_slot * kNPad + n];
        }
        P dsum = P(0);
        dispatch_unit<P, true, LS>(un, A.terms, sp, sgp, gim, gf, n, half, act, to_p(hv), dsum);
        const double ds = half_pair_sum(dsum);
        if (half == 0 && act && un.nl_slot < 0) eacc += hv * ds;
      }
    }
    if constexpr (!kFixG) {
      __syncthreads();
      if (A.unit_dyn && tid == 0)
        eacc += unit_energy(misc);
      break;
    }
    {
      // largest |scaled flush| of the CTA
      float vm = (float)gf.vmax;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) vm = fmaxf(vm, __shfl_xor_sync(0xffffffffu, vm, o));
      if (lane == 0) atomicMax(misc + 12, __float_as_int(vm));
    }
    __syncthreads();
    const float vm = __int_as_float(misc[12]);
    const bool out = !(vm < A.g_bound);   // also true for NaN
    // a scale that leaves more than 6 bits of the range unused is redone too
    const bool coarse = vm > 0.0f && vm < A.g_bound * (1.0f / 64.0f);
    if (tid == 0 && vm > 0.0f && vm < 3.0e38f) {
      // next scale: the largest flush at half the bound
      int lv = ilogbf(vm);
      if (vm > ldexpf(1.0f, lv)) ++lv;
      // (capped so that a coefficient times the scale stays finite)
      misc[16 + ti] = max(-120, min(100, gexp + ilogbf(A.g_bound) - 1 - lv));
    }
    if ((!out && !coarse) || attempt >= 2) {
      if (out && tid == 0) atomicOr(A.status, kStatusAdjointRange);
      if (A.unit_dyn && tid == 0)
        eacc += unit_energy(misc);
      eacc += (double)esum.s + (double)esum.c;
      break;
    }
    eacc = eacc0;
    __syncthreads();   // misc[12] read by all before the next attempt resets it
    }
    if (sizeof(R) == 4) {
      // fixed point -> float, in place
      __syncthreads();
      const float inv = ldexpf(1.0f, -gexp);
      const int* gi = reinterpret_cast<const int*>(sg);
      for (int e = tid; e < 2 * gim; e += kBlock)
        sg[e] = (R)(fmaf((float)gi[e], 65536.0f, (float)gi[e + 2 * gim]) * inv);
      __syncthreads();
    }
    // double-float path: the four words -> FP64 adjoint in the space of a
    // (not read again for this centre)
    R* gP6 = sg;
    if constexpr (kDF) {
      __syncthreads();
      const double inv = ldexp(1.0, -gexp);
      const int* gw = reinterpret_cast<const int*>(sg);
      double* gd = reinterpret_cast<double*>(sa);
      for (int e = tid; e < 2 * gim; e += kBlock) {
        const double lo2 = (double)gw[e + 4 * gim] * 65536.0 + (double)gw[e + 6 * gim];  // exact
        gd[e] = fma((double)gw[e], 0x1p48, fma((double)gw[e + 2 * gim], 0x1p32, lo2)) * inv;
      }
      gP6 = reinterpret_cast<R*>(gd);
      __syncthreads();
    }
    MLIPG_STAMP(4)
    // ---------------------------------------------------------------- P6
    double fix = 0.0, fiy = 0.0, fiz = 0.0;
    double va[6] = {0, 0, 0, 0, 0, 0};   // this centre's virial (reference order)
    if constexpr (sizeof(R) == 8) {
      // FP64 kernels: 32 neighbours per warp; the four warps of a group
      // split the m columns of the harmonics (each Y_lm and dY_lm computed
      // once, all 16 channels contracted per entry); the four partial forces
      // of a neighbour meet in shared memory (the space of a, at least 7 KB,
      // or of the adjoint words in the double-float kernel: neither is read
      // again for this centre) and are added in a fixed order.  (The FP32
      // form of this split measured 6.6 % slower on the mixed kernel: its
      // 16 channels do not fit the register budget of two CTAs per SM.)
      double* pf = reinterpret_cast<double*>(kDF ? static_cast<void*>(sg) : static_cast<void*>(sa));
      const int part = warp & 3, grp = warp >> 2;
      const int rounds = (nkeep + 2 * 32 - 1) / (2 * 32);
      for (int it = 0; it < rounds; ++it) {
        const int jj = it * 64 + grp * 32 + lane;
        const bool valid = jj < nkeep;
        const int k = valid ? nbk[jj] : nbk[0];
        const int j = __ldg(A.nbr_idx + k);
        const double4 xj = A.x4[j];
        const int tj = valid ? (int)xj.w : 0;
        double dx, dy, dz;
        pair_disp(A, c, k, xi, xj, dx, dy, dz);
        if (!valid) { dx = 1.0; dy = 0.0; dz = 0.0; }
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        double f[kNPad], fd[kNPad];
        radial64d(A, r, f, fd);
        const double ir = 1.0 / r;
        ForceVis16 v{gP6 + (size_t)tj * LS * kNPad, gim, f, fd, (R)(dx * ir), (R)(dy * ir),
                     (R)(dz * ir), R(0), R(0), R(0)};
        sh_visit_part<LCAP>((R)dx, (R)dy, (R)dz, (R)r, L, part, v);
        double* q = pf + ((grp * 32 + lane) * 4 + part) * 3;
        q[0] = (double)v.fx;
        q[1] = (double)v.fy;
        q[2] = (double)v.fz;
        __syncthreads();
        if (part == 0 && valid) {
          const double* q0 = pf + (grp * 32 + lane) * 12;
          const double fx = (q0[0] + q0[3]) + (q0[6] + q0[9]);
          const double fy = (q0[1] + q0[4]) + (q0[7] + q0[10]);
          const double fz = (q0[2] + q0[5]) + (q0[8] + q0[11]);
          fix += fx; fiy += fy; fiz += fz;
          const int fj = A.fold ? __ldg(A.fold + j) : j;
          atomicAdd(A.f + 3 * (size_t)fj, -fx);
          atomicAdd(A.f + 3 * (size_t)fj + 1, -fy);
          atomicAdd(A.f + 3 * (size_t)fj + 2, -fz);
          // reference component order: xx yy zz yz zx xy
          va[0] -= dx * fx; va[1] -= dy * fy; va[2] -= dz * fz;
          va[3] -= dy * fz; va[4] -= dz * fx; va[5] -= dx * fy;
        }
        __syncthreads();
      }
    } else {
      // 4 threads per neighbour; thread `sub` owns radial channels 4*sub..4*sub+3
      const int sub = tid & 3, n0 = 4 * sub;
      const int rounds = (nkeep + kBlock / 4 - 1) / (kBlock / 4);
      for (int it = 0; it < rounds; ++it) {
        const int jj = it * (kBlock / 4) + (tid >> 2);
        const bool valid = jj < nkeep;
        const int k = valid ? nbk[jj] : nbk[0];
        const int j = __ldg(A.nbr_idx + k);
        const double4 xj = A.x4[j];
        const int tj = valid ? (int)xj.w : 0;
        double dx, dy, dz;
        pair_disp(A, c, k, xi, xj, dx, dy, dz);
        if (!valid) { dx = 1.0; dy = 0.0; dz = 0.0; }
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        R f[4], fd[4];
        radial4(A.radial, F, n0, (R)r, rc, f, fd);
        const double ir = 1.0 / r;
        ForceVis v{gP6 + (size_t)tj * LS * kNPad + n0, gim, f, fd, (R)(dx * ir), (R)(dy * ir),
                   (R)(dz * ir), R(0), R(0), R(0)};
        sh_visit<LCAP, true>((R)dx, (R)dy, (R)dz, (R)r, L, v);
        double fx = v.fx, fy = v.fy, fz = v.fz;
        fx += __shfl_xor_sync(0xffffffffu, fx, 1);
        fy += __shfl_xor_sync(0xffffffffu, fy, 1);
        fz += __shfl_xor_sync(0xffffffffu, fz, 1);
        fx += __shfl_xor_sync(0xffffffffu, fx, 2);
        fy += __shfl_xor_sync(0xffffffffu, fy, 2);
        fz += __shfl_xor_sync(0xffffffffu, fz, 2);
        if (valid && sub == 0) {
          fix += fx; fiy += fy; fiz += fz;
          const int fj = A.fold ? __ldg(A.fold + j) : j;
          atomicAdd(A.f + 3 * (size_t)fj, -fx);
          atomicAdd(A.f + 3 * (size_t)fj + 1, -fy);
          atomicAdd(A.f + 3 * (size_t)fj + 2, -fz);
          // reference component order: xx yy zz yz zx xy
          va[0] -= dx * fx; va[1] -= dy * fy; va[2] -= dz * fz;
          va[3] -= dy * fz; va[4] -= dz * fx; va[5] -= dx * fy;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) vir[q] += va[q];
    // block reduction of the centre's energy, force and virial
    {
      double v10[10] = {eacc, fix, fiy, fiz, va[0], va[1], va[2], va[3], va[4], va[5]};
#pragma unroll
      for (int q = 0; q < 10; ++q) v10[q] = warp_sum(v10[q]);
      if (lane == 0)
        for (int q = 0; q < 10; ++q) red[warp * 16 + q] = v10[q];
    }
    __syncthreads();
    if (tid < 6 && A.vatom) {
      double v = 0;
      for (int w = 0; w < kBlock / 32; ++w) v += red[w * 16 + 4 + tid];
      // reference order xx yy zz yz zx xy -> LAMMPS xx yy zz xy xz yz
      const int dst = tid < 3 ? tid : (tid == 3 ? 5 : (tid == 4 ? 4 : 3));
      A.vatom[(size_t)c * 6 + dst] = v;
    }
    if (tid == 0) {
      double e = 0, gx = 0, gy = 0, gz = 0;
      for (int w = 0; w < kBlock / 32; ++w) {
        e += red[w * 16]; gx += red[w * 16 + 1]; gy += red[w * 16 + 2]; gz += red[w * 16 + 3];
      }
      if (A.eatom) A.eatom[c] = e;
      ecta += e;
      const int fi = A.fold ? __ldg(A.fold + i) : i;
      atomicAdd(A.f + 3 * (size_t)fi, gx);
      atomicAdd(A.f + 3 * (size_t)fi + 1, gy);
      atomicAdd(A.f + 3 * (size_t)fi + 2, gz);
    }
    __syncthreads();
    MLIPG_STAMP(5)
  }
#undef MLIPG_STAMP
  if (prof && tid == 0)
    for (int k = 0; k < 6; ++k) atomicAdd(A.phase_clocks + k, ph[k]);
  // CTA 0 leaves its adapted exponents for the next launch (any recent value
  // is a good start; the cache only saves redone centres)
  if (kFixG && blockIdx.x == 0 && tid < T && A.gexp_cache) A.gexp_cache[tid] = misc[16 + tid];
  // per-CTA partial sums: energy + virial (reference order)
  double vals[7] = {ecta, vir[0], vir[1], vir[2], vir[3], vir[4], vir[5]};
#pragma unroll
  for (int q = 0; q < 7; ++q) vals[q] = warp_sum(vals[q]);
  __syncthreads();
  if (lane == 0)
    for (int q = 0; q < 7; ++q) red[warp * 16 + q] = vals[q];
  __syncthreads();
  if (tid < 8) {
    double s = 0;
    if (tid < 7)
      for (int w = 0; w < kBlock / 32; ++w) s += red[w * 16 + tid];
    A.partials[(size_t)blockIdx.x * 8 + tid] = s;   // slot 7 zero (finalize writes the status there)
  }
}

size_t smem_bytes(int T, int L, int nb_cap, int nl_cap, int lh64) {
  const int lcap = L <= 6 ? 6 : (L <= 12 ? 12 : (L <= 16 ? 16 : 20));   // launch()'s pick
  return smem_layout(T, (lcap + 1) * (lcap + 2) / 2, nb_cap, nl_cap, sizeof(R) == 4 ? lh64 : 0)
      .total;
}

template <int LCAP>
static cudaError_t prepare(size_t smem) {
  return cudaFuncSetAttribute(fused_kernel<LCAP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem);
}

template <int LCAP>
static int occupancy(size_t smem) {
  if (prepare<LCAP>(smem) != cudaSuccess) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fused_kernel<LCAP>, kBlock, smem) !=
      cudaSuccess)
    return 0;
  return nb;
}

int max_blocks(int L, size_t smem) {
  if (L <= 6) return occupancy<6>(smem);
  if (L <= 12) return occupancy<12>(smem);
  if (L <= 16) return occupancy<16>(smem);
  return occupancy<20>(smem);
}

cudaError_t launch(int L, const KernelArgs& a, int grid, size_t smem, cudaStream_t s) {
  cudaError_t e;
  if (L <= 6) {
    if ((e = prepare<6>(smem)) != cudaSuccess) return e;
    fused_kernel<6><<<grid, kBlock, smem, s>>>(a);
  } else if (L <= 12) {
    if ((e = prepare<12>(smem)) != cudaSuccess) return e;
    fused_kernel<12><<<grid, kBlock, smem, s>>>(a);
  } else if (L <= 16) {
    if ((e = prepare<16>(smem)) != cudaSuccess) return e;
    fused_kernel<16><<<grid, kBlock, smem, s>>>(a);
  } else {
    if ((e = prepare<20>(smem)) != cudaSuccess) return e;
    fused_kernel<20><<<grid, kBlock, smem, s>>>(a);
  }
  return cudaGetLastError();
}

#endif  // MLIPG_NO_FUSED

cudaError_t init_constants() {
  R A[kLhMax] = {}, B[kLhMax] = {}, LM[kLhMax] = {}, dg[kMaxL + 2] = {}, of[kMaxL + 2] = {},
    ll[kMaxL + 1] = {};
  for (int l = 2; l <= kMaxL; ++l) {
    const double ls = l * l, lm1s = (l - 1) * (l - 1);
    for (int m = 0; m <= l - 2; ++m) {
      const double ms = m * m;
      A[l * (l + 1) / 2 + m] = (R)std::sqrt((4.0 * ls - 1.0) / (ls - ms));
      B[l * (l + 1) / 2 + m] = (R)(-std::sqrt((lm1s - ms) / (4.0 * lm1s - 1.0)));
    }
  }
  for (int l = 0; l <= kMaxL; ++l)
    for (int m = 0; m <= l; ++m) LM[l * (l + 1) / 2 + m] = (R)std::sqrt((double)(l - m) * (l + m + 1));
  for (int m = 1; m <= kMaxL + 1; ++m) dg[m] = (R)(-std::sqrt(1.0 + 0.5 / m));
  for (int m = 0; m <= kMaxL + 1; ++m) of[m] = (R)std::sqrt(2.0 * m + 3.0);
  // the m = 0 derivative factor sqrt(l (l+1)) h; the FP32 instantiation's
  // harmonics are normalised by Y_00 and carry no factor h = 1/sqrt(2)
  for (int l = 0; l <= kMaxL; ++l)
    ll[l] = (R)std::sqrt((sizeof(R) == 4 ? 1.0 : 0.5) * l * (l + 1));
  double A64[kLhMax] = {}, B64[kLhMax] = {}, dg64[kMaxL + 2] = {}, of64[kMaxL + 2] = {};
  for (int l = 2; l <= kMaxL; ++l) {
    const double ls = l * l, lm1s = (l - 1) * (l - 1);
    for (int m = 0; m <= l - 2; ++m) {
      const double ms = m * m;
      A64[l * (l + 1) / 2 + m] = std::sqrt((4.0 * ls - 1.0) / (ls - ms));
      B64[l * (l + 1) / 2 + m] = -std::sqrt((lm1s - ms) / (4.0 * lm1s - 1.0));
    }
  }
  for (int m = 1; m <= kMaxL + 1; ++m) dg64[m] = -std::sqrt(1.0 + 0.5 / m);
  for (int m = 0; m <= kMaxL + 1; ++m) of64[m] = std::sqrt(2.0 * m + 3.0);
  cudaError_t e;
  if ((e = cudaMemcpyToSymbol(cA64, A64, sizeof A64)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(cB64, B64, sizeof B64)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(cDiag64, dg64, sizeof dg64)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(cOff64, of64, sizeof of64)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(cA, A, sizeof A)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(cB, B, sizeof B)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(cLM, LM, sizeof LM)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(cDiag, dg, sizeof dg)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(cOff, of, sizeof of)) != cudaSuccess) return e;
  return cudaMemcpyToSymbol(cLL, ll, sizeof ll);
}

}  // namespace MLIPG_TAG
}  // namespace mlipg
