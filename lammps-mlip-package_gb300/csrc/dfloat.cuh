// Double-float arithmetic: a value is the unevaluated sum h + l of two FP32
// numbers with |l| <= ulp(h) / 2, which carries 48 significant bits on the
// FP32 pipe (GB300 issues FP32 FMAs 64 times faster than FP64 ones).
//
// The operations are the classical error-free transformations, written with
// explicit round-to-nearest intrinsics so that the compiler neither
// contracts a product into a following addition nor reassociates:
//   TwoSum (Knuth, TAOCP vol. 2, 4.2.2): s = a + b, e = exact rounding error;
//   TwoProd by FMA: p = a * b, e = fma(a, b, -p) exactly;
//   addition and multiplication as in Dekker (1971) / Hida, Li and Bailey's
//   double-double "sloppy" forms, with one final Fast2Sum renormalisation.
// Relative error per operation is a few units of 2^-47 of the operands.
// The exponent range is FP32's: contributions below ~1e-38 flush to zero,
// which is far below every quantity the kernels accumulate.
#pragma once

#include <cuda_runtime.h>

namespace mlipg {

struct DF {
  float h, l;
  DF() = default;
  __host__ __device__ constexpr explicit DF(float x) : h(x), l(0.0f) {}
  __host__ __device__ constexpr DF(float hi, float lo) : h(hi), l(lo) {}
};

// complex double-float, 16 bytes: (Re h, Re l, Im h, Im l)
struct __align__(16) DFc {
  DF x, y;
};

__device__ __forceinline__ DF df_renorm(float s, float t) {
  const float h = __fadd_rn(s, t);
  return DF(h, __fsub_rn(t, __fsub_rn(h, s)));
}

__device__ __forceinline__ DF operator+(DF a, DF b) {
  const float s = __fadd_rn(a.h, b.h);
  const float v = __fsub_rn(s, a.h);
  const float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, v)), __fsub_rn(b.h, v));
  return df_renorm(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ DF operator-(DF a) { return DF(-a.h, -a.l); }
__device__ __forceinline__ DF operator-(DF a, DF b) { return a + (-b); }

__device__ __forceinline__ DF operator*(DF a, DF b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return df_renorm(p, e);
}

// a * b + c with one renormalisation
__device__ __forceinline__ DF vfma(DF a, DF b, DF c) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  const float s = __fadd_rn(p, c.h);
  const float v = __fsub_rn(s, p);
  const float t = __fadd_rn(__fsub_rn(p, __fsub_rn(s, v)), __fsub_rn(c.h, v));
  return df_renorm(s, __fadd_rn(t, __fadd_rn(e, c.l)));
}
__device__ __forceinline__ float vfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double vfma(double a, double b, double c) { return fma(a, b, c); }

__device__ __forceinline__ DF& operator+=(DF& a, DF b) { return a = a + b; }
__device__ __forceinline__ DF& operator-=(DF& a, DF b) { return a = a - b; }

// exact scaling by a power of two (no overflow or underflow in use)
__device__ __forceinline__ DF df_scale(DF a, float s) { return DF(a.h * s, a.l * s); }

// Accumulator of double-float products: the unevaluated sum s + c, s the
// rounded running sum of the products' high parts, c the exact rounding
// error of every addition to s (TwoSum) plus the products' low parts
// (TwoProd and the cross terms).  Only s carries a dependency from one
// accumulation to the next (one FP32 add), and a single renormalisation
// gives the value; the error is a few 2^-47 of the sum of |products|.
struct DFA {
  float s = 0.0f, c = 0.0f;
};
__device__ __forceinline__ void acc_fma(DFA& a, DF x, DF y) {
  const float p = __fmul_rn(x.h, y.h);
  float e = __fmaf_rn(x.h, y.h, -p);
  e = __fmaf_rn(x.h, y.l, e);
  e = __fmaf_rn(x.l, y.h, e);
  const float t = __fadd_rn(a.s, p);
  const float v = __fsub_rn(t, a.s);
  const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, v)), __fsub_rn(p, v));
  a.c = __fadd_rn(a.c, __fadd_rn(err, e));
  a.s = t;
}
__device__ __forceinline__ void acc_add(DFA& a, DF x) {
  const float t = __fadd_rn(a.s, x.h);
  const float v = __fsub_rn(t, a.s);
  const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, v)), __fsub_rn(x.h, v));
  a.c = __fadd_rn(a.c, __fadd_rn(err, x.l));
  a.s = t;
}
__device__ __forceinline__ DF acc_val(const DFA& a) { return df_renorm(a.s, a.c); }
// (re, im) += (ar + i ai) (br + i bi)
__device__ __forceinline__ void cacc(DFA& re, DFA& im, DF ar, DF ai, DF br, DF bi) {
  acc_fma(re, ar, br);
  acc_fma(re, -ai, bi);
  acc_fma(im, ar, bi);
  acc_fma(im, ai, br);
}

__device__ __forceinline__ DF df_from_double(double v) {
  const float h = __double2float_rn(v);
  return DF(h, __double2float_rn(v - (double)h));
}
__device__ __forceinline__ double df_to_double(DF a) { return (double)a.h + (double)a.l; }

}  // namespace mlipg
