// Double-float ("float-float") arithmetic: a value is the unevaluated sum hi + lo of two floats
// with |lo| <= ulp(hi) / 2, about 48 significant bits (unit roundoff ~ 2^-47).  GB300 issues FP32
// at 64 times its FP64 rate, so a double-float multiply-add (about 14 FP32 instructions) costs a
// quarter of the FP64 pipe time of one DFMA; the mixed-precision solver uses it for the Schur
// factor and its triangular solves, where FP32 alone is far too inaccurate for the condition of S.
//
// Algorithms (published, restated here): Knuth's TwoSum and Dekker's Fast2Sum for exact sums,
// the FMA form of Dekker's TwoProduct for exact products (Dekker 1971, "A floating-point technique
// for extending the available precision"); the pair operations follow the "sloppy" double-double
// add and the standard product of Hida, Li and Bailey's double-double arithmetic.  Every elementary
// step uses the _rn intrinsics so that the compiler cannot contract or reassociate it.
#pragma once
#include <cuda_runtime.h>

#include "vh_common.cuh"

namespace vh {

using ::fma;   // keep the FP64 / FP32 overloads visible next to the pair overload below

// float -> double, exact, with integer operations: sign, exponent rebiased by 1023 - 127 and the
// 23 fraction bits moved to the top of the 52 (GB300 runs the conversion instruction on its slow
// FP64 pipe).  Zero, subnormal, infinite and NaN floats take the conversion instruction.
__host__ __device__ __forceinline__ double f2d_exact(float f) {
#ifdef __CUDA_ARCH__
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFFu;
  if (e - 1u < 254u) {
    const unsigned hw = (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7FFFFFu) >> 3);
    return __hiloint2double((int)hw, (int)((u & 7u) << 29));
  }
#endif
  return (double)f;
}

struct dfloat {
  float hi, lo;
  dfloat() = default;
  __host__ __device__ constexpr dfloat(float h) : hi(h), lo(0.0f) {}
  __host__ __device__ constexpr dfloat(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr dfloat(int v) : hi((float)v), lo(0.0f) {}
  // nearest pair to a double: hi = rn(d), lo = rn(d - hi) (d - hi is exact in double)
  __host__ __device__ explicit dfloat(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ double to_double() const { return f2d_exact(hi) + f2d_exact(lo); }
};

struct dcomplex {
  dfloat x, y;
};
template <> struct cplx_t<dfloat> { using type = dcomplex; };

__device__ __forceinline__ dcomplex to_c(double2 a, dcomplex) { return dcomplex{dfloat(a.x), dfloat(a.y)}; }
__device__ __forceinline__ dcomplex to_c(dcomplex a, dcomplex) { return a; }
__host__ __device__ __forceinline__ dcomplex mk(dfloat a, dfloat b) { return dcomplex{a, b}; }
__device__ __forceinline__ double2 to_d(dcomplex a) { return make_double2(a.x.to_double(), a.y.to_double()); }

// s + e = a + b exactly (Knuth)
__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// s + e = a + b exactly when |a| >= |b| or a == 0 (Dekker)
__device__ __forceinline__ void df_fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) {
  float s, e;
  df_two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  dfloat r;
  df_fast_two_sum(s, e, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ dfloat operator-(dfloat a) { return dfloat(-a.hi, -a.lo); }
__device__ __forceinline__ dfloat operator-(dfloat a, dfloat b) { return a + (-b); }
__device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);                       // exact error of a.hi * b.hi
  e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
  dfloat r;
  df_fast_two_sum(p, e, r.hi, r.lo);
  return r;
}
// a * b + c with one rounding to the pair format
__device__ __forceinline__ dfloat fma(dfloat a, dfloat b, dfloat c) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
  float s, t;
  df_two_sum(p, c.hi, s, t);
  t = __fadd_rn(t, __fadd_rn(e, c.lo));
  dfloat r;
  df_fast_two_sum(s, t, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ dfloat& operator+=(dfloat& a, dfloat b) { return a = a + b; }
__device__ __forceinline__ dfloat& operator-=(dfloat& a, dfloat b) { return a = a - b; }
__device__ __forceinline__ dfloat& operator*=(dfloat& a, dfloat b) { return a = a * b; }
__device__ __forceinline__ bool operator>(dfloat a, dfloat b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }

// Running dot product in pair precision with one normalisation at the end: Dot2 of Ogita, Rump
// and Oishi ("Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005), extended to pair
// operands by adding the cross terms hi*lo + lo*hi to each product's exact error.  `s` holds the
// rounded running sum and `c` the sum of every product and addition error, so the loop-carried
// dependency is a single addition per term (a pair fma carries about nine dependent operations).
struct df_dot {
  float s, c;
  df_dot() = default;   // uninitialised (arrays of accumulators set before use)
  __device__ __forceinline__ explicit df_dot(dfloat init) : s(init.hi), c(init.lo) {}
  // += a * b
  __device__ __forceinline__ void add(dfloat a, dfloat b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
    float s2, q;
    df_two_sum(s, p, s2, q);
    s = s2;
    c = __fadd_rn(c, __fadd_rn(q, e));
  }
  __device__ __forceinline__ dfloat value() const {
    dfloat r;
    df_two_sum(s, c, r.hi, r.lo);   // |c| may exceed |s| after cancellation
    df_fast_two_sum(r.hi, r.lo, r.hi, r.lo);
    return r;
  }
  // adds another partial dot product (the same accumulation rule: exact sum of the rounded parts)
  __device__ __forceinline__ void merge(float os, float oc) {
    float s2, q;
    df_two_sum(s, os, s2, q);
    s = s2;
    c = __fadd_rn(c, __fadd_rn(q, oc));
  }
  // sum over the 32 lanes of a warp (butterfly: every lane ends with the total)
  __device__ __forceinline__ void warp_sum() {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) merge(__shfl_xor_sync(0xffffffffu, s, o), __shfl_xor_sync(0xffffffffu, c, o));
  }
};

// The same interface over FP64 (plain fused multiply-adds), for templates over the factor type.
struct d_dot {
  double s;
  __device__ __forceinline__ explicit d_dot(double init) : s(init) {}
  __device__ __forceinline__ void add(double a, double b) { s = fma(a, b, s); }
  __device__ __forceinline__ double value() const { return s; }
  __device__ __forceinline__ void warp_sum() {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  }
};
template <typename T> struct dot_of;
template <> struct dot_of<double> { using type = d_dot; };
template <> struct dot_of<dfloat> { using type = df_dot; };

// double -> pair on the integer and FP32 pipes (GB300's FP64 pipe, which the conversion
// instructions use, runs at 1/64 of the FP32 rate).  hi takes the sign, the exponent and the top 23
// fraction bits of d (truncated); lo the remaining 29 fraction bits, rounded to a float.  hi + lo
// equals d to within 2^-47 |d| and |lo| < ulp(hi).  Zero (and FP64 subnormals) give zero; magnitudes
// outside [2^-74, 2^127) -- where lo would leave the normal float range or hi overflow -- take the
// conversion instructions.
__device__ __forceinline__ dfloat df_split(double d) {
  const unsigned hw = (unsigned)__double2hiint(d), lw = (unsigned)__double2loint(d);
  const unsigned e = (hw >> 20) & 0x7FFu;   // biased binary64 exponent
  if (e - 949u <= 1150u - 949u) {
    const unsigned s = hw & 0x80000000u;
    dfloat r;
    r.hi = __uint_as_float(s | ((e - 896u) << 23) | ((hw & 0xFFFFFu) << 3) | (lw >> 29));
    // the remainder's weight is 2^(e - 1075); e >= 949 keeps that power of two a normal float
    const float rem = __uint2float_rn(lw & 0x1FFFFFFFu) * __uint_as_float((e - 948u) << 23);
    r.lo = __uint_as_float(__float_as_uint(rem) | s);
    return r;
  }
  if (e == 0) return dfloat(0.0f);
  return dfloat(d);
}

// 1 / b: single-precision seed, then two Newton steps y <- y + y (1 - b y), each in pair arithmetic
__device__ __forceinline__ dfloat df_recip(dfloat b) {
  dfloat y(__frcp_rn(b.hi));
  const dfloat one(1.0f);
  for (int it = 0; it < 2; ++it) y = fma(y, one - b * y, y);
  return y;
}
__device__ __forceinline__ dfloat operator/(dfloat a, dfloat b) { return a * df_recip(b); }

// 1 / sqrt(p): single-precision seed, then two Newton steps y <- y + y (1 - p y^2) / 2
__device__ __forceinline__ dfloat df_rsqrt(dfloat p) {
  dfloat y(rsqrtf(p.hi));
  const dfloat one(1.0f), half(0.5f);
  for (int it = 0; it < 2; ++it) y = fma(y * half, one - p * y * y, y);
  return y;
}

}  // namespace vh
