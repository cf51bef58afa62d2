// Double-float ("float-float") arithmetic on the FP32 pipe.
//
// A df64 value is the unevaluated sum hi + lo of two floats with |lo| <=
// ulp(hi)/2, giving a ~48-bit significand with float's exponent range.  The
// error-free transformations are Knuth's TwoSum, Dekker's Fast2Sum and the
// FMA-based TwoProduct; the arithmetic follows the classic double-single
// algorithms (Dekker 1971; Hida, Li and Bailey, "Library for double-double
// and quad-double arithmetic", 2001), restated for float pairs.
//
// On GB300 an FP64 instruction issues at 1/64 of the FP32 rate, so the
// mixed path carries its high-precision quantities (positions, the stretch
// variable s, the residual chain, dot products) in df64 and touches native
// FP64 only once per warp or tile.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace mfem_gpu {

struct df64 {
  float hi, lo;
  __host__ __device__ df64() : hi(0.f), lo(0.f) {}
  __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ df64(float f) : hi(f), lo(0.f) {}
  __host__ __device__ df64(int i) : hi(float(i)), lo(0.f) {}
  // From double: exact for the constants the templates use (folded at
  // compile time); at run time it costs three FP64 instructions.
  __host__ __device__ explicit df64(double d) : hi(float(d)), lo(float(d - double(float(d)))) {}
  __host__ __device__ double to_double() const { return double(hi) + double(lo); }
};

__device__ __forceinline__ df64 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v));
  return df64(s, e);
}
__device__ __forceinline__ df64 fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  const float e = __fsub_rn(b, __fsub_rn(s, a));
  return df64(s, e);
}
__device__ __forceinline__ df64 two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  const float e = __fmaf_rn(a, b, -p);
  return df64(p, e);
}

// Addition: one TwoSum of the high parts with the low parts folded into
// its error term, then renormalised (Dekker's add2; the "sloppy" addition
// of Hida, Li and Bailey).  Its error is below about 2^-47 (|a| + |b|):
// relative to the operands, not to the result, which is as much as either
// operand's own representation error allows anyway -- the residual chains
// and dot products this type carries are bounded that way (S - s, b - A x,
// sums of products).  11 FP32 instructions instead of the 20 of the
// two-TwoSum form that is accurate relative to the result.
__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  const df64 s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  df64 p = two_prod(a.hi, b.hi);
  p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
  p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df64 operator/(df64 a, df64 b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const df64 r = a - b * df64(q1);
  const float q2 = __fdiv_rn(r.hi, b.hi);
  const df64 r2 = r - b * df64(q2);
  const float q3 = __fdiv_rn(r2.hi, b.hi);
  df64 q = fast_two_sum(q1, q2);
  return q + df64(q3);
}
__device__ __forceinline__ df64& operator+=(df64& a, df64 b) { return a = a + b; }
__device__ __forceinline__ df64& operator-=(df64& a, df64 b) { return a = a - b; }
__device__ __forceinline__ df64& operator*=(df64& a, df64 b) { return a = a * b; }
__device__ __forceinline__ bool operator<(df64 a, df64 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(df64 a, df64 b) { return b < a; }
__device__ __forceinline__ bool operator<=(df64 a, df64 b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(df64 a, df64 b) { return !(a < b); }
__device__ __forceinline__ bool operator==(df64 a, df64 b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(df64 a, df64 b) { return !(a == b); }
// The float/double overloads stay visible beside the df64 ones.
using ::fabs;
using ::fmax;
__device__ __forceinline__ df64 fabs(df64 a) { return a.hi < 0.f ? -a : a; }
__device__ __forceinline__ df64 fmax(df64 a, df64 b) { return a < b ? b : a; }

// acc + a b in one pass: the TwoProduct terms of a b go straight into the
// one-TwoSum addition, unnormalised (15 FP32 instructions, 14 with a float
// factor, against 7 + 11 for the product and the sum apart); the error
// bound is that of the addition, about 2^-47 of |acc| + |a b|.
__device__ __forceinline__ df64 madd(df64 acc, df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const df64 s = two_sum(acc.hi, p);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(acc.lo, e)));
}
__device__ __forceinline__ df64 madd(df64 acc, df64 a, float b) {
  const float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  const df64 s = two_sum(acc.hi, p);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(acc.lo, e)));
}

// Accumulation of float products into a df64 (exact products).
__device__ __forceinline__ void df_fma(df64& acc, float a, float b) { acc = acc + two_prod(a, b); }

// Storage conversions.
__device__ __forceinline__ df64 df_load(const float2 v) { return df64(v.x, v.y); }
__device__ __forceinline__ float2 df_store(df64 v) { return make_float2(v.hi, v.lo); }

}  // namespace mfem_gpu
