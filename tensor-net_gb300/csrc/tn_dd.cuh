// tn_dd.cuh -- double-float ("dd") arithmetic: a value is the unevaluated sum
// hi + lo of two float32 numbers with |lo| <= ulp(hi) / 2, about 48 significant
// bits, computed entirely on the FP32 pipes.
//
// GB300 issues FP64 at 1/64 of its FP32 rate, so FP64-class accuracy is
// cheaper as float pairs: the error-free transformations TwoSum (Knuth),
// FastTwoSum (Dekker) and TwoProduct (one FMA) give sums and products exact to
// the second float, and the usual double-float algorithms (Dekker 1971;
// Hida, Li and Bailey's double-double) build +, *, /, sqrt on them.
// Every primitive uses the explicitly rounded intrinsics (__fadd_rn, ...),
// which the compiler never contracts into FMAs: a contracted a*b + c would
// break the exactness the transformations rely on.
//
// Relative accuracy of a rounded operation here is about 2^-46..2^-47
// (Eps<dd>), against 2^-53 for float64; float64's exponent range is not
// kept (float32's is): the engine's values (Schmidt values down to the
// cutoff, Gamma = U / Lambda) stay well inside it.
#pragma once

#include <cuda_runtime.h>

namespace tn {

// the float / double overloads stay visible beside the dd ones declared here
using ::fabs;
using ::fma;
using ::isfinite;
using ::sqrt;

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// |a| >= |b| (or a == 0)
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

struct __align__(8) dd {
  float hi, lo;
  dd() = default;
  __host__ __device__ constexpr dd(float h, float l) : hi(h), lo(l) {}
  __device__ dd(float x) : hi(x), lo(0.f) {}
  __device__ dd(int x) : hi(float(x)), lo(float(x - int(float(x)))) {}
  __device__ dd(double x) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(x - double(hi));
  }
  __device__ explicit operator double() const { return double(hi) + double(lo); }
  __device__ explicit operator float() const { return __fadd_rn(hi, lo); }
};

// normalised sum of a raw pair (any magnitudes)
__device__ __forceinline__ dd dd_norm(float h, float l) {
  float s, e;
  two_sum(h, l, s, e);
  return dd(s, e);
}

__device__ __forceinline__ dd operator-(dd a) { return dd(-a.hi, -a.lo); }

// IEEE-style double-float addition (both halves summed with TwoSum), accurate
// also under cancellation
__device__ __forceinline__ dd operator+(dd a, dd b) {
  float s, e, t, f;
  two_sum(a.hi, b.hi, s, e);
  two_sum(a.lo, b.lo, t, f);
  e = __fadd_rn(e, t);
  fast_two_sum(s, e, s, e);
  e = __fadd_rn(e, f);
  fast_two_sum(s, e, s, e);
  return dd(s, e);
}
__device__ __forceinline__ dd operator-(dd a, dd b) { return a + (-b); }

__device__ __forceinline__ dd operator*(dd a, dd b) {
  float p, e;
  two_prod(a.hi, b.hi, p, e);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  fast_two_sum(p, e, p, e);
  return dd(p, e);
}

__device__ __forceinline__ dd operator/(dd a, dd b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  // r = a - q1 * b
  float p, e;
  two_prod(q1, b.hi, p, e);
  e = __fmaf_rn(q1, b.lo, e);
  float s, f;
  two_sum(a.hi, -p, s, f);
  f = __fadd_rn(f, __fsub_rn(a.lo, e));
  const float r = __fadd_rn(s, f);
  const float q2 = __fdiv_rn(r, b.hi);
  float h, l;
  fast_two_sum(q1, q2, h, l);
  return dd(h, l);
}

__device__ __forceinline__ dd &operator+=(dd &a, dd b) { return a = a + b; }
__device__ __forceinline__ dd &operator-=(dd &a, dd b) { return a = a - b; }
__device__ __forceinline__ dd &operator*=(dd &a, dd b) { return a = a * b; }

__device__ __forceinline__ bool operator<(dd a, dd b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(dd a, dd b) { return b < a; }
__device__ __forceinline__ bool operator<=(dd a, dd b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(dd a, dd b) { return !(a < b); }
__device__ __forceinline__ bool operator==(dd a, dd b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(dd a, dd b) { return !(a == b); }

__device__ __forceinline__ dd fabs(dd a) { return a.hi < 0.f ? -a : a; }

// sqrt(a) = x + (a - x^2) / (2x), x = sqrtf(a.hi) (one Newton step)
__device__ __forceinline__ dd sqrt(dd a) {
  if (!(a.hi > 0.f)) return dd(0.f, 0.f);
  const float x = __fsqrt_rn(a.hi);
  float p, e;
  two_prod(x, x, p, e);
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), e), a.lo);
  const float c = __fdiv_rn(r, __fmul_rn(2.f, x));
  float h, l;
  fast_two_sum(x, c, h, l);
  return dd(h, l);
}

// a * b + c
__device__ __forceinline__ dd fma(dd a, dd b, dd c) { return a * b + c; }

__device__ __forceinline__ bool isfinite(dd a) { return ::isfinite(a.hi) && ::isfinite(a.lo); }

// Accumulation of a sum of products into a raw pair (hi, lo): the leading
// product is split exactly (TwoProduct), the running sum exactly (TwoSum),
// and every rounding error, the cross terms a.hi*b.lo + a.lo*b.hi and the
// accumulator's own low part are collected in lo, which is never
// renormalised inside the loop (12 float operations per real product).
// The caller normalises with dd_norm(hi, lo) after the loop.
struct dacc {
  float hi, lo;
};
__device__ __forceinline__ void dacc_add_prod(dacc &s, dd a, dd b) {
  float p, e;
  two_prod(a.hi, b.hi, p, e);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  float h, t;
  two_sum(s.hi, p, h, t);
  s.hi = h;
  s.lo = __fadd_rn(s.lo, __fadd_rn(t, e));
}

template <typename T>
__device__ __forceinline__ T shfl_xor(T v, int o) {
  return __shfl_xor_sync(0xffffffffu, v, o);
}
template <>
__device__ __forceinline__ dd shfl_xor<dd>(dd v, int o) {
  return dd(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
}

}  // namespace tn
