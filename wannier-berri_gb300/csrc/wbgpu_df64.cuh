// Double-float ("df64") real arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2, giving a
// 48-bit significand (relative precision ~2^-48 = 3.6e-15) with the FP32 exponent range.
// GB300 issues FP32 at ~58x its FP64 rate, so kernels whose FP64 precision requirement is
// "well beyond FP32" but whose throughput is FP64-pipe-bound run several times faster in
// df64.  The algorithms are the classical error-free transformations (Knuth two-sum,
// Dekker/FMA two-product) and one Newton step for reciprocal and square root.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include "wbgpu_common.cuh"

struct df64 {
  float hi, lo;
};

__host__ __device__ __forceinline__ df64 df_from(double x) {
  const float h = (float)x;
  df64 r;
  r.hi = h;
  r.lo = (float)(x - (double)h);
  return r;
}
__host__ __device__ __forceinline__ df64 df_from_f(float x) {
  df64 r;
  r.hi = x;
  r.lo = 0.0f;
  return r;
}
__host__ __device__ __forceinline__ double df_to_double(df64 a) { return (double)a.hi + (double)a.lo; }

// s + e = a + b exactly
__device__ __forceinline__ df64 df_two_sum(float a, float b) {
  const float s = a + b;
  const float v = s - a;
  const float e = (a - (s - v)) + (b - v);
  df64 r;
  r.hi = s;
  r.lo = e;
  return r;
}
// requires |a| >= |b|
__device__ __forceinline__ df64 df_quick(float a, float b) {
  const float s = a + b;
  df64 r;
  r.hi = s;
  r.lo = b - (s - a);
  return r;
}

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  df64 s = df_two_sum(a.hi, b.hi);
  return df_quick(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ df64 operator-(df64 a) {
  a.hi = -a.hi;
  a.lo = -a.lo;
  return a;
}
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_quick(p, e);
}
__device__ __forceinline__ df64& operator+=(df64& a, df64 b) { return a = a + b; }
__device__ __forceinline__ df64& operator-=(df64& a, df64 b) { return a = a - b; }
__device__ __forceinline__ df64& operator*=(df64& a, df64 b) { return a = a * b; }

// a * b + c with one renormalisation
__device__ __forceinline__ df64 fma(df64 a, df64 b, df64 c) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const df64 s = df_two_sum(p, c.hi);
  return df_quick(s.hi, s.lo + (e + c.lo));
}

// Lazy multiply-add chains: acc += a b with the exact two-sum of the leading parts and every
// error term collected in acc.lo, without renormalising (12 instead of 15 FP32 instructions);
// df_lazy_done renormalises once at the end of the chain (a full two-sum: after cancellation
// |lo| may exceed |hi|).  Over a few hundred steps lo stays within a few hundred ulp(hi).
__device__ __forceinline__ void df_lazy_fma(df64& acc, df64 a, df64 b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const float s = acc.hi + p;
  const float v = s - acc.hi;
  const float t = (acc.hi - (s - v)) + (p - v);
  acc.hi = s;
  acc.lo = acc.lo + (t + e);
}
__device__ __forceinline__ df64 df_lazy_done(df64 acc) { return df_two_sum(acc.hi, acc.lo); }

__device__ __forceinline__ bool operator<(df64 a, df64 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(df64 a, df64 b) { return b < a; }
__device__ __forceinline__ bool operator<=(df64 a, df64 b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(df64 a, df64 b) { return !(a < b); }
__device__ __forceinline__ bool operator==(df64 a, df64 b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(df64 a, df64 b) { return !(a == b); }

__device__ __forceinline__ df64 fabs(df64 a) { return a.hi < 0.0f || (a.hi == 0.0f && a.lo < 0.0f) ? -a : a; }

// 1/a: FP32 seed, one Newton step r + r (1 - a r)
__device__ __forceinline__ df64 df_recip(df64 a) {
  const float r = 1.0f / a.hi;
  df64 one;
  one.hi = 1.0f;
  one.lo = 0.0f;
  const df64 rr = df_from_f(r);
  const df64 e = one - a * rr;
  return df_quick(r, r * e.hi + r * e.lo);
}
__device__ __forceinline__ df64 operator/(df64 a, df64 b) {
  const df64 r = df_recip(b);
  const df64 q = a * r;  // one correction of the quotient keeps ~2 ulp accuracy
  const df64 res = a - q * b;
  return df_quick(q.hi, q.lo + res.hi * r.hi);
}
// sqrt(a) for a >= 0: FP32 seed, one Newton step y + (a - y^2) / (2y)
__device__ __forceinline__ df64 sqrt(df64 a) {
  if (!(a.hi > 0.0f)) return df_from_f(0.0f);
  const float y = sqrtf(a.hi);
  const df64 yy = df_from_f(y) * df_from_f(y);
  const df64 d = a - yy;
  return df_quick(y, d.hi * (0.5f / y));
}
__device__ __forceinline__ df64 rsqrt(df64 a) { return df_recip(sqrt(a)); }
__device__ __forceinline__ df64 copysign(df64 a, df64 s) { return (s.hi < 0.0f) != (a.hi < 0.0f) ? -a : a; }
__device__ __forceinline__ df64 fmax(df64 a, df64 b) { return a < b ? b : a; }

// Arithmetic traits: constants and conversions for the two real types the solver runs in.
template <typename R> struct Arith;
template <> struct Arith<double> {
  static __device__ __forceinline__ double from(double x) { return x; }
  static __device__ __forceinline__ double to(double x) { return x; }
  static __device__ __forceinline__ double eps() { return 2.220446049250313e-16; }
  static __device__ __forceinline__ double tiny_norm() { return 2.2250738585072014e-308; }
  // relative floor for inverse-iteration pivots: growth per tiny pivot stays within range
  static __device__ __forceinline__ double pivot_floor() { return 2.220446049250313e-16; }
};
template <> struct Arith<float> {
  static __device__ __forceinline__ float from(double x) { return (float)x; }
  static __device__ __forceinline__ double to(float x) { return (double)x; }
  static __device__ __forceinline__ float eps() { return 5.9604644775390625e-08f; }  // 2^-24
  static __device__ __forceinline__ float tiny_norm() { return 1e-30f; }
  // FP32 exponent range: three consecutive pivots at the floor stay below 1e20
  static __device__ __forceinline__ float pivot_floor() { return 1e-6f; }
};
template <> struct Arith<df64> {
  static __device__ __forceinline__ df64 from(double x) { return df_from(x); }
  static __device__ __forceinline__ double to(df64 x) { return df_to_double(x); }
  static __device__ __forceinline__ df64 eps() { return df_from(7.105427357601002e-15); }  // 2^-47
  static __device__ __forceinline__ df64 tiny_norm() { return df_from(1e-30); }
  // FP32 exponent range: a floor of 1e-12 keeps three consecutive tiny pivots below 1e36
  static __device__ __forceinline__ df64 pivot_floor() { return df_from(1e-12); }
};

// complex df64 (same 16-byte footprint as double2)
struct cdf {
  df64 x, y;
};
template <> struct C2<df64> { typedef cdf t; };
template <> WBG_HD cdf czero<cdf>() {
  cdf r;
  r.x.hi = 0.0f; r.x.lo = 0.0f; r.y.hi = 0.0f; r.y.lo = 0.0f;
  return r;
}

// warp shuffles of the real types
__device__ __forceinline__ float shfl_xor(float v, int off) { return __shfl_xor_sync(0xffffffffu, v, off); }
__device__ __forceinline__ double shfl_xor(double v, int off) { return __shfl_xor_sync(0xffffffffu, v, off); }
__device__ __forceinline__ df64 shfl_xor(df64 v, int off) {
  v.hi = __shfl_xor_sync(0xffffffffu, v.hi, off);
  v.lo = __shfl_xor_sync(0xffffffffu, v.lo, off);
  return v;
}

// conversion of a double into each working real type
template <typename T> __device__ __forceinline__ T real_from_double(double x);
template <> __device__ __forceinline__ float real_from_double<float>(double x) { return (float)x; }
template <> __device__ __forceinline__ double real_from_double<double>(double x) { return x; }
template <> __device__ __forceinline__ df64 real_from_double<df64>(double x) { return df_from(x); }

