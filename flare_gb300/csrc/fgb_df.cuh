// Double-float arithmetic: a value is an unevaluated sum hi + lo of two
// FP32 numbers (|lo| <= ulp(hi)), about 46 significant bits.  FP64 runs at
// roughly 2 operations per clock per SM on this GPU and FP32 at 128, so the
// descriptor stages of the mixed-precision path compute in this type: an
// add costs 11 FP32 operations and a multiply 7, both far cheaper than one
// FP64 operation.  The algorithms are the classical error-free
// transformations (Knuth's TwoSum, Dekker's Fast2Sum, the FMA-based exact
// product) and the double-single division and square-root steps of the
// double-double literature (Hida, Li and Bailey), written here for FP32
// pairs.  Conversions to and from FP64 are done on the bit patterns with
// integer instructions.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "fgb_common.cuh"

namespace fgb {
// The type and its functions live in a nested namespace: argument-dependent
// lookup finds sqrt(df) and the operators from anywhere, while unqualified
// calls with FP64 or FP32 arguments inside namespace fgb still reach the
// CUDA math library.
namespace dfm {

struct df;
__device__ __forceinline__ df df_from_double(double d);

struct df {
  float hi, lo;
  df() = default;
  __device__ __forceinline__ constexpr df(float h, float l) : hi(h), lo(l) {}
  // integers used as constants are exact in FP32 below 2^24
  __device__ __forceinline__ explicit df(int v) : hi((float)v), lo(0.f) {}
  __device__ __forceinline__ explicit df(double d) : df(df_from_double(d)) {}
};

// s + e = a + b exactly (Knuth)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// s + e = a + b exactly, for |a| >= |b| (Dekker)
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s,
                                             float &e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ df operator+(df a, df b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  df r;
  fast_two_sum(s, e, r.hi, r.lo);
  return r;
}

__device__ __forceinline__ df operator-(df a) { return df(-a.hi, -a.lo); }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }

__device__ __forceinline__ df operator*(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);          // exact product error
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  df r;
  fast_two_sum(p, e, r.hi, r.lo);
  return r;
}

__device__ __forceinline__ df operator/(df a, df b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const df r = a - b * df(q1, 0.f);
  const float q2 = __fdiv_rn(r.hi, b.hi);
  df q;
  fast_two_sum(q1, q2, q.hi, q.lo);
  return q;
}

__device__ __forceinline__ df operator*(df a, int k) { return a * df(k); }
__device__ __forceinline__ df operator*(int k, df a) { return df(k) * a; }

__device__ __forceinline__ df &operator+=(df &a, df b) { return a = a + b; }
__device__ __forceinline__ df &operator-=(df &a, df b) { return a = a - b; }
__device__ __forceinline__ df &operator*=(df &a, df b) { return a = a * b; }
__device__ __forceinline__ df &operator/=(df &a, df b) { return a = a / b; }

__device__ __forceinline__ bool operator<(df a, df b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
__device__ __forceinline__ bool operator>(df a, df b) { return b < a; }
__device__ __forceinline__ bool operator<=(df a, df b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(df a, df b) { return !(a < b); }

// sqrt: one Newton correction of the FP32 root, with the exact square
__device__ __forceinline__ df sqrt(df a) {
  if (!(a.hi > 0.f)) return df(0.f, 0.f);
  const float s = __fsqrt_rn(a.hi);
  const float p = __fmul_rn(s, s);
  const float pe = __fmaf_rn(s, s, -p);
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), pe), a.lo);
  df q;
  fast_two_sum(s, __fdiv_rn(r, __fmul_rn(2.f, s)), q.hi, q.lo);
  return q;
}

// ------------------------------------------------ FP64 <-> double-float
// hi = d with its mantissa cut to 24 bits (exact), lo = the remaining 29
// bits rounded to FP32; |d - (hi + lo)| <= 2^-47 |d|.  Zero, subnormal and
// out-of-FP32-range inputs go through the FP64 conversion instead.
// Out of line so that the compiler cannot if-convert it into the common
// path: its FP64 instructions would then run on every call.
static __device__ __noinline__ df df_from_double_rare(double d) {
  const float h = __double2float_rn(d);
  return df(h, __double2float_rn(d - (double)h));
}

__device__ __forceinline__ df df_from_double(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const int E = (int)((b >> 52) & 0x7FF);
  const int e = E - 1023;
  if (E == 0 || e < -100 || e > 100) return df_from_double_rare(d);
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const unsigned long long m = b & 0xFFFFFFFFFFFFFULL;
  const float hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) |
                                   (unsigned)(m >> 29));
  const unsigned rem = (unsigned)(m & ((1ULL << 29) - 1));
  // rem * 2^(e - 52); e - 52 >= -152 needs two steps to stay normal
  float lo = __uint2float_rn(rem);
  lo = __fmul_rn(lo, __uint_as_float((unsigned)(e - 52 + 64 + 127) << 23));
  lo = __fmul_rn(lo, 0x1p-64f);
  return df(hi, sign ? -lo : lo);
}

// d with its mantissa cut to 24 bits (relative error below 2^-23); FP32
// range only, FP64 conversion otherwise.
static __device__ __noinline__ float trunc_float_rare(double d) {
  return __double2float_rn(d);
}

__device__ __forceinline__ float trunc_float(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const int E = (int)((b >> 52) & 0x7FF);
  const int e = E - 1023;
  if (E == 0 || e < -126 || e > 127) return trunc_float_rare(d);
  return __uint_as_float(((unsigned)(b >> 63) << 31) |
                         ((unsigned)(e + 127) << 23) |
                         (unsigned)((b & 0xFFFFFFFFFFFFFULL) >> 29));
}

// FP64 value of an FP32 number, on the bit patterns: exact for normal
// numbers, infinities and NaNs; FP32 subnormals become signed zeros.
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned E = (u >> 23) & 0xFF;
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  const unsigned long long field =
      E == 0 ? 0ULL : (E == 255 ? 2047ULL : (unsigned long long)(E - 127 + 1023));
  const unsigned long long mant =
      E == 0 ? 0ULL : (unsigned long long)(u & 0x7FFFFF) << 29;
  return __longlong_as_double((long long)(sign | (field << 52) | mant));
}

// hi + lo rounded once to FP64
__device__ __forceinline__ double to_double(df a) {
  return f2d_exact(a.hi) + f2d_exact(a.lo);
}
// K_lm as a double-float from the FP32 tables (no conversion)
__device__ __forceinline__ void ylm_norm(int i, df &k) {
  k = df(c_ylm_norm_f[i], c_ylm_norm_lo[i]);
}
__device__ __forceinline__ void dfact_const(int m, df &v) {
  v = df(c_dfact_f[m], c_dfact_lo[m]);
}
__device__ __forceinline__ df div_int(df x, int k) {
  return x * df(c_inv_f[k], c_inv_lo[k]);
}

// Rare-path functions (cutoffs other than quadratic and hard): evaluated in
// FP64 and split back.
__device__ __forceinline__ df cos(df a) { return df_from_double(::cos(to_double(a))); }
__device__ __forceinline__ df sin(df a) { return df_from_double(::sin(to_double(a))); }
__device__ __forceinline__ df pow(df a, df b) {
  return df_from_double(::pow(to_double(a), to_double(b)));
}
// radial bases other than Chebyshev are evaluated in FP64
__device__ __forceinline__ double rad_to_double(df a) { return to_double(a); }

}  // namespace dfm
using dfm::df;
using dfm::to_double;
using dfm::trunc_float;
using dfm::f2d_exact;
using dfm::two_sum;
using dfm::fast_two_sum;
__device__ __forceinline__ double to_double(double a) { return a; }
// The nearest float: the high part of a normalised double-float; an FP64
// value is rounded (a conversion on the FP64 pipe).
__device__ __forceinline__ float to_float(df a) { return a.hi; }
__device__ __forceinline__ float to_float(double a) { return (float)a; }
template <> __device__ __forceinline__ df rad_from_double<df>(double x) {
  return dfm::df_from_double(x);
}

}  // namespace fgb
