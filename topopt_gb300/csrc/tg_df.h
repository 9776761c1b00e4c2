// tg_df.h -- "double-float": a value carried as an unevaluated sum hi + lo of
// two FP32 numbers (|lo| <= ulp(hi)/2), about 48 significant bits, computed on
// the FP32 pipe.  GB300 issues FP32 at roughly 58x its FP64 rate, so an FP64-
// accuracy residual in double-float arithmetic costs a fraction of the native
// FP64 one.
//
// The algorithms are the classical error-free transformations: Knuth's TwoSum
// and Dekker's Fast2Sum for addition, the FMA-based exact product for
// multiplication, with the renormalisations of the double-double arithmetic of
// Hida, Li and Bailey ("Algorithms for quad-double precision floating point
// arithmetic", 2001), here on FP32 pairs.  Every step is an explicitly rounded
// intrinsic so the compiler can neither fuse nor reorder it.
#pragma once
#include <cuda_runtime.h>

namespace tg {

struct df {
  float hi, lo;
  df() = default;
  __host__ __device__ __forceinline__ constexpr df(float h, float l) : hi(h), lo(l) {}
};

// The nearest double-float to a double: hi = rn(v), lo = rn(v - hi).
__host__ __device__ __forceinline__ df df_from(double v) {
  const float h = float(v);
  return df(h, float(v - double(h)));
}
__host__ __device__ __forceinline__ double df_to_double(df a) {
  return double(a.hi) + double(a.lo);
}

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df(s, e);
}
// Fast2Sum, valid when |a| >= |b| (or a == 0).
__device__ __forceinline__ df quick_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df(s, __fsub_rn(b, __fsub_rn(s, a)));
}

// Addition: TwoSum of the high parts, the low parts and the exact error summed
// in FP32, one renormalisation (the "sloppy" double-double add).  Its error is
// bounded by about 2^-47 (|a| + |b|) -- relative to the operands, not to the
// sum, so a cancellation keeps the operands' absolute accuracy, which is what a
// residual b - A x needs -- at about half the operations of the variant whose
// error is relative to the sum.
__device__ __forceinline__ df operator+(df a, df b) {
  const df s = two_sum(a.hi, b.hi);
  return quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df operator-(df a) { return df(-a.hi, -a.lo); }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }
__device__ __forceinline__ df operator*(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);  // the exact rounding error of a.hi * b.hi
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return quick_two_sum(p, e);
}
__device__ __forceinline__ df mad(df a, df b, df c) { return a * b + c; }
__device__ __forceinline__ bool df_nonzero(df a) { return a.hi != 0.0f || a.lo != 0.0f; }

__device__ __forceinline__ df shfl_up(df v, int d) {
  return df(__shfl_up_sync(0xffffffffu, v.hi, d), __shfl_up_sync(0xffffffffu, v.lo, d));
}
__device__ __forceinline__ df shfl_down(df v, int d) {
  return df(__shfl_down_sync(0xffffffffu, v.hi, d), __shfl_down_sync(0xffffffffu, v.lo, d));
}

}  // namespace tg
