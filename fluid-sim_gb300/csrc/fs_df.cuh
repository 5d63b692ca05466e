// fs_df.cuh -- double-float ("df") arithmetic on the FP32 pipe.
//
// GB300 executes FP64 at 1.19 TFLOP/s against 64 TFLOP/s for FP32 (measured
// with dependent FMA chains on the device), so the high-precision part of the
// MIXED projection -- divergence, residual d - lap(p), pressure accumulation,
// gradient subtraction -- is carried as an unevaluated sum hi + lo of two
// floats (~48-bit significand, relative rounding ~1e-14) and computed with
// error-free transformations:
//   two_sum   (Knuth), fast_two_sum (Dekker), two_prod via FMA,
// as published in Dekker (1971), Knuth TAOCP vol. 2 sec. 4.2.2, and the QD
// library paper of Hida, Li & Bailey (2001).  The _rn intrinsics keep nvcc
// from contracting or reassociating the steps whose rounding errors the
// transformations recover.
#pragma once

#include <cuda_runtime.h>

namespace fs {

struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_make(float x) { return {x, 0.f}; }

// s + e == a + b exactly
__device__ __forceinline__ df two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ df fast_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}

// a - b exactly
__device__ __forceinline__ df two_diff(float a, float b) { return two_sum(a, -b); }

// p + e == a * b exactly
__device__ __forceinline__ df two_prod(float a, float b) {
  float p = __fmul_rn(a, b);
  float e = __fmaf_rn(a, b, -p);
  return {p, e};
}

// accurate df + df
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  df t = two_sum(a.lo, b.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = fast_two_sum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }

// df + float
__device__ __forceinline__ df df_add_f(df a, float b) {
  df s = two_sum(a.hi, b);
  s.lo = __fadd_rn(s.lo, a.lo);
  return fast_two_sum(s.hi, s.lo);
}

// df * df
__device__ __forceinline__ df df_mul(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  p.lo = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
  return fast_two_sum(p.hi, p.lo);
}

// df * float
__device__ __forceinline__ df df_mul_f(df a, float b) {
  df p = two_prod(a.hi, b);
  p.lo = __fmaf_rn(a.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ float df_to_f(df a) { return __fadd_rn(a.hi, a.lo); }

// df <-> double (only for host I/O and tests; FP64 pipe)
__device__ __forceinline__ df df_from_d(double x) {
  float hi = (float)x;
  float lo = (float)(x - (double)hi);
  return {hi, lo};
}
__device__ __forceinline__ double df_to_d(df a) { return (double)a.hi + (double)a.lo; }

// host: a double constant split into df
inline df df_host(double x) {
  float hi = (float)x;
  float lo = (float)(x - (double)hi);
  return {hi, lo};
}

}  // namespace fs
