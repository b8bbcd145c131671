// Double-float ("double-word") arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits.  On this GPU an FP64 instruction occupies the
// SM's FP64 pipe for 16 cycles per warp and a dependent FP64 operation takes
// about 64 cycles, against 4.5 for FP32, so short FP64-grade computations
// that are latency- or FP64-throughput-bound (the per-atom Newton solves)
// run in pairs of floats instead.
//
// Published building blocks, written here from their descriptions:
//   TwoSum (Knuth, TAOCP vol. 2, 4.2.2), FastTwoSum (Dekker, Numer. Math. 18,
//   1971), TwoProd with an FMA; the pair sum is Algorithm 6 ("AccurateDWPlusDW",
//   relative error <= 3u^2) and the pair product Algorithm 12 ("DWTimesDW3",
//   <= 4u^2) of Joldes, Muller and Popescu, "Tight and rigorous error bounds for
//   basic building blocks of double-word arithmetic", ACM TOMS 44 (2017),
//   u = 2^-24.  Reciprocal and reciprocal square root start from the FP32
//   approximations and take two Newton steps whose residual is formed in
//   pairs (each step squares the relative error).
// The error-free parts use the _rn intrinsics, which the compiler never
// contracts into FMAs (a contraction would break the error-free property).
#pragma once
#include <cuda_runtime.h>

namespace gr {

struct dfl {
  float hi, lo;
};

__device__ __forceinline__ dfl df_make(float a) { return {a, 0.f}; }

__device__ __forceinline__ dfl df_from_double(double v) {
  const float h = __double2float_rn(v);
  return {h, __double2float_rn(v - (double)h)};
}

__device__ __forceinline__ double df_to_double(dfl x) { return (double)x.hi + (double)x.lo; }

// |a| >= |b| (or a == 0)
__device__ __forceinline__ dfl df_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dfl df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ dfl df_add(dfl x, dfl y) {
  const dfl s = df_two_sum(x.hi, y.hi);
  const dfl t = df_two_sum(x.lo, y.lo);
  const dfl v = df_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return df_fast_two_sum(v.hi, __fadd_rn(t.lo, v.lo));
}

__device__ __forceinline__ dfl df_neg(dfl x) { return {-x.hi, -x.lo}; }

__device__ __forceinline__ dfl df_sub(dfl x, dfl y) { return df_add(x, df_neg(y)); }

__device__ __forceinline__ dfl df_mul(dfl x, dfl y) {
  const float ch = __fmul_rn(x.hi, y.hi);
  const float cl1 = __fmaf_rn(x.hi, y.hi, -ch);
  const float tl0 = __fmul_rn(x.lo, y.lo);
  const float tl1 = __fmaf_rn(x.hi, y.lo, tl0);
  const float cl2 = __fmaf_rn(x.lo, y.hi, tl1);
  return df_fast_two_sum(ch, __fadd_rn(cl1, cl2));
}

// x - y z
__device__ __forceinline__ dfl df_fms(dfl x, dfl y, dfl z) { return df_sub(x, df_mul(y, z)); }

// 1 - q for q within a few ulps of 1: 1 - q.hi is exact (Sterbenz)
__device__ __forceinline__ float df_one_minus(dfl q) {
  return __fsub_rn(__fsub_rn(1.f, q.hi), q.lo);
}

// 1 / x, x.hi != 0 and finite
__device__ __forceinline__ dfl df_rcp(dfl x) {
  const float y0 = __frcp_rn(x.hi);
  // y1 = y0 + y0 (1 - x y0): relative error ~ (2^-24)^2
  const float e0 = df_one_minus(df_mul(x, df_make(y0)));
  const dfl y1 = df_fast_two_sum(y0, __fmul_rn(y0, e0));
  const float e1 = df_one_minus(df_mul(x, y1));
  return df_add(y1, df_make(__fmul_rn(y1.hi, e1)));
}

// 1 / sqrt(x), x.hi > 0 and finite
__device__ __forceinline__ dfl df_rsqrt(dfl x) {
  const float y0 = rsqrtf(x.hi);
  // y1 = y0 + y0 (1 - x y0^2) / 2
  const float e0 = df_one_minus(df_mul(x, df_mul(df_make(y0), df_make(y0))));
  const dfl y1 = df_fast_two_sum(y0, __fmul_rn(0.5f * y0, e0));
  const float e1 = df_one_minus(df_mul(x, df_mul(y1, y1)));
  return df_add(y1, df_make(__fmul_rn(0.5f * y1.hi, e1)));
}

__device__ __forceinline__ dfl df_shfl(dfl v, int src, int width) {
  return {__shfl_sync(0xffffffffu, v.hi, src, width), __shfl_sync(0xffffffffu, v.lo, src, width)};
}

}  // namespace gr
