// fb_df.cuh -- double-float ("df") arithmetic on the FP32 pipe.
//
// GB300 executes FP64 at about 1/64 of its FP32 rate, so the table
// contractions of the three-center kernels are carried as unevaluated sums
// of two floats, a = hi + lo with |lo| <= ulp(hi)/2, giving a 48-bit
// significand (relative error ~ 2^-47 per operation).  The building blocks
// are the error-free transformations of Knuth (TwoSum), Dekker
// (Fast2Sum / quick-two-sum) and the FMA-based exact product; the operation
// sequences are those of the published double-double literature (Dekker
// 1971; Hida, Li & Bailey, "Library for double-double and quad-double
// arithmetic", 2001), written here for float pairs.  Every rounding step is
// an explicit __f*_rn intrinsic so the compiler cannot fuse or reorder it.
#pragma once
#include <cuda_runtime.h>

namespace fb {

struct df {
  float h, l;
};

__device__ __forceinline__ df df_make(float h, float l = 0.0f) { return df{h, l}; }

// split a double into hi + lo floats (three conversions and one DADD)
__device__ __forceinline__ df df_from(double x) {
  float h = __double2float_rn(x);
  float l = __double2float_rn(x - (double)h);
  return df{h, l};
}
__device__ __forceinline__ double df_to(df a) { return (double)a.h + (double)a.l; }

// Fast2Sum, valid when |a| >= |b| or a == 0
__device__ __forceinline__ df quick_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return df{s, e};
}
// TwoSum, valid for any a, b
__device__ __forceinline__ df two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df{s, e};
}

__device__ __forceinline__ df operator+(df a, df b) {
  df s = two_sum(a.h, b.h);
  float e = __fadd_rn(s.l, __fadd_rn(a.l, b.l));
  return quick_two_sum(s.h, e);
}
__device__ __forceinline__ df operator-(df a) { return df{-a.h, -a.l}; }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }
__device__ __forceinline__ df operator*(df a, df b) {
  float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return quick_two_sum(p, e);
}
__device__ __forceinline__ df operator*(df a, float b) {
  float p = __fmul_rn(a.h, b);
  float e = __fmaf_rn(a.h, b, -p);
  e = __fmaf_rn(a.l, b, e);
  return quick_two_sum(p, e);
}
__device__ __forceinline__ df df_fma(df a, df b, df c) { return a * b + c; }
__device__ __forceinline__ df &operator+=(df &a, df b) {
  a = a + b;
  return a;
}
__device__ __forceinline__ df &operator-=(df &a, df b) {
  a = a - b;
  return a;
}

// Accumulator of sum_n w_n t_n for df weights and df table values: the
// hi*hi products are exact (FMA remainder) and summed with TwoSum into s;
// everything of order 2^-24 relative (cross terms, product remainders, sum
// errors) goes to c.  12 FP32 operations per term.
struct dacc {
  float s, c;
};
__device__ __forceinline__ void dacc_first(dacc &a, df w, df t) {
  float p = __fmul_rn(w.h, t.h);
  float pe = __fmaf_rn(w.h, t.h, -p);
  float c = __fmaf_rn(w.h, t.l, pe);
  a.c = __fmaf_rn(w.l, t.h, c);
  a.s = p;
}
__device__ __forceinline__ void dacc_add(dacc &a, df w, df t) {
  float p = __fmul_rn(w.h, t.h);
  float pe = __fmaf_rn(w.h, t.h, -p);
  float c = __fmaf_rn(w.h, t.l, a.c);
  c = __fmaf_rn(w.l, t.h, c);
  df s = two_sum(a.s, p);
  a.c = __fadd_rn(c, __fadd_rn(pe, s.l));
  a.s = s.h;
}
__device__ __forceinline__ df dacc_val(const dacc &a) { return two_sum(a.s, a.c); }

// square root by one Newton step from the float square root (a >= 0)
__device__ __forceinline__ df df_sqrt(df a) {
  if (a.h <= 0.0f) return df{0.0f, 0.0f};
  float y = __fsqrt_rn(a.h);
  df e = a - df{y, 0.0f} * df{y, 0.0f};
  return df{y, 0.0f} + e * __fdiv_rn(0.5f, y);
}

}  // namespace fb
