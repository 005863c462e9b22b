// pg_df.cuh -- compensated FP32 pairs ("double-float"): value = hi + lo with
// |lo| <= ulp(hi)/2, about 48 significant bits, evaluated on the FP32 pipe.
//
// Error-free transformations: two_sum (Knuth), quick_two_sum (Dekker, needs
// |a| >= |b|), two_prod via fmaf.  These contain no multiply-add that a
// compiler could contract, except the explicit fmaf calls.
#pragma once

namespace pg {

struct df { float hi, lo; };

__device__ __forceinline__ df two_sum(float a, float b)
{
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}

__device__ __forceinline__ df quick_two_sum(float a, float b)
{
  float s = a + b;
  float e = b - (s - a);
  return {s, e};
}

__device__ __forceinline__ df two_prod(float a, float b)
{
  float p = a * b;
  float e = fmaf(a, b, -p);
  return {p, e};
}

__device__ __forceinline__ df df_add(df a, df b)
{
  df s = two_sum(a.hi, b.hi);
  df t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ df df_add_f(df a, float b)
{
  df s = two_sum(a.hi, b);
  s.lo += a.lo;
  return quick_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df df_mul_f(df a, float b)
{
  df p = two_prod(a.hi, b);
  p.lo = fmaf(a.lo, b, p.lo);
  return quick_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ df df_mul(df a, df b)
{
  df p = two_prod(a.hi, b.hi);
  p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
  return quick_two_sum(p.hi, p.lo);
}

// square root with one Newton correction from the FP32 root
__device__ __forceinline__ df df_sqrt(df a)
{
  if (!(a.hi > 0.0f)) return {sqrtf(fmaxf(a.hi, 0.0f)), 0.0f};
  float s = sqrtf(a.hi);
  df p = two_prod(s, s);
  float r = ((a.hi - p.hi) - p.lo + a.lo) * (0.5f / s);
  return quick_two_sum(s, r);
}

__device__ __forceinline__ df df_from(double d)
{
  float hi = (float)d;
  float lo = (float)(d - (double)hi);
  return {hi, lo};
}

__device__ __forceinline__ double df_to(df a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ float df_f(df a) { return a.hi + a.lo; }

// sign tests of hi + lo
__device__ __forceinline__ bool df_pos(df a) { return a.hi > 0.0f || (a.hi == 0.0f && a.lo > 0.0f); }
__device__ __forceinline__ bool df_neg_(df a) { return a.hi < 0.0f || (a.hi == 0.0f && a.lo < 0.0f); }

} // namespace pg
