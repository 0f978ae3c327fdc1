// Double-float ("df") arithmetic on the FP32 pipes: a value is hi + lo with two floats,
// about 48 significant bits (relative rounding ~3.6e-15 per operation).  On GB300 the FP64
// pipe runs at 1/62 of the FP32 rate, so FP64-accurate integrals done with these
// error-free transformations (Knuth two-sum, FMA two-product) cost several times less than
// native FP64.  Every operation uses round-to-nearest intrinsics, so the compiler can neither
// contract nor reassociate them.
//
// df_sincos: Cody-Waite reduction of the argument by multiples of pi/64 (pi/64 split in three
// floats, the first with 11 significant bits so the product with the multiple is exact for
// |m| < 2^13, i.e. |theta| < 400), a 128-entry df table of sin / cos at j pi/64, Taylor series
// of the remainder (|t| <= pi/128) and the angle-addition formulas.
#pragma once

#include <cuda_runtime.h>

namespace bgb {

struct dfl {
  float hi, lo;
};

__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void df_fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
__device__ __forceinline__ dfl df_from(float a) { return {a, 0.f}; }
__device__ __forceinline__ dfl df_neg(dfl a) { return {-a.hi, -a.lo}; }
// sum with error terms of both parts folded once (absolute error ~2^-48 max(|a|, |b|))
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
  float s, e;
  df_two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  dfl r;
  df_fast_two_sum(s, e, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ dfl df_sub(dfl a, dfl b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ dfl df_addf(dfl a, float b) {
  float s, e;
  df_two_sum(a.hi, b, s, e);
  e = __fadd_rn(e, a.lo);
  dfl r;
  df_fast_two_sum(s, e, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  dfl r;
  df_fast_two_sum(p, e, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ dfl df_mulf(dfl a, float b) {
  const float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  dfl r;
  df_fast_two_sum(p, e, r.hi, r.lo);
  return r;
}
// a * b + c
__device__ __forceinline__ dfl df_fma(dfl a, dfl b, dfl c) { return df_add(df_mul(a, b), c); }
__device__ __forceinline__ double df_to_double(dfl a) { return (double)a.hi + (double)a.lo; }

// 1 / sqrt(s), s > 0: FP32 estimate and one Newton step with the residual in df.
__device__ __forceinline__ dfl df_rsqrt(dfl s) {
  const float y = rsqrtf(s.hi);
  const float yy = __fmul_rn(y, y);
  const float yye = __fmaf_rn(y, y, -yy);
  const dfl sy2 = df_mul(s, dfl{yy, yye});
  const float r = __fsub_rn(__fsub_rn(1.0f, sy2.hi), sy2.lo);  // 1 - s y^2, ~1e-7
  const float c = __fmul_rn(__fmul_rn(0.5f, y), r);
  dfl out;
  df_fast_two_sum(y, c, out.hi, out.lo);
  // second step for ~1e-15
  const dfl o2 = df_mul(out, out);
  const dfl so2 = df_mul(s, o2);
  const float r2 = __fsub_rn(__fsub_rn(1.0f, so2.hi), so2.lo);
  return df_addf(out, __fmul_rn(__fmul_rn(0.5f, out.hi), r2));
}

// sin and cos of a df angle |theta| < 400.  tab[j] = (sin_hi, sin_lo, cos_hi, cos_lo) of
// j pi / 64, j = 0..127 (host-computed in FP64).  pi64 = pi/64 as three floats.
struct DfTrig {
  float inv_step;    // 64 / pi
  float p1, p2, p3;  // pi/64 = p1 + p2 + p3, p1 with 11 significant bits
  dfl s3, s5;        // -1/6, 1/120  (sin series)
  float s7;          // -1/5040
  float c4, c6;      // 1/24, -1/720
  dfl inv4pi;        // 1 / (4 pi)
};

__device__ __forceinline__ void df_sincos(dfl th, const float4* __restrict__ tab, const DfTrig& T, dfl& s, dfl& c) {
  const float m = rintf(__fmul_rn(th.hi, T.inv_step));
  // t = th - m * pi/64
  const float a = __fmaf_rn(-m, T.p1, th.hi);  // exact
  const float q2 = __fmul_rn(m, T.p2);
  const float q2e = __fmaf_rn(m, T.p2, -q2);
  dfl t = df_add(dfl{a, th.lo}, dfl{-q2, -q2e});
  t = df_addf(t, -__fmul_rn(m, T.p3));
  const int j = ((int)m) & 127;
  const float4 e = tab[j];
  const dfl t2 = df_mul(t, t);
  // sin t = t + t^3 (-1/6 + t^2/120 - t^4/5040)
  const float small = __fmaf_rn(t2.hi, __fmaf_rn(t2.hi, T.s7, T.s5.hi), 0.f);
  const dfl br = df_addf(T.s3, small);
  const dfl st = df_add(t, df_mul(df_mul(t, t2), br));
  // cos t = 1 + t^2 (-1/2 + t^2 (1/24 - t^2/720))
  const float q = __fmaf_rn(t2.hi, T.c6, T.c4);
  const dfl br2 = df_addf(df_mulf(t2, q), -0.5f);
  const dfl ct = df_addf(df_mul(t2, br2), 1.0f);
  const dfl sa{e.x, e.y}, ca{e.z, e.w};
  s = df_add(df_mul(sa, ct), df_mul(ca, st));
  c = df_sub(df_mul(ca, ct), df_mul(sa, st));
}

}  // namespace bgb
