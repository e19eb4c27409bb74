// cov_df.cuh -- double-float arithmetic (an unevaluated sum hi + lo of two
// FP32 values, ~48-bit significand) for the per-pair passes.  GB300 issues
// FP64 at 1/64 of its FP32 rate, so the pair statistics, marginals and
// scores are carried in double-float on the FP32 pipes.
//
// Error-free transformations: two_sum (Knuth), fast_two_sum (Dekker,
// |a| >= |b|), two_prod via FMA.  Their sums and the products that feed them
// are written with the round-to-nearest intrinsics (__fadd_rn, __fsub_rn,
// __fmul_rn), which the compiler never contracts into an FMA: a product
// fused into the sum of a transformation would leave its low word wrong by
// up to an FP32 rounding, and would do so differently in every kernel that
// inlines it.  df_log is a table-driven natural
// logarithm (argument reduction by a 128-entry reciprocal table, then the
// series of ln(1 + t) for |t| < 2^-7.9); its absolute error is below
// 2e-13 over the range the statistics use (1e-10 .. 2^40), against the
// 1e-12 that the pair statistics need from it.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace covgpu {

struct df { float hi, lo; };

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {   // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df df_norm(df a) { return fast_two_sum(a.hi, a.lo); }
__device__ __forceinline__ df df_add_f(df a, float b) {
  const df s = two_sum(a.hi, b);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}
__device__ __forceinline__ df df_add(df a, df b) {
  const df s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
// accumulation without renormalising: the low part gathers the rounding
// errors (each below ulp(hi)), renormalised once by the caller (df_norm)
__device__ __forceinline__ void df_acc(df& s, df b) {
  const df t = two_sum(s.hi, b.hi);
  s.hi = t.hi;
  s.lo = __fadd_rn(s.lo, __fadd_rn(t.lo, b.lo));
}
__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float e = fmaf(a.hi, b.hi, -p);
  return fast_two_sum(p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e)));
}
// product left unnormalised (for df_acc)
__device__ __forceinline__ df df_mul_u(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  return {p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p)))};
}
// a^2, unnormalised
__device__ __forceinline__ df df_sqr_u(df a) {
  const float p = __fmul_rn(a.hi, a.hi);
  return {p, fmaf(2.f * a.hi, a.lo, fmaf(a.hi, a.hi, -p))};
}
__device__ __forceinline__ df df_scale(df a, float s) {   // s a power of two
  return {__fmul_rn(a.hi, s), __fmul_rn(a.lo, s)};
}
__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
// 1/b and a/b: an FP32 estimate corrected by one residual step (relative
// error ~2^-46)
__device__ __forceinline__ df df_div(df a, df b) {
  const float r = 1.0f / b.hi;
  const float q1 = __fmul_rn(a.hi, r);
  const df pr = df_mul_u(b, {q1, 0.f});
  const df res = df_add(a, df_neg(df_norm(pr)));
  return fast_two_sum(q1, __fmul_rn(res.hi, r));
}
__device__ __forceinline__ df df_recip(df b) { return df_div({1.f, 0.f}, b); }
__device__ __forceinline__ df df_of(double x) {
  const float hi = (float)x;
  return {hi, (float)(x - (double)hi)};
}
__device__ __forceinline__ double df_to_d(df a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ df two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ df ld_df(const float2* p) { const float2 v = *p; return {v.x, v.y}; }
__device__ __forceinline__ void st_df(float2* p, df v) { *p = make_float2(v.hi, v.lo); }
// order of normalised double-float values (|lo| <= ulp(hi)/2)
__device__ __forceinline__ bool df_lt(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ df df_min(df a, df b) { return df_lt(b, a) ? b : a; }
__device__ __forceinline__ df df_max(df a, df b) { return df_lt(a, b) ? b : a; }

// ---------------------------------------------------------------------------
// natural logarithm of a positive, normal double-float a = hi + lo
//   hi = 2^k m, m in [1, 2); j = the top 7 bits of m's fraction;
//   r_j = fl(1 / c_j), c_j = 1 + (j + 1/2)/128; table entry j holds
//   {r_j, -ln r_j as hi + lo}.  m r_j = 1 + t exactly as a double-float
//   (FMA residual), |t| <= 2^-8 + 2^-24, and
//   ln a = k ln 2 - ln r_j + ln(1 + t) + ln(1 + lo/hi),
//   ln(1 + t) = t - t^2/2 + t^3/3 - t^4/4 + t^5/5 (next term < 1e-15),
//   ln(1 + lo/hi) = lo/hi (next term < 2e-15).
//   k ln 2 comes from a second table indexed by hi's biased exponent
//   (256 entries of k ln 2 as hi + lo, two to a float4), so it costs one
//   shared load instead of a three-piece product.
// ---------------------------------------------------------------------------
constexpr int LOGTAB_N = 128;                    // the 1/c_j entries
constexpr int LOGTAB_TOT = LOGTAB_N + 256 / 2;   // + the k ln 2 entries

__device__ __forceinline__ df df_log(df a, const float4* __restrict__ tab) {
  const int bits = __float_as_int(a.hi);
  const int j = (bits >> 16) & (LOGTAB_N - 1);
  const float m = __int_as_float((bits & 0x007FFFFF) | 0x3F800000);
  const float4 T = tab[j];
  const float2 K = reinterpret_cast<const float2*>(tab + LOGTAB_N)[((unsigned)bits >> 23) & 255u];   // k ln 2
  const float p = __fmul_rn(m, T.x);
  const float pe = fmaf(m, T.x, -p);
  const df t = fast_two_sum(__fsub_rn(p, 1.0f), pe);   // p - 1 is exact (p within 2^-7 of 1)
  const float s2 = __fmul_rn(t.hi, t.hi);
  const float s2e = fmaf(t.hi, t.hi, -s2);  // t.hi^2 = s2 + s2e exactly
  const float poly = __fmul_rn(__fmul_rn(t.hi, s2), fmaf(t.hi, fmaf(t.hi, 0.2f, -0.25f), 0.333333343f));
  const float corr = __fdividef(a.lo, a.hi);
  const float low = __fadd_rn(__fsub_rn(fmaf(-t.hi, t.lo, t.lo), __fmul_rn(0.5f, s2e)), __fadd_rn(poly, corr));
  const df l1p = fast_two_sum(t.hi, __fmul_rn(-0.5f, s2));
  const df r = df_add({K.x, K.y}, {T.y, T.z});
  return df_add(r, {l1p.hi, __fadd_rn(l1p.lo, low)});
}

// the table of df_log (LOGTAB_TOT float4), made on the host in FP64; each
// context keeps a copy in global memory and kernels stage it in shared
// memory (the index differs from lane to lane)
void logtab_host(float4* tab);

// ---------------------------------------------------------------------------
// Weighted counts from weight limbs.  Each weight is quantised to
// q = round(w 2^E) < 2^(3b) and split into three b-bit limbs,
// q = l0 + 2^b l1 + 2^2b l2, b = min(11, floor(log2((2^24 - 1) / N))), so a
// limb summed over N sequences is an exact integer in FP32 and an 11-bit limb
// is exact in FP16.  The three exact limb sums d0, d1, d2 are combined
// into a double-float count with two error-free sums, in this fixed order
// (every counting kernel uses it, so the tensor and SIMT paths give the same
// count for the same sums): c2 + c1, then + c0, then the low parts; the
// scale 2^-E is a power of two.
// ---------------------------------------------------------------------------
__device__ __forceinline__ df limb_count(float d0, float d1, float d2, float B, float scale) {
  const float c2 = __fmul_rn(d2, __fmul_rn(B, B)), c1 = __fmul_rn(d1, B);
  const df s1 = two_sum(c2, c1);
  const df s2 = two_sum(s1.hi, d0);
  const df r = fast_two_sum(s2.hi, __fadd_rn(s1.lo, s2.lo));
  return {__fmul_rn(r.hi, scale), __fmul_rn(r.lo, scale)};
}
// equal weights w (one limb: the unit count c times w as hi + lo)
__device__ __forceinline__ df unit_count(float c, float w_hi, float w_lo) {
  const float p = __fmul_rn(c, w_hi);
  return fast_two_sum(p, fmaf(c, w_lo, fmaf(c, w_hi, -p)));
}

}  // namespace covgpu
