// Float-float ("double-float") arithmetic on the FP32 pipe, for the kernels that would otherwise
// be bound by GB300's FP64 pipe (not in reference).
//
// Measured on GB300 per SM and clock: 117 FP32 FMAs, 1.6 FP64 FMAs, 1.7 double->float
// conversions (they run on the FP64 unit), 8.9 float->double conversions, 26 int->float
// conversions, 61 integer multiply-adds.  A value held as an unevaluated sum hi + lo of two
// floats carries about 48 significant bits, and its sums and products cost 3-20 FP32
// instructions, several times cheaper than one FP64 instruction here.  Doubles enter through an
// integer split of their bit pattern (no double->float conversion) and leave as
// (double)hi + (double)lo.
//
// The building blocks are the error-free transformations TwoSum (Knuth), Fast2Sum (Dekker) and
// TwoProd with an FMA, composed as in M. Joldes, J.-M. Muller, V. Popescu, "Tight and rigorous
// error bounds for basic building blocks of double-word arithmetic", ACM TOMS 44(2), 2017
// (relative error bounds in units of u^2 = 2^-48 stated per routine).  Every operation uses the
// round-to-nearest intrinsics, which the compiler never contracts or reassociates.
//
// The elementary functions follow the table-driven method of P. T. P. Tang (ACM TOMS 15(2),
// 1989 and 16(4), 1990) with float-float tables (ff32_tables.h): exp reduces to |r| <=
// ln2/256 with 128 entries, log to |r| <= 2^-9 with 256 entries; the leading polynomial terms
// are float-float, the tail (below 2^-24 of the result) is plain FP32.  Absolute error of log
// and relative error of exp are a few 2^-48 (bounds checked by tests/test_fastmath_gpu.py).
#pragma once

#include <cuda_runtime.h>

#include "ff32_tables.h"

namespace fg {

struct ff {
  float h, l;
};

__device__ __forceinline__ ff ff_make(float h, float l = 0.0f) {
  ff r;
  r.h = h;
  r.l = l;
  return r;
}

// s + e = a + b exactly
__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return ff_make(s, e);
}

// s + e = a + b exactly when |a| >= |b| (or a = 0)
__device__ __forceinline__ ff fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return ff_make(s, __fsub_rn(b, __fsub_rn(s, a)));
}

// p + e = a b exactly (barring underflow)
__device__ __forceinline__ ff two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return ff_make(p, __fmaf_rn(a, b, -p));
}

__device__ __forceinline__ ff ff_neg(ff a) { return ff_make(-a.h, -a.l); }

// exact scaling by a power of two
__device__ __forceinline__ ff ff_scale(ff a, float p2) {
  return ff_make(__fmul_rn(a.h, p2), __fmul_rn(a.l, p2));
}

// AccurateDWPlusDW (error <= 3u^2)
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const ff s = two_sum(a.h, b.h);
  const ff t = two_sum(a.l, b.l);
  const ff v = fast_two_sum(s.h, __fadd_rn(s.l, t.h));
  return fast_two_sum(v.h, __fadd_rn(t.l, v.l));
}

__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

// SloppyDWPlusDW: accurate (about 2u^2) when a and b have the same sign or |b| << |a|
__device__ __forceinline__ ff ff_add_fast(ff a, ff b) {
  const ff s = two_sum(a.h, b.h);
  return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}

// DWPlusFP (error <= 2u^2)
__device__ __forceinline__ ff ff_add_f(ff a, float b) {
  const ff s = two_sum(a.h, b);
  return fast_two_sum(s.h, __fadd_rn(a.l, s.l));
}

// DWTimesFP3 (error <= 2u^2)
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
  const ff c = two_prod(a.h, b);
  return fast_two_sum(c.h, __fmaf_rn(a.l, b, c.l));
}

// DWTimesDW3 (error <= 4u^2)
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const ff c = two_prod(a.h, b.h);
  const float t = __fmaf_rn(a.h, b.l, __fmul_rn(a.l, b.l));
  return fast_two_sum(c.h, __fadd_rn(c.l, __fmaf_rn(a.l, b.h, t)));
}

// ---- lean forms: no renormalisation -------------------------------------------------------
// For chains of sums and products whose end result is renormalised once.  Their results keep
// |lo| within a few ulp of hi when their inputs do, which the error bounds of the next lean
// operation allow for (a few 2^-48 relative, as the renormalised forms); a value that leaves
// float-float (ff_to_double, a comparison) passes through a renormalising operation first.
// A difference of nearly equal values is renormalised before it multiplies: its low word then
// holds most of its significant bits, which ff_mul_lean's FP32 cross term would round to 24
// (an error of 2^-48 of the operands instead of the difference; measured as 40 % more Krylov
// iterations in the late Picard solves of the heterogeneous-loam workload).

// a b: TwoProd of the leading words plus the two cross terms (a.l b.l, below 2^-46 of the
// product, is dropped)
__device__ __forceinline__ ff ff_mul_lean(ff a, ff b) {
  const ff c = two_prod(a.h, b.h);
  return ff_make(c.h, __fadd_rn(c.l, __fmaf_rn(a.l, b.h, __fmul_rn(a.h, b.l))));
}

// a - b: TwoSum of the leading words, the low words' difference added to its error term;
// antisymmetric, ff_dif_lean(a, b) = -ff_dif_lean(b, a) exactly (TwoSum's error is exact and
// rounding to nearest is symmetric)
__device__ __forceinline__ ff ff_dif_lean(ff a, ff b) {
  const ff s = two_sum(a.h, -b.h);
  return ff_make(s.h, __fadd_rn(s.l, __fsub_rn(a.l, b.l)));
}

// a + b
__device__ __forceinline__ ff ff_add_lean(ff a, ff b) {
  const ff s = two_sum(a.h, b.h);
  return ff_make(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}

// A running sum of float-float terms: the leading words are summed with TwoSum and every error
// term and low word is collected in one float, so the absolute error is a few 2^-48 of the
// largest term (as a chain of SloppyDWPlusDW, at 8 instead of 11 instructions a term).
struct FfSum {
  float s, e;
};

__device__ __forceinline__ FfSum ff_sum_of(ff x) {
  FfSum q;
  q.s = x.h;
  q.e = x.l;
  return q;
}

__device__ __forceinline__ void ff_sum_add(FfSum& q, ff x) {
  const ff t = two_sum(q.s, x.h);
  q.s = t.h;
  q.e = __fadd_rn(q.e, __fadd_rn(t.l, x.l));
}

// the sum, renormalised (TwoSum of the two words)
__device__ __forceinline__ ff ff_sum_value(const FfSum& q) { return two_sum(q.s, q.e); }

__device__ __forceinline__ ff ff_sqr(ff a) {
  const ff c = two_prod(a.h, a.h);
  return fast_two_sum(c.h, __fmaf_rn(__fmul_rn(2.0f, a.h), a.l, c.l));
}

// DWDivDW2 with a correctly rounded reciprocal in place of the float division (error a few
// 2^-46): q = a.h/b.h, then one correction from the float-float remainder a - q b
__device__ __forceinline__ ff ff_div(ff a, ff b) {
  const float r = __frcp_rn(b.h);
  const float q = __fmul_rn(a.h, r);
  const ff qb = ff_mul_f(b, q);
  const float pi = __fsub_rn(a.h, qb.h);
  const float d = __fadd_rn(pi, __fsub_rn(a.l, qb.l));
  return fast_two_sum(q, __fmul_rn(d, r));
}

// The rare cases of the conversions below, kept out of line: inlined, the compiler evaluates
// them for every value (predicated) and their FP64 instructions then bound the kernels.
static __device__ __noinline__ ff ff_from_double_rare(double x) {
  const float h = (float)x;
  return ff_make(h, isfinite(h) ? (float)(x - (double)h) : 0.0f);
}

static __device__ __noinline__ double ff_to_double_rare(ff a) { return (double)a.h + (double)a.l; }

// double -> float-float without a double->float conversion: hi = the top 24 bits of the
// significand (truncated), lo = the next 29 bits (rounded to 24 by the int->float conversion),
// 0 <= |lo| < ulp(hi), lo of the sign of hi.  ff_from_double renormalises the pair;
// ff_from_double_lean leaves it as a lean operand.  Values below 2^-100 or above 2^127 in
// magnitude (and 0, inf, NaN) take the conversion instructions instead.
__device__ __forceinline__ ff ff_split_bits(int hx, int lx, int E) {
  const int sign = hx & (int)0x80000000;
  const float h = __int_as_float(sign | ((E - 1023 + 127) << 23) | ((hx & 0x000fffff) << 3) |
                                 (int)((unsigned)lx >> 29));
  // remainder r * 2^(E - 1075), r < 2^29: (float)r * 2^-52 * 2^(E - 1023)
  const float p2 = __int_as_float((E - 1023 + 127) << 23);
  float l = __fmul_rn(__fmul_rn(__uint2float_rn((unsigned)lx & 0x1fffffffu), 0x1p-52f), p2);
  l = __int_as_float(__float_as_int(l) | sign);
  return ff_make(h, l);
}

__device__ __forceinline__ ff ff_from_double_lean(double x) {
  const int hx = __double2hiint(x);
  const int E = (hx >> 20) & 0x7ff;
  // one unsigned compare for 1023 - 100 <= E <= 1023 + 127
  if ((unsigned)(E - (1023 - 100)) > 227u) return ff_from_double_rare(x);
  return ff_split_bits(hx, __double2loint(x), E);
}

__device__ __forceinline__ ff ff_from_double(double x) {
  const int hx = __double2hiint(x);
  const int E = (hx >> 20) & 0x7ff;
  if ((unsigned)(E - (1023 - 100)) > 227u) return ff_from_double_rare(x);
  const ff r = ff_split_bits(hx, __double2loint(x), E);
  return fast_two_sum(r.h, r.l);
}

// x rounded to a float (to nearest, ties away from zero) without a double->float conversion:
// the significand's leading 24 bits plus the first dropped bit, added as an integer (a carry
// moves into the exponent).  |x| below the normal float range gives a signed zero; huge, inf and
// NaN x take the conversion instruction.
__device__ __forceinline__ float ff_hi_of(double x) {
  const int hx = __double2hiint(x);
  const int E = (hx >> 20) & 0x7ff;
  if (E < 1023 - 126) return __int_as_float(hx & (int)0x80000000);
  if (E > 1023 + 126) return ff_from_double_rare(x).h;
  const unsigned lx = (unsigned)__double2loint(x);
  return __int_as_float(((hx & (int)0x80000000) | ((E - 1023 + 127) << 23) |
                         ((hx & 0x000fffff) << 3) | (int)(lx >> 29)) +
                        (int)((lx >> 28) & 1u));
}

// float-float -> double without an FP64 addition: the two significands are added as integers
// (a.l shifted to the double's last place, truncated there), so the result is within an ulp of
// the double nearest to a.h + a.l.  Valid for a normal a.h and a normalised pair.
__device__ __forceinline__ double ff_to_double_core(ff a) {
  const int bh = __float_as_int(a.h);
  const int eh = (bh >> 23) & 0xff;
  // a.h = mh 2^(eh-150): the double's significand M = mh 2^29 in units of 2^(eh-179)
  unsigned long long M = (unsigned long long)((bh & 0x007fffff) | 0x00800000) << 29;
  const int bl = __float_as_int(a.l);
  const int el = (bl >> 23) & 0xff;
  // a.l = ml 2^(el-150) (subnormal: ml 2^-149) = ml 2^(el-eh+29) units; a normalised pair
  // (|a.l| <= ulp(a.h)/2) has el <= eh - 24, so the shift below is at most 5 to the left
  const unsigned ml = el ? (unsigned)((bl & 0x007fffff) | 0x00800000) : (unsigned)(bl & 0x007fffff);
  const int d = eh - (el ? el : 1) - 29;
  const unsigned long long L = d <= 0 ? (unsigned long long)ml << min(-d, 29)
                                      : (d < 32 ? (unsigned long long)(ml >> d) : 0ull);
  M = ((bh ^ bl) < 0) ? M - L : M + L;
  int e = eh - 127 + 1023;
  if (M < (1ull << 52)) {  // a.h a power of two and a.l of the opposite sign
    M <<= 1;
    e -= 1;
  }
  const unsigned long long bits = ((unsigned long long)((unsigned)bh & 0x80000000u) << 32) |
                                  ((unsigned long long)e << 52) | (M & ((1ull << 52) - 1));
  return __longlong_as_double((long long)bits);
}

// Zero, subnormal, infinite and NaN a.h take the conversion instructions.
__device__ __forceinline__ double ff_to_double(ff a) {
  const int eh = (__float_as_int(a.h) >> 23) & 0xff;
  if (eh == 0 || eh == 0xff) return ff_to_double_rare(a);
  return ff_to_double_core(a);
}

// ---- branch-free conversions --------------------------------------------------------------
// For kernels whose values stay within the normal float range: no out-of-line call and no
// branch (the special cases are selected), so that the calling kernel keeps no call site.
// Outside that range they flush: |x| < 2^-126 (and 0) gives a signed zero, an absolute error
// below 2^-126; |x| >= 2^128, inf and NaN give NaN.

// as ff_from_double_lean
__device__ __forceinline__ ff ff_from_double_nb(double x) {
  const int hx = __double2hiint(x);
  const int lx = __double2loint(x);
  const int fe = ((hx >> 20) & 0x7ff) - (1023 - 127);  // the float's biased exponent
  const int sign = hx & (int)0x80000000;
  float h = __int_as_float(sign | (fe << 23) | ((hx & 0x000fffff) << 3) |
                           (int)((unsigned)lx >> 29));
  const float p2 = __int_as_float((fe & 0xff) << 23);
  float l = __fmul_rn(__fmul_rn(__uint2float_rn((unsigned)lx & 0x1fffffffu), 0x1p-52f), p2);
  l = __int_as_float(__float_as_int(l) | sign);
  if (fe < 1) {
    h = __int_as_float(sign);
    l = h;
  }
  if (fe > 254) {
    h = __int_as_float(0x7fc00000);
    l = 0.0f;
  }
  return ff_make(h, l);
}

// as ff_hi_of (|x| >= 2^127 gives NaN)
__device__ __forceinline__ float ff_hi_of_nb(double x) {
  const int hx = __double2hiint(x);
  const int fe = ((hx >> 20) & 0x7ff) - (1023 - 127);
  const unsigned lx = (unsigned)__double2loint(x);
  float r = __int_as_float(((hx & (int)0x80000000) | (fe << 23) | ((hx & 0x000fffff) << 3) |
                            (int)(lx >> 29)) +
                           (int)((lx >> 28) & 1u));
  if (fe < 1) r = __int_as_float(hx & (int)0x80000000);
  if (fe > 253) r = __int_as_float(0x7fc00000);
  return r;
}

// as ff_to_double for a normalised pair; a.h zero or subnormal gives a signed zero, infinite
// or NaN a.h gives NaN
__device__ __forceinline__ double ff_to_double_nb(ff a) {
  const int bh = __float_as_int(a.h);
  const int eh = (bh >> 23) & 0xff;
  double r = ff_to_double_core(a);
  const unsigned long long zero = (unsigned long long)((unsigned)bh & 0x80000000u) << 32;
  if (eh == 0) r = __longlong_as_double((long long)zero);
  if (eh == 0xff) r = __longlong_as_double(0x7ff8000000000000ll);
  return r;
}

static __device__ __noinline__ double f2d_scaled_rare(float f, int k) {
  return ldexp((double)f, k);
}

// (double)f * 2^k exactly, without the FP64 pipe (GB300 converts float -> double there): the
// float's exponent re-biased by 1023 - 127 + k, its significand moved to the top of the double's.
// Zero gives a signed zero; subnormal, infinite and NaN f, and results outside the normal
// double range, take the conversion instruction.
__device__ __forceinline__ double f2d_scaled(float f, int k) {
  const unsigned b = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
  if ((b << 1) == 0u) return __longlong_as_double((long long)sign);
  const int e = (int)((b >> 23) & 0xffu);
  const int E = e + (1023 - 127) + k;
  if (e == 0 || e == 0xff || E <= 0 || E >= 0x7ff) return f2d_scaled_rare(f, k);
  return __longlong_as_double((long long)(sign | ((unsigned long long)E << 52) |
                                          ((unsigned long long)(b & 0x007fffffu) << 29)));
}

// k with 2^(k-1) <= v < 2^k for a positive normal double v (0 otherwise), clamped to
// [-120, 120] so that 2^-k is a normal float
__device__ __host__ __forceinline__ int pow2_above(double v) {
  union {
    double d;
    unsigned long long u;
  } w;
  w.d = v;
  const unsigned long long b = w.u;
  const int E = (int)((b >> 52) & 0x7ffu);
  if ((b >> 63) || E == 0 || E == 0x7ff) return 0;
  const int k = E - 1022;
  return k < -120 ? -120 : (k > 120 ? 120 : k);
}

// 2^k as a double and as a float (|k| <= 120)
__device__ __host__ __forceinline__ double pow2d(int k) {
  union {
    unsigned long long u;
    double d;
  } w;
  w.u = (unsigned long long)(k + 1023) << 52;
  return w.d;
}
__device__ __host__ __forceinline__ float pow2f_of(int k) {
  union {
    unsigned u;
    float f;
  } w;
  w.u = (unsigned)(k + 127) << 23;
  return w.f;
}

// a >= 1 (a normalised)
__device__ __forceinline__ bool ff_ge1(ff a) { return a.h > 1.0f || (a.h == 1.0f && a.l >= 0.0f); }

// ---- elementary functions ----------------------------------------------------------------

// e^r - 1 for |r| <= ln2/256 (|r| <= 0.0028): r + r^2/2 in float-float, r^3/6 + r^4/24 + r^5/120
// in FP32 (below 3.3e-9; its rounding below 1e-15 absolute: a few u^2 relative to e^r)
__device__ __forceinline__ ff ff_expm1_small(ff r) {
  const ff r2 = ff_sqr(r);
  float t = __fmaf_rn(r.h, 1.0f / 120.0f, 1.0f / 24.0f);
  t = __fmaf_rn(t, r.h, 1.0f / 6.0f);
  t = __fmul_rn(__fmul_rn(t, r.h), r2.h);
  return ff_add_f(ff_add_fast(r, ff_scale(r2, 0.5f)), t);
}

// the same series with r^3/6 in float-float as well (FP32 tail below 2.2e-12): a few u^2
// relative to e^r - 1 itself, as expm1 needs
__device__ __forceinline__ ff ff_expm1_small_rel(ff r) {
  const ff r2 = ff_sqr(r);
  const ff r3 = ff_mul(r2, r);
  float t = __fmaf_rn(r.h, 1.0f / 120.0f, 1.0f / 24.0f);
  t = __fmul_rn(__fmul_rn(t, r.h), r3.h);
  // 1/6 = 0x1.555556p-3 - 0x1.555556p-28 (float-float)
  const ff s3 = ff_add_f(ff_mul(r3, ff_make(0x1.555556p-3f, -0x1.555556p-28f)), t);
  return ff_add_fast(ff_add_fast(r, ff_scale(r2, 0.5f)), s3);
}

// x = k ln2/128 + r, |r| <= ln2/256 (about), k = 128 m + j; returns r, sets k
__device__ __forceinline__ ff ff_exp_reduce(ff x, int* k_out) {
  const float kf = rintf(__fmul_rn(x.h, kFfInvLn2x128));
  *k_out = (int)kf;
  // x.h - k C1 is exact (k C1 has at most 24 bits and lies within a factor of x.h's range)
  const float rh = __fmaf_rn(-kf, kFfLn2x128C1, x.h);
  const ff p = two_prod(kf, kFfLn2x128C2);
  const ff s = two_sum(rh, -p.h);
  const ff s2 = two_sum(s.h, x.l);
  const float lo = __fsub_rn(__fsub_rn(__fadd_rn(s.l, s2.l), p.l), __fmul_rn(kf, kFfLn2x128C3));
  return two_sum(s2.h, lo);
}

// 2^m as a float, -126 <= m <= 127
__device__ __forceinline__ float ff_pow2f(int m) { return __int_as_float((m + 127) << 23); }

// e^x, |x| <= 87 (e^x = 0 below -87, inf above 88)
__device__ __forceinline__ ff ff_exp(ff x) {
  if (!(x.h <= 88.0f)) return x.h != x.h ? x : ff_make(__int_as_float(0x7f800000));
  if (!(x.h >= -87.0f)) return ff_make(0.0f);
  int k;
  const ff r = ff_exp_reduce(x, &k);
  const ff q = ff_expm1_small(r);
  const float2 T = kFfExp2Tab[k & 127];
  const ff t = ff_make(T.x, T.y);
  const ff e = ff_add_fast(t, ff_mul(t, q));  // |T q| <= 0.003 T
  return ff_scale(e, ff_pow2f(k >> 7));
}

// e^x - 1: the series for |x| <= ln2/256; T_j 2^m - 1 (exact) + 2^m (T_j q + T_lo) up to
// |x| <= ln 2; e^x - 1 directly beyond (|result| >= 1/2: no cancellation)
__device__ __forceinline__ ff ff_expm1(ff x) {
  const float ax = fabsf(x.h);
  if (ax <= 0.0027f) return ff_expm1_small_rel(x);
  if (!(ax <= 0.6931f)) {
    const ff e = ff_exp(x);
    return ff_add_f(e, -1.0f);
  }
  int k;
  const ff r = ff_exp_reduce(x, &k);
  const ff q = ff_expm1_small_rel(r);
  const float2 T = kFfExp2Tab[k & 127];
  const float sc = ff_pow2f(k >> 7);
  const float a = __fmaf_rn(T.x, sc, -1.0f);  // exact: T.x 2^m in [1/2, 2]
  // 2^m (T q + (T - T.x)): the table's remainder to a third float, since the result can be
  // 200 times smaller than T and would inherit the float-float table's 2^-49 relative error
  const ff rest = ff_scale(
      ff_add(ff_mul(ff_make(T.x, T.y), q), fast_two_sum(T.y, kFfExp2Lo2[k & 127])), sc);
  return ff_add(ff_make(a), rest);
}

// ln(1 + r) for |r| <= 2^-9: r - r^2/2 in float-float, r^3/3 - r^4/4 + r^5/5 in FP32
__device__ __forceinline__ ff ff_log1p_small(ff r) {
  const ff r2 = ff_sqr(r);
  float t = __fmaf_rn(r.h, 0.2f, -0.25f);
  t = __fmaf_rn(t, r.h, 1.0f / 3.0f);
  t = __fmul_rn(__fmul_rn(t, r.h), r2.h);
  return ff_add_f(ff_add_fast(r, ff_scale(r2, -0.5f)), t);
}

// ln x, x > 0: x = 2^e m, c = centre of m's 1/256 interval, ln x = e ln2 + ln c + ln(1 + r),
// r = (m - c)/c, |r| <= 2^-9
__device__ __forceinline__ ff ff_log(ff x) {
  int bits = __float_as_int(x.h);
  if (bits <= 0 || bits >= 0x7f800000) {  // zero, negative, infinite, NaN
    if (x.h == 0.0f) return ff_make(-__int_as_float(0x7f800000));
    if (x.h != x.h || x.h > 0.0f) return x;
    return ff_make(__int_as_float(0x7fc00000));
  }
  int e = 0;
  if (bits < 0x00800000) {  // subnormal hi: normalise
    x = ff_scale(x, 0x1p24f);
    bits = __float_as_int(x.h);
    e = -24;
  }
  e += (bits >> 23) - 127;
  const int j = (bits >> 15) & 255;
  const float m = __int_as_float((bits & 0x007fffff) | 0x3f800000);
  const float c = __int_as_float(0x3f800000 | (j << 15) | (1 << 14));
  // x.l 2^-e (e <= 127: the scale is a normal float for e >= -126; below, x.l is negligible)
  const float xl = e >= -126 ? __fmul_rn(x.l, ff_pow2f(-e)) : 0.0f;
  const ff d = two_sum(__fsub_rn(m, c), xl);  // m - c exact
  const float4 L = kFfLogTab[j];
  const ff r = ff_mul(d, ff_make(L.x, L.y));
  const ff p = ff_log1p_small(r);
  // e ln2 = e L1 (exact) + e L2 (exact as a product pair) + e L3
  const float ef = (float)e;
  const ff el2 = two_prod(ef, kFfLn2L2);
  // the sums need absolute accuracy only (every logarithm here feeds an exponential): the
  // double-word additions whose error is a few u^2 of the operands serve
  ff a = ff_add_fast(ff_make(__fmul_rn(ef, kFfLn2L1)),
                     ff_make(el2.h, __fmaf_rn(ef, kFfLn2L3, el2.l)));
  a = ff_add_fast(a, ff_make(L.z, L.w));
  return ff_add_fast(a, p);
}

// ln(1 + t), t >= 0 (or t > -1)
__device__ __forceinline__ ff ff_log1p(ff t) {
  if (fabsf(t.h) <= 0x1p-9f) return ff_log1p_small(t);
  const ff s = two_sum(1.0f, t.h);
  return ff_log(fast_two_sum(s.h, __fadd_rn(s.l, t.l)));
}

}  // namespace fg
