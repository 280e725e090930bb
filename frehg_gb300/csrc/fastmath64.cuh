// Table-driven FP64 exponential and logarithm for the constitutive kernels (own
// implementation of the published method of P. T. P. Tang: "Table-driven implementation of the
// exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989, and
// "Table-driven implementation of the logarithm function ...", ACM TOMS 16(4), 1990).
//
// On GB300 the FP64 pipe runs at ~1/64 of the FP32 rate and the van Genuchten kernels are bound
// by it (ncu: 85 % FP64-pipe active, 1-9 % DRAM), so the instruction count of exp/log is their
// cost.  A 64-entry table of 2^(j/64) reduces exp to a degree-5 polynomial on |r| <= ln2/128,
// a 128-entry table of 1/c_j and ln(c_j) reduces log to a degree-7 polynomial on |r| <= 2^-8;
// both need about 12-16 FP64 instructions.  Accuracy against the CUDA math library is checked by
// tests/test_fastmath_gpu.py (bound stated there).  Tables: fastmath64_tables.h, generated by
// gen_fastmath_tables.py.
#pragma once

#include <cuda_runtime.h>

#include "fastmath64_tables.h"

namespace fg {

constexpr double kInvLn2x64 = 0x1.71547652b82fep+6;  // 64 / ln 2
constexpr double kLn2x64Hi = 0x1.62e42p-7;           // ln2/64 to 21 bits: k * hi is exact
constexpr double kLn2x64Lo = 0x1.fdf473de6af28p-28;  // ln2/64 - hi
constexpr double kLn2Hi = 0x1.62e42p-1;              // ln 2 to 21 bits: e * hi is exact
constexpr double kLn2Lo = 0x1.fdf473de6af28p-22;     // ln 2 - hi
constexpr double kRoundShift = 0x1.8p52;             // x + this rounds x to an integer

// 2^m for -1022 <= m <= 1023 from its exponent field
__device__ __forceinline__ double fm_pow2i(int m) {
  return __hiloint2double((m + 1023) << 20, 0);
}

// Argument reduction shared by exp and expm1: x = (64 m + j) ln2/64 + r, |r| <= ln2/128, and
// p = e^r - 1 by its Taylor polynomial of degree 5 (truncation below 4e-17 relative).
struct FmExpParts {
  int j, m;
  double r, p;
};

__device__ __forceinline__ FmExpParts fm_exp_reduce(double x) {
  const double t = fma(x, kInvLn2x64, kRoundShift);
  const int k = __double2loint(t);  // the low word of the shifted value holds round(x*64/ln2)
  const double kd = t - kRoundShift;
  double r = fma(-kd, kLn2x64Hi, x);
  r = fma(-kd, kLn2x64Lo, r);
  double q = fma(r, 1.0 / 120.0, 1.0 / 24.0);
  q = fma(q, r, 1.0 / 6.0);
  q = fma(q, r, 0.5);
  FmExpParts s;
  s.r = r;
  s.p = fma(q, r * r, r);
  s.j = k & 63;
  s.m = k >> 6;  // arithmetic shift: floor(k / 64)
  return s;
}

__device__ __forceinline__ double fexp(double x) {
  if (!(fabs(x) <= 708.0)) {
    if (x != x) return x;
    if (x > 709.782712893384) return INFINITY;
    if (x < -745.1332191019412) return 0.0;
  }
  const FmExpParts s = fm_exp_reduce(x);
  const double th = kExp2Tab[s.j][0], tl = kExp2Tab[s.j][1];
  const double e = th + fma(th, s.p, tl);  // 2^(j/64) e^r
  if (s.m >= -1022 && s.m <= 1023) return e * fm_pow2i(s.m);
  const int m1 = s.m / 2;  // results near overflow or subnormal: scale in two steps
  return (e * fm_pow2i(m1)) * fm_pow2i(s.m - m1);
}

// e^x - 1: Taylor polynomial for |x| < 1/64; for 1/64 <= |x| <= ln 2 the reduced form
// (2^m T_hi - 1) + 2^m (T_hi p + T_lo) with p = e^r - 1 to degree 8, whose first term is
// exact (2^m T_hi in [1/2, 2]);
// beyond, e^x - 1 directly (|result| >= 1/2, no cancellation).
__device__ __forceinline__ double fexpm1(double x) {
  const double ax = fabs(x);
  if (ax < 0x1p-6) {
    double q = fma(x, 1.0 / 40320.0, 1.0 / 5040.0);
    q = fma(q, x, 1.0 / 720.0);
    q = fma(q, x, 1.0 / 120.0);
    q = fma(q, x, 1.0 / 24.0);
    q = fma(q, x, 1.0 / 6.0);
    q = fma(q, x, 0.5);
    return fma(q, x * x, x);
  }
  if (!(ax <= 0.6931471805599453)) return fexp(x) - 1.0;
  const FmExpParts s = fm_exp_reduce(x);
  const double th = kExp2Tab[s.j][0], tl = kExp2Tab[s.j][1];
  const double sc = fm_pow2i(s.m);
  // the result can be as small as 1/64, so e^r - 1 needs degree 8 here (truncation below
  // 1e-23 absolute) rather than exp's degree 5
  const double r = s.r;
  double q = fma(r, 1.0 / 40320.0, 1.0 / 5040.0);
  q = fma(q, r, 1.0 / 720.0);
  q = fma(q, r, 1.0 / 120.0);
  q = fma(q, r, 1.0 / 24.0);
  q = fma(q, r, 1.0 / 6.0);
  q = fma(q, r, 0.5);
  const double p = fma(q, r * r, r);
  return (th * sc - 1.0) + sc * fma(th, p, tl);
}

// ln(1 + f) for |f| < 1/64 by its Taylor polynomial of degree 11 (truncation below 2^-70
// relative); f exact.
__device__ __forceinline__ double fm_log1p_small(double f) {
  double q = fma(f, -1.0 / 11.0, 1.0 / 10.0);
  q = fma(q, f, -1.0 / 9.0);
  q = fma(q, f, 1.0 / 8.0);
  q = fma(q, f, -1.0 / 7.0);
  q = fma(q, f, 1.0 / 6.0);
  q = fma(q, f, -1.0 / 5.0);
  q = fma(q, f, 1.0 / 4.0);
  q = fma(q, f, -1.0 / 3.0);
  q = fma(q, f, 0.5);
  return fma(-q, f * f, f);
}

// ln x: x = 2^e m, m in [1, 2), c = centre of m's 1/128 interval, r = (m - c)/c,
// ln x = e ln2 + ln c + ln(1 + r) with |r| <= 2^-8; near x = 1 the series on x - 1 directly.
__device__ __forceinline__ double flog(double x) {
  int hx = __double2hiint(x);
  int lx = __double2loint(x);
  int e = 0;
  if (hx < 0x00100000 || hx >= 0x7ff00000) {  // zero, negative, subnormal, infinite, NaN
    if (x != x || x == INFINITY) return x;
    if (x == 0.0) return -INFINITY;
    if (x < 0.0) return __longlong_as_double(0x7ff8000000000000ll);
    x *= 0x1p54;  // subnormal: normalise
    hx = __double2hiint(x);
    lx = __double2loint(x);
    e = -54;
  }
  const double f1 = x - 1.0;
  if (fabs(f1) < 0x1p-6) return fm_log1p_small(f1);
  e += (hx >> 20) - 1023;
  const int j = (hx >> 13) & 127;
  const double m = __hiloint2double((hx & 0x000fffff) | 0x3ff00000, lx);
  const double c = __hiloint2double(0x3ff00000 | (j << 13) | (1 << 12), 0);
  const double r = (m - c) * kLogTab[j][0];  // m - c is exact (Sterbenz)
  double q = fma(r, 1.0 / 7.0, -1.0 / 6.0);
  q = fma(q, r, 1.0 / 5.0);
  q = fma(q, r, -0.25);
  q = fma(q, r, 1.0 / 3.0);
  q = fma(q, r, -0.5);
  const double ed = (double)e;
  const double hi = fma(ed, kLn2Hi, kLogTab[j][1]);
  const double lo = fma(ed, kLn2Lo, kLogTab[j][2]);
  return hi + (r + fma(q, r * r, lo));
}

// ln(1 + t), t > -1: the series for |t| < 1/64; else ln(s) with s = 1 + t plus the rounding
// of s, (t - (s - 1))/s (Goldberg), whose size (an ulp of s at most) needs only a float 1/s.
__device__ __forceinline__ double flog1p(double t) {
  if (fabs(t) < 0x1p-6) return fm_log1p_small(t);
  if (!(t < 1e300)) return flog(t);
  const double s = 1.0 + t;
  const double corr = (t - (s - 1.0)) * (double)__frcp_rn((float)s);
  return flog(s) + corr;
}

}  // namespace fg
