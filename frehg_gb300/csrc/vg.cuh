// van Genuchten / Mualem constitutive relations on the device (FP64).
//
// Same relations and formula order as VanGenuchten (src/re/VanGenuchten.hpp:18-137); the
// conductivity is returned relative to Ks (kr = K/Ks, with the reference's cap K <= Ks and
// K = Ks above zero head (VG) or above the air-entry head (MVG)), so one evaluation per cell
// serves the three directional conductivities Ks_x/y/z * kr.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/frehg_gb300.h"
#include "fastmath64.cuh"
#include "ff32.cuh"

namespace fg {

// One soil class with the constants the relations reuse precomputed (same values the
// reference recomputes per call: m = 1 - 1/n, 1/m, 1/n).
struct SoilClass {
  double alpha, n, ths, thr, Ksx, Ksy, Ksz, Ss, aev;
  double m, inv_m, inv_n, inv_ths;
  int32_t use_vg, use_mvg;
  // float-float copies (hi, lo) for vg_constit_ff: alpha, n, m, theta_r, theta_s - theta_r,
  // n m (theta_s - theta_r); for the float-float Picard kernels: Ks_x, Ks_y, Ks_z, Ss/theta_s
  float ff_alpha[2], ff_n[2], ff_m[2], ff_thr[2], ff_dth[2], ff_nmdth[2];
  float ff_ks[3][2], ff_ss_ths[2];
  int32_t ks_iso;  // Ks_x == Ks_y == Ks_z
};

// SoilClass of one parameter block (host)
inline SoilClass make_soil_class(const frehg_soil_params& s) {
  SoilClass k;
  k.alpha = s.alpha;
  k.n = s.n;
  k.ths = s.theta_s;
  k.thr = s.theta_r;
  k.Ksx = s.Ks_x;
  k.Ksy = s.Ks_y;
  k.Ksz = s.Ks_z;
  k.Ss = s.Ss;
  k.aev = s.air_entry;
  k.m = 1.0 - 1.0 / s.n;
  k.inv_m = 1.0 / k.m;
  k.inv_n = 1.0 / s.n;
  k.inv_ths = 1.0 / s.theta_s;
  k.use_vg = s.use_vg;
  k.use_mvg = s.use_mvg;
  auto split = [](double v, float* out) {
    out[0] = (float)v;
    out[1] = (float)(v - (double)out[0]);
  };
  split(k.alpha, k.ff_alpha);
  split(k.n, k.ff_n);
  split(k.m, k.ff_m);
  split(k.thr, k.ff_thr);
  split(k.ths - k.thr, k.ff_dth);
  split(k.n * k.m * (k.ths - k.thr), k.ff_nmdth);
  split(k.Ksx, k.ff_ks[0]);
  split(k.Ksy, k.ff_ks[1]);
  split(k.Ksz, k.ff_ks[2]);
  split(k.Ss / k.ths, k.ff_ss_ths);
  k.ks_iso = (k.Ksx == k.Ksy && k.Ksx == k.Ksz) ? 1 : 0;
  return k;
}

// Soil of one cell after the per-cell overrides (not in reference: continuous Ks / alpha).
struct CellSoil {
  double alpha, n, ths, thr, Ss, aev, m, inv_m, inv_n, inv_ths;
  double Ksx, Ksy, Ksz;
  int32_t use_vg, use_mvg;
};

// Where the soil of a cell comes from: class table + optional class-id map (per column or per
// cell, uint8) + optional per-cell Ks and alpha fields.
struct SoilView {
  const SoilClass* cls = nullptr;
  const uint8_t* cid = nullptr;
  const double* Ks = nullptr;
  const double* alpha = nullptr;
  int cid3d = 0;
  // Picard scheme: van Genuchten theta(h) without the air-entry switch (theta = theta_s only
  // for h > 0).  The reference's switch (VanGenuchten.hpp:38-41) is a jump in theta of up to
  // 0.008 (sand) at h = air_entry that a Picard iteration cannot converge across; K and C of
  // the VG branch already switch at h = 0.
  int continuous_theta = 0;
};

__device__ __forceinline__ CellSoil soil_of(const SoilView& v, size_t cell, size_t col) {
  const int id = v.cid ? (int)v.cid[v.cid3d ? cell : col] : 0;
  const SoilClass& k = v.cls[id];
  CellSoil s;
  s.alpha = v.alpha ? v.alpha[cell] : k.alpha;
  s.n = k.n;
  s.ths = k.ths;
  s.thr = k.thr;
  s.Ss = k.Ss;
  s.aev = (v.continuous_theta && !k.use_mvg) ? 0.0 : k.aev;
  s.m = k.m;
  s.inv_m = k.inv_m;
  s.inv_n = k.inv_n;
  s.inv_ths = k.inv_ths;
  if (v.Ks) {
    const double K = v.Ks[cell];
    s.Ksx = K;
    s.Ksy = K;
    s.Ksz = K;
  } else {
    s.Ksx = k.Ksx;
    s.Ksy = k.Ksy;
    s.Ksz = k.Ksz;
  }
  s.use_vg = k.use_vg;
  s.use_mvg = k.use_mvg;
  return s;
}

// VanGenuchten::wcm (VanGenuchten.hpp:22-29)
__device__ __forceinline__ double vg_wcm(const CellSoil& s) {
  if (s.use_mvg) return s.thr + (s.ths - s.thr) * pow(1.0 + pow(fabs(s.aev) * s.alpha, s.n), s.m);
  return s.ths;
}

// waterContentFromHead (VanGenuchten.hpp:31-47)
__device__ __forceinline__ double vg_theta(const CellSoil& s, double h) {
  double wc;
  if (s.use_vg) {
    const double wcm_val = vg_wcm(s);
    const double se = pow(1.0 + pow(fabs(s.alpha * h), s.n), -s.m);
    if (h > s.aev)
      wc = s.ths;
    else
      wc = s.thr + (wcm_val - s.thr) * se;
  } else {
    wc = s.thr + (s.ths - s.thr) * exp(0.1634 * h);
  }
  if (wc > s.ths) wc = s.ths;
  if (wc < s.thr) wc = s.thr;
  return wc;
}

// headFromWaterContent (VanGenuchten.hpp:50-65).  The reference's
// pow(pow(q, 1/m) - 1, 1/n) with q = (wcm - thr)/(theta - thr) is evaluated as
// exp(log(expm1(log(q)/m)) / n): q^{1/m} - 1 without cancellation near saturation, and
// exp/log instead of the (costlier, extended-precision) FP64 pow.
__device__ __forceinline__ double vg_head(const CellSoil& s, double wc) {
  const double eps = 1.0e-7;
  if (s.use_vg) {
    const double wcm_val = vg_wcm(s);
    double theta = wc;
    if (theta - s.thr < eps) theta = s.thr + eps;
    if (theta < s.ths) {
      const double q = (wcm_val - s.thr) / (theta - s.thr);
      const double x = fexpm1(s.inv_m * flog(q));
      return -(1.0 / s.alpha) * fexp(s.inv_n * flog(x));
    }
    return 0.0;
  }
  return log((wc - s.thr) / (s.ths - s.thr)) / 0.1634;
}

// specificMoistureCapacity (VanGenuchten.hpp:68-81)
__device__ __forceinline__ double vg_capacity(const CellSoil& s, double h) {
  const double mm = s.m;
  const double wcm_val = vg_wcm(s);
  const double ah = fabs(s.alpha * h);
  const double nume = s.alpha * s.n * mm * (wcm_val - s.thr) * pow(ah, s.n - 1.0);
  const double deno = pow(1.0 + pow(ah, s.n), mm + 1.0);
  double c = nume / deno;
  if (s.use_mvg) {
    if (h > s.aev) c = 0.0;
  } else if (h > 0.0) {
    c = 0.0;
  }
  return c;
}

// conductivityFromHead / Ks (VanGenuchten.hpp:84-111)
__device__ __forceinline__ double vg_kr(const CellSoil& s, double h) {
  if (!s.use_vg) return exp(0.1634 * h);
  const double mm = s.m;
  const double se = pow(1.0 + pow(fabs(s.alpha * h), s.n), -mm);
  double kr;
  if (s.use_mvg) {
    const double wcm_val = vg_wcm(s);
    const double nume =
        1.0 - pow(1.0 - pow(se * (s.ths - s.thr) / (wcm_val - s.thr), s.inv_m), mm);
    const double deno = 1.0 - pow(1.0 - pow((s.ths - s.thr) / (wcm_val - s.thr), s.inv_m), mm);
    kr = (deno == 0.0) ? 1.0 : pow(se, 0.5) * pow(nume / deno, 2.0);
  } else {
    kr = pow(se, 0.5) * pow(1.0 - pow(1.0 - pow(se, s.inv_m), mm), 2.0);
  }
  if (kr > 1.0) kr = 1.0;
  if (s.use_mvg) {
    if (h > s.aev) kr = 1.0;
  } else if (h > 0.0) {
    kr = 1.0;
  }
  return kr;
}

// kr, theta and C at one head from one set of transcendental calls (VG, not MVG).  With
// L = ln|alpha h|, t = e^{nL} = |alpha h|^n, u = ln(1 + t):
//   se = (1+t)^-m = e^{-mu},  se^{1/m} = 1/(1+t),  1 - se^{1/m} = t/(1+t),
//   (1 - se^{1/m})^m = e^{m(nL - u)},  kr = e^{-mu/2} (1 - e^{m(nL-u)})^2,
//   C = alpha n m (ths - thr) |alpha h|^{n-1} (1+t)^{-(m+1)} = alpha n m (ths-thr) t se / (|alpha h| (1+t)).
// The same relations as the reference's pow() forms (VanGenuchten.hpp:31-111), evaluated with
// 2 logarithms, 2 exponentials and one expm1 instead of 11 pow() calls (se = e^{-mu/2}
// squared); 1 - e^{x} is formed as -expm1(x) so no digits cancel when the soil is dry.  The
// elementary functions are the table-driven ones of fastmath64.cuh (fewer FP64 instructions).  The caps and the saturated branches are the
// reference's.  MVG and the exponential model use the reference forms above.
struct Constit {
  double kr, theta, cap;
};

template <bool WANT_THETA, bool WANT_CAP>
__device__ __forceinline__ Constit vg_constit(const CellSoil& s, double h) {
  Constit r;
  if (!s.use_vg || s.use_mvg) {
    r.kr = vg_kr(s, h);
    r.theta = WANT_THETA ? vg_theta(s, h) : 0.0;
    r.cap = WANT_CAP ? vg_capacity(s, h) : 0.0;
    return r;
  }
  const double mm = s.m;
  const double ah = fabs(s.alpha * h);
  const double L = flog(ah);
  const double nL = s.n * L;
  const double t = fexp(nL);
  const double u = flog1p(t);
  const double mu = mm * u;
  // kr; se = e^{-mu} = (e^{-mu/2})^2 serves theta
  const double one_minus = -fexpm1(mm * (nL - u));
  const double se_half = fexp(-0.5 * mu);
  double kr = se_half * (one_minus * one_minus);
  if (kr > 1.0) kr = 1.0;
  if (h > 0.0) kr = 1.0;
  r.kr = kr;
  if (WANT_THETA) {
    double wc;
    if (h > s.aev)
      wc = s.ths;
    else
      wc = s.thr + (s.ths - s.thr) * (se_half * se_half);
    if (wc > s.ths) wc = s.ths;
    if (wc < s.thr) wc = s.thr;
    r.theta = wc;
  } else {
    r.theta = 0.0;
  }
  if (WANT_CAP) {
    // |alpha h|^{n-1} (1+t)^{-(m+1)} = t * se / (|alpha h| (1 + t)): one division, no exp
    double c = ah > 0.0 ? s.alpha * s.n * mm * (s.ths - s.thr) *
                              (t * (se_half * se_half) / (ah * (1.0 + t)))
                        : 0.0;
    if (h > 0.0) c = 0.0;
    r.cap = c;
  } else {
    r.cap = 0.0;
  }
  return r;
}

// vg_constit in float-float arithmetic on the FP32 pipe (ff32.cuh): the same relations, caps and
// saturated branches, about 48 significant bits per operation instead of 53 for K and theta,
// FP32 for C (which enters only the matrix diagonal), for the VG branch (MVG and the
// exponential model take vg_constit).  Where the soil is drier than |alpha h| = 1,
// (1 - se^{1/m})^m is formed from ln(1 + 1/t) rather than from the difference nL - u, so dry
// cells keep the relative accuracy of K that the FP64 forms (and the reference's pow forms)
// lose there.  k: the cell's class (its
// float-float constants); alpha: the cell's alpha, float-float (class value or per-cell
// field); aev: the head above which theta = theta_s.  Heads h >= 0 (and |alpha h| too small for the float range)
// give kr = 1, C = 0 and theta_s exactly, as the FP64 forms do.
template <bool WANT_THETA, bool WANT_CAP>
__device__ __forceinline__ Constit vg_constit_ff(const SoilClass& k, ff alpha, double aev,
                                                 double h) {
  Constit r;
  r.kr = 1.0;
  r.theta = k.ths;
  r.cap = 0.0;
  const ff ah = ff_mul(alpha, ff_from_double_nb(-h));  // |alpha h| for h < 0
  if (!(ah.h > 0.0f)) return r;
  const ff n = ff_make(k.ff_n[0], k.ff_n[1]);
  const ff m = ff_make(k.ff_m[0], k.ff_m[1]);
  const ff L = ff_log(ah);
  const ff nL = ff_mul(n, L);
  const ff t = ff_exp(nL);
  // u = ln(1 + t) and y = m (nL - u) = m ln(t / (1 + t)); for t > 1 (drier than |alpha h| = 1)
  // as u = nL + v, y = -m v with v = ln(1 + 1/t), so that y keeps its relative accuracy where
  // nL and u nearly cancel (the FP64 forms lose about log10(t) digits there)
  ff u, y;
  if (t.h > 1.0f) {
    const ff v = ff_log1p(ff_div(ff_make(1.0f), t));
    u = ff_add_fast(nL, v);
    y = ff_neg(ff_mul(m, v));
  } else {
    u = ff_log1p(t);
    y = ff_mul(m, ff_sub(nL, u));
  }
  const ff mu = ff_mul(m, u);
  const ff one_minus = ff_neg(ff_expm1(y));
  const ff se_half = ff_exp(ff_scale(mu, -0.5f));
  const ff kr = ff_mul(se_half, ff_sqr(one_minus));
  r.kr = ff_ge1(kr) ? 1.0 : ff_to_double_nb(kr);
  const ff se = ff_sqr(se_half);
  if (WANT_THETA && !(h > aev)) {
    // theta_r + (theta_s - theta_r) se with se in [0, 1]: theta_s where se rounds to >= 1
    const ff wc = ff_add_fast(ff_make(k.ff_thr[0], k.ff_thr[1]),
                              ff_mul(ff_make(k.ff_dth[0], k.ff_dth[1]), se));
    r.theta = ff_ge1(se) ? k.ths : ff_to_double_nb(wc);
  }
  if (WANT_CAP) {
    // alpha n m (ths - thr) t se / (|alpha h| (1 + t)) from the leading floats: C enters only
    // the matrix diagonal, which the float-float Picard path forms in FP32
    const float num = alpha.h * k.ff_nmdth[0] * (t.h * se.h);
    r.cap = (double)__fdividef(num, ah.h * (1.0f + t.h));
  }
  return r;
}

// dKdwc (VanGenuchten.hpp:114-136)
__device__ __forceinline__ double vg_dKdwc(const CellSoil& s, double wc, double Ks) {
  double theta = wc;
  if (theta > 0.9999 * s.ths && theta < s.ths) theta = 0.9999 * s.ths;
  const double mm = s.m;
  const double se = (theta - s.thr) / (s.ths - s.thr);
  if (s.use_mvg) {
    const double wcm_val = vg_wcm(s);
    const double c2 = (s.ths - s.thr) / (wcm_val - s.thr);
    const double c1 = 1.0 / pow(1.0 - pow(1.0 - pow(c2, s.inv_m), mm), 2.0);
    const double term0 = pow(1.0 - pow(c2 * se, s.inv_m), mm);
    const double term1 = 0.5 * c1 * Ks * pow(se, -0.5) * (1.0 - term0) * (1.0 - term0);
    const double term2 = 2.0 * c1 * Ks * c2 * pow(se, 0.5) * pow(c2 * se, s.inv_m - 1.0) *
                         (1.0 - term0) * pow(1.0 - pow(c2 * se, s.inv_m), mm - 1.0);
    return (term1 + term2) / (s.ths - s.thr);
  }
  const double term0 = pow(1.0 - pow(se, s.inv_m), mm);
  const double term1 = 0.5 * Ks * pow(se, -0.5) * (1.0 - term0) * (1.0 - term0);
  const double term2 = 2.0 * Ks * pow(se, (2.0 - mm) / (2.0 * mm)) * (1.0 - term0) *
                       pow(1.0 - pow(se, s.inv_m), mm - 1.0);
  return (term1 + term2) / (s.ths - s.thr);
}

}  // namespace fg
