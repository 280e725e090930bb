// Vertical line (column) preconditioner for the FP32 inner solve (not in reference).
//
// The scaled operator A~ = I + couplings is dominated by its vertical couplings (dz << dx, dy:
// the axis-2 transmissibility is (dx/dz)^2 = 400x the lateral one on 1 m x 1 m x 5 cm cells),
// which is what makes Jacobi-PCG slow.  M = blockdiag over columns of the tridiagonal part of A~
// (its axis-2 couplings and unit diagonal) is SPD whenever A~ is (principal submatrices), and
// M^-1 r is one Thomas solve per column.  Each thread owns one column; cells of a column are
// n0*n1 apart, so a warp's loads at one level are consecutive (coalesced).
//
// Factorisation (once per solve, FP64, stored FP32): M_col = L D L^T with unit lower
// bidiagonal L,
//   d_0 = 1,  l_k = a2_{k-1} / d_{k-1},  d_k = 1 - l_k a2_{k-1}      (l_0 = 0)
// Solve: y_k = r_k - l_k y_{k-1};  u_k = y_k / d_k;  z_k = u_k - l_{k+1} z_{k+1}.
// r . z = sum_k y_k^2 / d_k = sum_k y_k u_k comes out of the forward sweep, so the backward
// sweep needs neither r nor a reduction and can form the next search direction in place.
//
// PCG iteration (3 kernels, no separate direction kernel):
//   k32_spmv_v4 / k32_spmv : w = A~ p,  alpha = (r.z) / (p.w)
//   k32_line_fwd<true>     : x += alpha p, r -= alpha w, u = D^-1 L^-1 r, r.z, r.r, test, beta
//   k32_line_bwd           : z = L^-T u and p = z + beta p in the same sweep
#pragma once

#include "internal.h"
#include "reduce.cuh"

namespace fg {

constexpr int kLineBatch = 4;  // levels whose loads are issued together

__global__ void k_line_factor(const double* __restrict__ a2, float* __restrict__ lk,
                              float* __restrict__ dinv, int ncol, int nz) {
  const size_t sk = (size_t)ncol;
  for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < ncol;
       col += gridDim.x * blockDim.x) {
    size_t c = (size_t)col;
    double d = 1.0;
    lk[c] = 0.0f;
    dinv[c] = 1.0f;
    for (int k = 1; k < nz; ++k) {
      c += sk;
      const double a = a2[c - sk];
      const double l = a / d;
      d = 1.0 - l * a;
      // an SPD operator keeps d in (0, 1]; a non-positive pivot (an operator that is not
      // SPD) degrades that row to the Jacobi step instead of dividing by it
      if (!(d > 0.0)) d = 1.0;
      lk[c] = (float)l;
      dinv[c] = (float)(1.0 / d);
    }
  }
}

// Forward sweep.  UPDATE: first x += alpha p, r -= alpha w (the CG update of this iteration);
// then u = D^-1 L^-1 r and the sums r.z (as y.u) and r.r.  The last block runs the inner
// convergence test (on ||r||) and forms beta = (r.z)_new / (r.z)_old.  Without UPDATE it is
// the initial application: st->beta = r0.z0.
template <bool UPDATE>
__global__ void __launch_bounds__(128) k32_line_fwd(float* __restrict__ x, float* __restrict__ r,
                                                    const float* __restrict__ p,
                                                    const float* __restrict__ w,
                                                    const float* __restrict__ lk,
                                                    const float* __restrict__ dinv,
                                                    float* __restrict__ u, int ncol, int nz,
                                                    CgDevState* st, double* partials) {
  if (st->status) return;
  const float a = UPDATE ? (float)st->a : 0.0f;
  // the first update writes x = alpha p (x is not initialised)
  const bool xfirst = UPDATE && st->iter == 0;
  const size_t sk = (size_t)ncol;
  Kahan32 rz, rr;
  for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < ncol;
       col += gridDim.x * blockDim.x) {
    float y = 0.0f;
    for (int k0 = 0; k0 < nz; k0 += kLineBatch) {
      float rv[kLineBatch], lv[kLineBatch], dv[kLineBatch], xv[kLineBatch], pv[kLineBatch],
          wv[kLineBatch];
#pragma unroll
      for (int q = 0; q < kLineBatch; ++q) {
        if (k0 + q < nz) {
          const size_t c = (size_t)col + sk * (k0 + q);
          rv[q] = r[c];
          lv[q] = lk[c];
          dv[q] = dinv[c];
          if (UPDATE) {
            xv[q] = xfirst ? 0.0f : x[c];
            pv[q] = p[c];
            wv[q] = w[c];
          }
        }
      }
#pragma unroll
      for (int q = 0; q < kLineBatch; ++q) {
        if (k0 + q < nz) {
          const size_t c = (size_t)col + sk * (k0 + q);
          float rk = rv[q];
          if (UPDATE) {
            x[c] = fmaf(a, pv[q], xv[q]);
            rk = fmaf(-a, wv[q], rk);
            r[c] = rk;
          }
          y = fmaf(-lv[q], y, rk);
          const float uk = y * dv[q];
          u[c] = uk;
          rz.add(y * uk);
          rr.add(rk * rk);
        }
      }
    }
  }
  double loc[2] = {rz.value(), rr.value()};
  double tot[2];
  if (!grid_sum<2>(loc, partials, &st->arrive[2], tot)) return;
  if (flat_tid() == 0) {
    const double rzn = tot[0];
    const double rn = sqrt(tot[1]);
    if (!UPDATE) {
      st->beta = rzn;
      st->bcoef = 0.0;
      if (!(rzn > 0.0)) st->status = rzn == 0.0 ? kConvergedAtol : kDivergedIndefinitePc;
      return;
    }
    st->dp = rn;
    st->iter += 1;
    if (isnan(rn) || isnan(rzn)) {
      st->status = kDivergedNanOrInf;
    } else if (rn <= st->ttol) {
      st->status = kConvergedRtol;
    } else if (st->iter >= st->max_it) {
      st->status = kDivergedIts;
    } else if (!(rzn > 0.0)) {
      st->status = kDivergedIndefinitePc;
    } else {
      st->bcoef = rzn / st->beta;
      st->beta = rzn;
      st->its = st->iter + 1;
    }
  }
}

// Backward sweep z = L^-T u fused with the direction update p = z + beta p (p = z on the first
// iteration).
__global__ void __launch_bounds__(128) k32_line_bwd(const float* __restrict__ u,
                                                    const float* __restrict__ lk,
                                                    float* __restrict__ p, int ncol, int nz,
                                                    const CgDevState* st) {
  if (st->status) return;
  const float bc = (float)st->bcoef;
  const bool first = st->iter == 0;
  const size_t sk = (size_t)ncol;
  for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < ncol;
       col += gridDim.x * blockDim.x) {
    float z = 0.0f, lnext = 0.0f;
    for (int k0 = nz - 1; k0 >= 0; k0 -= kLineBatch) {
      float uv[kLineBatch], lv[kLineBatch], pv[kLineBatch];
#pragma unroll
      for (int q = 0; q < kLineBatch; ++q) {
        if (k0 - q >= 0) {
          const size_t c = (size_t)col + sk * (k0 - q);
          uv[q] = u[c];
          lv[q] = lk[c];
          pv[q] = first ? 0.0f : p[c];
        }
      }
#pragma unroll
      for (int q = 0; q < kLineBatch; ++q) {
        if (k0 - q >= 0) {
          const size_t c = (size_t)col + sk * (k0 - q);
          z = fmaf(-lnext, z, uv[q]);
          lnext = lv[q];
          p[c] = first ? z : fmaf(bc, pv[q], z);
        }
      }
    }
  }
}

// z (+)= M^-1 r for the flexible-CG path (u is scratch).
__global__ void __launch_bounds__(128) k32_line_apply(const float* __restrict__ r,
                                                      const float* __restrict__ lk,
                                                      const float* __restrict__ dinv,
                                                      float* __restrict__ u,
                                                      float* __restrict__ z, int ncol, int nz,
                                                      int accumulate) {
  const size_t sk = (size_t)ncol;
  for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < ncol;
       col += gridDim.x * blockDim.x) {
    float y = 0.0f;
    size_t c = (size_t)col;
    for (int k = 0; k < nz; ++k, c += sk) {
      y = fmaf(-lk[c], y, r[c]);
      u[c] = y * dinv[c];
    }
    float zz = 0.0f, lnext = 0.0f;
    for (int k = nz - 1; k >= 0; --k) {
      c -= sk;
      zz = fmaf(-lnext, zz, u[c]);
      lnext = lk[c];
      z[c] = accumulate ? z[c] + zz : zz;
    }
  }
}

}  // namespace fg
