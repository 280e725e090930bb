// Mixed-precision Krylov path (not in reference): FP32 Jacobi-PCG under FP64 iterative
// refinement.
//
// The operator is the same unit-diagonal scaled stencil as the FP64 path (A~ = D^-1/2 A D^-1/2,
// b~ = D^-1/2 b); its couplings are rounded once to FP32.  Each refinement sweep
//   1. forms the true residual r~ = b~ - A~ x~ in FP64 (FP64 couplings) and its unscaled norm
//      ||b - A x|| = ||r~ / s||; stops when ||b - A x|| <= ir_rtol * ||b||;
//   2. solves A~32 e = fp32(r~ 2^-k) with FP32 CG to a relative reduction inner_rtol (dot
//      products in FP32 with Kahan compensation per thread, combined in FP64 across
//      threads/blocks; 2^-k, a power of two near 1/||r~||, keeps FP32 away from underflow);
//   3. updates x~ += 2^k e in FP64.
// The FP32 inner iteration moves 56 B/cell (vs 120 B/cell in FP64) and leaves the FP64 pipe,
// the limiter of the FP64 path on GB300, idle.  Convergence is always to the FP64 true
// residual, so the inner precision changes the iteration count, not the accuracy.
#include "ff32.cuh"
#include "internal.h"
#include "krylov_kernels.cuh"
#include "line.cuh"
#include "reduce.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace fg {

// The inner state after the line preconditioner's first application, z0 = M^-1 r0, as
// k32_line_fwd<false> leaves it: beta = r0 . z0, no direction yet.
__device__ __forceinline__ void line_first_state(CgDevState* in, double rz) {
  in->beta = rz;
  in->bcoef = 0.0;
  if (!(rz > 0.0)) in->status = rz == 0.0 ? kConvergedAtol : kDivergedIndefinitePc;
}

// r~ = s b - A~ x~ (FP64); sums of r~^2 (scale of the inner system),
// (r~/s)^2 = (sq r~)^2 for the true residual (sq = 1/s) and b^2 for ||b||.  The last block
// runs the refinement test.  The inner solution e needs no zeroing: the inner solve's first
// update writes it.
// FIRST (the first sweep, x~ = 0): r~ = s b without the stencil product, kept in rres for
// k_ir_scale (x~ is not read: the first k_ir_update writes it), and the b^2 sum that ||b||
// needs (with x~ = 0 the true residual is b itself).  Later sweeps write the next inner
// right-hand side themselves and form the stencil product in FP64: the residual is a
// difference of nearly equal terms, and the refinement converges only as far as this product
// is accurate (a float-float form, 2^-48, was both slower here and short of 1e-12 on
// ill-conditioned systems).
// (Applying the line preconditioner to the new right-hand side in the same column march, as
// k_prep_ff does for the first sweep, made this kernel slower by more than the separate
// k32_line_fwd<false> takes.)
template <bool FIRST, bool INV_S = false>
__global__ void __launch_bounds__(256) k_ir_residual(
    const double* __restrict__ a0, const double* __restrict__ a1, const double* __restrict__ a2,
    const double* __restrict__ s, const double* __restrict__ sq, const double* __restrict__ b,
    double* __restrict__ x, double* __restrict__ rres, int n0, int n1, int n2, int planes,
    int tiles, CgDevState* ir, double* partials, double ir_rtol,
    float* __restrict__ rfo = nullptr, CgDevState* in = nullptr, double inner_rtol = 0.0) {
  if (ir->status) return;
  const int t0 = (n0 + 31) / 32;
  const size_t s01 = (size_t)n0 * n1;
  double v[3] = {0.0, 0.0, 0.0};
  if (FIRST) {
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
      const int i0 = (tile % t0) * 32 + threadIdx.x;
      const int i1 = (tile / t0) * 8 + threadIdx.y;
      if (i0 >= n0 || i1 >= n1) continue;
      const int kb = blockIdx.y * planes, ke = min(n2, kb + planes);
      size_t c = (size_t)i0 + (size_t)n0 * i1 + s01 * kb;
      for (int k = kb; k < ke; ++k, c += s01) {
        const double bc = b[c];
        const double r = s[c] * bc;
        rres[c] = r;
        v[0] = fma(r, r, v[0]);
        v[2] = fma(bc, bc, v[2]);
      }
    }
    v[1] = v[2];
  } else {
    // the sums of squares in FP32 (compensated), after scaling by the previous sweep's norms,
    // which keeps the terms far from the FP32 range limits: they only set the inner scale and
    // the stopping test, and the FP64 pipe stays with the stencil product
    // the right-hand side's scale a power of two (2^(k-1) <= previous ||r~|| < 2^k)
    const float sig0 = pow2f_of(-pow2_above(ir->a));
    const double rs1 = ir->ir_rnorm;
    const float sig1 = (float)(1.0 / rs1);
    Kahan32 k0, k1;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
      const int i0 = (tile % t0) * 32 + threadIdx.x;
      const int i1 = (tile / t0) * 8 + threadIdx.y;
      if (i0 >= n0 || i1 >= n1) continue;
      const int kb = blockIdx.y * planes, ke = min(n2, kb + planes);
      size_t c = (size_t)i0 + (size_t)n0 * i1 + s01 * kb;
      for (int k = kb; k < ke; ++k, c += s01) {
        double ax = x[c];
        if (i0 > 0) ax = fma(a0[c - 1], x[c - 1], ax);
        if (i0 + 1 < n0) ax = fma(a0[c], x[c + 1], ax);
        if (i1 > 0) ax = fma(a1[c - n0], x[c - n0], ax);
        if (i1 + 1 < n1) ax = fma(a1[c], x[c + n0], ax);
        if (k > 0) ax = fma(a2[c - s01], x[c - s01], ax);
        if (k + 1 < n2) ax = fma(a2[c], x[c + s01], ax);
        const double r = fma(s[c], b[c], -ax);
        const float rf = ff_hi_of(r);
        // sq r~ = r~ / s (INV_S: s holds floats and sq is not stored)
        const float sqc = INV_S ? __frcp_rn(ff_hi_of(s[c])) : ff_hi_of(sq[c]);
        const float q0 = rf * sig0, q1 = rf * sqc * sig1;
        rfo[c] = q0;  // the next inner solve's right-hand side, r~ / rs0 (rs0 = 2^k)
        k0.add(q0 * q0);
        k1.add(q1 * q1);
      }
    }
    v[0] = k0.value();
    v[1] = k1.value() * rs1 * rs1;
  }
  double tot[3];
  if (!grid_sum<3>(v, partials, &ir->arrive[0], tot)) return;
  if (flat_tid() == 0) {
    const double rn = sqrt(tot[1]);
    if (ir->ir_its == 0) ir->ir_bnorm = sqrt(tot[2]);
    ir->ir_rnorm = rn;
    ir->dp = rn;
    // ||r~||; later sweeps summed (r~ / rs0)^2, the FP32 right-hand side they wrote
    const double rs0 = FIRST ? 1.0 : pow2d(pow2_above(ir->a));
    ir->a = sqrt(tot[0]) * rs0;
    if (isnan(rn) || isinf(rn)) {
      ir->status = kDivergedNanOrInf;
    } else if (rn <= fmax(ir_rtol * ir->ir_bnorm, ir->atol) || tot[0] == 0.0) {
      ir->status = rn < ir->atol ? kConvergedAtol : kConvergedRtol;
    }
    if (!FIRST && ir->status == 0) {
      // the inner CG state, as k_ir_scale sets it, for the right-hand side r~ / rs0
      ir->rscale = rs0;
      in->beta = tot[0];
      in->rnorm0 = sqrt(tot[0]);
      in->ttol = inner_rtol * in->rnorm0;
      in->iter = 0;
      in->its = 0;
      in->dpi = 0.0;
      in->status = 0;
    }
  }
}

// Inner right-hand side rf = fp32(r~ 2^-k), 2^(k-1) <= ||r~|| < 2^k: norm in [1/2, 1), so FP32
// products cannot underflow however small the refinement residual is.  The last block
// initialises the inner CG state.
__global__ void k_ir_scale(const double* __restrict__ rres, float* __restrict__ rf, size_t n,
                           CgDevState* ir, CgDevState* in, double* partials,
                           double inner_rtol) {
  if (ir->status) return;
  // 2^-k with 2^(k-1) <= ||r~|| < 2^k: the right-hand side's norm in [1/2, 1), and the scale
  // a power of two (exact, and the refinement update forms rscale e without FP64 arithmetic)
  const int k = pow2_above(ir->a);
  const float sig = pow2f_of(-k);
  Kahan32 acc;
  // the FP32 right-hand side from the residual's leading 24 bits (integer split: GB300's
  // double->float conversion runs on the FP64 pipe); four cells per step, 16-byte accesses
  const size_t gid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const double2* r2 = reinterpret_cast<const double2*>(rres);
  float4* f4 = reinterpret_cast<float4*>(rf);
  for (size_t q = gid; q < n / 4; q += stride) {
    const double2 lo = r2[2 * q], hi = r2[2 * q + 1];
    const float4 v = make_float4(ff_hi_of(lo.x) * sig, ff_hi_of(lo.y) * sig,
                                 ff_hi_of(hi.x) * sig, ff_hi_of(hi.y) * sig);
    f4[q] = v;
    acc.add(v.x * v.x);
    acc.add(v.y * v.y);
    acc.add(v.z * v.z);
    acc.add(v.w * v.w);
  }
  for (size_t c = (n & ~(size_t)3) + gid; c < n; c += stride) {
    const float r32 = ff_hi_of(rres[c]) * sig;
    rf[c] = r32;
    acc.add(r32 * r32);
  }
  double loc[1] = {acc.value()};
  double tot[1];
  if (!grid_sum<1>(loc, partials, &in->arrive[0], tot)) return;
  if (flat_tid() == 0) {
    ir->rscale = pow2d(k);
    in->beta = tot[0];
    in->rnorm0 = sqrt(tot[0]);
    in->ttol = inner_rtol * in->rnorm0;
    in->iter = 0;
    in->its = 0;
    in->dpi = 0.0;
    in->status = tot[0] == 0.0 ? kConvergedAtol : 0;
  }
}

__global__ void k32_p(const float* __restrict__ r, float* __restrict__ p, size_t n,
                      const CgDevState* st) {
  if (st->status) return;
  const float bc = (float)st->bcoef;
  const bool first = st->iter == 0;
  const size_t gid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const float4* r4 = reinterpret_cast<const float4*>(r);
  float4* p4 = reinterpret_cast<float4*>(p);
  for (size_t q = gid; q < n / 4; q += stride) {
    const float4 rv = r4[q];
    float4 pv;
    if (first) {
      pv = rv;
    } else {
      pv = p4[q];
      pv.x = fmaf(bc, pv.x, rv.x);
      pv.y = fmaf(bc, pv.y, rv.y);
      pv.z = fmaf(bc, pv.z, rv.z);
      pv.w = fmaf(bc, pv.w, rv.w);
    }
    p4[q] = pv;
  }
  if (gid < (n & 3)) {
    const size_t c = (n & ~(size_t)3) + gid;
    p[c] = first ? r[c] : fmaf(bc, p[c], r[c]);
  }
}

__global__ void __launch_bounds__(256) k32_spmv(const float* __restrict__ a0,
                                                const float* __restrict__ a1,
                                                const float* __restrict__ a2,
                                                const float* __restrict__ p, float* __restrict__ w,
                                                int n0, int n1, int n2, int planes, int tiles,
                                                CgDevState* st, double* partials) {
  if (st->status) return;
  const int t0 = (n0 + 31) / 32;
  Kahan32 acc;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int i0 = (tile % t0) * 32 + threadIdx.x;
    const int i1 = (tile / t0) * 8 + threadIdx.y;
    if (i0 >= n0 || i1 >= n1) continue;
    const size_t s01 = (size_t)n0 * n1;
    const int kb = blockIdx.y * planes, ke = min(n2, kb + planes);
    size_t c = (size_t)i0 + (size_t)n0 * i1 + s01 * kb;
    float pm = 0.0f, am = 0.0f;
    if (kb > 0) {
      pm = p[c - s01];
      am = a2[c - s01];
    }
    float pc = p[c];
    for (int k = kb; k < ke; ++k) {
      const float pp = (k + 1 < n2) ? p[c + s01] : 0.0f;
      const float ac = a2[c];
      float v = pc;
      if (i0 > 0) v = fmaf(a0[c - 1], p[c - 1], v);
      if (i0 + 1 < n0) v = fmaf(a0[c], p[c + 1], v);
      if (i1 > 0) v = fmaf(a1[c - n0], p[c - n0], v);
      if (i1 + 1 < n1) v = fmaf(a1[c], p[c + n0], v);
      v = fmaf(am, pm, v);
      v = fmaf(ac, pp, v);
      w[c] = v;
      acc.add(pc * v);
      pm = pc;
      pc = pp;
      am = ac;
      c += s01;
    }
  }
  double loc[1] = {acc.value()};
  double tot[1];
  if (!grid_sum<1>(loc, partials, &st->arrive[1], tot)) return;
  if (flat_tid() == 0) {
    const double dpi = tot[0];
    st->its = st->iter + 1;
    if (!(dpi > 0.0)) {  // breakdown (or NaN): end the inner solve, refinement decides
      st->status = isnan(dpi) ? kDivergedNanOrInf : kDivergedIndefiniteMat;
      return;
    }
    st->dpi = dpi;
    st->a = st->beta / dpi;
  }
}

// Vectorised variant for n0 % 4 == 0: a thread owns 4 consecutive cells along axis 0 (16-byte
// loads of p and the couplings); the axis-0 neighbours across threads come from warp shuffles,
// the axis-2 neighbours roll in registers while the thread marches through its planes.
__device__ __forceinline__ float4 ld4(const float* __restrict__ a, size_t c) {
  return *reinterpret_cast<const float4*>(a + c);
}

__global__ void __launch_bounds__(128) k32_spmv_v4(const float* __restrict__ a0,
                                                   const float* __restrict__ a1,
                                                   const float* __restrict__ a2,
                                                   const float* __restrict__ p,
                                                   float* __restrict__ w, int n0, int n1, int n2,
                                                   int planes, int tiles, CgDevState* st,
                                                   double* partials) {
  if (st->status) return;
  const int t0 = (n0 + 127) / 128;
  const int lane = threadIdx.x;
  const unsigned full = 0xffffffffu;
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  Kahan32 acc;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int i0 = (tile % t0) * 128 + lane * 4;
    const int i1 = (tile / t0) * 4 + threadIdx.y;
    const bool act = i0 < n0 && i1 < n1;
    const size_t s01 = (size_t)n0 * n1;
    const int kb = blockIdx.y * planes, ke = min(n2, kb + planes);
    size_t c = act ? (size_t)i0 + (size_t)n0 * i1 + s01 * kb : 0;
    float4 pc = act ? ld4(p, c) : z4;
    float4 pm = z4, am = z4;
    if (act && kb > 0) {
      pm = ld4(p, c - s01);
      am = ld4(a2, c - s01);
    }
    for (int k = kb; k < ke; ++k) {
      const bool up = act && k + 1 < n2;
      const float4 pp = up ? ld4(p, c + s01) : z4;
      const float4 A0 = act ? ld4(a0, c) : z4;
      const float4 A1 = act ? ld4(a1, c) : z4;
      const float4 A2 = act ? ld4(a2, c) : z4;
      const bool hs = act && i1 > 0, hn = act && i1 + 1 < n1;
      const float4 PS = hs ? ld4(p, c - n0) : z4;
      const float4 AS = hs ? ld4(a1, c - n0) : z4;
      const float4 PN = hn ? ld4(p, c + n0) : z4;
      float pl = __shfl_up_sync(full, pc.w, 1);
      float al = __shfl_up_sync(full, A0.w, 1);
      float pr = __shfl_down_sync(full, pc.x, 1);
      if (lane == 0) {
        const bool l = act && i0 > 0;
        pl = l ? p[c - 1] : 0.f;
        al = l ? a0[c - 1] : 0.f;
      }
      if (lane == 31) pr = (act && i0 + 4 < n0) ? p[c + 4] : 0.f;
      float4 v;
      v.x = pc.x;
      v.x = fmaf(al, pl, v.x);
      v.x = fmaf(A0.x, pc.y, v.x);
      v.y = fmaf(A0.x, pc.x, pc.y);
      v.y = fmaf(A0.y, pc.z, v.y);
      v.z = fmaf(A0.y, pc.y, pc.z);
      v.z = fmaf(A0.z, pc.w, v.z);
      v.w = fmaf(A0.z, pc.z, pc.w);
      v.w = fmaf(A0.w, pr, v.w);
      v.x = fmaf(AS.x, PS.x, v.x);
      v.y = fmaf(AS.y, PS.y, v.y);
      v.z = fmaf(AS.z, PS.z, v.z);
      v.w = fmaf(AS.w, PS.w, v.w);
      v.x = fmaf(A1.x, PN.x, v.x);
      v.y = fmaf(A1.y, PN.y, v.y);
      v.z = fmaf(A1.z, PN.z, v.z);
      v.w = fmaf(A1.w, PN.w, v.w);
      v.x = fmaf(am.x, pm.x, v.x);
      v.y = fmaf(am.y, pm.y, v.y);
      v.z = fmaf(am.z, pm.z, v.z);
      v.w = fmaf(am.w, pm.w, v.w);
      v.x = fmaf(A2.x, pp.x, v.x);
      v.y = fmaf(A2.y, pp.y, v.y);
      v.z = fmaf(A2.z, pp.z, v.z);
      v.w = fmaf(A2.w, pp.w, v.w);
      if (act) {
        *reinterpret_cast<float4*>(w + c) = v;
        acc.add(pc.x * v.x);
        acc.add(pc.y * v.y);
        acc.add(pc.z * v.z);
        acc.add(pc.w * v.w);
      }
      pm = pc;
      pc = pp;
      am = A2;
      c += s01;
    }
  }
  double loc[1] = {acc.value()};
  double tot[1];
  if (!grid_sum<1>(loc, partials, &st->arrive[1], tot)) return;
  if (flat_tid() == 0) {
    const double dpi = tot[0];
    st->its = st->iter + 1;
    if (!(dpi > 0.0)) {
      st->status = isnan(dpi) ? kDivergedNanOrInf : kDivergedIndefiniteMat;
      return;
    }
    st->dpi = dpi;
    st->a = st->beta / dpi;
  }
}

// launch geometry of k32_spmv_v4: (32 x 4) threads cover 128 x 4 cells of a plane
static StencilLaunch launch_v4(int n0, int n1, int n2) {
  StencilLaunch L;
  L.block = dim3(32, 4, 1);
  const long tiles = (long)((n0 + 127) / 128) * ((n1 + 3) / 4);
  const long target = (long)kNumSMs * 16 * 2;
  long z = target / (tiles > 0 ? tiles : 1);
  if (z < 1) z = 1;
  if (z > n2) z = n2;
  int planes = (int)((n2 + z - 1) / z);
  z = (n2 + planes - 1) / planes;
  long gx = tiles;
  const long cap = kMaxRedBlocks / z;
  if (gx > cap) gx = cap;
  L.planes = planes;
  L.tiles = (int)tiles;
  L.grid = dim3((unsigned)gx, (unsigned)z, 1);
  return L;
}

__global__ void k32_update(float* __restrict__ e, float* __restrict__ r,
                           const float* __restrict__ p, const float* __restrict__ w, size_t n,
                           CgDevState* st, double* partials) {
  if (st->status) return;
  const float a = (float)st->a;
  // the first iteration writes e = a p (e is not initialised)
  const bool first = st->iter == 0;
  Kahan32 acc;
  const size_t gid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  float4* e4 = reinterpret_cast<float4*>(e);
  float4* r4 = reinterpret_cast<float4*>(r);
  const float4* p4 = reinterpret_cast<const float4*>(p);
  const float4* w4 = reinterpret_cast<const float4*>(w);
  for (size_t q = gid; q < n / 4; q += stride) {
    float4 ev = first ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : e4[q], rv = r4[q];
    const float4 pv = p4[q], wv = w4[q];
    ev.x = fmaf(a, pv.x, ev.x);
    ev.y = fmaf(a, pv.y, ev.y);
    ev.z = fmaf(a, pv.z, ev.z);
    ev.w = fmaf(a, pv.w, ev.w);
    rv.x = fmaf(-a, wv.x, rv.x);
    rv.y = fmaf(-a, wv.y, rv.y);
    rv.z = fmaf(-a, wv.z, rv.z);
    rv.w = fmaf(-a, wv.w, rv.w);
    e4[q] = ev;
    r4[q] = rv;
    acc.add(rv.x * rv.x);
    acc.add(rv.y * rv.y);
    acc.add(rv.z * rv.z);
    acc.add(rv.w * rv.w);
  }
  if (gid < (n & 3)) {
    const size_t c = (n & ~(size_t)3) + gid;
    e[c] = fmaf(a, p[c], first ? 0.0f : e[c]);
    const float rc = fmaf(-a, w[c], r[c]);
    r[c] = rc;
    acc.add(rc * rc);
  }
  double loc[1] = {acc.value()};
  double tot[1];
  if (!grid_sum<1>(loc, partials, &st->arrive[2], tot)) return;
  if (flat_tid() == 0) {
    const double rr = tot[0];
    const double rn = sqrt(rr);
    st->dp = rn;
    st->iter += 1;
    if (isnan(rn)) {
      st->status = kDivergedNanOrInf;
    } else if (rn <= st->ttol) {
      st->status = kConvergedRtol;
    } else if (st->iter >= st->max_it) {
      st->status = kDivergedIts;
    } else {
      st->bcoef = rr / st->beta;
      st->beta = rr;
      st->its = st->iter + 1;
    }
  }
}

// x~ += rscale e (the inner system was solved for the residual divided by rscale); FIRST:
// x~ = rscale e (x~ was 0 and is not read).  The inner solve's first update writes e without
// reading it, so e holds nothing before it: an inner solve that stopped before its first
// iteration (in->iter == 0) contributes e = 0.  Four cells per step with 16-byte loads and
// stores (the buffers are whole cudaMalloc allocations: 256-byte aligned).
// rscale is a power of two 2^k: rscale e is formed by integer operations (f2d_scaled), which
// leaves FIRST without FP64 instructions and the others with one addition per cell.
template <bool FIRST>
__device__ __forceinline__ double ir_step(int k, float e, double x) {
  const double v = f2d_scaled(e, k);
  return FIRST ? v : x + v;
}

template <bool FIRST>
__global__ void k_ir_update(double* __restrict__ x, const float* __restrict__ e, size_t n,
                            const CgDevState* ir, const CgDevState* in) {
  const size_t gid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  if (in->iter == 0) {
    if (FIRST)
      for (size_t c = gid; c < n; c += stride) x[c] = 0.0;
    return;
  }
  const double rs = ir->rscale;
  const int scale = pow2_above(rs) - 1;  // rscale = 2^scale
  if (rs != pow2d(scale)) {  // not a power of two (no path sets one): FP64 arithmetic
    for (size_t c = gid; c < n; c += stride)
      x[c] = FIRST ? rs * (double)e[c] : fma(rs, (double)e[c], x[c]);
    return;
  }
  const float4* e4 = reinterpret_cast<const float4*>(e);
  double2* x2 = reinterpret_cast<double2*>(x);
  for (size_t q = gid; q < n / 4; q += stride) {
    const float4 ev = e4[q];
    double2 lo = make_double2(0.0, 0.0), hi = lo;
    if (!FIRST) {
      lo = x2[2 * q];
      hi = x2[2 * q + 1];
    }
    lo.x = ir_step<FIRST>(scale, ev.x, lo.x);
    lo.y = ir_step<FIRST>(scale, ev.y, lo.y);
    hi.x = ir_step<FIRST>(scale, ev.z, hi.x);
    hi.y = ir_step<FIRST>(scale, ev.w, hi.y);
    x2[2 * q] = lo;
    x2[2 * q + 1] = hi;
  }
  for (size_t c = (n & ~(size_t)3) + gid; c < n; c += stride)
    x[c] = ir_step<FIRST>(scale, e[c], FIRST ? 0.0 : x[c]);
}

__global__ void k_to_f32(const double* __restrict__ a0, const double* __restrict__ a1,
                         const double* __restrict__ a2, float* __restrict__ f0,
                         float* __restrict__ f1, float* __restrict__ f2, size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
       c += (size_t)gridDim.x * blockDim.x) {
    f0[c] = (float)a0[c];
    f1[c] = (float)a1[c];
    f2[c] = (float)a2[c];
  }
}

__global__ void k_zero64(double* __restrict__ x, size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
       c += (size_t)gridDim.x * blockDim.x)
    x[c] = 0.0;
}

// ---- flexible CG (FCG(1), Notay 2000) with a nonlinear preconditioner z = M(r) ----------
//   beta = -(z . A p_prev) / (p_prev . A p_prev);  p = z + beta p_prev;  alpha = (p . r)/(p . A p)
// k_fcg_beta forms beta from z . w_prev (w_prev = A p_prev still holds the previous SpMV);
// k_fcg_p forms p and p . r, stored as st->beta so that k32_spmv* yields alpha = (p.r)/(p.Ap).
__global__ void k_fcg_beta(const float* __restrict__ z, const float* __restrict__ w, size_t n,
                           CgDevState* st, double* partials) {
  if (st->status) return;
  Kahan32 acc;
  if (st->iter > 0)
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
         c += (size_t)gridDim.x * blockDim.x)
      acc.add(z[c] * w[c]);
  double loc[1] = {acc.value()};
  double tot[1];
  if (!grid_sum<1>(loc, partials, &st->arrive[3], tot)) return;
  if (flat_tid() == 0) st->bcoef = st->iter > 0 ? -tot[0] / st->dpi : 0.0;
}

__global__ void k_fcg_p(const float* __restrict__ z, float* __restrict__ p,
                        const float* __restrict__ r, size_t n, CgDevState* st, double* partials) {
  if (st->status) return;
  const float bc = (float)st->bcoef;
  const bool first = st->iter == 0;
  Kahan32 acc;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
       c += (size_t)gridDim.x * blockDim.x) {
    const float pv = first ? z[c] : fmaf(bc, p[c], z[c]);
    p[c] = pv;
    acc.add(pv * r[c]);
  }
  double loc[1] = {acc.value()};
  double tot[1];
  if (!grid_sum<1>(loc, partials, &st->arrive[4], tot)) return;
  if (flat_tid() == 0) st->beta = tot[0];
}

// z += r: the network supplies the correction on top of the (unit-diagonal) Jacobi step
__global__ void k_add_f32(float* __restrict__ z, const float* __restrict__ r, size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
       c += (size_t)gridDim.x * blockDim.x)
    z[c] += r[c];
}

// ------------------------------------------------------------------------------------------

int KrylovSolver::ensure32(size_t n) {
  if (n <= cap32 && xf) return FREHG_OK;
  cudaFree(xf);
  cudaFree(rf);
  cudaFree(pf);
  cudaFree(wf);
  xf = rf = pf = wf = nullptr;
  if (g32) {
    cudaGraphExecDestroy(g32);
    g32 = nullptr;
  }
  if (g32s) {
    cudaGraphExecDestroy(g32s);
    g32s = nullptr;
  }
  FG_CUDA(cudaMalloc(&xf, n * sizeof(float)));
  FG_CUDA(cudaMalloc(&rf, n * sizeof(float)));
  FG_CUDA(cudaMalloc(&pf, n * sizeof(float)));
  FG_CUDA(cudaMalloc(&wf, n * sizeof(float)));
  cudaFree(rres);
  rres = nullptr;
  FG_CUDA(cudaMalloc(&rres, n * sizeof(double)));
  FG_TRY(op32.alloc(n));
  if (!dst32) {
    FG_CUDA(cudaMalloc(&dst32, sizeof(CgDevState)));
    FG_CUDA(cudaMemset(dst32, 0, sizeof(CgDevState)));
    FG_TRY(alloc_mapped(reinterpret_cast<void**>(&hst32), sizeof(CgDevState)));
  }
  cap32 = n;
  return FREHG_OK;
}

// Scaling of a fresh operator for the mixed path in two passes (solves whose result is the
// solution itself): s = D^-1/2 with sq = D^1/2 in FP64 (d s^2 = 1 to rounding, as the
// refinement residual's unit diagonal assumes), then one pass per column that scales the
// couplings in place (FP64, for the refinement residual), writes their FP32 copies (leading 24
// bits, without a double->float conversion: GB300 runs those on the FP64 pipe) and, with the
// line preconditioner, the column factors
//   l_k = v2_{k-1} / d_{k-1},  d_k = 1 - l_k v2_{k-1}   (d_0 = 1)
// in float-float, stored as floats.  The float-float path's update solves take k_prep_ff.
__global__ void k_diag_rsqrt_sq(double* __restrict__ s, double* __restrict__ sq, size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
       c += (size_t)gridDim.x * blockDim.x) {
    const double d = s[c];
    const double dd = d == 0.0 ? 1.0 : d;  // PCJacobi replaces a zero diagonal entry by 1
    const double r = rsqrt(dd);
    s[c] = r;
    sq[c] = dd * r;
  }
}

__device__ __forceinline__ ff scaled_coupling64(double* a, size_t c, double sc, double sn) {
  const double v = a[c] * sc * sn;
  a[c] = v;
  return ff_make(ff_hi_of(v));
}

// the float-float path's scale factors are floats, and so are the couplings the float-float
// Picard assembly writes: a s_c s_n = a (p_h + p_l) with p = s_c s_n exact, one float-float by
// float product, stored in FP64 for the refinement residual
__device__ __forceinline__ ff scaled_coupling_f(float af, double* a, size_t c, float sc,
                                                float sn) {
  const ff v = ff_mul_f(two_prod(sc, sn), af);
  a[c] = ff_to_double(v);
  return v;
}

__global__ void __launch_bounds__(128) k_scale_mixed(double* __restrict__ a0,
                                                     double* __restrict__ a1,
                                                     double* __restrict__ a2,
                                                     const double* __restrict__ s,
                                                     float* __restrict__ f0,
                                                     float* __restrict__ f1,
                                                     float* __restrict__ f2,
                                                     float* __restrict__ lk,
                                                     float* __restrict__ dinv, int n0, int n1,
                                                     int n2, int line) {
  const int ncol = n0 * n1;
  const size_t sk = (size_t)ncol;
  const ff zero = ff_make(0.0f);
  for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < ncol;
       col += gridDim.x * blockDim.x) {
    const int i0 = col % n0, i1 = col / n0;
    ff inv_d = ff_make(1.0f), aprev = zero;
    size_t c = (size_t)col;
    double sc = s[c];
    for (int k = 0; k < n2; ++k, c += sk) {
      const double sb = (k + 1 < n2) ? s[c + sk] : 0.0;
      ff v0 = zero, v1 = zero, v2 = zero;
      if (i0 + 1 < n0) v0 = scaled_coupling64(a0, c, sc, s[c + 1]);
      else a0[c] = 0.0;
      if (i1 + 1 < n1) v1 = scaled_coupling64(a1, c, sc, s[c + n0]);
      else a1[c] = 0.0;
      if (k + 1 < n2) v2 = scaled_coupling64(a2, c, sc, sb);
      else a2[c] = 0.0;
      f0[c] = v0.h;
      f1[c] = v1.h;
      f2[c] = v2.h;
      if (line) {
        ff l = zero;
        if (k > 0) {
          l = ff_mul(aprev, inv_d);
          ff d = ff_add_f(ff_neg(ff_mul(l, aprev)), 1.0f);
          if (!(d.h > 1e-30f)) d = ff_make(1.0f);  // not SPD: that row falls back to Jacobi
          inv_d = ff_div(ff_make(1.0f), d);
        }
        lk[c] = l.h;
        dinv[c] = inv_d.h;
        aprev = v2;
      }
      sc = sb;
    }
  }
}

// The float-float path's preparation in one pass per column (update solves, ff_operator): the
// scale factors s = D^-1/2 rounded to FP32 (a similarity transform: any s applied consistently
// gives the same solution, and FP32 s make s_c s_n an exact float product; d s^2 is then 1 only
// to FP32 precision while the refinement takes it as 1, which perturbs the update, not the
// iterate's fixed point), formed from the diagonal by each thread for itself and its neighbours
// (the same rounding everywhere, so the diagonal stays in place) and written to s_out; the
// scaled couplings a s_c s_n in float-float and their FP32 copies; the line factors as in
// k_scale_mixed; and the first refinement sweep (x~ = 0): the inner right-hand side
// fp32(s b) 2^-e with its CG state (k_ir_scale's job) and the norms ||s b||, ||b|| and the
// stopping test (k_ir_residual<true>'s), all in FP32 arithmetic: the scale 2^-e comes from the
// previous solve's first residual, which keeps the scaled values and their squares far from
// the FP32 range limits (a power of two changes no rounding).  When a scaled sum of squares
// leaves [2^-60, 2^60] (the first solve, a jump in scale) the last block sets
// ir->rhs_rescale and the host runs k_ir_residual<true> and k_ir_scale instead (FP64).  The
// kernel has no FP64 arithmetic: GB300's FP64 pipe would bound it.
// This replaces k_diag_rsqrt_sq, k_scale_mixed, the first k_ir_residual and k_ir_scale: the
// diagonal, the couplings and b are read once.  The assembly wrote
// the diagonal (dg) and the unscaled couplings (f0-f2) as floats; f0-f2 are overwritten in
// place by the scaled FP32 copies, and the FP64 scaled couplings go to a0-a2.
__device__ __forceinline__ float scale_of(float d) { return rsqrtf(d == 0.0f ? 1.0f : d); }

__global__ void __launch_bounds__(128) k_prep_ff(
    double* __restrict__ a0, double* __restrict__ a1, double* __restrict__ a2,
    const float* __restrict__ dg, const double* __restrict__ b, double* __restrict__ s_out,
    float* __restrict__ f0,
    float* __restrict__ f1, float* __restrict__ f2, float* __restrict__ lk,
    float* __restrict__ dinv, int n0, int n1, int n2, int line, CgDevState* ir,
    double* partials, double ir_rtol, float* __restrict__ rf, CgDevState* in, int sig_exp,
    double inner_rtol, float* __restrict__ u) {
  const int ncol = n0 * n1;
  const size_t sk = (size_t)ncol;
  const ff zero = ff_make(0.0f);
  const float sig = pow2f_of(-sig_exp);
  Kahan32 kq, kb, kz;
  for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < ncol;
       col += gridDim.x * blockDim.x) {
    const int i0 = col % n0, i1 = col / n0;
    const bool hx = i0 + 1 < n0, hy = i1 + 1 < n1;
    ff inv_d = ff_make(1.0f), aprev = zero;
    float y = 0.0f;  // u != nullptr: forward substitution of the first right-hand side
    size_t c = (size_t)col;
    // level k's inputs are loaded one level ahead (two levels of loads in flight per thread)
    float sc = scale_of(dg[c]);
    float q0 = f0[c], q1 = f1[c], q2 = f2[c];
    float dx = hx ? dg[c + 1] : 1.0f, dy = hy ? dg[c + n0] : 1.0f;
    float dz = n2 > 1 ? dg[c + sk] : 1.0f;
    double bq = b[c];
    for (int k = 0; k < n2; ++k, c += sk) {
      const float e0 = q0, e1 = q1, e2 = q2, ex = dx, ey = dy, ez = dz;
      const double bc = bq;
      if (k + 1 < n2) {
        const size_t cn = c + sk;
        q0 = f0[cn];
        q1 = f1[cn];
        q2 = f2[cn];
        dx = hx ? dg[cn + 1] : 1.0f;
        dy = hy ? dg[cn + n0] : 1.0f;
        dz = k + 2 < n2 ? dg[cn + sk] : 1.0f;
        bq = b[cn];
      }
      const float sb = (k + 1 < n2) ? scale_of(ez) : 0.0f;
      s_out[c] = f2d_scaled(sc, 0);
      ff v0 = zero, v1 = zero, v2 = zero;
      if (hx) v0 = scaled_coupling_f(e0, a0, c, sc, scale_of(ex));
      else a0[c] = 0.0;
      if (hy) v1 = scaled_coupling_f(e1, a1, c, sc, scale_of(ey));
      else a1[c] = 0.0;
      if (k + 1 < n2) v2 = scaled_coupling_f(e2, a2, c, sc, sb);
      else a2[c] = 0.0;
      f0[c] = v0.h;
      f1[c] = v1.h;
      f2[c] = v2.h;
      ff l = zero;
      if (line) {
        if (k > 0) {
          l = ff_mul(aprev, inv_d);
          ff d = ff_add_f(ff_neg(ff_mul(l, aprev)), 1.0f);
          if (!(d.h > 1e-30f)) d = ff_make(1.0f);  // not SPD: that row falls back to Jacobi
          inv_d = ff_div(ff_make(1.0f), d);
        }
        lk[c] = l.h;
        dinv[c] = inv_d.h;
        aprev = v2;
      }
      // first sweep: x~ = 0 (the first k_ir_update writes x~ without reading it), r~ = s b,
      // kept only as its FP32 form r~ 2^-e (the inner right-hand side), with the sums of
      // squares of r~ 2^-e and b 2^-e (with x~ = 0 the true residual is b) compensated in FP32
      const float qb = ff_hi_of(bc) * sig;
      const float q = sc * qb;
      rf[c] = q;
      kq.add(q * q);
      kb.add(qb * qb);
      if (u) {  // the line preconditioner's first application (k32_line_fwd<false>)
        y = fmaf(-l.h, y, q);
        const float uk = y * inv_d.h;
        u[c] = uk;
        kz.add(y * uk);
      }
      sc = sb;
    }
  }
  double v[3] = {kq.value(), kb.value(), kz.value()};
  double tot[3];
  if (!grid_sum<3>(v, partials, &ir->arrive[0], tot)) return;
  if (flat_tid() == 0) {
    ir->rhs_rescale = 0;
    if (!(tot[0] >= 0x1p-60 && tot[0] <= 0x1p60 && tot[1] >= 0x1p-60 && tot[1] <= 0x1p60)) {
      // the scaled sums left the FP32 margin (or are 0, inf, NaN): the host recomputes this
      // sweep's residual, norms and test in FP64 (k_ir_residual<true>, k_ir_scale)
      ir->rhs_rescale = 1;
      return;
    }
    const double inv_sig = pow2d(sig_exp);
    const double rn = sqrt(tot[1]) * inv_sig;
    ir->ir_bnorm = rn;
    ir->ir_rnorm = rn;
    ir->dp = rn;
    ir->a = sqrt(tot[0]) * inv_sig;
    if (rn <= fmax(ir_rtol * ir->ir_bnorm, ir->atol))
      ir->status = rn < ir->atol ? kConvergedAtol : kConvergedRtol;
    if (ir->status == 0) {
      ir->rscale = inv_sig;
      in->beta = tot[0];
      in->rnorm0 = sqrt(tot[0]);
      in->ttol = inner_rtol * in->rnorm0;
      in->iter = 0;
      in->its = 0;
      in->dpi = 0.0;
      in->status = 0;
      if (u) line_first_state(in, tot[2]);
    }
  }
}

// sq = 1 / s for an operator scaled earlier (s already holds D^-1/2)
__global__ void k_inv64(const double* __restrict__ s, double* __restrict__ sq, size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
       c += (size_t)gridDim.x * blockDim.x)
    sq[c] = 1.0 / s[c];
}

int KrylovSolver::prep_mixed(Stencil64& A, cudaStream_t st, bool line,
                             const frehg_solver_config& cfg) {
  const size_t n = A.n;
  FG_TRY(ensure32(n));
  if (line) FG_TRY(ensure_line(n));
  const int nb = reduction_blocks(n, 256, 4);
  const double dn = (double)n;
  const int ncol = A.n0 * A.n1;
  const int lb = (int)std::min<long>((ncol + 127) / 128, kMaxRedBlocks);
  first_done = false;
  first_line_done = false;
  if (A.f32_entries && (A.scaled || !ff_operator)) {
    set_error("FP32-form operator outside the float-float preparation");
    return FREHG_ERR_STATE;
  }
  if (!A.scaled) {
    if (ff_operator) {
      if (!A.f32_entries) {
        set_error("the float-float preparation needs the assembly's FP32-form operator");
        return FREHG_ERR_STATE;
      }
      // the refinement state, then one pass: scale factors, scaled operator, FP32 copy, line
      // factors and the first sweep's residual
      CgDevState ir0, in0;
      memset(&ir0, 0, sizeof(ir0));
      memset(&in0, 0, sizeof(in0));
      ir0.atol = cfg.atol;
      in0.max_it = cfg.max_it;
      FG_CUDA(cudaMemcpyAsync(dst, &ir0, sizeof(CgDevState), cudaMemcpyHostToDevice, st));
      FG_CUDA(cudaMemcpyAsync(dst32, &in0, sizeof(CgDevState), cudaMemcpyHostToDevice, st));
      // the first inner right-hand side's scale: 2^-e with 2^(e-1) <= the previous solve's
      // first residual norm < 2^e
      const int sig_exp = pow2_above(first_rnorm[rnorm_slot & 1]);
      // the line preconditioner's first application as well, unless the network runs
      const bool first_line = line && net.net == nullptr;
      FG_LAUNCH(prof, st, "k_prep_ff",
                (4.0 + 12.0 + 8.0 + 24.0 + 12.0 + 8.0 + 4.0 + (line ? 8.0 : 0.0) +
                 (first_line ? 4.0 : 0.0)) * dn,
                k_prep_ff<<<lb, 128, 0, st>>>(A.a0, A.a1, A.a2, reinterpret_cast<const float*>(A.s),
                                              A.b, r, op32.a0, op32.a1, op32.a2, lkf, dinvf,
                                              A.n0, A.n1, A.n2, line ? 1 : 0, dst, partials,
                                              cfg.ir_rtol, rf, dst32, sig_exp, cfg.inner_rtol,
                                              first_line ? uf : nullptr));
      FG_CUDA(cudaGetLastError());
      first_line_done = first_line;
      A.scaled = true;
      A.s_in_r = true;
      A.f32_entries = false;
      first_done = true;
      return FREHG_OK;
    }
    FG_LAUNCH(prof, st, "k_diag_rsqrt_sq", 24.0 * dn,
              k_diag_rsqrt_sq<<<nb, 256, 0, st>>>(A.s, r, n));
    FG_LAUNCH(prof, st, "k_scale_mixed", (56.0 + 12.0 + (line ? 8.0 : 0.0)) * dn,
              k_scale_mixed<<<lb, 128, 0, st>>>(A.a0, A.a1, A.a2, A.s, op32.a0, op32.a1,
                                                op32.a2, lkf, dinvf, A.n0, A.n1, A.n2,
                                                line ? 1 : 0));
    FG_CUDA(cudaGetLastError());
    A.scaled = true;
    return FREHG_OK;
  }
  // an operator scaled by an earlier solve: derive sq (unless r holds s), the FP32 copy and
  // the factors from it
  if (!A.s_in_r) FG_LAUNCH(prof, st, "k_inv64", 16.0 * dn, k_inv64<<<nb, 256, 0, st>>>(A.s, r, n));
  FG_LAUNCH(prof, st, "k_to_f32", 36.0 * dn,
            k_to_f32<<<nb, 256, 0, st>>>(A.a0, A.a1, A.a2, op32.a0, op32.a1, op32.a2, n));
  if (line)
    FG_LAUNCH(prof, st, "k_line_factor", 16.0 * dn,
              k_line_factor<<<lb, 128, 0, st>>>(A.a2, lkf, dinvf, ncol, A.n2));
  FG_CUDA(cudaGetLastError());
  return FREHG_OK;
}

int KrylovSolver::ensure_line(size_t n) {
  if (lkf && n <= cap_line) return FREHG_OK;
  cudaFree(lkf);
  cudaFree(dinvf);
  cudaFree(uf);
  lkf = dinvf = uf = nullptr;
  FG_CUDA(cudaMalloc(&lkf, n * sizeof(float)));
  FG_CUDA(cudaMalloc(&dinvf, n * sizeof(float)));
  FG_CUDA(cudaMalloc(&uf, n * sizeof(float)));
  cap_line = n;
  return FREHG_OK;
}

int KrylovSolver::solve_mixed(Stencil64& A, double* x_out, const frehg_solver_config& cfg,
                              cudaStream_t st, CgResult* res) {
  const size_t n = A.n;
  FG_TRY(ensure32(n));
  const int nb = reduction_blocks(n, 256, 4);
  const double dn = (double)n;
  const StencilLaunch L = stencil_launch(A.n0, A.n1, A.n2);
  const bool vec4 = (A.n0 % 4) == 0 && getenv("FREHG_NO_VEC4") == nullptr;
  const StencilLaunch L4 = launch_v4(A.n0, A.n1, A.n2);
  FG_CUDA(cudaGetLastError());
  // inner preconditioner: Jacobi (unit diagonal, z = r) or vertical lines
  const bool line = !strcmp(cfg.pc_type, "line");
  const int ncol = A.n0 * A.n1, nzl = A.n2;
  const int lb = (int)std::min<long>((ncol + 127) / 128, kMaxRedBlocks);
  CgDevState ir0, in0;
  memset(&ir0, 0, sizeof(ir0));
  memset(&in0, 0, sizeof(in0));
  ir0.atol = cfg.atol;
  in0.max_it = cfg.max_it;
  // prep_mixed may have formed the first sweep's residual and its state already, and the
  // line preconditioner's first application to it
  const bool first_done_here = first_done;
  const bool first_line_here = first_line_done;
  first_done = false;
  first_line_done = false;
  if (!first_done_here) {
    FG_CUDA(cudaMemcpyAsync(dst, &ir0, sizeof(CgDevState), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(dst32, &in0, sizeof(CgDevState), cudaMemcpyHostToDevice, st));
  }
  // where the scale factors are: A.s, or r (as floats) after the float-float preparation
  const double* sv = A.s_in_r ? r : A.s;

  const int chunk = 32;
  const long shape_key = (long)A.n0 * 1000003L + A.n1;
  const bool rebuild = !g32 || g32_key != (const void*)op32.a0 || g_stream32 != st || g_n32 != n ||
                       g32_shape != shape_key || g32_line != (line ? 1 : 0);
  auto spmv32 = [&](cudaStream_t s) {
    if (vec4)
      k32_spmv_v4<<<L4.grid, L4.block, 0, s>>>(op32.a0, op32.a1, op32.a2, pf, wf, A.n0, A.n1,
                                                A.n2, L4.planes, L4.tiles, dst32, partials);
    else
      k32_spmv<<<L.grid, L.block, 0, s>>>(op32.a0, op32.a1, op32.a2, pf, wf, A.n0, A.n1, A.n2,
                                          L.planes, L.tiles, dst32, partials);
  };
  // inner iterations run as CUDA graphs: a first chunk of 4 (easy systems converge in a few),
  // then chunks of 32; iterations after convergence return at once
  const int chunk0 = 4;
  auto capture = [&](int iters, cudaGraphExec_t* out) -> int {
    if (*out) cudaGraphExecDestroy(*out);
    *out = nullptr;
    cudaStream_t cap_st;
    FG_CUDA(cudaStreamCreateWithFlags(&cap_st, cudaStreamNonBlocking));
    cudaGraph_t graph;
    FG_CUDA(cudaStreamBeginCapture(cap_st, cudaStreamCaptureModeThreadLocal));
    for (int q = 0; q < iters; ++q) {
      if (line) {
        spmv32(cap_st);
        k32_line_fwd<true><<<lb, 128, 0, cap_st>>>(xf, rf, pf, wf, lkf, dinvf, uf, ncol, nzl,
                                                   dst32, partials);
        k32_line_bwd<<<lb, 128, 0, cap_st>>>(uf, lkf, pf, ncol, nzl, dst32);
      } else {
        k32_p<<<nb, 256, 0, cap_st>>>(rf, pf, n, dst32);
        spmv32(cap_st);
        k32_update<<<nb, 256, 0, cap_st>>>(xf, rf, pf, wf, n, dst32, partials);
      }
    }
    cudaError_t e = cudaStreamEndCapture(cap_st, &graph);
    cudaStreamDestroy(cap_st);
    if (e != cudaSuccess) {
      set_error("graph capture failed: %s", cudaGetErrorString(e));
      return FREHG_ERR_CUDA;
    }
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      set_error("graph instantiate failed: %s", cudaGetErrorString(e));
      return FREHG_ERR_CUDA;
    }
    return FREHG_OK;
  };
  if (!(prof && prof->on) && rebuild) {
    FG_TRY(capture(chunk, &g32));
    FG_TRY(capture(chunk0, &g32s));
    g32_key = op32.a0;
    g_stream32 = st;
    g_n32 = n;
    g32_shape = shape_key;
    g32_line = line ? 1 : 0;
  }

  const int max_sweeps = 60;
  int inner_total = 0, sweeps = 0;
  bool fcg_fallback = false;
  const bool dbg = getenv("FREHG_DEBUG_IR") != nullptr;
  for (;;) {
    // whether this sweep's right-hand side producer also applied the line preconditioner
    // once (k32_line_fwd<false>): k_prep_ff does in the first sweep
    bool fwd0_done = false;
    if (sweeps == 0) {
      if (!first_done_here)
        FG_LAUNCH(prof, st, "k_ir_residual0", 24.0 * dn,
                  k_ir_residual<true><<<L.grid, L.block, 0, st>>>(
                      A.a0, A.a1, A.a2, sv, r, A.b, x, rres, A.n0, A.n1, A.n2, L.planes,
                      L.tiles, dst, partials, cfg.ir_rtol));
      else
        fwd0_done = first_line_here;
    } else if (A.s_in_r) {
      FG_LAUNCH(prof, st, "k_ir_residual", 52.0 * dn,
                (k_ir_residual<false, true><<<L.grid, L.block, 0, st>>>(
                    A.a0, A.a1, A.a2, sv, sv, A.b, x, rres, A.n0, A.n1, A.n2, L.planes,
                    L.tiles, dst, partials, cfg.ir_rtol, rf, dst32, cfg.inner_rtol)));
    } else {
      FG_LAUNCH(prof, st, "k_ir_residual", 52.0 * dn,
                k_ir_residual<false><<<L.grid, L.block, 0, st>>>(
                    A.a0, A.a1, A.a2, A.s, r, A.b, x, rres, A.n0, A.n1, A.n2, L.planes,
                    L.tiles, dst, partials, cfg.ir_rtol, rf, dst32, cfg.inner_rtol));
    }
    // the first sweep's right-hand side (norm in [1/2, 1); k_prep_ff wrote it already); later
    // residual kernels write theirs
    if (sweeps == 0 && !first_done_here)
      FG_LAUNCH(prof, st, "k_ir_scale", 12.0 * dn,
                k_ir_scale<<<nb, 256, 0, st>>>(rres, rf, n, dst, dst32, partials,
                                               cfg.inner_rtol));
    FG_CUDA(cudaGetLastError());
    FG_TRY(fetch_small(hst, dst, sizeof(CgDevState), st));
    FG_CUDA(cudaStreamSynchronize(st));
    if (prof && prof->on) FG_TRY(prof->flush());
    if (sweeps == 0 && first_done_here && hst->rhs_rescale) {
      // k_prep_ff's scale left the FP32 margin: this sweep's residual, norms and test in FP64
      fwd0_done = false;
      FG_LAUNCH(prof, st, "k_ir_residual0", 24.0 * dn,
                k_ir_residual<true><<<L.grid, L.block, 0, st>>>(
                    A.a0, A.a1, A.a2, sv, r, A.b, x, rres, A.n0, A.n1, A.n2, L.planes,
                    L.tiles, dst, partials, cfg.ir_rtol));
      FG_LAUNCH(prof, st, "k_ir_scale", 12.0 * dn,
                k_ir_scale<<<nb, 256, 0, st>>>(rres, rf, n, dst, dst32, partials,
                                               cfg.inner_rtol));
      FG_CUDA(cudaGetLastError());
      FG_TRY(fetch_small(hst, dst, sizeof(CgDevState), st));
      FG_CUDA(cudaStreamSynchronize(st));
      if (prof && prof->on) FG_TRY(prof->flush());
    }
    if (sweeps == 0 && hst->a > 0.0 && std::isfinite(hst->a))
      first_rnorm[rnorm_slot & 1] = hst->a;
    if (hst->status != 0) break;
    if (sweeps >= max_sweeps) break;
    // inner FP32 solve: flexible CG with the learned preconditioner, or Jacobi CG
    FG_TRY(fetch_small(hst32, dst32, sizeof(CgDevState), st));
    FG_CUDA(cudaStreamSynchronize(st));
    // a sweep that starts with the network's budget (twice the reference solve's inner
    // iterations) spent runs without it, as do the later ones
    if (net.net != nullptr && !fcg_fallback && net.max_inner > 0 &&
        inner_total >= net.max_inner)
      fcg_fallback = true;
    const bool use_net = net.net != nullptr && !fcg_fallback;
    if (use_net) {
      if (!zf) {
        FG_CUDA(cudaMalloc(&zf, cap32 * sizeof(float)));
      }
      const int check = 4;
      for (int it = 0; it < cfg.max_it && hst32->status == 0; ++it) {
        FG_TRY(unet_apply(net.net, A.n0, A.n1, A.n2, rf, net.lnk, net.cap, zf, st));
        if (line)
          FG_LAUNCH(prof, st, "k32_line_apply", 32.0 * dn,
                    k32_line_apply<<<lb, 128, 0, st>>>(rf, lkf, dinvf, uf, zf, ncol, nzl, 1));
        else
          FG_LAUNCH(prof, st, "k_add_f32", 12.0 * dn, k_add_f32<<<nb, 256, 0, st>>>(zf, rf, n));
        FG_LAUNCH(prof, st, "k_fcg_beta", 8.0 * dn,
                  k_fcg_beta<<<nb, 256, 0, st>>>(zf, wf, n, dst32, partials));
        FG_LAUNCH(prof, st, "k_fcg_p", 16.0 * dn,
                  k_fcg_p<<<nb, 256, 0, st>>>(zf, pf, rf, n, dst32, partials));
        FG_LAUNCH(prof, st, vec4 ? "k32_spmv_v4" : "k32_spmv", 20.0 * dn, spmv32(st));
        FG_LAUNCH(prof, st, "k32_update", 24.0 * dn,
                  k32_update<<<nb, 256, 0, st>>>(xf, rf, pf, wf, n, dst32, partials));
        FG_CUDA(cudaGetLastError());
        if ((it + 1) % check == 0) {
          FG_TRY(fetch_small(hst32, dst32, sizeof(CgDevState), st));
          FG_CUDA(cudaStreamSynchronize(st));
          if (prof && prof->on) FG_TRY(prof->flush());
          if (net.max_inner > 0 && inner_total + hst32->its > net.max_inner) {
            fcg_fallback = true;  // too slow: Jacobi CG from here on (the iterate is kept)
            break;
          }
        }
      }
      FG_TRY(fetch_small(hst32, dst32, sizeof(CgDevState), st));
      FG_CUDA(cudaStreamSynchronize(st));
      if (prof && prof->on) FG_TRY(prof->flush());
    }
    if (!use_net && line) {
      // z0 = M^-1 r0, r0.z0 (unless the right-hand side's producer formed them) and p0 = z0
      if (!fwd0_done)
        FG_LAUNCH(prof, st, "k32_line_fwd0", 16.0 * dn,
                  (k32_line_fwd<false><<<lb, 128, 0, st>>>(xf, rf, pf, wf, lkf, dinvf, uf, ncol,
                                                           nzl, dst32, partials)));
      FG_LAUNCH(prof, st, "k32_line_bwd", 12.0 * dn,
                k32_line_bwd<<<lb, 128, 0, st>>>(uf, lkf, pf, ncol, nzl, dst32));
      FG_CUDA(cudaGetLastError());
    }
    for (int q = 0; !use_net && q < cfg.max_it / chunk + 2 && hst32->status == 0; ++q) {
      const int iters = q == 0 ? chunk0 : chunk;
      const int its_before = hst32->its;
      if (prof && prof->on) {
        for (int it = 0; it < iters; ++it) {
          if (line) {
            FG_LAUNCH(prof, st, vec4 ? "k32_spmv_v4" : "k32_spmv", 20.0 * dn, spmv32(st));
            FG_LAUNCH(prof, st, "k32_line_fwd", 36.0 * dn,
                      (k32_line_fwd<true><<<lb, 128, 0, st>>>(xf, rf, pf, wf, lkf, dinvf, uf,
                                                              ncol, nzl, dst32, partials)));
            FG_LAUNCH(prof, st, "k32_line_bwd", 16.0 * dn,
                      k32_line_bwd<<<lb, 128, 0, st>>>(uf, lkf, pf, ncol, nzl, dst32));
          } else {
            FG_LAUNCH(prof, st, "k32_p", 12.0 * dn,
                      k32_p<<<nb, 256, 0, st>>>(rf, pf, n, dst32));
            FG_LAUNCH(prof, st, vec4 ? "k32_spmv_v4" : "k32_spmv", 20.0 * dn, spmv32(st));
            FG_LAUNCH(prof, st, "k32_update", 24.0 * dn,
                      k32_update<<<nb, 256, 0, st>>>(xf, rf, pf, wf, n, dst32, partials));
          }
        }
        FG_CUDA(cudaGetLastError());
      } else {
        FG_CUDA(cudaGraphLaunch(q == 0 ? g32s : g32, st));
        if (prof) prof->launches += 3 * iters;
      }
      FG_TRY(fetch_small(hst32, dst32, sizeof(CgDevState), st));
      FG_CUDA(cudaStreamSynchronize(st));
      if (prof && prof->on) {
        FG_TRY(prof->flush());
        // the chunk's iterations after convergence returned at once (the line solve's backward
        // sweep of the converging iteration too: the forward sweep's kernel ran the test)
        const int done = std::min(iters, std::max(0, hst32->its - its_before));
        const int64_t idle = iters - done;
        if (line) {
          prof->idle(vec4 ? "k32_spmv_v4" : "k32_spmv", idle);
          prof->idle("k32_line_fwd", idle);
          prof->idle("k32_line_bwd", std::min<int64_t>(iters, idle + (hst32->status != 0 &&
                                                                       done > 0 ? 1 : 0)));
        } else {
          prof->idle("k32_p", idle);
          prof->idle(vec4 ? "k32_spmv_v4" : "k32_spmv", idle);
          prof->idle("k32_update", idle);
        }
      }
    }
    inner_total += hst32->its;
    if (dbg)
      fprintf(stderr, "ir sweep %d: true |r| %.3e / |b| %.3e ; inner its %d status %d |r0| %.3e -> %.3e\n",
              sweeps, hst->ir_rnorm, hst->ir_bnorm, hst32->its, hst32->status, hst32->rnorm0,
              hst32->dp);
    if (sweeps == 0)
      FG_LAUNCH(prof, st, "k_ir_update", 12.0 * dn,
                k_ir_update<true><<<nb, 256, 0, st>>>(x, xf, n, dst, dst32));
    else
      FG_LAUNCH(prof, st, "k_ir_update", 20.0 * dn,
                k_ir_update<false><<<nb, 256, 0, st>>>(x, xf, n, dst, dst32));
    FG_CUDA(cudaGetLastError());
    ++sweeps;
    // next sweep's residual kernel re-arms the refinement bookkeeping
    FG_CUDA(cudaMemcpyAsync(&dst->ir_its, &sweeps, sizeof(int), cudaMemcpyHostToDevice, st));
  }
  // stopped before the first update: x~ = 0
  if (sweeps == 0)
    FG_LAUNCH(prof, st, "k_zero64", 8.0 * dn, k_zero64<<<nb, 256, 0, st>>>(x, n));
  FG_TRY(finish64(A, x_out, st, res, nb));
  res->its = inner_total;
  res->inner_its = inner_total;
  res->ir_its = sweeps;
  res->fallback = fcg_fallback ? 1 : 0;
  res->rnorm = hst->ir_rnorm;
  res->reason = hst->status;
  if (hst->status <= 0) {
    set_error("mixed-precision refinement stopped after %d sweeps: true residual %g vs %g * %g "
              "(reason %d)", sweeps, hst->ir_rnorm, cfg.ir_rtol, hst->ir_bnorm, hst->status);
    return hst->status == kDivergedNanOrInf ? FREHG_ERR_NONFINITE : FREHG_ERR_NOT_CONVERGED;
  }
  return FREHG_OK;
}

}  // namespace fg
