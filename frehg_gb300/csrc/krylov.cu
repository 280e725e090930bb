// Krylov solver on the GPU: Jacobi-preconditioned CG for a 7-point SPD stencil.
//
// Replaces the PETSc KSP solve behind PetscLinearSolver::solve
// (src/linear/backends/PetscLinearSolver.cpp:200-220): KSPSolve_CG with the preconditioned
// residual norm, zero initial guess and KSPConvergedDefault (converged when
// ||B r|| <= max(rtol*||B b||, atol); divergence when ||B r|| >= 1e4*||B b||, NaN/Inf,
// indefinite matrix or preconditioner, or max_it).
//
// GB300 design:
//  * The operator is scaled once per solve to unit diagonal: A~ = D^-1/2 A D^-1/2.  CG on A~
//    is Jacobi-PCG on A (x~ = D^1/2 x, r~ = D^-1/2 r, beta = r.z = r~.r~, p'Ap = p~'A~p~,
//    ||B r|| = ||s r~|| with s = D^-1/2), so the diagonal is never stored or multiplied and
//    no divisions remain in the loop.
//  * Three phases per iteration (p-update, stencil SpMV + p.w, update + two norms), as one
//    cooperative launch (k_cg_iter, the phases separated by two bounded grid barriers; by
//    default for systems of up to kFusedAutoCells unknowns) or as three kernels (larger
//    systems, or devices without cooperative launch); the last reduction ends in the
//    last-arriving block, which also runs the scalar part of the algorithm (beta, stopping
//    test) on the device.  Launches of a converged solve return at once, so
//    iterations are captured in a CUDA graph of `chunk` iterations and the host only reads
//    the status between chunks.  Reductions are deterministic (fixed block partition, fixed
//    summation tree).
//  * FP64 is 1/64 of the FP32 rate on GB300, so the kernels are arranged to keep the FP64
//    instruction count per cell low (13 FMA-class ops per iteration) as well as the bytes.
#include "internal.h"
#include "reduce.cuh"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace fg {

// KSPConvergedDefault
__device__ __forceinline__ int converged_test(CgDevState* s, double rnorm) {
  if (isnan(rnorm) || isinf(rnorm)) return kDivergedNanOrInf;
  if (rnorm <= s->ttol) return rnorm < s->atol ? kConvergedAtol : kConvergedRtol;
  if (s->divtol > 0.0 && rnorm >= s->divtol * s->rnorm0) return kDivergedDtol;
  return 0;
}

// ------------------------------------------------------------------------------------------
// geometry helpers

StencilLaunch stencil_launch(int n0, int n1, int n2) {
  StencilLaunch L;
  L.block = dim3(32, 8, 1);
  const int t0 = (n0 + 31) / 32, t1 = (n1 + 7) / 8;
  const long tiles = (long)t0 * t1;
  // about two waves of 8 resident (32 x 8)-thread blocks per SM; the launch shape, and with
  // it the summation tree of the reductions, depends on the grid sizes only
  const long target = (long)kNumSMs * 8 * 2;
  long z = target / (tiles > 0 ? tiles : 1);
  if (z < 1) z = 1;
  if (z > n2) z = n2;
  int planes = (int)((n2 + z - 1) / z);
  z = (n2 + planes - 1) / planes;
  // blocks stride over tiles when there are more tiles than reduction partial slots
  long gx = tiles;
  const long cap = kMaxRedBlocks / z;
  if (gx > cap) gx = cap;
  L.planes = planes;
  L.tiles = (int)tiles;
  L.grid = dim3((unsigned)gx, (unsigned)z, 1);
  return L;
}

namespace {
__global__ void k_fetch_words(const unsigned* __restrict__ src, unsigned* __restrict__ dst,
                              int words) {
  for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
}
}  // namespace

int alloc_mapped(void** host, size_t bytes) {
  FG_CUDA(cudaHostAlloc(host, bytes, cudaHostAllocMapped));
  return FREHG_OK;
}

int fetch_small(void* host_mapped, const void* dev, size_t bytes, cudaStream_t st) {
  void* d = nullptr;
  FG_CUDA(cudaHostGetDevicePointer(&d, host_mapped, 0));
  k_fetch_words<<<1, 32, 0, st>>>(static_cast<const unsigned*>(dev), static_cast<unsigned*>(d),
                                  (int)(bytes / 4));
  FG_CUDA(cudaGetLastError());
  return FREHG_OK;
}

int reduction_blocks(size_t n, int threads, int per_thread) {
  size_t b = (n + (size_t)threads * per_thread - 1) / ((size_t)threads * per_thread);
  if (b < 1) b = 1;
  if (b > (size_t)kNumSMs * 8) b = (size_t)kNumSMs * 8;
  return (int)b;
}

// ------------------------------------------------------------------------------------------
// operator scaling

__global__ void k_diag_rsqrt(double* __restrict__ s, size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
       c += (size_t)gridDim.x * blockDim.x) {
    double d = s[c];
    if (d == 0.0) d = 1.0;  // PCJacobi replaces a zero diagonal entry by 1
    s[c] = rsqrt(d);        // NaN for d < 0: the solve then stops with DIVERGED_NANORINF
  }
}

__global__ void k_scale_offdiag(double* __restrict__ a0, double* __restrict__ a1,
                                double* __restrict__ a2, const double* __restrict__ s, int n0,
                                int n1, int n2, int planes, int tiles) {
  const int t0 = (n0 + 31) / 32;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int i0 = (tile % t0) * 32 + threadIdx.x;
    const int i1 = (tile / t0) * 8 + threadIdx.y;
    if (i0 >= n0 || i1 >= n1) continue;
    const size_t s01 = (size_t)n0 * n1;
    const int kb = blockIdx.y * planes;
    const int ke = min(n2, kb + planes);
    for (int k = kb; k < ke; ++k) {
      const size_t c = (size_t)i0 + (size_t)n0 * i1 + s01 * k;
      const double sc = s[c];
      if (i0 + 1 < n0) a0[c] *= sc * s[c + 1]; else a0[c] = 0.0;
      if (i1 + 1 < n1) a1[c] *= sc * s[c + n0]; else a1[c] = 0.0;
      if (k + 1 < n2) a2[c] *= sc * s[c + s01]; else a2[c] = 0.0;
    }
  }
}

// ------------------------------------------------------------------------------------------
// FP64 CG kernels

// r~ = s b, x~ = 0; ||B b|| and beta = r~.r~; iteration-0 stopping test.
__global__ void k_cg_init(const double* __restrict__ s, const double* __restrict__ b,
                          double* __restrict__ x, double* __restrict__ r, size_t n,
                          CgDevState* st, double* partials) {
  double v[2] = {0.0, 0.0};
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
       c += (size_t)gridDim.x * blockDim.x) {
    const double sc = s[c];
    const double rc = sc * b[c];
    r[c] = rc;
    x[c] = 0.0;
    v[0] = fma(rc, rc, v[0]);
    const double z = sc * rc;
    v[1] = fma(z, z, v[1]);
  }
  double tot[2];
  if (!grid_sum<2>(v, partials, &st->arrive[0], tot)) return;
  if (flat_tid() == 0) {
    const double dp = sqrt(tot[1]);
    st->dp = dp;
    st->rnorm0 = dp;
    st->ttol = fmax(st->rtol * dp, st->atol);
    st->its = 0;
    st->iter = 0;
    st->dpi = 0.0;
    st->beta = tot[0];
    st->status = converged_test(st, dp);
    if (!st->status && st->beta == 0.0) {  // loop top of iteration 0
      st->its = 1;
      st->status = kConvergedAtol;
    }
  }
}

// p = r~ (first iteration) or p = r~ + bcoef p   (16-byte vector accesses)
__global__ void k_cg_p(const double* __restrict__ r, double* __restrict__ p, size_t n,
                       const CgDevState* st) {
  if (st->status) return;
  const double bc = st->bcoef;
  const bool first = st->iter == 0;
  const size_t gid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const double2* r2 = reinterpret_cast<const double2*>(r);
  double2* p2 = reinterpret_cast<double2*>(p);
  for (size_t q = gid; q < n / 2; q += stride) {
    const double2 rv = r2[q];
    double2 pv;
    if (first) {
      pv = rv;
    } else {
      pv = p2[q];
      pv.x = fma(bc, pv.x, rv.x);
      pv.y = fma(bc, pv.y, rv.y);
    }
    p2[q] = pv;
  }
  if ((n & 1) && gid == 0) p[n - 1] = first ? r[n - 1] : fma(bc, p[n - 1], r[n - 1]);
}

// w = A~ p (unit diagonal) and p.w; the last block forms alpha.
template <typename T, typename Acc>
__device__ __forceinline__ Acc spmv_cell(const T* __restrict__ p, const T* __restrict__ a0,
                                         const T* __restrict__ a1, size_t c, int i0, int i1,
                                         int n0, int n1, T pc) {
  Acc v = (Acc)pc;
  if (i0 > 0) v = fma((Acc)a0[c - 1], (Acc)p[c - 1], v);
  if (i0 + 1 < n0) v = fma((Acc)a0[c], (Acc)p[c + 1], v);
  if (i1 > 0) v = fma((Acc)a1[c - n0], (Acc)p[c - n0], v);
  if (i1 + 1 < n1) v = fma((Acc)a1[c], (Acc)p[c + n0], v);
  return v;
}

__global__ void __launch_bounds__(256) k_cg_spmv(const double* __restrict__ a0,
                                                 const double* __restrict__ a1,
                                                 const double* __restrict__ a2,
                                                 const double* __restrict__ p,
                                                 double* __restrict__ w, int n0, int n1, int n2,
                                                 int planes, int tiles, CgDevState* st,
                                                 double* partials) {
  if (st->status) return;
  const int t0 = (n0 + 31) / 32;
  double acc[1] = {0.0};
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int i0 = (tile % t0) * 32 + threadIdx.x;
    const int i1 = (tile / t0) * 8 + threadIdx.y;
    if (i0 >= n0 || i1 >= n1) continue;
    const size_t s01 = (size_t)n0 * n1;
    const int kb = blockIdx.y * planes;
    const int ke = min(n2, kb + planes);
    size_t c = (size_t)i0 + (size_t)n0 * i1 + s01 * kb;
    double pm = 0.0, am = 0.0;
    if (kb > 0) {
      pm = p[c - s01];
      am = a2[c - s01];
    }
    double pc = p[c];
    for (int k = kb; k < ke; ++k) {
      const double pp = (k + 1 < n2) ? p[c + s01] : 0.0;
      const double ac = a2[c];
      double v = spmv_cell<double, double>(p, a0, a1, c, i0, i1, n0, n1, pc);
      v = fma(am, pm, v);
      v = fma(ac, pp, v);
      w[c] = v;
      acc[0] = fma(pc, v, acc[0]);
      pm = pc;
      pc = pp;
      am = ac;
      c += s01;
    }
  }
  double tot[1];
  if (!grid_sum<1>(acc, partials, &st->arrive[1], tot)) return;
  if (flat_tid() == 0) {
    const double dpi = tot[0];
    st->its = st->iter + 1;
    if (dpi == 0.0 || (st->iter > 0 && ((dpi > 0.0) != (st->dpi > 0.0))) || isnan(dpi)) {
      st->status = isnan(dpi) ? kDivergedNanOrInf : kDivergedIndefiniteMat;
      return;
    }
    st->dpiold = st->dpi;
    st->dpi = dpi;
    st->a = st->beta / dpi;
  }
}

// The scalar end of an iteration (last block): ||B r|| = sqrt(tot[1]) and the stopping test,
// beta = r~.r~ = tot[0] and the next direction's coefficient.
__device__ __forceinline__ void cg_update_tail(CgDevState* st, const double (&tot)[2]) {
  const double dp = sqrt(tot[1]);
  st->dp = dp;
  const int reason = converged_test(st, dp);
  if (reason) {
    st->status = reason;
    return;
  }
  st->betaold = st->beta;
  st->beta = tot[0];
  st->iter += 1;
  if (st->iter >= st->max_it) {
    st->status = kDivergedIts;
    return;
  }
  st->its = st->iter + 1;
  if (st->beta == 0.0) {
    st->status = kConvergedAtol;
    return;
  }
  st->bcoef = st->beta / st->betaold;
  if (st->bcoef < 0.0) st->status = kDivergedIndefinitePc;
}

// x~ += a p, r~ -= a w, then ||B r|| and beta = r~.r~; the last block runs the stopping test
// and prepares the next iteration's beta ratio.
__global__ void k_cg_update(double* __restrict__ x, double* __restrict__ r,
                            const double* __restrict__ p, const double* __restrict__ w,
                            const double* __restrict__ s, size_t n, CgDevState* st,
                            double* partials) {
  if (st->status) return;
  const double a = st->a;
  double v[2] = {0.0, 0.0};
  const size_t gid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  double2* x2 = reinterpret_cast<double2*>(x);
  double2* r2 = reinterpret_cast<double2*>(r);
  const double2* p2 = reinterpret_cast<const double2*>(p);
  const double2* w2 = reinterpret_cast<const double2*>(w);
  const double2* s2 = reinterpret_cast<const double2*>(s);
  for (size_t q = gid; q < n / 2; q += stride) {
    double2 xv = x2[q], rv = r2[q];
    const double2 pv = p2[q], wv = w2[q], sv = s2[q];
    xv.x = fma(a, pv.x, xv.x);
    xv.y = fma(a, pv.y, xv.y);
    rv.x = fma(-a, wv.x, rv.x);
    rv.y = fma(-a, wv.y, rv.y);
    x2[q] = xv;
    r2[q] = rv;
    v[0] = fma(rv.x, rv.x, v[0]);
    v[0] = fma(rv.y, rv.y, v[0]);
    const double zx = sv.x * rv.x, zy = sv.y * rv.y;
    v[1] = fma(zx, zx, v[1]);
    v[1] = fma(zy, zy, v[1]);
  }
  if ((n & 1) && gid == 0) {
    const size_t c = n - 1;
    x[c] = fma(a, p[c], x[c]);
    const double rc = fma(-a, w[c], r[c]);
    r[c] = rc;
    v[0] = fma(rc, rc, v[0]);
    const double z = s[c] * rc;
    v[1] = fma(z, z, v[1]);
  }
  double tot[2];
  if (!grid_sum<2>(v, partials, &st->arrive[2], tot)) return;
  if (flat_tid() == 0) cg_update_tail(st, tot);
}

// One Jacobi-PCG iteration (KSPSolve_CG's loop body) in one cooperative launch, all blocks
// resident: the direction p = r~ + bcoef p (p = r~ in iteration 0), a grid barrier, w = A~ p
// with the block partials of p.w, a grid barrier after which every block sums the same
// partials in the same order and forms alpha itself, then x~ += alpha p, r~ -= alpha w and the
// two norms, reduced by the last block to arrive, which runs the stopping test (cg_update_tail).
// The arithmetic per cell is that of k_cg_p, k_cg_spmv and k_cg_update.  Work units (a
// 32 x 8-column tile over a chunk of `planes` planes) are dealt round-robin to the blocks, the
// same units to the same block in all three phases, so the only values a block reads that
// another block wrote in this launch are the neighbours' directions of the stencil product;
// every direction read goes through L2 (ld.global.cg), since L1 is not coherent within a
// launch.  The iteration's scalars are read once at the start, before the first barrier, so
// that block 0 may update them after the second.
__global__ void __launch_bounds__(256) k_cg_iter(const double* __restrict__ a0,
                                                 const double* __restrict__ a1,
                                                 const double* __restrict__ a2,
                                                 const double* __restrict__ s,
                                                 double* __restrict__ x, double* __restrict__ r,
                                                 double* __restrict__ p, double* __restrict__ w,
                                                 int n0, int n1, int n2, int planes, int tiles,
                                                 CgDevState* st, double* partials) {
  if (st->status) return;
  const double bc = st->bcoef, beta = st->beta, dpi_prev = st->dpi;
  const int iter = st->iter;
  const int t0 = (n0 + 31) / 32;
  const size_t s01 = (size_t)n0 * n1;
  const int units = tiles * ((n2 + planes - 1) / planes);
  const int nb = flat_nblocks(), bid = flat_bid();
  // 1. direction
  for (int u = bid; u < units; u += nb) {
    const int tile = u % tiles, kb = (u / tiles) * planes, ke = min(n2, kb + planes);
    const int i0 = (tile % t0) * 32 + threadIdx.x;
    const int i1 = (tile / t0) * 8 + threadIdx.y;
    if (i0 >= n0 || i1 >= n1) continue;
    size_t c = (size_t)i0 + (size_t)n0 * i1 + s01 * kb;
    for (int k = kb; k < ke; ++k, c += s01) {
      const double rc = r[c];
      p[c] = iter == 0 ? rc : fma(bc, __ldcg(p + c), rc);
    }
  }
  if (!grid_barrier(&st->bar_count, &st->bar_gen, &st->bar_timeout)) {
    if (flat_tid() == 0) atomicExch(&st->status, (int)kGridBarrierTimeout);
    return;
  }
  // 2. stencil product and p.w
  double acc[1] = {0.0};
  for (int u = bid; u < units; u += nb) {
    const int tile = u % tiles, kb = (u / tiles) * planes, ke = min(n2, kb + planes);
    const int i0 = (tile % t0) * 32 + threadIdx.x;
    const int i1 = (tile / t0) * 8 + threadIdx.y;
    if (i0 >= n0 || i1 >= n1) continue;
    size_t c = (size_t)i0 + (size_t)n0 * i1 + s01 * kb;
    double pm = 0.0, am = 0.0;
    if (kb > 0) {
      pm = __ldcg(p + c - s01);
      am = a2[c - s01];
    }
    double pc = __ldcg(p + c);
    for (int k = kb; k < ke; ++k) {
      const double pp = (k + 1 < n2) ? __ldcg(p + c + s01) : 0.0;
      const double ac = a2[c];
      double v = pc;
      if (i0 > 0) v = fma(a0[c - 1], __ldcg(p + c - 1), v);
      if (i0 + 1 < n0) v = fma(a0[c], __ldcg(p + c + 1), v);
      if (i1 > 0) v = fma(a1[c - n0], __ldcg(p + c - n0), v);
      if (i1 + 1 < n1) v = fma(a1[c], __ldcg(p + c + n0), v);
      v = fma(am, pm, v);
      v = fma(ac, pp, v);
      w[c] = v;
      acc[0] = fma(pc, v, acc[0]);
      pm = pc;
      pc = pp;
      am = ac;
      c += s01;
    }
  }
  __shared__ double sh[32];
  __shared__ double dpi_sh;
  double* pw = partials + 3 * (size_t)kMaxRedBlocks;
  block_sum<1>(acc, sh);
  if (flat_tid() == 0) pw[bid] = acc[0];
  if (!grid_barrier(&st->bar_count, &st->bar_gen, &st->bar_timeout)) {
    if (flat_tid() == 0) atomicExch(&st->status, (int)kGridBarrierTimeout);
    return;
  }
  double t[1] = {0.0};
  for (int b = flat_tid(); b < nb; b += flat_nthreads()) t[0] += __ldcg(&pw[b]);
  block_sum<1>(t, sh);
  if (flat_tid() == 0) dpi_sh = t[0];
  __syncthreads();
  const double dpi = dpi_sh;
  const bool lead = bid == 0 && flat_tid() == 0;
  if (dpi == 0.0 || (iter > 0 && ((dpi > 0.0) != (dpi_prev > 0.0))) || isnan(dpi)) {
    if (lead) {
      st->its = iter + 1;
      st->status = isnan(dpi) ? kDivergedNanOrInf : kDivergedIndefiniteMat;
    }
    return;
  }
  const double a = beta / dpi;
  if (lead) {
    st->its = iter + 1;
    st->dpiold = dpi_prev;
    st->dpi = dpi;
    st->a = a;
  }
  // 3. update and norms
  double v[2] = {0.0, 0.0};
  for (int u = bid; u < units; u += nb) {
    const int tile = u % tiles, kb = (u / tiles) * planes, ke = min(n2, kb + planes);
    const int i0 = (tile % t0) * 32 + threadIdx.x;
    const int i1 = (tile / t0) * 8 + threadIdx.y;
    if (i0 >= n0 || i1 >= n1) continue;
    size_t c = (size_t)i0 + (size_t)n0 * i1 + s01 * kb;
    for (int k = kb; k < ke; ++k, c += s01) {
      x[c] = fma(a, __ldcg(p + c), x[c]);
      const double rc = fma(-a, w[c], r[c]);
      r[c] = rc;
      v[0] = fma(rc, rc, v[0]);
      const double z = s[c] * rc;
      v[1] = fma(z, z, v[1]);
    }
  }
  double tot[2];
  if (!grid_sum<2>(v, partials, &st->arrive[2], tot)) return;
  if (flat_tid() == 0) cg_update_tail(st, tot);
}

__global__ void k_unscale(const double* __restrict__ s, const double* __restrict__ xs,
                          double* __restrict__ x, size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
       c += (size_t)gridDim.x * blockDim.x)
    x[c] = s[c] * xs[c];
}

// ------------------------------------------------------------------------------------------
// host side

int Stencil64::alloc(int n0_, int n1_, int n2_) {
  release();
  n0 = n0_;
  n1 = n1_;
  n2 = n2_;
  n = (size_t)n0 * n1 * n2;
  FG_CUDA(cudaMalloc(&a0, n * sizeof(double)));
  FG_CUDA(cudaMalloc(&a1, n * sizeof(double)));
  FG_CUDA(cudaMalloc(&a2, n * sizeof(double)));
  FG_CUDA(cudaMalloc(&s, n * sizeof(double)));
  FG_CUDA(cudaMalloc(&b, n * sizeof(double)));
  scaled = false;
  s_in_r = false;
  return FREHG_OK;
}

void Stencil64::release() {
  cudaFree(a0);
  cudaFree(a1);
  cudaFree(a2);
  cudaFree(s);
  cudaFree(b);
  a0 = a1 = a2 = s = b = nullptr;
  n = 0;
}

int Stencil32::alloc(size_t n_) {
  release();
  n = n_;
  FG_CUDA(cudaMalloc(&a0, n * sizeof(float)));
  FG_CUDA(cudaMalloc(&a1, n * sizeof(float)));
  FG_CUDA(cudaMalloc(&a2, n * sizeof(float)));
  return FREHG_OK;
}

void Stencil32::release() {
  cudaFree(a0);
  cudaFree(a1);
  cudaFree(a2);
  a0 = a1 = a2 = nullptr;
  n = 0;
}

KrylovSolver::~KrylovSolver() {
  if (g64) cudaGraphExecDestroy(g64);
  if (g32) cudaGraphExecDestroy(g32);
  if (g32s) cudaGraphExecDestroy(g32s);
  if (gsor) cudaGraphExecDestroy(gsor);
  cudaFree(invd);
  cudaFree(zs);
  cudaFree(x);
  cudaFree(r);
  cudaFree(p);
  cudaFree(w);
  cudaFree(partials);
  cudaFree(dst);
  cudaFreeHost(hst);
  cudaFree(xf);
  cudaFree(rf);
  cudaFree(pf);
  cudaFree(wf);
  cudaFree(rres);
  cudaFree(dst32);
  cudaFreeHost(hst32);
  cudaFree(zf);
  cudaFree(lkf);
  cudaFree(dinvf);
  cudaFree(uf);
  op32.release();
}

int KrylovSolver::ensure(size_t n) {
  if (n <= cap && x) return FREHG_OK;
  cudaFree(x);
  cudaFree(r);
  cudaFree(p);
  cudaFree(w);
  x = r = p = w = nullptr;
  if (g64) {
    cudaGraphExecDestroy(g64);
    g64 = nullptr;
  }
  FG_CUDA(cudaMalloc(&x, n * sizeof(double)));
  FG_CUDA(cudaMalloc(&r, n * sizeof(double)));
  FG_CUDA(cudaMalloc(&p, n * sizeof(double)));
  FG_CUDA(cudaMalloc(&w, n * sizeof(double)));
  if (!partials) FG_CUDA(cudaMalloc(&partials, 4 * kMaxRedBlocks * sizeof(double)));
  if (!dst) {
    FG_CUDA(cudaMalloc(&dst, sizeof(CgDevState)));
    FG_CUDA(cudaMemset(dst, 0, sizeof(CgDevState)));
    FG_TRY(alloc_mapped(reinterpret_cast<void**>(&hst), sizeof(CgDevState)));
  }
  cap = n;
  return FREHG_OK;
}

int KrylovSolver::scale(Stencil64& A, cudaStream_t st) {
  if (A.scaled && A.s_in_r) {
    set_error("operator prepared for the float-float mixed-precision solve; reassemble it");
    return FREHG_ERR_STATE;
  }
  if (A.scaled) return FREHG_OK;
  if (A.f32_entries) {
    set_error("operator assembled in FP32 form for the mixed-precision solve (precision 1)");
    return FREHG_ERR_STATE;
  }
  const int nb = reduction_blocks(A.n, 256, 4);
  const double n = (double)A.n;
  FG_LAUNCH(prof, st, "k_diag_rsqrt", 16.0 * n, k_diag_rsqrt<<<nb, 256, 0, st>>>(A.s, A.n));
  FG_CUDA(cudaGetLastError());
  const StencilLaunch L = stencil_launch(A.n0, A.n1, A.n2);
  FG_LAUNCH(prof, st, "k_scale_offdiag", 56.0 * n,
            k_scale_offdiag<<<L.grid, L.block, 0, st>>>(A.a0, A.a1, A.a2, A.s, A.n0, A.n1, A.n2,
                                                        L.planes, L.tiles));
  FG_CUDA(cudaGetLastError());
  A.scaled = true;
  return FREHG_OK;
}

// Run a captured chunk graph until the device status leaves "running" or max_it is reached.
int KrylovSolver::run_chunks(cudaGraphExec_t g, cudaStream_t st, int max_it, int chunk,
                            int launches_per_it) {
  const int max_launch = max_it / chunk + 2;
  for (int q = 0; q < max_launch; ++q) {
    FG_CUDA(cudaGraphLaunch(g, st));
    if (prof) prof->launches += (int64_t)launches_per_it * chunk;
    FG_TRY(fetch_small(hst, dst, sizeof(CgDevState), st));
    FG_CUDA(cudaStreamSynchronize(st));
    if (hst->status != 0) return FREHG_OK;
  }
  set_error("Krylov loop: device status still running after %d chunk launches", max_launch);
  return FREHG_ERR_STATE;
}

int KrylovSolver::solve(Stencil64& A, double* x_out, const frehg_solver_config& cfg,
                        cudaStream_t st, CgResult* res) {
  FG_TRY(ensure(A.n));
  if (!strcmp(cfg.pc_type, "sor")) {
    if (cfg.precision != 0) {
      set_error("pc_type 'sor' runs in FP64 (precision 0)");
      return FREHG_ERR_UNSUPPORTED;
    }
    if (keep_scaled) {
      set_error("pc_type 'sor' returns the unscaled solution");
      return FREHG_ERR_STATE;
    }
    return solve_sor(A, x_out, cfg, st, res);
  }
  if (cfg.precision == 1) {
    FG_TRY(prep_mixed(A, st, !strcmp(cfg.pc_type, "line"), cfg));
    return solve_mixed(A, x_out, cfg, st, res);
  }
  FG_TRY(scale(A, st));
  if (strcmp(cfg.pc_type, "jacobi") != 0) {
    set_error("pc_type '%s' needs the mixed-precision solve (precision 1)", cfg.pc_type);
    return FREHG_ERR_UNSUPPORTED;
  }
  return solve64(A, x_out, cfg, st, res);
}

// Self-check of the grid barrier: every block but skip_block waits at one barrier with a
// bound of `polls` polls; with a block that never arrives the others' waits run out and set
// *timeout, and the kernel returns normally.
__global__ void k_barrier_check(unsigned int* count, unsigned int* gen, int* timeout,
                                int skip_block, long polls) {
  if ((int)blockIdx.x == skip_block) return;
  grid_barrier(count, gen, timeout, polls);
}

// Launch shape of k_cg_iter: the stencil tiles over at most the blocks the device holds at
// once (a cooperative launch may not exceed them).  False where the device has no cooperative
// launch or the shape does not fit.
static bool cg_iter_launch(int n0, int n1, int n2, StencilLaunch* L) {
  int dev = 0, coop = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_iter, 256, 0) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (!coop || per_sm < 1 || sms < 1) return false;
  const long resident = std::min<long>((long)per_sm * sms, kMaxRedBlocks);
  const long t0 = (n0 + 31) / 32, t1 = (n1 + 7) / 8, tiles = t0 * t1;
  // plane chunks short enough for about 16 work units per block (the blocks' shares then
  // differ by at most a sixteenth), long enough to keep the stencil's march along axis 2
  long planes = (tiles * n2 + 16 * resident - 1) / (16 * resident);
  planes = std::max<long>(1, std::min<long>(planes, n2));
  const long units = tiles * ((n2 + planes - 1) / planes);
  if (units > (long)INT32_MAX - resident) return false;
  // as few blocks as give every block the same number of units (small systems: fewer blocks
  // to wait for at the grid barriers)
  const long per_block = (units + resident - 1) / resident;
  const long blocks = (units + per_block - 1) / per_block;
  L->block = dim3(32, 8, 1);
  L->grid = dim3((unsigned)blocks, 1, 1);
  L->planes = (int)planes;
  L->tiles = (int)tiles;
  return true;
}

static cudaError_t launch_cg_iter(const StencilLaunch& L, cudaStream_t st, const Stencil64& A,
                                  double* x, double* r, double* p, double* w, CgDevState* dst,
                                  double* partials) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = L.grid;
  cfg.blockDim = L.block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_cg_iter, (const double*)A.a0, (const double*)A.a1,
                            (const double*)A.a2, (const double*)A.s, x, r, p, w, A.n0, A.n1,
                            A.n2, L.planes, L.tiles, dst, partials);
}

static int chunk_for(size_t n) {
  if (n >= (size_t)4 << 20) return 16;
  if (n >= (size_t)1 << 18) return 32;
  return 64;
}

int KrylovSolver::solve64(Stencil64& A, double* x_out, const frehg_solver_config& cfg,
                          cudaStream_t st, CgResult* res) {
  const size_t n = A.n;
  // stopping parameters
  CgDevState init;
  memset(&init, 0, sizeof(init));
  init.rtol = cfg.rtol;
  init.atol = cfg.atol;
  init.divtol = 1.0e4;
  init.max_it = cfg.max_it;
  FG_CUDA(cudaMemcpyAsync(dst, &init, sizeof(CgDevState), cudaMemcpyHostToDevice, st));
  const int nb = reduction_blocks(n, 256, 4);
  const double dn = (double)n;
  FG_LAUNCH(prof, st, "k_cg_init", 32.0 * dn,
            k_cg_init<<<nb, 256, 0, st>>>(A.s, A.b, x, r, n, dst, partials));
  FG_CUDA(cudaGetLastError());

  const int chunk = chunk_for(n);
  const StencilLaunch L = stencil_launch(A.n0, A.n1, A.n2);
  StencilLaunch LF;
  const bool want = !coop_failed && (fused64 > 0 || (fused64 < 0 && n <= kFusedAutoCells));
  const int form = want && cg_iter_launch(A.n0, A.n1, A.n2, &LF) ? 1 : 0;
  if (prof && prof->on) {
    // profiled path: the same kernels launched one by one between CUDA events
    FG_TRY(fetch_small(hst, dst, sizeof(CgDevState), st));
    FG_CUDA(cudaStreamSynchronize(st));
    for (int q = 0; q < cfg.max_it / chunk + 2 && hst->status == 0; ++q) {
      for (int it = 0; it < chunk; ++it) {
        if (form) {
          FG_LAUNCH(prof, st, "k_cg_iter", 120.0 * dn,
                    FG_CUDA(launch_cg_iter(LF, st, A, x, r, p, w, dst, partials)));
          continue;
        }
        FG_LAUNCH(prof, st, "k_cg_p", 24.0 * dn, k_cg_p<<<nb, 256, 0, st>>>(r, p, n, dst));
        FG_LAUNCH(prof, st, "k_cg_spmv", 40.0 * dn,
                  k_cg_spmv<<<L.grid, L.block, 0, st>>>(A.a0, A.a1, A.a2, p, w, A.n0, A.n1, A.n2,
                                                        L.planes, L.tiles, dst, partials));
        FG_LAUNCH(prof, st, "k_cg_update", 56.0 * dn,
                  k_cg_update<<<nb, 256, 0, st>>>(x, r, p, w, A.s, n, dst, partials));
      }
      FG_CUDA(cudaGetLastError());
      FG_TRY(fetch_small(hst, dst, sizeof(CgDevState), st));
      FG_CUDA(cudaStreamSynchronize(st));
      FG_TRY(prof->flush());
    }
    return finish64(A, x_out, st, res, nb);
  }
  const bool rebuild = !g64 || g64_key != (const void*)A.a0 || g64_key2 != (const void*)A.s ||
                       g_stream != st || g_n != n || g64_form != form;
  if (rebuild) {
    if (g64) cudaGraphExecDestroy(g64);
    g64 = nullptr;
    cudaStream_t cap_st;
    FG_CUDA(cudaStreamCreateWithFlags(&cap_st, cudaStreamNonBlocking));
    cudaGraph_t graph;
    FG_CUDA(cudaStreamBeginCapture(cap_st, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = cudaSuccess;
    for (int q = 0; q < chunk; ++q) {
      if (form) {
        const cudaError_t e1 = launch_cg_iter(LF, cap_st, A, x, r, p, w, dst, partials);
        if (le == cudaSuccess) le = e1;
        continue;
      }
      k_cg_p<<<nb, 256, 0, cap_st>>>(r, p, n, dst);
      k_cg_spmv<<<L.grid, L.block, 0, cap_st>>>(A.a0, A.a1, A.a2, p, w, A.n0, A.n1, A.n2,
                                                L.planes, L.tiles, dst, partials);
      k_cg_update<<<nb, 256, 0, cap_st>>>(x, r, p, w, A.s, n, dst, partials);
    }
    cudaError_t e = cudaStreamEndCapture(cap_st, &graph);
    cudaStreamDestroy(cap_st);
    if (le != cudaSuccess) {
      // the cooperative launch was refused (e.g. under MPS): three kernels from now on
      if (e == cudaSuccess) cudaGraphDestroy(graph);
      cudaGetLastError();
      coop_failed = true;
      return solve64(A, x_out, cfg, st, res);
    }
    if (e != cudaSuccess) {
      set_error("graph capture failed: %s", cudaGetErrorString(e));
      return FREHG_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&g64, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      set_error("graph instantiate failed: %s", cudaGetErrorString(e));
      return FREHG_ERR_CUDA;
    }
    g64_key = A.a0;
    g64_key2 = A.s;
    g_stream = st;
    g_n = n;
    g64_form = form;
  }
  // iteration 0 may already have converged
  FG_TRY(fetch_small(hst, dst, sizeof(CgDevState), st));
  FG_CUDA(cudaStreamSynchronize(st));
  if (hst->status == 0) FG_TRY(run_chunks(g64, st, cfg.max_it, chunk, form ? 1 : 3));
  return finish64(A, x_out, st, res, nb);
}

int KrylovSolver::finish64(Stencil64& A, double* x_out, cudaStream_t st, CgResult* res, int nb) {
  if (!keep_scaled) {
    FG_LAUNCH(prof, st, "k_unscale", 24.0 * (double)A.n,
              k_unscale<<<nb, 256, 0, st>>>(scale_vector(A), x, x_out, A.n));
    FG_CUDA(cudaGetLastError());
  }
  res->its = hst->its;
  res->reason = hst->status;
  res->rnorm = hst->dp;
  res->inner_its = hst->its;
  res->ir_its = 0;
  if (hst->bar_timeout || hst->status == kGridBarrierTimeout) {
    set_error("Krylov loop: a grid barrier of the one-launch CG iteration timed out after %d "
              "iterations", hst->its);
    return FREHG_ERR_CUDA;
  }
  if (hst->status < 0) {
    set_error("KSP diverged (reason %d) after %d iterations, residual norm %g", hst->status,
              hst->its, hst->dp);
    return hst->status == kDivergedNanOrInf ? FREHG_ERR_NONFINITE : FREHG_ERR_NOT_CONVERGED;
  }
  return FREHG_OK;
}

}  // namespace fg

extern "C" int frehg_check_grid_barrier(int skip_block, long long polls, int* timed_out) {
  using namespace fg;
  clear_error();
  FG_ARG(timed_out && polls > 0 && skip_block >= -1 && skip_block < 2,
         "timed_out required, polls > 0, skip_block in {-1, 0, 1}");
  int dev = 0, coop = 0;
  FG_CUDA(cudaGetDevice(&dev));
  FG_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  if (!coop) {
    set_error("the device has no cooperative launch");
    return FREHG_ERR_UNSUPPORTED;
  }
  unsigned int* w = nullptr;  // count, generation, timeout flag
  FG_CUDA(cudaMalloc(&w, 3 * sizeof(unsigned int)));
  cudaError_t e = cudaMemset(w, 0, 3 * sizeof(unsigned int));
  if (e == cudaSuccess) {
    unsigned int* count = w;
    unsigned int* gen = w + 1;
    int* flag = reinterpret_cast<int*>(w + 2);
    long npolls = (long)polls;
    void* args[] = {&count, &gen, &flag, &skip_block, &npolls};
    e = cudaLaunchCooperativeKernel((const void*)k_barrier_check, dim3(2), dim3(32), args, 0,
                                    nullptr);
  }
  int host_flag = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&host_flag, w + 2, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(w);
  if (e != cudaSuccess) {
    set_error("grid barrier check: %s", cudaGetErrorString(e));
    return FREHG_ERR_CUDA;
  }
  *timed_out = host_flag;
  return FREHG_OK;
}
