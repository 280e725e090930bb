// PCSOR on the GPU: CG preconditioned by PETSc's local symmetric SOR sweep (omega = 1, one
// sweep, zero initial guess), the groundwater default of the reference
// (groundwater.solver.pc_type = "sor", src/driver/Orchestrator.cpp:489, applied by
// PCSetType / KSPSolve in src/linear/backends/PetscLinearSolver.cpp:193,204).
//
// M^-1 r = (D+U)^-1 D (D+L)^-1 r in the owned row order of Decomp3D on one rank
// (row = (j*nx + i)*nz + k, DomainDecomposition.cpp:109-119):
//   forward   y_c = (r_c - a_S y_S - a_W y_W - a_Up y_Up) / d_c     (lower neighbours)
//   backward  z_c = (d_c y_c - a_Down z_Down - a_E z_E - a_N z_N) / d_c
// with 1/d formed once as PETSc's MatSOR does (a zero diagonal entry taken as 1), the product
// d y formed as y / (1/d), and the neighbour terms in the reference's column order.
//
// Lexicographic Gauss-Seidel is sequential in row order, but on the 7-point stencil a cell
// depends only on its -1 neighbours along each axis (forward) or +1 neighbours (backward), so
// all cells of one hyperplane a0 + a1 + a2 = w are independent once the planes before it are
// done: sweeping the planes in order reproduces the sequential result exactly.  Small systems
// run both sweeps in one block, the planes separated by __syncthreads (one launch per
// application, no inter-block synchronisation); larger ones launch one kernel per plane, all
// captured in the iteration graph.  The Krylov part is the unscaled PETSc KSPSolve_CG: the
// operator keeps its diagonal (SOR needs D and L, not D^-1/2 A D^-1/2).
#include "internal.h"
#include "reduce.cuh"

#include <cmath>
#include <cstring>

namespace fg {

namespace {

struct SorGeom {
  int n[3];
  size_t stride[3];
  int ord[3];  // axes from the slowest to the fastest of the reference's row order
  int w_end;   // number of hyperplanes, n0 + n1 + n2 - 2
};

SorGeom sor_geom(const Stencil64& A) {
  SorGeom g;
  g.n[0] = A.n0;
  g.n[1] = A.n1;
  g.n[2] = A.n2;
  g.stride[0] = 1;
  g.stride[1] = (size_t)A.n0;
  g.stride[2] = (size_t)A.n0 * A.n1;
  for (int q = 0; q < 3; ++q) g.ord[q] = A.ref_order[q];
  g.w_end = A.n0 + A.n1 + A.n2 - 2;
  return g;
}

__device__ __forceinline__ const double* coupling(const double* a0, const double* a1,
                                                  const double* a2, int ax) {
  return ax == 0 ? a0 : (ax == 1 ? a1 : a2);
}

// forward update of one cell: z_c = (r_c - sum of lower terms) * invd_c
__device__ __forceinline__ void sor_fwd_cell(const SorGeom& g, const int (&idx)[3], size_t c,
                                             const double* __restrict__ a0,
                                             const double* __restrict__ a1,
                                             const double* __restrict__ a2,
                                             const double* __restrict__ invd,
                                             const double* __restrict__ r, double* z) {
  double sum = r[c];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const int ax = g.ord[q];
    if (idx[ax] > 0) {
      const size_t m = c - g.stride[ax];
      sum = __dsub_rn(sum, __dmul_rn(coupling(a0, a1, a2, ax)[m], __ldcg(&z[m])));
    }
  }
  z[c] = __dmul_rn(sum, invd[c]);
}

// backward update: z_c = (z_c / invd_c - sum of upper terms) * invd_c
__device__ __forceinline__ void sor_bwd_cell(const SorGeom& g, const int (&idx)[3], size_t c,
                                             const double* __restrict__ a0,
                                             const double* __restrict__ a1,
                                             const double* __restrict__ a2,
                                             const double* __restrict__ invd, double* z) {
  const double id = invd[c];
  double sum = __ddiv_rn(__ldcg(&z[c]), id);
#pragma unroll
  for (int q = 2; q >= 0; --q) {
    const int ax = g.ord[q];
    if (idx[ax] + 1 < g.n[ax]) {
      sum = __dsub_rn(sum, __dmul_rn(coupling(a0, a1, a2, ax)[c], __ldcg(&z[c + g.stride[ax]])));
    }
  }
  z[c] = __dmul_rn(sum, id);
}

// cells of hyperplane w: one per (a1, a2) pair with a0 = w - a1 - a2 inside the box
__device__ __forceinline__ bool plane_cell(const SorGeom& g, int w, long t, int (&idx)[3],
                                           size_t& c) {
  idx[1] = (int)(t % g.n[1]);
  idx[2] = (int)(t / g.n[1]);
  idx[0] = w - idx[1] - idx[2];
  if (idx[0] < 0 || idx[0] >= g.n[0]) return false;
  c = (size_t)idx[0] + g.stride[1] * idx[1] + g.stride[2] * idx[2];
  return true;
}

// both sweeps in one block (small systems)
__global__ void k_sor_block(SorGeom g, const double* __restrict__ a0,
                            const double* __restrict__ a1, const double* __restrict__ a2,
                            const double* __restrict__ invd, const double* __restrict__ r,
                            double* z, const CgDevState* st) {
  if (st->status) return;
  const long cols = (long)g.n[1] * g.n[2];
  for (int w = 0; w < g.w_end + 1; ++w) {
    for (long t = threadIdx.x; t < cols; t += blockDim.x) {
      int idx[3];
      size_t c;
      if (plane_cell(g, w, t, idx, c)) sor_fwd_cell(g, idx, c, a0, a1, a2, invd, r, z);
    }
    __syncthreads();
  }
  for (int w = g.w_end; w >= 0; --w) {
    for (long t = threadIdx.x; t < cols; t += blockDim.x) {
      int idx[3];
      size_t c;
      if (plane_cell(g, w, t, idx, c)) sor_bwd_cell(g, idx, c, a0, a1, a2, invd, z);
    }
    __syncthreads();
  }
}

// one hyperplane of one sweep (larger systems; one launch per plane)
template <bool FWD>
__global__ void k_sor_plane(SorGeom g, int w, const double* __restrict__ a0,
                            const double* __restrict__ a1, const double* __restrict__ a2,
                            const double* __restrict__ invd, const double* __restrict__ r,
                            double* z, const CgDevState* st) {
  if (st->status) return;
  const long cols = (long)g.n[1] * g.n[2];
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < cols;
       t += (long)gridDim.x * blockDim.x) {
    int idx[3];
    size_t c;
    if (!plane_cell(g, w, t, idx, c)) continue;
    if (FWD)
      sor_fwd_cell(g, idx, c, a0, a1, a2, invd, r, z);
    else
      sor_bwd_cell(g, idx, c, a0, a1, a2, invd, z);
  }
}

// 1/d (a zero diagonal entry replaced by 1, MatSOR / PCJacobi), x = 0, r = b
__global__ void k_sor_prep(const double* __restrict__ d, const double* __restrict__ b,
                           double* __restrict__ invd, double* __restrict__ x,
                           double* __restrict__ r, size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
       c += (size_t)gridDim.x * blockDim.x) {
    const double dc = d[c];
    invd[c] = 1.0 / (dc == 0.0 ? 1.0 : dc);
    x[c] = 0.0;
    r[c] = b[c];
  }
}

__device__ __forceinline__ int sor_converged(CgDevState* s, double rnorm) {
  if (isnan(rnorm) || isinf(rnorm)) return kDivergedNanOrInf;
  if (rnorm <= s->ttol) return rnorm < s->atol ? kConvergedAtol : kConvergedRtol;
  if (s->divtol > 0.0 && rnorm >= s->divtol * s->rnorm0) return kDivergedDtol;
  return 0;
}

// ||z|| and beta = z.r after a preconditioner application; the last block runs
// KSPSolve_CG's scalar steps (stopping test, beta ratio) as in the Jacobi path.
template <bool INIT>
__global__ void k_sor_dots(const double* __restrict__ z, const double* __restrict__ r, size_t n,
                           CgDevState* st, double* partials) {
  if (st->status) return;
  double v[2] = {0.0, 0.0};
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
       c += (size_t)gridDim.x * blockDim.x) {
    const double zc = z[c];
    v[0] = fma(zc, zc, v[0]);
    v[1] = fma(zc, r[c], v[1]);
  }
  double tot[2];
  if (!grid_sum<2>(v, partials, &st->arrive[3], tot)) return;
  if (flat_tid() != 0) return;
  const double dp = sqrt(tot[0]);
  st->dp = dp;
  if (INIT) {
    st->rnorm0 = dp;
    st->ttol = fmax(st->rtol * dp, st->atol);
    st->its = 0;
    st->iter = 0;
    st->dpi = 0.0;
    st->status = sor_converged(st, dp);
    if (st->status) return;
    st->beta = tot[1];
    st->its = 1;
    if (st->beta == 0.0) st->status = kConvergedAtol;
    return;
  }
  const int reason = sor_converged(st, dp);
  if (reason) {
    st->status = reason;
    return;
  }
  st->betaold = st->beta;
  st->beta = tot[1];
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

// p = z (first iteration) or z + (beta/betaold) p
__global__ void k_sor_p(const double* __restrict__ z, double* __restrict__ p, size_t n,
                        const CgDevState* st) {
  if (st->status) return;
  const double bc = st->bcoef;
  const bool first = st->iter == 0;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
       c += (size_t)gridDim.x * blockDim.x)
    p[c] = first ? z[c] : fma(bc, p[c], z[c]);
}

// w = A p with the diagonal, p.w, alpha = beta / p.w
__global__ void __launch_bounds__(256) k_sor_spmv(const double* __restrict__ d,
                                                  const double* __restrict__ a0,
                                                  const double* __restrict__ a1,
                                                  const double* __restrict__ a2,
                                                  const double* __restrict__ p,
                                                  double* __restrict__ w, int n0, int n1, int n2,
                                                  CgDevState* st, double* partials) {
  if (st->status) return;
  const size_t s1 = (size_t)n0, s2 = (size_t)n0 * n1, n = s2 * n2;
  double acc[1] = {0.0};
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
       c += (size_t)gridDim.x * blockDim.x) {
    const int i0 = (int)(c % s1);
    const int i1 = (int)((c / s1) % n1);
    const int i2 = (int)(c / s2);
    const double pc = p[c];
    double v = d[c] * pc;
    if (i0 > 0) v = fma(a0[c - 1], p[c - 1], v);
    if (i0 + 1 < n0) v = fma(a0[c], p[c + 1], v);
    if (i1 > 0) v = fma(a1[c - s1], p[c - s1], v);
    if (i1 + 1 < n1) v = fma(a1[c], p[c + s1], v);
    if (i2 > 0) v = fma(a2[c - s2], p[c - s2], v);
    if (i2 + 1 < n2) v = fma(a2[c], p[c + s2], v);
    w[c] = v;
    acc[0] = fma(pc, v, acc[0]);
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

// x += a p, r -= a w
__global__ void k_sor_update(double* __restrict__ x, double* __restrict__ r,
                             const double* __restrict__ p, const double* __restrict__ w,
                             size_t n, const CgDevState* st) {
  if (st->status) return;
  const double a = st->a;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
       c += (size_t)gridDim.x * blockDim.x) {
    x[c] = fma(a, p[c], x[c]);
    r[c] = fma(-a, w[c], r[c]);
  }
}

// systems up to this many unknowns sweep in one block
constexpr size_t kSorBlockMax = 1u << 16;

}  // namespace

int KrylovSolver::ensure_sor(size_t n) {
  if (n <= cap_sor && invd) return FREHG_OK;
  cudaFree(invd);
  cudaFree(zs);
  invd = zs = nullptr;
  FG_CUDA(cudaMalloc(&invd, n * sizeof(double)));
  FG_CUDA(cudaMalloc(&zs, n * sizeof(double)));
  cap_sor = n;
  return FREHG_OK;
}

// one preconditioner application r -> z on stream st
static void sor_apply(const SorGeom& g, const Stencil64& A, const double* invd, const double* r,
                      double* z, const CgDevState* dst, cudaStream_t st, Profiler* prof) {
  const size_t n = A.n;
  const long cols = (long)g.n[1] * g.n[2];
  if (n <= kSorBlockMax) {
    int bs = (int)((cols + 31) / 32 * 32);
    bs = bs < 32 ? 32 : (bs > 1024 ? 1024 : bs);
    FG_LAUNCH(prof, st, "k_sor_block", 56.0 * (double)n,
              k_sor_block<<<1, bs, 0, st>>>(g, A.a0, A.a1, A.a2, invd, r, z, dst));
    return;
  }
  const int nb = (int)((cols + 255) / 256);
  for (int w = 0; w <= g.w_end; ++w)
    FG_LAUNCH(prof, st, "k_sor_plane_fwd", 48.0 * (double)n / (g.w_end + 1),
              k_sor_plane<true><<<nb, 256, 0, st>>>(g, w, A.a0, A.a1, A.a2, invd, r, z, dst));
  for (int w = g.w_end; w >= 0; --w)
    FG_LAUNCH(prof, st, "k_sor_plane_bwd", 48.0 * (double)n / (g.w_end + 1),
              k_sor_plane<false><<<nb, 256, 0, st>>>(g, w, A.a0, A.a1, A.a2, invd, nullptr, z,
                                                     dst));
}

int KrylovSolver::solve_sor(Stencil64& A, double* x_out, const frehg_solver_config& cfg,
                            cudaStream_t st, CgResult* res) {
  if (A.scaled || A.f32_entries) {
    set_error("pc_type 'sor' needs the unscaled FP64 operator; reassemble the system");
    return FREHG_ERR_STATE;
  }
  const size_t n = A.n;
  FG_TRY(ensure_sor(n));
  const SorGeom g = sor_geom(A);
  CgDevState init;
  memset(&init, 0, sizeof(init));
  init.rtol = cfg.rtol;
  init.atol = cfg.atol;
  init.divtol = 1.0e4;
  init.max_it = cfg.max_it;
  FG_CUDA(cudaMemcpyAsync(dst, &init, sizeof(CgDevState), cudaMemcpyHostToDevice, st));
  const int nb = reduction_blocks(n, 256, 4);
  const double dn = (double)n;
  double* xs = x;  // the graph keeps fixed pointers; x_out receives a copy
  FG_LAUNCH(prof, st, "k_sor_prep", 40.0 * dn,
            k_sor_prep<<<nb, 256, 0, st>>>(A.s, A.b, invd, xs, r, n));
  sor_apply(g, A, invd, r, zs, dst, st, prof);
  FG_LAUNCH(prof, st, "k_sor_dots", 16.0 * dn,
            k_sor_dots<true><<<nb, 256, 0, st>>>(zs, r, n, dst, partials));
  FG_CUDA(cudaGetLastError());

  // one iteration: p, w = A p (alpha), x/r update, z = M r, norms and beta
  auto iteration = [&](cudaStream_t s, Profiler* pr) {
    FG_LAUNCH(pr, s, "k_sor_p", 24.0 * dn, k_sor_p<<<nb, 256, 0, s>>>(zs, p, n, dst));
    FG_LAUNCH(pr, s, "k_sor_spmv", 48.0 * dn,
              k_sor_spmv<<<nb, 256, 0, s>>>(A.s, A.a0, A.a1, A.a2, p, w, A.n0, A.n1, A.n2, dst,
                                            partials));
    FG_LAUNCH(pr, s, "k_sor_update", 48.0 * dn,
              k_sor_update<<<nb, 256, 0, s>>>(xs, r, p, w, n, dst));
    sor_apply(g, A, invd, r, zs, dst, s, pr);
    FG_LAUNCH(pr, s, "k_sor_dots", 16.0 * dn,
              k_sor_dots<false><<<nb, 256, 0, s>>>(zs, r, n, dst, partials));
  };
  const int per_it = 4 + (n <= kSorBlockMax ? 1 : 2 * (g.w_end + 1));
  int chunk = 4096 / per_it;
  chunk = chunk < 1 ? 1 : (chunk > 32 ? 32 : chunk);

  FG_CUDA(cudaMemcpyAsync(hst, dst, sizeof(CgDevState), cudaMemcpyDeviceToHost, st));
  FG_CUDA(cudaStreamSynchronize(st));
  if (prof && prof->on) {
    for (int q = 0; q < cfg.max_it + 1 && hst->status == 0; ++q) {
      iteration(st, prof);
      FG_CUDA(cudaGetLastError());
      FG_CUDA(cudaMemcpyAsync(hst, dst, sizeof(CgDevState), cudaMemcpyDeviceToHost, st));
      FG_CUDA(cudaStreamSynchronize(st));
      FG_TRY(prof->flush());
    }
  } else if (hst->status == 0) {
    const bool rebuild = !gsor || gsor_key != (const void*)A.a0 || gsor_key2 != (const void*)invd ||
                         gsor_stream != st || gsor_n != n;
    if (rebuild) {
      if (gsor) cudaGraphExecDestroy(gsor);
      gsor = nullptr;
      cudaStream_t cap_st;
      FG_CUDA(cudaStreamCreateWithFlags(&cap_st, cudaStreamNonBlocking));
      cudaGraph_t graph;
      FG_CUDA(cudaStreamBeginCapture(cap_st, cudaStreamCaptureModeThreadLocal));
      for (int q = 0; q < chunk; ++q) iteration(cap_st, nullptr);
      cudaError_t e = cudaStreamEndCapture(cap_st, &graph);
      cudaStreamDestroy(cap_st);
      if (e != cudaSuccess) {
        set_error("SOR graph capture failed: %s", cudaGetErrorString(e));
        return FREHG_ERR_CUDA;
      }
      e = cudaGraphInstantiate(&gsor, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) {
        set_error("SOR graph instantiate failed: %s", cudaGetErrorString(e));
        return FREHG_ERR_CUDA;
      }
      gsor_key = A.a0;
      gsor_key2 = invd;
      gsor_stream = st;
      gsor_n = n;
    }
    const int max_launch = cfg.max_it / chunk + 2;
    int q = 0;
    for (; q < max_launch; ++q) {
      FG_CUDA(cudaGraphLaunch(gsor, st));
      if (prof) prof->launches += (int64_t)per_it * chunk;
      FG_CUDA(cudaMemcpyAsync(hst, dst, sizeof(CgDevState), cudaMemcpyDeviceToHost, st));
      FG_CUDA(cudaStreamSynchronize(st));
      if (hst->status != 0) break;
    }
    if (q == max_launch) {
      set_error("SOR Krylov loop: device status still running after %d chunk launches",
                max_launch);
      return FREHG_ERR_STATE;
    }
  }
  res->its = hst->its;
  res->reason = hst->status;
  res->rnorm = hst->dp;
  res->inner_its = hst->its;
  res->ir_its = 0;
  if (hst->status < 0) {
    set_error("KSP diverged (reason %d) after %d iterations, residual norm %g", hst->status,
              hst->its, hst->dp);
    return hst->status == kDivergedNanOrInf ? FREHG_ERR_NONFINITE : FREHG_ERR_NOT_CONVERGED;
  }
  if (x_out && x_out != x)
    FG_CUDA(cudaMemcpyAsync(x_out, x, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  return FREHG_OK;
}

}  // namespace fg
