// Shared internals of libfrehg_gb300: error plumbing, the device Krylov solver, soil tables.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/frehg_gb300.h"

namespace fg {

// ------------------------------------------------------------------------------------------
// errors: every C entry point returns an int status and records text for frehg_last_error().
void set_error(const char* fmt, ...);
void clear_error();

#define FG_CUDA(call)                                                                    \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      ::fg::set_error("%s:%d: %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
      return FREHG_ERR_CUDA;                                                             \
    }                                                                                    \
  } while (0)

#define FG_TRY(expr)            \
  do {                          \
    int rc_ = (expr);           \
    if (rc_ != FREHG_OK) return rc_; \
  } while (0)

#define FG_ARG(cond, ...)                  \
  do {                                     \
    if (!(cond)) {                         \
      ::fg::set_error(__VA_ARGS__);        \
      return FREHG_ERR_BAD_ARG;            \
    }                                      \
  } while (0)

// ------------------------------------------------------------------------------------------
// Launch accounting and optional per-kernel event timing.
class Profiler {
 public:
  bool on = false;
  int64_t launches = 0;
  ~Profiler();
  void reset();
  // bracket one launch: begin() before, end() after (no-ops while off)
  int begin(cudaStream_t st);
  void end(int slot, cudaStream_t st, const char* name, double bytes);
  // after the stream has been synchronised: fold finished event pairs into the table
  int flush();
  // n launches of `name` (already flushed) returned without work
  void idle(const char* name, int64_t n);
  struct Stat {
    std::string name;
    int64_t launches = 0;
    double ms = 0.0;
    double bytes = 0.0;
    int64_t idle = 0;
  };
  std::vector<Stat> stats;

 private:
  struct Pending {
    cudaEvent_t a, b;
    std::string name;
    double bytes;
  };
  std::vector<Pending> pending_;
  std::vector<cudaEvent_t> pool_;
  cudaEvent_t get_event();
};

// Launch bracket: counts the launch and, while profiling, times it with CUDA events.
#define FG_LAUNCH(prof, st, name, bytes, ...)           \
  do {                                                  \
    const int slot_ = (prof) ? (prof)->begin(st) : -1; \
    __VA_ARGS__;                                        \
    if (prof) (prof)->end(slot_, st, name, bytes);      \
  } while (0)

// Upper bound of the blocks any reduction kernel launches (partials buffers are sized to it).
constexpr int kMaxRedBlocks = 32768;
// largest system the FP64 Jacobi-PCG runs as one launch per iteration by default: on GB300 the
// one-launch form is up to 8 % faster up to about 32k unknowns; beyond, its two grid barriers
// and half occupancy weigh about as much as the three kernels' launch gaps (25 % slower at
// 262k, 5 % faster at 1M, 6 % slower at 2M and 8.4M unknowns)
constexpr size_t kFusedAutoCells = 65536;
constexpr int kNumSMs = 152;

// ------------------------------------------------------------------------------------------
// 7-point symmetric stencil operator on an n0 x n1 x n2 box (axis 0 fastest).
// Before scaling: d = diagonal, a0/a1/a2 = coupling of cell c with its +1 neighbour along each
// axis (0 where that neighbour does not exist).  After scale(): a* hold D^-1/2 A D^-1/2
// couplings and s = D^-1/2, so the operator has a unit diagonal (Jacobi PCG == CG on it).
struct Stencil64 {
  int n0 = 0, n1 = 0, n2 = 0;
  size_t n = 0;
  double* a0 = nullptr;
  double* a1 = nullptr;
  double* a2 = nullptr;
  double* s = nullptr;  // holds d before scale(), D^-1/2 after
  double* b = nullptr;  // right-hand side (unscaled)
  bool scaled = false;
  // the float-float path's preparation left s = D^-1/2 in the mixed solver's FP64 vector r
  // (as floats) and d itself in s
  bool s_in_r = false;
  // the float-float Picard assembly wrote the diagonal as floats into the first n floats of s
  // and the couplings (unscaled, as floats) into the mixed solver's FP32 operator; only the
  // float-float preparation (k_prep_ff) reads this form
  bool f32_entries = false;
  // axes from the slowest to the fastest of the reference's row order (Decomp3D: j, i, k);
  // PCSOR subtracts its neighbour terms in that order.  RE handles store (i, j, k) as axes
  // (0, 1, 2), the linear seam stores owned order (k, i, j)
  int ref_order[3] = {1, 0, 2};
  int alloc(int n0, int n1, int n2);
  void release();
};

// Single-precision copy of a scaled operator (the inner solve of the mixed-precision path).
struct Stencil32 {
  size_t n = 0;
  float* a0 = nullptr;
  float* a1 = nullptr;
  float* a2 = nullptr;
  int alloc(size_t n);
  void release();
};

// Device-resident Krylov state (PETSc KSPSolve_CG + KSPConvergedDefault scalars).
struct CgDevState {
  double beta, betaold, bcoef, a, dpi, dpiold, dp, rnorm0, ttol;
  double rtol, atol, divtol;
  int its, max_it, status, iter;
  unsigned int arrive[8];
  double ir_bnorm, ir_rnorm;  // refinement loop norms (mixed precision)
  double rscale;              // the inner right-hand side is r~ / rscale (mixed precision)
  int ir_its;
  int rhs_rescale;  // k_prep_ff: its power-of-two scaled right-hand side needs k_ir_scale instead
  // grid barrier of the one-launch CG iteration (k_cg_iter): arrival count, generation, and
  // the flag a block sets when its bounded wait ran out
  unsigned int bar_count, bar_gen;
  int bar_timeout;
  int pad_;
};

// KSPConvergedReason values
enum {
  kConvergedRtol = 2,
  kConvergedAtol = 3,
  kDivergedIts = -3,
  kDivergedDtol = -4,
  kDivergedIndefinitePc = -8,
  kDivergedNanOrInf = -9,
  kDivergedIndefiniteMat = -10,
  // not a PETSc reason: a grid barrier of the one-launch CG iteration did not complete in time
  kGridBarrierTimeout = -90,
};

struct CgResult {
  int fallback = 0;   // the learned preconditioner was dropped for Jacobi during this solve
  int its = 0;
  int reason = 0;
  double rnorm = 0.0;
  int inner_its = 0;  // mixed precision: total fp32 iterations
  int ir_its = 0;     // mixed precision: refinement sweeps
};

// Learned preconditioner context of a solve (the network and its per-cell input fields).
}  // namespace fg
struct frehg_unet;
namespace fg {
int unet_apply(frehg_unet* net, int nx, int ny, int nz, const float* r, const float* lnk,
               const float* cap, float* z, cudaStream_t st);
struct NetPrecond {
  frehg_unet* net = nullptr;
  const float* lnk = nullptr;
  const float* cap = nullptr;
  int max_inner = 0;  // fall back to Jacobi CG beyond this many inner iterations (0 = never)
};

// Jacobi-preconditioned CG in FP64 (one cooperative launch or three kernels per iteration,
// CUDA-graph chunks), with an optional FP32 inner solve under FP64 iterative refinement.
class KrylovSolver {
 public:
  ~KrylovSolver();
  int ensure(size_t n);  // work vectors for up to n unknowns
  // Scale the operator in place (s = D^-1/2, a* -> D^-1/2 A D^-1/2).  Idempotent.
  int scale(Stencil64& A, cudaStream_t st);
  // Solve A x = b (A scaled, b unscaled in A.b).  x_out receives the unscaled solution.
  int solve(Stencil64& A, double* x_out, const frehg_solver_config& cfg, cudaStream_t st,
            CgResult* res);

  size_t cap = 0;
  double *x = nullptr, *r = nullptr, *p = nullptr, *w = nullptr;
  double* partials = nullptr;
  CgDevState* dst = nullptr;
  CgDevState* hst = nullptr;  // pinned mirror
  // mixed precision buffers
  int ensure32(size_t n);
  size_t cap32 = 0;
  float *xf = nullptr, *rf = nullptr, *pf = nullptr, *wf = nullptr;
  double* rres = nullptr;  // fp64 true residual
  Stencil32 op32;
  CgDevState* dst32 = nullptr;  // inner FP32 solve state
  CgDevState* hst32 = nullptr;
  cudaStream_t g_stream32 = nullptr;
  size_t g_n32 = 0;
  long g32_shape = 0;
  // graphs
  cudaGraphExec_t g64 = nullptr;
  cudaGraphExec_t g32 = nullptr;
  cudaGraphExec_t g32s = nullptr;  // first, short chunk of the inner solve
  const void* g64_key = nullptr;
  const void* g64_key2 = nullptr;
  // the FP64 Jacobi-PCG iteration as one cooperative launch (k_cg_iter) rather than three
  // kernels, where the device has cooperative launches: 1 always, 0 never, -1 (default) for
  // systems of at most kFusedAutoCells unknowns (larger ones run faster as three kernels);
  // g64_form: the form g64 holds; coop_failed: a cooperative capture failed, use three kernels
  int fused64 = -1;
  int g64_form = -1;
  bool coop_failed = false;
  Profiler* prof = nullptr;  // owner's profiler (launch counts, optional event timing)
  NetPrecond net;            // learned preconditioner (FCG inner solves when set)
  // the mixed path's scaled couplings in float-float (2^-48) instead of FP64 products: for
  // solves whose result is an update of an iterate (Picard), where the operator's last bits
  // change the update, not the fixed point; solves whose result is the solution keep FP64
  bool ff_operator = false;
  // leave the solution scaled: x_out is not written, the caller applies x = s x~ itself from
  // x (x~) and scale_vector(A) (the Picard update fuses it into h += x)
  bool keep_scaled = false;
  const double* scale_vector(const Stencil64& A) const { return A.s_in_r ? r : A.s; }
  float* zf = nullptr;
  // vertical-line preconditioner (FP32 factors and sweep scratch)
  int ensure_line(size_t n);
  // scaling of the operator for the mixed path (sq = D^1/2 into r, FP32 copy, line factors)
  int prep_mixed(Stencil64& A, cudaStream_t st, bool line, const frehg_solver_config& cfg);
  bool first_done = false;  // prep_mixed formed the first refinement residual and its state
  bool first_line_done = false;  // ... and the line preconditioner's first application
  // first residual norms of earlier solves, the scale of the next one's: slot 0 for the first
  // solve of a time step (its residual is orders of magnitude above the previous step's last
  // one), slot 1 for the later (Picard) solves; the caller picks the slot
  double first_rnorm[2] = {0.0, 0.0};
  int rnorm_slot = 1;
  size_t cap_line = 0;
  float *lkf = nullptr, *dinvf = nullptr, *uf = nullptr;
  // PCSOR (pc_type "sor", precision 0): 1/d, the preconditioned residual, iteration graph
  int ensure_sor(size_t n);
  size_t cap_sor = 0;
  double *invd = nullptr, *zs = nullptr;
  cudaGraphExec_t gsor = nullptr;
  const void* gsor_key = nullptr;
  const void* gsor_key2 = nullptr;
  cudaStream_t gsor_stream = nullptr;
  size_t gsor_n = 0;
  int g32_line = 0;
  const void* g32_key = nullptr;
  cudaStream_t g_stream = nullptr;
  size_t g_n = 0;

 private:
  int solve64(Stencil64& A, double* x_out, const frehg_solver_config& cfg, cudaStream_t st,
              CgResult* res);
  int solve_mixed(Stencil64& A, double* x_out, const frehg_solver_config& cfg, cudaStream_t st,
                  CgResult* res);
  // CG + PCSOR on the unscaled operator; the solution is left in x and copied to x_out
  int solve_sor(Stencil64& A, double* x_out, const frehg_solver_config& cfg, cudaStream_t st,
                CgResult* res);
  int run_chunks(cudaGraphExec_t g, cudaStream_t st, int max_it, int chunk,
                 int launches_per_it = 3);
  int finish64(Stencil64& A, double* x_out, cudaStream_t st, CgResult* res, int nb);
};

// Launch helpers shared by the stencil kernels: a (32 x 8) thread tile over axes 0/1 marching
// along axis 2 in slabs.
struct StencilLaunch {
  dim3 grid, block;
  int planes;  // axis-2 planes per block
  int tiles;   // 32 x 8 tiles over axes 0/1 (blocks stride over them)
};
StencilLaunch stencil_launch(int n0, int n1, int n2);

int reduction_blocks(size_t n, int threads, int per_thread);

// Small device-to-host read-backs (the solvers' control state, a few hundred bytes) ordered on
// st: a one-warp kernel writes them into mapped page-locked host memory (host_mapped, from
// alloc_mapped), so that they do not queue on the copy engines behind a bulk result copy in
// flight.  The caller synchronises st before reading.  bytes: a multiple of 4.
int fetch_small(void* host_mapped, const void* dev, size_t bytes, cudaStream_t st);
int alloc_mapped(void** host, size_t bytes);

}  // namespace fg
