// frehg_cg_solve_noalloc: the Jacobi-preconditioned CG solve of the linear-solver seam, with
// no device allocation of its own.
//
// Who needs it: a caller that is not allowed to allocate GPU memory -- for example a component
// running inside a host framework that reserves the device memory budget up front and forbids
// its plug-ins any allocation of their own, or a time-critical loop that cannot afford the
// device-wide synchronisation cudaMalloc/cudaFree may cause.  Such a caller brings the operator,
// the right-hand side and the solution array in device memory it already owns; the solver's
// work space (scaled operator copy, four Krylov vectors, reduction partials, scalar state) lives
// in one file-scope device array of fixed size, declared below.
//
// What to know before calling it:
//  * Size limit: at most kNoAllocMaxCells unknowns.  Larger systems are refused with
//    FREHG_ERR_BAD_ARG; use frehg_cg_solve for them.
//  * The array exists once per GPU that loads this library and stays reserved until the
//    process exits: 8 x kNoAllocMaxCells doubles + 2 x 32,768 reduction slots + the scalar
//    state = 17,302,016 bytes (about 17.3 MB, 16.5 MiB).
//  * Every call looks up the array's device address (cudaGetSymbolAddress, which allocates
//    nothing) on the device that is current, so the address stays right after a device reset
//    reloads the module.  The first call on a device loads the module there; make that first
//    call before any stream capture on the device.
//  * Every call on a device shares the one array and overwrites what the previous call left
//    there; the scalar state is reset at the start of each call.  Calls that overlap on the GPU
//    (two streams, or two host threads on one device) race on the array and corrupt each
//    other -- serialise them.
//  * No cudaMalloc, cudaFree or allocating library routine is called.
#include "internal.h"
#include "krylov_kernels.cuh"

#include <cstring>

namespace {

constexpr size_t kNoAllocMaxCells = (size_t)1 << 18;  // 262,144 unknowns (e.g. 64 x 64 x 64)
constexpr size_t kStateDoubles = 64;                  // room for fg::CgDevState
constexpr size_t kScratchDoubles =
    8 * kNoAllocMaxCells + 2 * (size_t)fg::kMaxRedBlocks + kStateDoubles;
static_assert(sizeof(fg::CgDevState) <= kStateDoubles * sizeof(double), "state slot too small");

// the work space: s, a0, a1, a2 (scaled operator copy), x~, r, p, w, partials, state
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

// Device address of the work space on the current device.  In host code the array's name is
// only a host-side stand-in; kernels must be given this address.
int scratch_address(double** out) {
  int dev = -1;
  FG_CUDA(cudaGetDevice(&dev));
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || p == nullptr) {
    fg::set_error("frehg_cg_solve_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                  cudaGetErrorString(e));
    return FREHG_ERR_CUDA;
  }
  *out = static_cast<double*>(p);
  return FREHG_OK;
}

}  // namespace

extern "C" int frehg_cg_solve_noalloc(int nx, int ny, int nz, const double* diag,
                                      const double* a_k, const double* a_i, const double* a_j,
                                      const double* b, double* x, const frehg_solver_config* cfg,
                                      void* stream, int* its, double* rnorm) {
  using namespace fg;
  clear_error();
  FG_ARG(diag && a_k && a_i && a_j && b && x && cfg, "frehg_cg_solve_noalloc: null argument");
  FG_ARG(nx > 0 && ny > 0 && nz > 0, "frehg_cg_solve_noalloc: grid sizes must be positive");
  const size_t n = (size_t)nx * ny * nz;
  FG_ARG(n <= kNoAllocMaxCells,
         "frehg_cg_solve_noalloc: %zu unknowns exceed the fixed work space of %zu unknowns; "
         "use frehg_cg_solve for larger systems", n, kNoAllocMaxCells);
  if (strcmp(cfg->ksp_type, "cg") != 0 || strcmp(cfg->pc_type, "jacobi") != 0 ||
      cfg->precision != 0) {
    set_error("frehg_cg_solve_noalloc: only ksp_type cg, pc_type jacobi, fp64");
    return FREHG_ERR_UNSUPPORTED;
  }
  FG_ARG(cfg->rtol > 0 && cfg->max_it > 0, "rtol and max_it must be positive");
  double* base = nullptr;
  FG_TRY(scratch_address(&base));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t M = kNoAllocMaxCells;
  double* s = base;
  double* a0 = base + M;
  double* a1 = base + 2 * M;
  double* a2 = base + 3 * M;
  double* xs = base + 4 * M;
  double* r = base + 5 * M;
  double* p = base + 6 * M;
  double* w = base + 7 * M;
  double* partials = base + 8 * M;
  CgDevState* dst = reinterpret_cast<CgDevState*>(base + 8 * M + 2 * (size_t)kMaxRedBlocks);

  // the caller's operator is copied, never modified; axis order is the owned order (k fastest)
  FG_CUDA(cudaMemcpyAsync(s, diag, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  FG_CUDA(cudaMemcpyAsync(a0, a_k, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  FG_CUDA(cudaMemcpyAsync(a1, a_i, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  FG_CUDA(cudaMemcpyAsync(a2, a_j, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  // fresh scalar state: stopping parameters set, every arrival counter zero
  CgDevState init;
  memset(&init, 0, sizeof(init));
  init.rtol = cfg->rtol;
  init.atol = cfg->atol;
  init.divtol = 1.0e4;
  init.max_it = cfg->max_it;
  FG_CUDA(cudaMemcpyAsync(dst, &init, sizeof(init), cudaMemcpyHostToDevice, st));

  const int n0 = nz, n1 = nx, n2 = ny;
  const int nb = reduction_blocks(n, 256, 4);
  const StencilLaunch L = stencil_launch(n0, n1, n2);
  k_diag_rsqrt<<<nb, 256, 0, st>>>(s, n);
  k_scale_offdiag<<<L.grid, L.block, 0, st>>>(a0, a1, a2, s, n0, n1, n2, L.planes, L.tiles);
  k_cg_init<<<nb, 256, 0, st>>>(s, b, xs, r, n, dst, partials);
  FG_CUDA(cudaGetLastError());
  CgDevState h;
  FG_CUDA(cudaMemcpyAsync(&h, dst, sizeof(h), cudaMemcpyDeviceToHost, st));
  FG_CUDA(cudaStreamSynchronize(st));
  const int chunk = 16;
  for (int q = 0; q < cfg->max_it / chunk + 2 && h.status == 0; ++q) {
    for (int it = 0; it < chunk; ++it) {
      k_cg_p<<<nb, 256, 0, st>>>(r, p, n, dst);
      k_cg_spmv<<<L.grid, L.block, 0, st>>>(a0, a1, a2, p, w, n0, n1, n2, L.planes, L.tiles,
                                            dst, partials);
      k_cg_update<<<nb, 256, 0, st>>>(xs, r, p, w, s, n, dst, partials);
    }
    FG_CUDA(cudaGetLastError());
    FG_CUDA(cudaMemcpyAsync(&h, dst, sizeof(h), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
  }
  k_unscale<<<nb, 256, 0, st>>>(s, xs, x, n);
  FG_CUDA(cudaGetLastError());
  FG_CUDA(cudaStreamSynchronize(st));
  if (its) *its = h.its;
  if (rnorm) *rnorm = h.dp;
  if (h.status == 0) {
    set_error("frehg_cg_solve_noalloc: iteration loop ended with the solve still running");
    return FREHG_ERR_STATE;
  }
  if (h.status < 0) {
    set_error("frehg_cg_solve_noalloc: KSP diverged (reason %d) after %d iterations", h.status,
              h.its);
    return h.status == kDivergedNanOrInf ? FREHG_ERR_NONFINITE : FREHG_ERR_NOT_CONVERGED;
  }
  return FREHG_OK;
}
