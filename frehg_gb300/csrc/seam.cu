// frehg_cg_* / frehg_system_*: the linear-solver seam on the GPU.
//
// Replaces LinearSolver / SparseSystem / makeLinearSolver
// (include/frehg2/linear/LinearSolver.hpp:18-33, SparseSystem.hpp:15-40,
// src/linear/backends/LinearSolverFactory.cpp:9-16, PetscLinearSolver.cpp:30-220) for callers
// that assemble a 7-point system row by row in Decomp3D's owned order (k fastest,
// row = (j*nx + i)*nz + k, src/linear/DomainDecomposition.cpp:235-256).  The rows are decoded
// into the stencil form the device solver uses (diagonal + one coupling per axis); the device
// arrays use the owned order directly, with axis 0 = k, axis 1 = i, axis 2 = j.
#include "internal.h"

#include <cmath>
#include <cstdarg>
#include <cstring>
#include <vector>

using namespace fg;

// ------------------------------------------------------------------------------------------
// errors / defaults (shared by every entry point of the library)

namespace fg {
static thread_local char g_err[1024] = {0};
void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
void clear_error() { g_err[0] = 0; }
}  // namespace fg

struct frehg_cg {
  frehg_solver_config cfg;
  KrylovSolver ksp;
  CgResult last;
  cudaStream_t stream = nullptr;
  ~frehg_cg() {
    if (stream) cudaStreamDestroy(stream);
  }
};

struct frehg_system {
  frehg_cg* cg = nullptr;
  int nx = 0, ny = 0, nz = 0;
  size_t n = 0;
  // host staging of the 7 coefficients per row: diag, +/- along k, i, j
  std::vector<double> diag, up0, dn0, up1, dn1, up2, dn2;
  Stencil64 A;
  double* x = nullptr;  // device solution
  bool assembled = false;
  bool have_rhs = false;
  ~frehg_system() {
    A.release();
    cudaFree(x);
  }
};

extern "C" {

const char* frehg_last_error(void) { return fg::g_err; }

void frehg_soil_params_default(frehg_soil_params* s) {
  s->alpha = 1.43;
  s->n = 1.56;
  s->theta_s = 0.33;
  s->theta_r = 0.0;
  s->Ks_x = 0.0;
  s->Ks_y = 0.0;
  s->Ks_z = 2.89e-6;
  s->Ss = 1.0e-5;
  s->use_vg = 1;
  s->use_mvg = 0;
  s->air_entry = -0.02;
}

void frehg_re_params_default(frehg_re_params* p) {
  memset(p, 0, sizeof(*p));
  frehg_soil_params_default(&p->soil);
  p->dx = 1.0;
  p->dy = 1.0;
  p->dz = 0.01;
  p->botz = -1.0;
  p->dt = 1.0e-4;
  p->dt_min = 1.0e-4;
  p->dt_max = 2.0;
  p->co_max = 2.0;
  p->adaptive_dt = 1;
  p->use_corrector = 1;
  p->bc_type[5] = 1;
  p->picard_max_it = 50;
  p->picard_tol = 1.0e-6;
  p->picard_fp64 = -1;
}

void frehg_solver_config_default(frehg_solver_config* c) {
  memset(c, 0, sizeof(*c));
  strcpy(c->ksp_type, "cg");
  strcpy(c->pc_type, "jacobi");
  c->rtol = 1.0e-8;
  c->atol = 1.0e-50;
  c->max_it = 10000;
  c->precision = 0;
  c->ir_rtol = 1.0e-10;
  c->inner_rtol = 1.0e-4;
}

int frehg_build_arch(void) {
#ifdef FREHG_BUILD_ARCH
  return FREHG_BUILD_ARCH;
#else
  return 0;
#endif
}

int frehg_cg_create(const frehg_solver_config* cfg, frehg_cg** out) {
  clear_error();
  FG_ARG(cfg && out, "null argument");
  if (strcmp(cfg->ksp_type, "cg") != 0 && strcmp(cfg->ksp_type, "fcg") != 0) {
    set_error("makeLinearSolver: ksp_type '%s' is not available on the gb300 backend (cg, fcg)",
              cfg->ksp_type);
    return FREHG_ERR_UNSUPPORTED;
  }
  if (strcmp(cfg->pc_type, "jacobi") != 0 && strcmp(cfg->pc_type, "sor") != 0) {
    set_error("makeLinearSolver: pc_type '%s' is not available on the gb300 backend (jacobi, sor)",
              cfg->pc_type);
    return FREHG_ERR_UNSUPPORTED;
  }
  if (!strcmp(cfg->pc_type, "sor") && cfg->precision != 0) {
    set_error("makeLinearSolver: pc_type 'sor' runs in FP64 (precision 0)");
    return FREHG_ERR_UNSUPPORTED;
  }
  FG_ARG(cfg->rtol > 0 && cfg->max_it > 0, "rtol and max_it must be positive");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    set_error("no CUDA device");
    return FREHG_ERR_NO_DEVICE;
  }
  frehg_cg* cg = new frehg_cg();
  cg->cfg = *cfg;
  if (cudaStreamCreateWithFlags(&cg->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete cg;
    set_error("cudaStreamCreate failed");
    return FREHG_ERR_CUDA;
  }
  *out = cg;
  return FREHG_OK;
}

int frehg_cg_destroy(frehg_cg* cg) {
  clear_error();
  if (cg) {
    cudaStreamSynchronize(cg->stream);
    delete cg;
  }
  return FREHG_OK;
}

int frehg_system_create(frehg_cg* cg, int nx, int ny, int nz, frehg_system** out) {
  clear_error();
  FG_ARG(cg && out, "null argument");
  FG_ARG(nx > 0 && ny > 0 && nz > 0, "grid sizes must be positive");
  frehg_system* s = new frehg_system();
  s->cg = cg;
  s->nx = nx;
  s->ny = ny;
  s->nz = nz;
  s->n = (size_t)nx * ny * nz;
  for (auto* v : {&s->diag, &s->up0, &s->dn0, &s->up1, &s->dn1, &s->up2, &s->dn2})
    v->assign(s->n, 0.0);
  if (s->A.alloc(nz, nx, ny) != FREHG_OK || cudaMalloc(&s->x, s->n * sizeof(double)) != cudaSuccess) {
    delete s;
    set_error("device allocation for the system failed");
    return FREHG_ERR_CUDA;
  }
  // owned order (k, i, j) on axes (0, 1, 2): the reference's row order is j slowest, then i, k
  s->A.ref_order[0] = 2;
  s->A.ref_order[1] = 1;
  s->A.ref_order[2] = 0;
  *out = s;
  return FREHG_OK;
}

int frehg_system_destroy(frehg_system* s) {
  clear_error();
  delete s;
  return FREHG_OK;
}

int frehg_system_zero_entries(frehg_system* s) {
  clear_error();
  FG_ARG(s, "null handle");
  for (auto* v : {&s->diag, &s->up0, &s->dn0, &s->up1, &s->dn1, &s->up2, &s->dn2})
    std::fill(v->begin(), v->end(), 0.0);
  s->assembled = false;
  return FREHG_OK;
}

int frehg_system_begin_assembly(frehg_system* s) {
  clear_error();
  FG_ARG(s, "null handle");
  return FREHG_OK;
}

// place one (row, col, val) triplet; ADD_VALUES semantics
static int place(frehg_system* s, long row, long col, double v) {
  FG_ARG(row >= 0 && (size_t)row < s->n, "row %ld outside [0,%zu)", row, s->n);
  FG_ARG(col >= 0 && (size_t)col < s->n, "column %ld outside [0,%zu)", col, s->n);
  const long n0 = s->nz, n1 = s->nx;
  const long k = row % n0, i = (row / n0) % n1, j = row / (n0 * n1);
  const long d = col - row;
  if (d == 0) {
    s->diag[row] += v;
    return FREHG_OK;
  }
  if (d == 1 && k + 1 < n0) { s->up0[row] += v; return FREHG_OK; }
  if (d == -1 && k > 0) { s->dn0[row] += v; return FREHG_OK; }
  if (d == n0 && i + 1 < n1) { s->up1[row] += v; return FREHG_OK; }
  if (d == -n0 && i > 0) { s->dn1[row] += v; return FREHG_OK; }
  if (d == n0 * n1 && j + 1 < s->ny) { s->up2[row] += v; return FREHG_OK; }
  if (d == -n0 * n1 && j > 0) { s->dn2[row] += v; return FREHG_OK; }
  set_error("column %ld is not a 7-point neighbour of row %ld", col, row);
  return FREHG_ERR_BAD_ARG;
}

int frehg_system_add_row(frehg_system* s, int global_row, int ncols, const int* cols,
                         const double* vals) {
  clear_error();
  FG_ARG(s && (ncols == 0 || (cols && vals)), "null argument");
  FG_ARG(ncols >= 0 && ncols <= 7, "ncols must be in [0,7]");
  for (int q = 0; q < ncols; ++q) FG_TRY(place(s, global_row, cols[q], vals[q]));
  s->assembled = false;
  return FREHG_OK;
}

int frehg_system_add_coo(frehg_system* s, const int* rows, const int* cols, const double* vals,
                         int64_t n, int on_device) {
  clear_error();
  FG_ARG(s && n >= 0 && (n == 0 || (rows && cols && vals)), "bad argument");
  std::vector<int> hr, hc;
  std::vector<double> hv;
  if (on_device) {
    hr.resize(n);
    hc.resize(n);
    hv.resize(n);
    FG_CUDA(cudaMemcpy(hr.data(), rows, n * sizeof(int), cudaMemcpyDeviceToHost));
    FG_CUDA(cudaMemcpy(hc.data(), cols, n * sizeof(int), cudaMemcpyDeviceToHost));
    FG_CUDA(cudaMemcpy(hv.data(), vals, n * sizeof(double), cudaMemcpyDeviceToHost));
    rows = hr.data();
    cols = hc.data();
    vals = hv.data();
  }
  for (int64_t q = 0; q < n; ++q) FG_TRY(place(s, rows[q], cols[q], vals[q]));
  s->assembled = false;
  return FREHG_OK;
}

int frehg_system_end_assembly(frehg_system* s) {
  clear_error();
  FG_ARG(s, "null handle");
  const long n0 = s->nz, n01 = (long)s->nz * s->nx;
  // the Krylov method needs a symmetric operator: every coupling must match its transpose
  for (size_t r = 0; r < s->n; ++r) {
    const double pairs[3][2] = {{s->up0[r], r + 1 < s->n ? s->dn0[r + 1] : 0.0},
                                {s->up1[r], r + n0 < s->n ? s->dn1[r + n0] : 0.0},
                                {s->up2[r], r + n01 < s->n ? s->dn2[r + n01] : 0.0}};
    for (int q = 0; q < 3; ++q) {
      const double a = pairs[q][0], b = pairs[q][1];
      if (std::fabs(a - b) > 1e-12 * std::fmax(std::fabs(a), std::fabs(b))) {
        set_error("operator is not symmetric at row %zu (%g vs %g): CG needs an SPD matrix", r, a,
                  b);
        return FREHG_ERR_UNSUPPORTED;
      }
    }
  }
  FG_CUDA(cudaMemcpy(s->A.s, s->diag.data(), s->n * sizeof(double), cudaMemcpyHostToDevice));
  FG_CUDA(cudaMemcpy(s->A.a0, s->up0.data(), s->n * sizeof(double), cudaMemcpyHostToDevice));
  FG_CUDA(cudaMemcpy(s->A.a1, s->up1.data(), s->n * sizeof(double), cudaMemcpyHostToDevice));
  FG_CUDA(cudaMemcpy(s->A.a2, s->up2.data(), s->n * sizeof(double), cudaMemcpyHostToDevice));
  s->A.scaled = false;
  s->A.s_in_r = false;
  s->A.f32_entries = false;
  s->assembled = true;
  return FREHG_OK;
}

int frehg_system_set_rhs(frehg_system* s, const double* b, int on_device) {
  clear_error();
  FG_ARG(s && b, "null argument");
  FG_CUDA(cudaMemcpyAsync(s->A.b, b, s->n * sizeof(double),
                          on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                          s->cg->stream));
  s->have_rhs = true;
  return FREHG_OK;
}

int frehg_system_get_solution(frehg_system* s, double* x, int on_device) {
  clear_error();
  FG_ARG(s && x, "null argument");
  FG_CUDA(cudaMemcpyAsync(x, s->x, s->n * sizeof(double),
                          on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                          s->cg->stream));
  FG_CUDA(cudaStreamSynchronize(s->cg->stream));
  return FREHG_OK;
}

int frehg_cg_setup(frehg_cg* cg, frehg_system* s) {
  clear_error();
  FG_ARG(cg && s, "null argument");
  if (!s->assembled) {
    set_error("setup before end_assembly");
    return FREHG_ERR_STATE;
  }
  FG_TRY(cg->ksp.ensure(s->n));
  // PCSOR works on the unscaled operator (D and L); Jacobi-PCG on D^-1/2 A D^-1/2
  if (!strcmp(cg->cfg.pc_type, "sor")) return FREHG_OK;
  return cg->ksp.scale(s->A, cg->stream);
}

int frehg_cg_solve(frehg_cg* cg, frehg_system* s, const double* b, double* x, int on_device) {
  clear_error();
  FG_ARG(cg && s, "null argument");
  FG_TRY(frehg_cg_setup(cg, s));
  if (b) FG_TRY(frehg_system_set_rhs(s, b, on_device));
  if (!s->have_rhs) {
    set_error("solve without a right-hand side");
    return FREHG_ERR_STATE;
  }
  CgResult res;
  const int rc = cg->ksp.solve(s->A, s->x, cg->cfg, cg->stream, &res);
  cg->last = res;
  if (rc != FREHG_OK) return rc;
  if (x) FG_TRY(frehg_system_get_solution(s, x, on_device));
  FG_CUDA(cudaStreamSynchronize(cg->stream));
  return FREHG_OK;
}

int frehg_cg_iteration_count(const frehg_cg* cg, int* its) {
  clear_error();
  FG_ARG(cg && its, "null argument");
  *its = cg->last.its;
  return FREHG_OK;
}

int frehg_cg_residual_norm(const frehg_cg* cg, double* rnorm) {
  clear_error();
  FG_ARG(cg && rnorm, "null argument");
  *rnorm = cg->last.rnorm;
  return FREHG_OK;
}

int frehg_cg_converged_reason(const frehg_cg* cg, int* reason) {
  clear_error();
  FG_ARG(cg && reason, "null argument");
  *reason = cg->last.reason;
  return FREHG_OK;
}

int frehg_cg_set_fused_iteration(frehg_cg* cg, int on) {
  clear_error();
  FG_ARG(cg, "null handle");
  FG_ARG(on >= -1 && on <= 1, "on must be -1, 0 or 1");
  cg->ksp.fused64 = on;
  return FREHG_OK;
}

}  // extern "C"
