// frehg_re_*: the Richards-equation step on one GPU (replaces class ReSolver,
// src/re/ReSolver.hpp:48-156 / src/re/ReSolver.cpp).  The whole step runs on the device; the
// host only issues launches and reads the Krylov / reallocation status words.
#include "internal.h"
#include "re_kernels.cuh"
#include "picard.cuh"
#include "picard_ff.cuh"
#include "picard_tma.cuh"
#include "krylov_kernels.cuh"

#include <algorithm>
#include <cmath>
#include <chrono>
#include <cstring>
#include <vector>

using namespace fg;

struct frehg_re {
  int nx = 0, ny = 0, nz = 0;
  size_t n = 0, ncol = 0;
  frehg_re_params p;
  frehg_solver_config cfg;
  bool attached = false;
  bool have_geometry = false;
  bool have_state = false;
  bool finalized = false;
  bool ghosts_valid = false;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  int cur = 0;
  // asynchronous result copies (frehg_re_get_interior_async): their stream, the event after the
  // last copy out of state buffer q (H[q], W[q]) and whether it may still be in flight
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_ev[2] = {nullptr, nullptr};
  cudaEvent_t issue_ev = nullptr;
  bool copy_pending[2] = {false, false};
  // state
  double* H[2] = {nullptr, nullptr};
  double* W[2] = {nullptr, nullptr};
  double* kr = nullptr;
  double* wch = nullptr;
  double* cap = nullptr;
  // second set for the float-float Picard update that also forms the next iteration's
  // constitutive values (allocated on first use; swapped with the first set when taken)
  double* kr2 = nullptr;
  double* wch2 = nullptr;
  double* cap2 = nullptr;
  double* qx = nullptr;
  double* qy = nullptr;
  double* qz = nullptr;
  double* qztop = nullptr;
  double* qtop_field = nullptr;
  bool has_qtop = false;
  uint8_t* flags = nullptr;
  double* scratch = nullptr;  // n doubles for exports / Picard increments
  bool staged = false;        // Picard assembly staged through TMA (frehg_re_set_assembly_staging)
  // kr, wch, cap hold the values at the current head: set by a converged float-float Picard
  // step (its last update formed them), taken by the next step's first iteration, and cleared
  // by every call that changes the head, the soil, the parameters or the solver
  bool constit_fresh = false;
  ReScalars* sc = nullptr;
  ReScalars* sc_host = nullptr;
  double* partials = nullptr;
  double* xch = nullptr;  // surface-exchange staging (eta, bottom, q, total), on first use
  double* gh_top = nullptr;    // top-layer ghost copies (h then wc) from before an exchange
  bool top_ghost_stale = false;
  // soil
  SoilClass* cls = nullptr;
  std::vector<SoilClass> cls_host;  // host copy of the class table
  int nclass = 0;
  uint8_t* cid = nullptr;
  int cid3d = 0;
  double* fKs = nullptr;
  double* falpha = nullptr;
  // operator + Krylov
  Stencil64 A;
  KrylovSolver ksp;
  // learned preconditioner
  frehg_unet* net = nullptr;
  float* lnk_f = nullptr;  // network input fields of the current system
  float* cap_f = nullptr;
  int plain_its_ref = 0;   // inner iterations of the last network-free solve (fallback bound)
  // time policy of the learned preconditioner
  int probe_every = 32;      // a probe solve applies the network every probe_every solves
  double max_ratio = 1.0;    // network kept while its solve time <= max_ratio * plain time
  bool net_on = false;       // outcome of the last probe
  bool probe_pending = true; // the next solve with a network-free reference probes
  long solves_since_probe = 0;
  bool probe_now = false;
  double last_plain_ms = 0.0;
  double apply_ms = -1.0;    // host time of one network application at this grid (once)
  // counters / profiling
  frehg_re_counters cnt;
  Profiler prof;
  ~frehg_re();
};

frehg_re::~frehg_re() {
  for (int q = 0; q < 2; ++q) {
    cudaFree(H[q]);
    cudaFree(W[q]);
  }
  cudaFree(kr);
  cudaFree(wch);
  cudaFree(cap);
  cudaFree(kr2);
  cudaFree(wch2);
  cudaFree(cap2);
  cudaFree(qx);
  cudaFree(qy);
  cudaFree(qz);
  cudaFree(qztop);
  cudaFree(xch);
  cudaFree(gh_top);
  cudaFree(qtop_field);
  cudaFree(flags);
  cudaFree(scratch);
  cudaFree(sc);
  cudaFreeHost(sc_host);
  cudaFree(partials);
  cudaFree(cls);
  cudaFree(cid);
  cudaFree(fKs);
  cudaFree(falpha);
  cudaFree(lnk_f);
  cudaFree(cap_f);
  A.release();
  if (copy_stream) {
    cudaStreamSynchronize(copy_stream);
    cudaStreamDestroy(copy_stream);
  }
  for (cudaEvent_t e : {copy_ev[0], copy_ev[1], issue_ev})
    if (e) cudaEventDestroy(e);
  if (own_stream) cudaStreamDestroy(own_stream);
}

// Before work that writes state buffer q (-1: both): the handle's stream waits on the device for
// the result copies still reading it; host: the host waits for them (entry points that write
// the buffers with synchronous copies).
static int wait_copies(frehg_re* re, int q, bool host) {
  for (int b = 0; b < 2; ++b) {
    if ((q >= 0 && b != q) || !re->copy_pending[b]) continue;
    if (host) {
      FG_CUDA(cudaEventSynchronize(re->copy_ev[b]));
    } else {
      FG_CUDA(cudaStreamWaitEvent(re->stream, re->copy_ev[b], 0));
    }
    re->copy_pending[b] = false;
  }
  return FREHG_OK;
}


static int validate_params(const frehg_re_params* p) {
  FG_ARG(p->dx > 0 && p->dy > 0 && p->dz > 0, "dx, dy, dz must be positive");
  FG_ARG(p->scheme == 0 || p->scheme == 1, "scheme must be 0 (pca) or 1 (picard)");
  for (int q = 0; q < 4; ++q)
    if (p->bc_type[q] != 0) {
      set_error(
          "bc_type[%d]: lateral Dirichlet/fixed-flux GW boundaries are not implemented; only "
          "no-flux (0) is supported on lateral faces",
          q);
      return FREHG_ERR_UNSUPPORTED;
    }
  const int bmax = p->scheme == 1 ? 3 : 2;
  FG_ARG(p->bc_type[4] >= 0 && p->bc_type[4] <= bmax, "bc_type[4] (bottom) must be in [0,%d]", bmax);
  FG_ARG(p->bc_type[5] >= 0 && p->bc_type[5] <= 2, "bc_type[5] (top) must be 0, 1 or 2");
  if (p->baroclinic) {
    set_error("baroclinic (density-driven) coupling is not implemented");
    return FREHG_ERR_UNSUPPORTED;
  }
  if (p->sim_shallowwater) {
    set_error("sim_shallowwater: the coupled top face belongs to the SW-GW coupling, not built");
    return FREHG_ERR_UNSUPPORTED;
  }
  if (p->follow_terrain) {
    set_error("follow_terrain is not realised by the groundwater step");
    return FREHG_ERR_UNSUPPORTED;
  }
  return FREHG_OK;
}

static int upload_class0(frehg_re* re) {
  if (re->nclass > 0 && re->cid) return FREHG_OK;  // a soil map owns the table
  const SoilClass k = make_soil_class(re->p.soil);
  if (!re->cls) FG_CUDA(cudaMalloc(&re->cls, sizeof(SoilClass) * 256));
  FG_CUDA(cudaMemcpy(re->cls, &k, sizeof(SoilClass), cudaMemcpyHostToDevice));
  re->cls_host.assign(1, k);
  re->nclass = 1;
  return FREHG_OK;
}

static ReArgs make_args(frehg_re* re) {
  ReArgs a;
  memset(&a, 0, sizeof(a));
  a.nx = re->nx;
  a.ny = re->ny;
  a.nz = re->nz;
  a.n = re->n;
  a.ncol = re->ncol;
  a.dx = re->p.dx;
  a.dy = re->p.dy;
  a.dz = re->p.dz;
  a.htop = re->p.htop;
  a.hbot = re->p.hbot;
  a.qtop = re->p.qtop;
  a.qbot = re->p.qbot;
  a.co_max = re->p.co_max;
  a.dt_min = re->p.dt_min;
  a.dt_max = re->p.dt_max;
  a.bc4 = re->p.bc_type[4];
  a.bc5 = re->p.bc_type[5];
  a.full3d = re->p.use_full3d;
  a.ghosts_valid = re->ghosts_valid;
  a.adaptive = re->p.adaptive_dt;
  a.use_corrector = re->p.use_corrector;
  a.has_qtop = re->has_qtop;
  a.face_mean = re->p.face_mean;
  a.rain_rate = re->p.rain_rate;
  a.rain_until = re->p.rain_until;
  a.picard_dh_max = re->p.picard_dh_max;
  // geometric factors, so that the kernels multiply instead of dividing in FP64
  {
    const double dx = re->p.dx, dy = re->p.dy, dz = re->p.dz;
    a.inv_dx = 1.0 / dx;
    a.inv_dy = 1.0 / dy;
    a.inv_dz = 1.0 / dz;
    a.cx = dy * dz / dx;
    a.cy = dx * dz / dy;
    a.cz = dx * dy / dz;
    a.v_dz = dx * dy * dz / dz;
    a.inv_Ax = 1.0 / (dy * dz);
    a.inv_Ay = 1.0 / (dx * dz);
    a.inv_Az = 1.0 / (dx * dy);
    a.vol_cell = dx * dy * dz;
  }
  a.soil.cls = re->cls;
  a.soil.cid = re->cid;
  a.soil.cid3d = re->cid3d;
  a.soil.Ks = re->fKs;
  a.soil.alpha = re->falpha;
  a.soil.continuous_theta = re->p.scheme == 1;
  a.gh_top_h = re->top_ghost_stale ? re->gh_top : nullptr;
  a.gh_top_w = re->top_ghost_stale ? re->gh_top + re->ncol : nullptr;
  a.h_old = re->H[re->cur];
  a.w_old = re->W[re->cur];
  a.h_new = re->H[1 - re->cur];
  a.w_new = re->W[1 - re->cur];
  a.kr = re->kr;
  a.wch = re->wch;
  a.cap = re->cap;
  a.qx = re->qx;
  a.qy = re->qy;
  a.qz = re->qz;
  a.qztop = re->qztop;
  a.qtop_field = re->qtop_field;
  a.flags = re->flags;
  a.sc = re->sc;
  a.partials = re->partials;
  return a;
}

// ------------------------------------------------------------------------------------------
// simple device helpers for the C API

namespace {
__global__ void k_theta_of_h(ReArgs a, const double* __restrict__ h, double* __restrict__ w) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < a.n;
       c += (size_t)gridDim.x * blockDim.x) {
    const CellSoil s = soil_of(a.soil, c, c % a.ncol);
    w[c] = vg_theta(s, h[c]);
  }
}
__global__ void k_h_of_theta(ReArgs a, const double* __restrict__ w, double* __restrict__ h) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < a.n;
       c += (size_t)gridDim.x * blockDim.x) {
    const CellSoil s = soil_of(a.soil, c, c % a.ncol);
    h[c] = vg_head(s, w[c]);
  }
}
__global__ void k_cap_of_h(ReArgs a, const double* __restrict__ h, double* __restrict__ o) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < a.n;
       c += (size_t)gridDim.x * blockDim.x) {
    const CellSoil s = soil_of(a.soil, c, c % a.ncol);
    o[c] = vg_capacity(s, h[c]);
  }
}
// face conductances Kx/Ky/Kz as computeKFace leaves them after the step (post-solve head = the
// kr array, vertical-only closure by the step's starting water content)
__global__ void k_faces_export(ReArgs a, const double* __restrict__ wstart, int which,
                               double* __restrict__ o) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < a.n;
       c += (size_t)gridDim.x * blockDim.x) {
    const size_t col = c % a.ncol;
    const int k = (int)(c / a.ncol), i = (int)(col % a.nx), j = (int)(col / a.nx);
    const CellSoil s = soil_of(a.soil, c, col);
    const double krc = a.kr[c];
    const bool sat_c = a.full3d ? true : wstart[c] >= s.ths;
    double v = 0.0;
    if (which == 0) {
      double Kn = 0.0;
      bool sat_n = true;
      if (i + 1 < a.nx) {
        const CellSoil sn = soil_of(a.soil, c + 1, col + 1);
        Kn = sn.Ksx * a.kr[c + 1];
        if (!a.full3d) sat_n = wstart[c + 1] >= sn.ths;
      }
      v = face_x(a, i, s.Ksx * krc, Kn, s.Ksx * krc, sat_c, sat_n);
    } else if (which == 1) {
      double Kn = 0.0;
      bool sat_n = true;
      if (j + 1 < a.ny) {
        const CellSoil sn = soil_of(a.soil, c + a.nx, col + a.nx);
        Kn = sn.Ksy * a.kr[c + a.nx];
        if (!a.full3d) sat_n = wstart[c + a.nx] >= sn.ths;
      }
      v = face_y(a, j, s.Ksy * krc, Kn, s.Ksy * krc, sat_c, sat_n);
    } else {
      double Kn = 0.0;
      if (k + 1 < a.nz) {
        const CellSoil sn = soil_of(a.soil, c + a.ncol, col);
        Kn = sn.Ksz * a.kr[c + a.ncol];
      }
      v = face_z(a, k, s.Ksz * krc, Kn);
    }
    o[c] = v;
  }
}
__global__ void k_volume(ReArgs a, const double* __restrict__ w, double* out) {
  double v[1] = {0.0};
  const double V = a.dx * a.dy * a.dz;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < a.n;
       c += (size_t)gridDim.x * blockDim.x)
    v[0] += w[c] * V;
  double tot[1];
  if (grid_sum<1>(v, a.partials, &a.sc->arrive[3], tot) && flat_tid() == 0) *out = tot[0];
}
}  // namespace

static int nblocks(size_t n) { return reduction_blocks(n, 256, 4); }

namespace {
// Surface-water exchange through the top face (Coupling::exchange, src/coupling/Coupling.cpp:
// 25-166): per column the rate from the top cell's head and the ponded depth, limited by the
// ponded volume / headroom (infiltration) or the drainable volume (seepage), applied to the
// surface level and to the top cell (water content clamped, head from the water content).
// The reference takes the uniform soil parameters (re.params().soil) and dz for the top cell.
__global__ void k_surface_exchange(double* __restrict__ h, double* __restrict__ wc,
                                   double* __restrict__ eta, const double* __restrict__ bottom,
                                   double* __restrict__ q_out, SoilClass k0, int ncol, double Az,
                                   double dz, double dt, double visc, double min_depth,
                                   double* partials, unsigned int* arrive, double* total) {
  CellSoil s;
  s.alpha = k0.alpha;
  s.n = k0.n;
  s.ths = k0.ths;
  s.thr = k0.thr;
  s.Ss = k0.Ss;
  s.aev = k0.aev;
  s.m = k0.m;
  s.inv_m = k0.inv_m;
  s.inv_n = k0.inv_n;
  s.inv_ths = k0.inv_ths;
  s.Ksx = k0.Ksx;
  s.Ksy = k0.Ksy;
  s.Ksz = k0.Ksz;
  s.use_vg = k0.use_vg;
  s.use_mvg = k0.use_mvg;
  const double V = Az * dz;
  double v[1] = {0.0};
  for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < ncol;
       col += gridDim.x * blockDim.x) {
    const double dept = fmax(eta[col] - bottom[col], 0.0);
    const double wc_top = wc[col];
    // computeExchangeRates (:48-57)
    double q = Az * s.Ksz * visc * (h[col] - dept) / (0.5 * dz);
    if (dept <= min_depth && q < 0.0) q = 0.0;
    // limitExchange (:82-97); a cell filled to its headroom (drained to theta_r) is set to
    // theta_s (theta_r) exactly, which wc - q dt / V reaches only up to rounding
    int bound = 0;
    if (q < 0.0) {
      const double q_min_surf = -dept * Az / dt;
      const double q_min_gw = -(s.ths - wc_top) * V / dt;
      if (q <= q_min_gw && q_min_gw >= q_min_surf) bound = 1;
      q = fmax(q, fmax(q_min_surf, q_min_gw));
    } else if (q > 0.0) {
      const double q_max_gw = (wc_top - s.thr) * V / dt;
      if (q >= q_max_gw) bound = -1;
      q = fmin(q, q_max_gw);
    }
    q_out[col] = q;
    // applyExchangeToSurface (:113-117) and applyExchangeToGroundwater (:133-140)
    eta[col] += q * dt / Az;
    double w = fmin(fmax(wc_top - q * dt / V, s.thr), s.ths);
    if (bound) w = bound > 0 ? s.ths : s.thr;
    wc[col] = w;
    h[col] = vg_head(s, w);
    v[0] += q * dt;
  }
  double tot[1];
  if (grid_sum<1>(v, partials, arrive, tot) && flat_tid() == 0) *total = tot[0];
}

// network input fields: ln of the vertical conductivity and the moisture capacity
__global__ void k_net_fields(ReArgs a, float* __restrict__ lnk, float* __restrict__ cap) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < a.n;
       c += (size_t)gridDim.x * blockDim.x) {
    const CellSoil s = soil_of(a.soil, c, c % a.ncol);
    const double K = s.Ksz * a.kr[c];
    lnk[c] = (float)log(K > 1e-300 ? K : 1e-300);
    cap[c] = (float)a.cap[c];
  }
}
// z = M^-1 r in FP64, M the vertical-line (column tridiagonal) part of the scaled operator,
// factorised on the fly as in the FP32 inner solve's line preconditioner (training targets of
// the learned correction over the line solve; u is scratch).
__global__ void k_line_apply64(const double* __restrict__ a2, const double* __restrict__ r,
                               double* __restrict__ u, double* __restrict__ z, int ncol,
                               int nz) {
  const size_t sk = (size_t)ncol;
  for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < ncol;
       col += gridDim.x * blockDim.x) {
    size_t c = (size_t)col;
    double d = 1.0, y = r[c];
    u[c] = y;
    z[c] = 0.0;  // holds l_k until the backward sweep overwrites it
    for (int k = 1; k < nz; ++k) {
      c += sk;
      const double a = a2[c - sk];
      const double l = a / d;
      d = 1.0 - l * a;
      if (!(d > 0.0)) d = 1.0;
      y = r[c] - l * y;
      u[c] = y / d;
      z[c] = l;
    }
    // u_0 = y_0 / d_0 with d_0 = 1 already holds
    double zz = 0.0, lnext = 0.0;
    for (int k = nz - 1; k >= 0; --k) {
      const double lk = z[c];
      zz = u[c] - lnext * zz;
      lnext = lk;
      z[c] = zz;
      c -= (k > 0) ? sk : 0;
    }
  }
}

// one training pair: r~_k and the target e~_k - sub_k with e~_k = x~* - x~_k (sub = 0, r~ or
// the line solve of r~), FP32
__global__ void k_pair(const double* __restrict__ xstar, const double* __restrict__ x,
                       const double* __restrict__ r, const double* __restrict__ sub,
                       float* __restrict__ rout, float* __restrict__ eout, size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
       c += (size_t)gridDim.x * blockDim.x) {
    rout[c] = (float)r[c];
    const double e = xstar[c] - x[c];
    eout[c] = (float)(sub ? e - sub[c] : e);
  }
}
}  // namespace

// Host time of one network application on this grid (second of two calls: the first sizes
// the activation buffers).  The input is the ln K field; the cost does not depend on values.
static int time_network(frehg_re* re) {
  cudaStream_t st = re->stream;
  ReArgs a = make_args(re);
  k_net_fields<<<nblocks(re->n), 256, 0, st>>>(a, re->lnk_f, re->cap_f);
  FG_CUDA(cudaGetLastError());
  float* z = reinterpret_cast<float*>(re->scratch);  // n doubles hold n floats
  double ms = 0.0;
  for (int q = 0; q < 2; ++q) {
    FG_CUDA(cudaStreamSynchronize(st));
    const auto t0 = std::chrono::steady_clock::now();
    FG_TRY(unet_apply(re->net, re->nx, re->ny, re->nz, re->lnk_f, re->lnk_f, re->cap_f, z, st));
    FG_CUDA(cudaStreamSynchronize(st));
    ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  re->apply_ms = ms;
  return FREHG_OK;
}

// Krylov solve of the assembled system with the handle's configuration.  The learned
// preconditioners run flexible CG inside the mixed-precision refinement with
// z = M(r) + NN(r, ln K, C): M = I for pc_type "unet" (unit-diagonal Jacobi step, Jacobi-PCG
// fallback), M = the vertical-line solve for "unet-line" (line-PCG fallback).  The first solve
// runs the fallback method and sets the threshold (2x its inner iterations) beyond which a
// solve switches to it.
// whether solve_system takes the mixed-precision path (the learned preconditioners run in it)
static bool mixed_solve(const frehg_re* re) {
  return re->cfg.precision == 1 || !strncmp(re->cfg.pc_type, "unet", 4);
}

// the Picard kernels in float-float arithmetic: picard_fp64 = 0, or -1 (the default) with the
// mixed-precision solve.  With the FP64 solve the float-float kernels' noise floor in K
// (about 1e-12 relative) leaves the late Picard solves right-hand sides that an FP64 CG to
// rtol 1e-12 reduces only slowly, so the default keeps that path FP64 throughout.
static bool picard_ff(const frehg_re* re) {
  return re->p.picard_fp64 == 0 || (re->p.picard_fp64 < 0 && mixed_solve(re));
}

static int solve_system(frehg_re* re, double* x_out, CgResult* res) {
  cudaStream_t st = re->stream;
  frehg_solver_config cfg = re->cfg;
  // a Picard solve yields an update of the iterate: its operator may carry 48 bits
  re->ksp.ff_operator = re->p.scheme == 1 && picard_ff(re);
  const bool learned = !strncmp(cfg.pc_type, "unet", 4);
  re->ksp.net = NetPrecond();
  bool use_net = false;
  if (learned) {
    cfg.precision = 1;
    strcpy(cfg.pc_type, strcmp(re->cfg.pc_type, "unet-line") ? "jacobi" : "line");
    bool probe = false;
    if (re->net && re->plain_its_ref > 0) {
      // time policy: probe the network every probe_every solves (always with probe_every 0)
      probe = re->probe_every <= 0 || re->probe_pending ||
              re->solves_since_probe >= re->probe_every;
      if (probe && re->probe_every > 0) {
        // a solve applies the network at least once: when one application alone takes longer
        // than max_ratio times the whole network-free solve, no probe can pay
        if (re->apply_ms < 0.0) FG_TRY(time_network(re));
        if (re->apply_ms >= re->max_ratio * re->last_plain_ms) {
          probe = false;
          re->net_on = false;
          re->probe_pending = false;
          re->solves_since_probe = 0;
        }
      }
      use_net = probe || re->net_on;
    }
    re->probe_now = probe;
    if (use_net) {
      ReArgs a = make_args(re);
      k_net_fields<<<nblocks(re->n), 256, 0, st>>>(a, re->lnk_f, re->cap_f);
      FG_CUDA(cudaGetLastError());
      re->ksp.net.net = re->net;
      re->ksp.net.lnk = re->lnk_f;
      re->ksp.net.cap = re->cap_f;
      re->ksp.net.max_inner = 2 * re->plain_its_ref;
    } else if (re->net && re->plain_its_ref > 0) {
      re->cnt.net_skipped += 1;
    }
  }
  const auto t0 = std::chrono::steady_clock::now();
  const int rc = re->ksp.solve(re->A, x_out, cfg, st, res);
  const double ms =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (learned && rc == FREHG_OK) {
    if (use_net) {
      re->cnt.net_solves += 1;
      re->cnt.net_ms += ms;
      if (re->probe_now) {
        re->net_on = re->probe_every <= 0 || re->last_plain_ms <= 0.0 ||
                     ms <= re->max_ratio * re->last_plain_ms;
        re->probe_pending = false;
        re->solves_since_probe = 0;
      }
    } else {
      re->last_plain_ms = ms;
    }
    ++re->solves_since_probe;
    // the reference count comes from network-free solves only (a fallback solve's count also
    // holds the network's iterations)
    if (!use_net) re->plain_its_ref = res->its;
  }
  if (!use_net) re->cnt.plain_ms += ms;
  if (res->fallback) re->cnt.fcg_fallbacks += 1;
  return rc;
}

// bytes one cell's soil lookup reads (per-cell Ks / alpha fields, class ids)
static double soil_bytes(const frehg_re* re) {
  return (re->fKs ? 8.0 : 0.0) + (re->falpha ? 8.0 : 0.0) + (re->cid && re->cid3d ? 1.0 : 0.0);
}

// ------------------------------------------------------------------------------------------
// PCA step (ReSolver::advanceStep, ReSolver.cpp:931-969)

static int pca_step(frehg_re* re) {
  re->constit_fresh = false;  // the step writes kr and cap at other heads
  cudaStream_t st = re->stream;
  ReArgs a = make_args(re);
  const int nb = nblocks(re->n);
  Profiler* prof = &re->prof;
  const double n = (double)re->n, sb = soil_bytes(re);
  FG_LAUNCH(prof, st, "k_step_begin", 0.0, k_step_begin<<<1, 1, 0, st>>>(re->sc));
  // computeKFace inputs at h^n
  FG_LAUNCH(prof, st, "k_kr", (24.0 + sb) * n,
            (k_constit<false, true><<<nb, 256, 0, st>>>(a, a.h_old, re->kr, nullptr, re->cap)));
  // groundwaterMatCoeff + groundwaterRhs + assembly
  const StencilLaunch L = stencil_launch(re->nx, re->ny, re->nz);
  re->A.scaled = false;
  re->A.s_in_r = false;
  re->A.f32_entries = false;
  FG_LAUNCH(prof, st, "k_assemble", (72.0 + sb) * n,
            k_assemble<<<L.grid, L.block, 0, st>>>(a, re->A.s, re->A.a0, re->A.a1, re->A.a2,
                                                   re->A.b, L.planes, L.tiles));
  FG_CUDA(cudaGetLastError());
  // LinearSolver::solve
  CgResult res;
  const int rc = solve_system(re, a.h_new, &res);
  re->cnt.last_ksp_iterations = res.its;
  re->cnt.last_residual_norm = res.rnorm;
  re->cnt.ksp_iterations += res.its;
  re->cnt.ir_sweeps += res.ir_its;
  if (rc != FREHG_OK) return rc;
  // enforceHeadBc + computeKFace + updateDiagnostics at h^{n+1} (the solve wrote h^{n+1})
  FG_LAUNCH(prof, st, "k_post", (24.0 + sb) * n, k_post<<<nb, 256, 0, st>>>(a));
  FG_CUDA(cudaGetLastError());
  // groundwaterFlux + updateWaterContent (+ dq of adaptiveTimeStep, boundary budgets)
  FG_LAUNCH(prof, st, "k_correct", (73.0 + sb) * n,
            k_correct<<<L.grid, L.block, 0, st>>>(a, L.planes, L.tiles));
  FG_CUDA(cudaGetLastError());
  // reallocateWaterContent: relax to the sequential sweep's fixed point
  const int top_sat = (re->p.bc_type[5] == 1 && re->p.htop >= 0.0) ? 1 : 0;
  const int cb = (int)((re->ncol + 127) / 128);
  const int max_sweeps = (int)re->n + 2;
  int sweeps = 0;
  for (;;) {
    FG_CUDA(cudaMemsetAsync(&re->sc->changed, 0, sizeof(int), st));
    FG_LAUNCH(prof, st, "k_realloc_sweep", 2.0 * n,
              k_realloc_sweep<<<cb, 128, 0, st>>>(a, top_sat));
    FG_CUDA(cudaGetLastError());
    ++sweeps;
    int changed = 0;
    FG_TRY(fetch_small(&re->sc_host->changed, &re->sc->changed, sizeof(int), st));
    FG_CUDA(cudaStreamSynchronize(st));
    if (prof->on) FG_TRY(prof->flush());
    changed = re->sc_host->changed;
    if (!changed) break;
    if (sweeps > max_sweeps) {
      set_error("reallocation relaxation did not settle after %d sweeps", sweeps);
      return FREHG_ERR_STATE;
    }
  }
  re->cnt.realloc_sweeps += sweeps;
  // apply reallocation, clampWaterContent, adaptiveTimeStep
  FG_LAUNCH(prof, st, "k_finalize", (25.0 + sb) * n,
            k_finalize<<<L.grid, L.block, 0, st>>>(a, top_sat, L.planes, L.tiles));
  FG_CUDA(cudaGetLastError());
  if (prof->on) {
    FG_CUDA(cudaStreamSynchronize(st));
    FG_TRY(prof->flush());
  }
  re->cur = 1 - re->cur;
  re->ghosts_valid = true;
  re->top_ghost_stale = false;  // the step re-enforced the ghosts
  return FREHG_OK;
}

// ------------------------------------------------------------------------------------------
// Tensor maps of the staged (TMA) Picard assembly: cuTensorMapEncodeTiled through the runtime's
// driver entry point (the library does not link libcuda).

namespace {
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static const EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return static_cast<EncodeTiledFn>(nullptr);
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

// an nx x ny x nz FP64 array (x fastest), boxes of bx x by x 1; out-of-range elements read 0
bool encode_box(CUtensorMap* m, const double* base, int nx, int ny, int nz, int bx, int by) {
  const EncodeTiledFn f = encode_tiled();
  if (!f || (reinterpret_cast<uintptr_t>(base) & 15u)) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
  const cuuint64_t strides[2] = {(cuuint64_t)nx * 8u, (cuuint64_t)nx * ny * 8u};
  const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1u};
  const cuuint32_t es[3] = {1u, 1u, 1u};
  return f(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double*>(base), dims, strides, box,
           es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the staged arrays' tensor maps; false when the layout does not qualify (the row stride of nx
// doubles must be a multiple of 16 bytes)
bool pic_tma_maps(const ReArgs& a, const double* ks, PicTmaMaps* m) {
  if (!ks || (a.nx & 1)) return false;
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  return encode_box(&m->h, a.h_new, nx, ny, nz, kPtWideX, kPtWideY) &&
         encode_box(&m->kr, a.kr, nx, ny, nz, kPtWideX, kPtWideY) &&
         encode_box(&m->ks, ks, nx, ny, nz, kPtWideX, kPtWideY) &&
         encode_box(&m->wo, a.w_old, nx, ny, nz, 32, 8) &&
         encode_box(&m->ho, a.h_old, nx, ny, nz, 32, 8) &&
         encode_box(&m->wch, a.wch, nx, ny, nz, 32, 8) &&
         encode_box(&m->cap, a.cap, nx, ny, nz, 32, 8);
}
}  // namespace

// Launch the staged assembly (mixed-precision form: float matrix entries).  *launched stays
// false when the handle's layout does not qualify; the caller then launches k_pic_assemble_ff.
static int launch_staged_assembly(frehg_re* re, const ReArgs& a, const StencilLaunch& PL,
                                  float* dgf, const Stencil32& o, double* b, bool* launched,
                                  int stall_producer = 0) {
  *launched = false;
  PicTmaMaps maps;
  if (!pic_tma_maps(a, re->fKs, &maps)) return FREHG_OK;
  static bool attr_set = false;
  if (!attr_set) {
    FG_CUDA(cudaFuncSetAttribute(k_pic_assemble_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kPtSmemBytes + 128));
    attr_set = true;
  }
  const double n = (double)re->n;
  // persistent: three blocks per SM stride over the tiles, so each block's copy pipeline runs on
  // from one tile into the next
  const long per_slab = (long)kNumSMs * 3 / (long)PL.grid.y;
  const dim3 grid((unsigned)std::max(1L, std::min((long)PL.tiles, per_slab)), PL.grid.y, 1);
  FG_LAUNCH(&re->prof, re->stream, "k_pic_assemble_ff", (72.0 + soil_bytes(re)) * n,
            (k_pic_assemble_tma<<<grid, dim3(32, 9), kPtSmemBytes + 128, re->stream>>>(
                a, maps, dgf, o.a0, o.a1, o.a2, b, PL.planes, PL.tiles, &re->sc->stage_err,
                stall_producer)));
  FG_CUDA(cudaGetLastError());
  *launched = true;
  return FREHG_OK;
}

static int read_scalars(const frehg_re* re) {
  FG_TRY(fetch_small(re->sc_host, re->sc, sizeof(ReScalars), re->stream));
  FG_CUDA(cudaStreamSynchronize(re->stream));
  return FREHG_OK;
}

// ------------------------------------------------------------------------------------------
// Mixed-form modified Picard step (not in reference).  Host loop over Picard iterations: each
// iteration assembles on the device, solves with the Krylov solver, updates h and reads |d|_inf.

static int picard_step(frehg_re* re) {
  cudaStream_t st = re->stream;
  Profiler* prof = &re->prof;
  const double n = (double)re->n, sb = soil_bytes(re);
  const int nb = nblocks(re->n);
  FG_TRY(read_scalars(re));
  double dt = re->sc_host->dt;
  ReArgs a = make_args(re);
  const StencilLaunch PL = stencil_launch(re->nx, re->ny, re->nz);
  // one conductivity serves all axes: a per-cell Ks field, or isotropic classes only
  bool iso = re->fKs != nullptr;
  if (!iso) {
    iso = true;
    for (const SoilClass& k : re->cls_host) iso = iso && k.ks_iso;
  }
  // every class van Genuchten (not MVG): the float-float constitutive kernel without FP64 forms
  bool all_ff = true;
  for (const SoilClass& k : re->cls_host) all_ff = all_ff && k.use_vg && !k.use_mvg;
  // a float-float assembly solved in mixed precision writes its matrix entries as floats
  const bool f32 = picard_ff(re) && mixed_solve(re);
  if (f32) FG_TRY(re->ksp.ensure32(re->n));
  int its = 0;
  // the previous step's last update formed the constitutive values at this step's start
  bool reuse = re->constit_fresh && picard_ff(re);
  re->constit_fresh = false;
  bool last_fused = false;
  for (;;) {
    FG_CUDA(cudaMemcpyAsync(&re->sc->dt, &dt, sizeof(double), cudaMemcpyHostToDevice, st));
    FG_LAUNCH(prof, st, "k_step_begin", 0.0, k_step_begin<<<1, 1, 0, st>>>(re->sc));
    FG_LAUNCH(prof, st, "k_copy64", 16.0 * n,
              k_copy64<<<nb, 256, 0, st>>>(a.h_new, a.h_old, re->n));
    bool converged = false;
    int fail = FREHG_OK;
    // the previous iteration's update formed this iteration's constitutive values (or the
    // previous step's, for the first attempt's first iteration)
    bool constit_ready = reuse;
    reuse = false;
    last_fused = false;
    for (its = 0; its < re->p.picard_max_it; ++its) {
      if (!picard_ff(re))
        FG_LAUNCH(prof, st, "k_kr", (32.0 + sb) * n,
                  (k_constit<true, true><<<nb, 256, 0, st>>>(a, a.h_new, re->kr, re->wch,
                                                             re->cap)));
      else if (constit_ready) {
      } else if (all_ff)
        FG_LAUNCH(prof, st, "k_kr_ff", (32.0 + sb) * n,
                  (k_constit_ff<true, true, true><<<nb, 256, 0, st>>>(a, a.h_new, re->kr,
                                                                      re->wch, re->cap)));
      else
        FG_LAUNCH(prof, st, "k_kr_ff", (32.0 + sb) * n,
                  (k_constit_ff<true, true, false><<<nb, 256, 0, st>>>(a, a.h_new, re->kr,
                                                                       re->wch, re->cap)));
      re->A.scaled = false;
      re->A.s_in_r = false;
      re->A.f32_entries = f32;
      if (!picard_ff(re))
        FG_LAUNCH(prof, st, "k_pic_assemble", (88.0 + sb) * n,
                  k_pic_assemble<<<PL.grid, PL.block, 0, st>>>(a, re->A.s, re->A.a0, re->A.a1,
                                                               re->A.a2, re->A.b, PL.planes,
                                                               PL.tiles));
      else if (f32) {
        // diagonal and couplings as floats (the float-float preparation's input)
        float* dgf = reinterpret_cast<float*>(re->A.s);
        const Stencil32& o = re->ksp.op32;
        bool staged = false;
        if (iso && re->staged) FG_TRY(launch_staged_assembly(re, a, PL, dgf, o, re->A.b, &staged));
        if (staged) {
        } else if (iso)
          FG_LAUNCH(prof, st, "k_pic_assemble_ff", (72.0 + sb) * n,
                    (k_pic_assemble_ff<true, false, float><<<PL.grid, PL.block, 0, st>>>(
                        a, dgf, o.a0, o.a1, o.a2, re->A.b, PL.planes, PL.tiles)));
        else
          FG_LAUNCH(prof, st, "k_pic_assemble_ff", (72.0 + sb) * n,
                    (k_pic_assemble_ff<false, false, float><<<PL.grid, PL.block, 0, st>>>(
                        a, dgf, o.a0, o.a1, o.a2, re->A.b, PL.planes, PL.tiles)));
      } else if (iso)
        FG_LAUNCH(prof, st, "k_pic_assemble_ff", (88.0 + sb) * n,
                  k_pic_assemble_ff<true><<<PL.grid, PL.block, 0, st>>>(
                      a, re->A.s, re->A.a0, re->A.a1, re->A.a2, re->A.b, PL.planes, PL.tiles));
      else
        FG_LAUNCH(prof, st, "k_pic_assemble_ff", (88.0 + sb) * n,
                  k_pic_assemble_ff<false><<<PL.grid, PL.block, 0, st>>>(
                      a, re->A.s, re->A.a0, re->A.a1, re->A.a2, re->A.b, PL.planes, PL.tiles));
      FG_CUDA(cudaGetLastError());
      CgResult res;
      // the update below applies x = s x~ (PCSOR solves the unscaled system into scratch)
      const bool sor = !strcmp(re->cfg.pc_type, "sor");
      re->ksp.keep_scaled = !sor;
      re->ksp.rnorm_slot = its == 0 ? 0 : 1;
      const int rc = solve_system(re, re->scratch, &res);
      re->ksp.keep_scaled = false;
      re->ksp.rnorm_slot = 1;
      re->cnt.last_ksp_iterations = res.its;
      re->cnt.last_residual_norm = res.rnorm;
      re->cnt.ksp_iterations += res.its;
      re->cnt.ir_sweeps += res.ir_its;
      if (rc != FREHG_OK) {
        fail = rc;
        break;
      }
      // float-float kernels: the update also forms the constitutive values at the new head
      // into the second set, which the next iteration takes (a converged step keeps the first
      // set, at the head its final update needs)
      const bool fused_update = !sor && picard_ff(re);
      last_fused = fused_update;
      if (fused_update && !re->kr2) {
        FG_CUDA(cudaMalloc(&re->kr2, re->n * sizeof(double)));
        FG_CUDA(cudaMalloc(&re->wch2, re->n * sizeof(double)));
        FG_CUDA(cudaMalloc(&re->cap2, re->n * sizeof(double)));
      }
      if (sor)
        FG_LAUNCH(prof, st, "k_pic_update", 24.0 * n,
                  k_pic_update<false><<<nb, 256, 0, st>>>(a, re->scratch));
      else if (fused_update && all_ff)
        FG_LAUNCH(prof, st, "k_pic_update_kr_ff", (56.0 + sb) * n,
                  k_pic_update_constit_ff<true><<<nb, 256, 0, st>>>(
                      a, re->ksp.x, re->ksp.scale_vector(re->A), re->kr2, re->wch2, re->cap2));
      else if (fused_update)
        FG_LAUNCH(prof, st, "k_pic_update_kr_ff", (56.0 + sb) * n,
                  k_pic_update_constit_ff<false><<<nb, 256, 0, st>>>(
                      a, re->ksp.x, re->ksp.scale_vector(re->A), re->kr2, re->wch2, re->cap2));
      else
        FG_LAUNCH(prof, st, "k_pic_update", 32.0 * n,
                  k_pic_update<true><<<nb, 256, 0, st>>>(a, re->ksp.x,
                                                         re->ksp.scale_vector(re->A)));
      FG_CUDA(cudaGetLastError());
      FG_TRY(fetch_small(&re->sc_host->dq_max, &re->sc->dq_max, sizeof(double), st));
      FG_TRY(fetch_small(&re->sc_host->stage_err, &re->sc->stage_err, sizeof(int), st));
      FG_CUDA(cudaStreamSynchronize(st));
      if (re->sc_host->stage_err) {
        set_error("staged Picard assembly: a bounded wait on its copy pipeline ran out (%d)",
                  re->sc_host->stage_err);
        return FREHG_ERR_CUDA;
      }
      if (prof->on) FG_TRY(prof->flush());
      re->cnt.picard_iterations += 1;
      if (re->sc_host->dq_max < re->p.picard_tol) {
        converged = true;
        ++its;
        break;
      }
      if (fused_update) {
        std::swap(re->kr, re->kr2);
        std::swap(re->wch, re->wch2);
        std::swap(re->cap, re->cap2);
        a.kr = re->kr;
        a.wch = re->wch;
        a.cap = re->cap;
        constit_ready = true;
      }
    }
    if (converged) break;
    // a failed step is retried at half the time step, down to an emergency floor of
    // dt_min / 16 below the controller's range
    const double dt_floor = re->p.dt_min / 16.0;
    if (!re->p.picard_dt_adapt || dt <= dt_floor) {
      if (fail == FREHG_OK) {
        set_error("Picard iteration did not reach |dh| < %g in %d iterations (dt %g)",
                  re->p.picard_tol, re->p.picard_max_it, dt);
        fail = FREHG_ERR_NOT_CONVERGED;
      }
      re->cnt.last_picard_iterations = its;
      return fail;
    }
    dt = fmax(0.5 * dt, dt_floor);
  }
  if (!picard_ff(re))
    FG_LAUNCH(prof, st, "k_pic_final", (40.0 + sb) * n,
              k_pic_final<<<PL.grid, PL.block, 0, st>>>(a, PL.planes, PL.tiles));
  else if (iso)
    FG_LAUNCH(prof, st, "k_pic_final_ff", (40.0 + sb) * n,
              (k_pic_assemble_ff<true, true, double><<<PL.grid, PL.block, 0, st>>>(
                  a, nullptr, nullptr, nullptr, nullptr, nullptr, PL.planes, PL.tiles)));
  else
    FG_LAUNCH(prof, st, "k_pic_final_ff", (40.0 + sb) * n,
              (k_pic_assemble_ff<false, true, double><<<PL.grid, PL.block, 0, st>>>(
                  a, nullptr, nullptr, nullptr, nullptr, nullptr, PL.planes, PL.tiles)));
  FG_CUDA(cudaGetLastError());
  if (last_fused) {
    // the last update formed the values at the step's final head (the final update above,
    // launched with the frozen set, leaves the head as it is): the next step starts with them
    std::swap(re->kr, re->kr2);
    std::swap(re->wch, re->wch2);
    std::swap(re->cap, re->cap2);
    re->constit_fresh = true;
  }
  re->cnt.last_picard_iterations = its;
  if (re->p.picard_dt_adapt) {
    // Picard-count controller: grow after <= 3 iterations, shrink after >= 8, within
    // [dt_min, dt_max] (a dt below dt_min after a retry only grows back)
    double nd = dt;
    if (its <= 3)
      nd = fmin(dt * 1.25, re->p.dt_max);
    else if (its >= 8)
      nd = fmax(dt * 0.7, fmin(dt, re->p.dt_min));
    FG_CUDA(cudaMemcpyAsync(&re->sc->dt, &nd, sizeof(double), cudaMemcpyHostToDevice, st));
    re->p.dt = nd;
  }
  FG_CUDA(cudaStreamSynchronize(st));
  if (prof->on) FG_TRY(prof->flush());
  re->cur = 1 - re->cur;
  re->ghosts_valid = true;
  re->top_ghost_stale = false;  // the step re-enforced the ghosts
  return FREHG_OK;
}

static int advance_one(frehg_re* re) {
  // the step writes the other state buffer: copies of the current one run on during it
  FG_TRY(wait_copies(re, 1 - re->cur, false));
  if (!re->finalized) {
    set_error("advance_step before finalize_initial_state");
    return FREHG_ERR_STATE;
  }
  if (!re->attached) {
    set_error("advance_step before attach_solver");
    return FREHG_ERR_STATE;
  }
  int rc;
  if (re->p.scheme == 1)
    rc = picard_step(re);
  else
    rc = pca_step(re);
  if (rc != FREHG_OK) return rc;
  re->cnt.steps += 1;
  re->cnt.cells_touched += (int64_t)re->n;
  return FREHG_OK;
}

// ------------------------------------------------------------------------------------------
// C API

extern "C" {

int frehg_re_create(int nx, int ny, int nz, const frehg_re_params* p, frehg_re** out) {
  clear_error();
  FG_ARG(out != nullptr && p != nullptr, "null argument");
  FG_ARG(nx > 0 && ny > 0 && nz > 0, "grid sizes must be positive");
  // the kernels index cells with 32-bit integers; 2^31 cells would need over 280 GB of state
  FG_ARG((size_t)nx * ny * nz < ((size_t)1 << 31), "more than 2^31 - 1 cells");
  FG_TRY(validate_params(p));
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    set_error("no CUDA device");
    return FREHG_ERR_NO_DEVICE;
  }
  frehg_re* re = new frehg_re();
  re->nx = nx;
  re->ny = ny;
  re->nz = nz;
  re->ncol = (size_t)nx * ny;
  re->n = re->ncol * nz;
  re->p = *p;
  frehg_solver_config_default(&re->cfg);
  memset(&re->cnt, 0, sizeof(re->cnt));
  auto fail = [&](int rc) {
    delete re;
    return rc;
  };
  const size_t n = re->n;
#define ALLOC(ptr, bytes)                                      \
  do {                                                         \
    if (cudaMalloc(&(ptr), (bytes)) != cudaSuccess) {          \
      set_error("cudaMalloc of %zu bytes failed", (size_t)(bytes)); \
      return fail(FREHG_ERR_CUDA);                             \
    }                                                          \
  } while (0)
  for (int q = 0; q < 2; ++q) {
    ALLOC(re->H[q], n * sizeof(double));
    ALLOC(re->W[q], n * sizeof(double));
  }
  ALLOC(re->kr, n * sizeof(double));
  ALLOC(re->wch, n * sizeof(double));
  ALLOC(re->cap, n * sizeof(double));
  ALLOC(re->qx, n * sizeof(double));
  ALLOC(re->qy, n * sizeof(double));
  ALLOC(re->qz, n * sizeof(double));
  ALLOC(re->qztop, re->ncol * sizeof(double));
  ALLOC(re->qtop_field, re->ncol * sizeof(double));
  ALLOC(re->flags, n);
  ALLOC(re->scratch, n * sizeof(double));
  ALLOC(re->sc, sizeof(ReScalars));
  ALLOC(re->partials, 4 * kMaxRedBlocks * sizeof(double));
#undef ALLOC
  if (alloc_mapped(reinterpret_cast<void**>(&re->sc_host), sizeof(ReScalars)) != FREHG_OK)
    return fail(FREHG_ERR_CUDA);
  if (re->A.alloc(nx, ny, nz) != FREHG_OK) return fail(FREHG_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&re->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(FREHG_ERR_CUDA);
  re->stream = re->own_stream;
  ReScalars s0;
  memset(&s0, 0, sizeof(s0));
  s0.dt = p->dt;
  s0.dtn = 0.0;
  if (cudaMemcpy(re->sc, &s0, sizeof(s0), cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(FREHG_ERR_CUDA);
  for (int q = 0; q < 2; ++q) {
    cudaMemset(re->H[q], 0, n * sizeof(double));
    cudaMemset(re->W[q], 0, n * sizeof(double));
  }
  cudaMemset(re->qx, 0, n * sizeof(double));
  cudaMemset(re->qy, 0, n * sizeof(double));
  cudaMemset(re->qz, 0, n * sizeof(double));
  cudaMemset(re->qztop, 0, re->ncol * sizeof(double));
  if (upload_class0(re) != FREHG_OK) return fail(FREHG_ERR_CUDA);
  if (re->ksp.ensure(n) != FREHG_OK) return fail(FREHG_ERR_CUDA);
  re->ksp.prof = &re->prof;
  *out = re;
  return FREHG_OK;
}

int frehg_re_destroy(frehg_re* re) {
  clear_error();
  if (re) {
    cudaStreamSynchronize(re->stream);
    if (re->copy_stream) cudaStreamSynchronize(re->copy_stream);
    delete re;
  }
  return FREHG_OK;
}

int frehg_re_set_params(frehg_re* re, const frehg_re_params* p) {
  clear_error();
  if (re) re->constit_fresh = false;
  FG_ARG(re && p, "null argument");
  FG_TRY(validate_params(p));
  const double old_dt = re->p.dt;
  re->p = *p;
  FG_TRY(upload_class0(re));
  if (p->dt != old_dt) {
    FG_CUDA(cudaStreamSynchronize(re->stream));
    FG_CUDA(cudaMemcpy(&re->sc->dt, &p->dt, sizeof(double), cudaMemcpyHostToDevice));
  }
  return FREHG_OK;
}

int frehg_re_get_params(const frehg_re* re, frehg_re_params* p) {
  clear_error();
  FG_ARG(re && p, "null argument");
  *p = re->p;
  FG_CUDA(cudaStreamSynchronize(re->stream));
  FG_CUDA(cudaMemcpy(&p->dt, &re->sc->dt, sizeof(double), cudaMemcpyDeviceToHost));
  return FREHG_OK;
}

int frehg_re_set_soil_map(frehg_re* re, const frehg_soil_params* classes, int nclass,
                          const int32_t* class_index, int is3d) {
  clear_error();
  if (re) re->constit_fresh = false;
  FG_ARG(re && classes && class_index, "null argument");
  FG_ARG(nclass >= 1 && nclass <= 256, "nclass must be in [1, 256]");
  const size_t cnt = is3d ? re->n : re->ncol;
  std::vector<uint8_t> ids(cnt);
  for (size_t c = 0; c < cnt; ++c) {
    FG_ARG(class_index[c] >= 0 && class_index[c] < nclass,
           "soil class id %d at %zu is out of range [0,%d)", class_index[c], c, nclass);
    ids[c] = (uint8_t)class_index[c];
  }
  std::vector<SoilClass> tab(nclass);
  for (int q = 0; q < nclass; ++q) tab[q] = make_soil_class(classes[q]);
  if (!re->cls) FG_CUDA(cudaMalloc(&re->cls, sizeof(SoilClass) * 256));
  FG_CUDA(cudaStreamSynchronize(re->stream));
  FG_CUDA(cudaMemcpy(re->cls, tab.data(), sizeof(SoilClass) * nclass, cudaMemcpyHostToDevice));
  re->cls_host = tab;
  cudaFree(re->cid);
  re->cid = nullptr;
  FG_CUDA(cudaMalloc(&re->cid, cnt));
  FG_CUDA(cudaMemcpy(re->cid, ids.data(), cnt, cudaMemcpyHostToDevice));
  re->cid3d = is3d ? 1 : 0;
  re->nclass = nclass;
  return FREHG_OK;
}

int frehg_re_set_cell_fields(frehg_re* re, const double* Ks, const double* alpha) {
  clear_error();
  if (re) re->constit_fresh = false;
  FG_ARG(re, "null handle");
  FG_CUDA(cudaStreamSynchronize(re->stream));
  cudaFree(re->fKs);
  cudaFree(re->falpha);
  re->fKs = re->falpha = nullptr;
  if (Ks) {
    FG_CUDA(cudaMalloc(&re->fKs, re->n * sizeof(double)));
    FG_CUDA(cudaMemcpy(re->fKs, Ks, re->n * sizeof(double), cudaMemcpyHostToDevice));
  }
  if (alpha) {
    FG_CUDA(cudaMalloc(&re->falpha, re->n * sizeof(double)));
    FG_CUDA(cudaMemcpy(re->falpha, alpha, re->n * sizeof(double), cudaMemcpyHostToDevice));
  }
  return FREHG_OK;
}

int frehg_re_attach_solver(frehg_re* re, const frehg_solver_config* cfg) {
  clear_error();
  if (re) re->constit_fresh = false;
  FG_ARG(re && cfg, "null argument");
  if (strcmp(cfg->ksp_type, "cg") != 0 && strcmp(cfg->ksp_type, "fcg") != 0) {
    set_error("ksp_type '%s' is not available (cg, fcg)", cfg->ksp_type);
    return FREHG_ERR_UNSUPPORTED;
  }
  const char* pcs[] = {"jacobi", "sor", "line", "unet", "unet-line"};
  bool known = false;
  for (const char* q : pcs) known = known || !strcmp(cfg->pc_type, q);
  if (!known) {
    set_error("pc_type '%s' is not available on the GPU path (jacobi, sor, line, unet, "
              "unet-line)", cfg->pc_type);
    return FREHG_ERR_UNSUPPORTED;
  }
  if (!strcmp(cfg->pc_type, "sor") && cfg->precision != 0) {
    set_error("pc_type 'sor' runs in FP64 (precision 0)");
    return FREHG_ERR_UNSUPPORTED;
  }
  FG_ARG(cfg->rtol > 0 && cfg->max_it > 0, "rtol and max_it must be positive");
  FG_ARG(cfg->precision == 0 || cfg->precision == 1, "precision must be 0 or 1");
  if (!strcmp(cfg->pc_type, "line") && cfg->precision != 1) {
    set_error("pc_type 'line' runs in the FP32 inner solve: it needs precision 1 (mixed)");
    return FREHG_ERR_UNSUPPORTED;
  }
  re->cfg = *cfg;
  re->attached = true;
  return FREHG_OK;
}

int frehg_re_initialize_geometry(frehg_re* re) {
  clear_error();
  if (re) re->constit_fresh = false;
  FG_ARG(re, "null handle");
  re->have_geometry = true;  // uniform dz per layer, every cell active (ReSolver.cpp:104-131)
  return FREHG_OK;
}

int frehg_re_set_initial_head(frehg_re* re, const double* h) {
  clear_error();
  if (re) re->constit_fresh = false;
  FG_ARG(re && h, "null argument");
  FG_TRY(wait_copies(re, -1, true));
  FG_CUDA(cudaStreamSynchronize(re->stream));
  FG_CUDA(cudaMemcpy(re->H[re->cur], h, re->n * sizeof(double), cudaMemcpyHostToDevice));
  ReArgs a = make_args(re);
  k_theta_of_h<<<nblocks(re->n), 256, 0, re->stream>>>(a, re->H[re->cur], re->W[re->cur]);
  FG_CUDA(cudaGetLastError());
  FG_CUDA(cudaStreamSynchronize(re->stream));
  re->have_state = true;
  return FREHG_OK;
}

int frehg_re_set_initial_water_content(frehg_re* re, const double* wc) {
  clear_error();
  if (re) re->constit_fresh = false;
  FG_ARG(re && wc, "null argument");
  FG_TRY(wait_copies(re, -1, true));
  FG_CUDA(cudaStreamSynchronize(re->stream));
  FG_CUDA(cudaMemcpy(re->W[re->cur], wc, re->n * sizeof(double), cudaMemcpyHostToDevice));
  ReArgs a = make_args(re);
  k_h_of_theta<<<nblocks(re->n), 256, 0, re->stream>>>(a, re->W[re->cur], re->H[re->cur]);
  FG_CUDA(cudaGetLastError());
  FG_CUDA(cudaStreamSynchronize(re->stream));
  re->have_state = true;
  return FREHG_OK;
}

int frehg_re_finalize_initial_state(frehg_re* re) {
  clear_error();
  if (re) re->constit_fresh = false;
  FG_ARG(re, "null handle");
  FG_TRY(wait_copies(re, -1, true));
  if (!re->have_state) {
    set_error("finalize_initial_state before an initial head or water content");
    return FREHG_ERR_STATE;
  }
  FG_CUDA(cudaStreamSynchronize(re->stream));
  // dtn_ = params_.dt (ReSolver.cpp:175-178)
  FG_CUDA(cudaMemcpy(&re->sc->dtn, &re->sc->dt, sizeof(double), cudaMemcpyDeviceToDevice));
  // a finalized initial state starts a run, also on a handle that has stepped before: ghost
  // values as freshly allocated (zero until the first step writes them), simulated time and
  // the boundary / elastic budgets at zero
  FG_CUDA(cudaMemcpy(re->sc_host, re->sc, sizeof(ReScalars), cudaMemcpyDeviceToHost));
  re->sc_host->time = 0.0;
  re->sc_host->vol_top = 0.0;
  re->sc_host->vol_bot = 0.0;
  re->sc_host->vol_elastic = 0.0;
  FG_CUDA(cudaMemcpy(re->sc, re->sc_host, sizeof(ReScalars), cudaMemcpyHostToDevice));
  re->ghosts_valid = false;
  re->top_ghost_stale = false;
  // the refinement's right-hand-side scales carried from solve to solve start afresh
  re->ksp.first_rnorm[0] = re->ksp.first_rnorm[1] = 0.0;
  re->ksp.first_done = false;
  re->finalized = true;
  return FREHG_OK;
}

int frehg_re_initialize_uniform_column(frehg_re* re, double init_wc) {
  clear_error();
  if (re) re->constit_fresh = false;
  FG_ARG(re, "null handle");
  FG_TRY(frehg_re_initialize_geometry(re));
  std::vector<double> w(re->n, init_wc);
  FG_TRY(frehg_re_set_initial_water_content(re, w.data()));
  return frehg_re_finalize_initial_state(re);
}

int frehg_re_set_top_flux_field(frehg_re* re, const double* q) {
  clear_error();
  FG_ARG(re && q, "null argument");
  FG_CUDA(cudaMemcpyAsync(re->qtop_field, q, re->ncol * sizeof(double), cudaMemcpyHostToDevice,
                          re->stream));
  re->has_qtop = true;
  return FREHG_OK;
}

int frehg_re_advance_step(frehg_re* re) {
  clear_error();
  FG_ARG(re, "null handle");
  return advance_one(re);
}

int frehg_re_advance_steps(frehg_re* re, int nsteps) {
  clear_error();
  FG_ARG(re && nsteps >= 0, "bad argument");
  for (int q = 0; q < nsteps; ++q) FG_TRY(advance_one(re));
  return FREHG_OK;
}


int frehg_re_dt(const frehg_re* re, double* dt) {
  clear_error();
  FG_ARG(re && dt, "null argument");
  FG_TRY(read_scalars(re));
  *dt = re->sc_host->dt;
  return FREHG_OK;
}

int frehg_re_dt_used(const frehg_re* re, double* dt) {
  clear_error();
  FG_ARG(re && dt, "null argument");
  FG_TRY(read_scalars(re));
  *dt = re->sc_host->dt_used;
  return FREHG_OK;
}

int frehg_re_time(const frehg_re* re, double* t) {
  clear_error();
  FG_ARG(re && t, "null argument");
  FG_TRY(read_scalars(re));
  *t = re->sc_host->time;
  return FREHG_OK;
}

int frehg_re_set_dt(frehg_re* re, double dt) {
  clear_error();
  FG_ARG(re && dt > 0, "bad argument");
  FG_CUDA(cudaStreamSynchronize(re->stream));
  FG_CUDA(cudaMemcpy(&re->sc->dt, &dt, sizeof(double), cudaMemcpyHostToDevice));
  re->p.dt = dt;
  return FREHG_OK;
}

int frehg_re_prime_adaptive_dt(frehg_re* re, double dt) {
  clear_error();
  FG_ARG(re && dt > 0, "bad argument");
  FG_CUDA(cudaStreamSynchronize(re->stream));
  FG_CUDA(cudaMemcpy(&re->sc->dt, &dt, sizeof(double), cudaMemcpyHostToDevice));
  FG_CUDA(cudaMemcpy(&re->sc->dtn, &dt, sizeof(double), cudaMemcpyHostToDevice));
  re->p.dt = dt;
  return FREHG_OK;
}

int frehg_re_surface_exchange(frehg_re* re, double* eta, const double* bottom, double dt,
                              double visc, double min_depth, double* q_out, double* total,
                              int on_device) {
  clear_error();
  if (re) re->constit_fresh = false;
  FG_ARG(re && eta && bottom && q_out && total, "null argument");
  FG_TRY(wait_copies(re, -1, true));
  FG_ARG(dt > 0.0, "dt must be positive");
  FG_ARG(re->finalized, "surface exchange before an initial state");
  cudaStream_t st = re->stream;
  const size_t nc = re->ncol;
  double *d_eta = eta, *d_q = q_out;
  const double* d_bot = bottom;
  if (!on_device) {
    if (!re->xch) FG_CUDA(cudaMalloc(&re->xch, (3 * nc + 1) * sizeof(double)));
    FG_CUDA(cudaMemcpyAsync(re->xch, eta, nc * sizeof(double), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(re->xch + nc, bottom, nc * sizeof(double), cudaMemcpyHostToDevice,
                            st));
    d_eta = re->xch;
    d_bot = re->xch + nc;
    d_q = re->xch + 2 * nc;
  } else if (!re->xch) {
    FG_CUDA(cudaMalloc(&re->xch, (3 * nc + 1) * sizeof(double)));
  }
  double* d_total = re->xch + 3 * nc;
  // the reference's halo keeps the top layer's ghost copies from before the exchange until its
  // next step re-enforces them; keep them (the first exchange since the last step decides)
  if (re->ghosts_valid && !re->top_ghost_stale) {
    if (!re->gh_top) FG_CUDA(cudaMalloc(&re->gh_top, 2 * nc * sizeof(double)));
    FG_CUDA(cudaMemcpyAsync(re->gh_top, re->H[re->cur], nc * sizeof(double),
                            cudaMemcpyDeviceToDevice, st));
    FG_CUDA(cudaMemcpyAsync(re->gh_top + nc, re->W[re->cur], nc * sizeof(double),
                            cudaMemcpyDeviceToDevice, st));
    re->top_ghost_stale = true;
  }
  const SoilClass k0 = make_soil_class(re->p.soil);
  const int nb = (int)std::min<size_t>((nc + 255) / 256, (size_t)kNumSMs * 8);
  k_surface_exchange<<<nb, 256, 0, st>>>(re->H[re->cur], re->W[re->cur], d_eta, d_bot, d_q, k0,
                                         (int)nc, re->p.dx * re->p.dy, re->p.dz, dt, visc,
                                         min_depth, re->partials, &re->sc->arrive[5], d_total);
  FG_CUDA(cudaGetLastError());
  if (!on_device) {
    FG_CUDA(cudaMemcpyAsync(eta, d_eta, nc * sizeof(double), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaMemcpyAsync(q_out, d_q, nc * sizeof(double), cudaMemcpyDeviceToHost, st));
  }
  FG_CUDA(cudaMemcpyAsync(total, d_total, sizeof(double), cudaMemcpyDeviceToHost, st));
  FG_CUDA(cudaStreamSynchronize(st));
  return FREHG_OK;
}

int frehg_re_checkpoint(frehg_re* re, double* h, double* wc, double* state) {
  clear_error();
  FG_ARG(re && h && wc && state, "null argument");
  FG_ARG(re->finalized, "checkpoint of a handle without a finalized state");
  if (re->top_ghost_stale) {
    set_error("checkpoint between a surface exchange and the next step: the top layer's "
              "pre-exchange ghost copies are not part of the state");
    return FREHG_ERR_STATE;
  }
  FG_CUDA(cudaStreamSynchronize(re->stream));
  FG_CUDA(cudaMemcpy(h, re->H[re->cur], re->n * sizeof(double), cudaMemcpyDeviceToHost));
  FG_CUDA(cudaMemcpy(wc, re->W[re->cur], re->n * sizeof(double), cudaMemcpyDeviceToHost));
  FG_CUDA(cudaMemcpy(re->sc_host, re->sc, sizeof(ReScalars), cudaMemcpyDeviceToHost));
  const ReScalars& s = *re->sc_host;
  const double v[FREHG_CHECKPOINT_SCALARS] = {s.time,    s.dt,      s.dtn,
                                              s.dt_used, s.vol_top, s.vol_bot,
                                              s.vol_elastic, re->ghosts_valid ? 1.0 : 0.0,
                                              re->ksp.first_rnorm[0], re->ksp.first_rnorm[1]};
  memcpy(state, v, sizeof(v));
  return FREHG_OK;
}

int frehg_re_restart(frehg_re* re, const double* h, const double* wc, const double* state) {
  clear_error();
  if (re) re->constit_fresh = false;
  FG_ARG(re && h && wc && state, "null argument");
  FG_TRY(wait_copies(re, -1, true));
  FG_ARG(state[1] > 0.0 && state[2] > 0.0, "checkpoint state has no positive dt");
  FG_CUDA(cudaStreamSynchronize(re->stream));
  FG_CUDA(cudaMemcpy(re->H[re->cur], h, re->n * sizeof(double), cudaMemcpyHostToDevice));
  FG_CUDA(cudaMemcpy(re->W[re->cur], wc, re->n * sizeof(double), cudaMemcpyHostToDevice));
  FG_CUDA(cudaMemcpy(re->sc_host, re->sc, sizeof(ReScalars), cudaMemcpyDeviceToHost));
  ReScalars& s = *re->sc_host;
  s.time = state[0];
  s.dt = state[1];
  s.dtn = state[2];  // primeAdaptiveDt's dtn_ (ReSolver.hpp:95-98)
  s.dt_used = state[3];
  s.vol_top = state[4];
  s.vol_bot = state[5];
  s.vol_elastic = state[6];
  FG_CUDA(cudaMemcpy(re->sc, re->sc_host, sizeof(ReScalars), cudaMemcpyHostToDevice));
  re->p.dt = state[1];
  re->ghosts_valid = state[7] != 0.0;
  re->ksp.first_rnorm[0] = state[8];
  re->ksp.first_rnorm[1] = state[9];
  re->ksp.first_done = false;
  re->top_ghost_stale = false;
  re->have_state = true;
  re->finalized = true;
  return FREHG_OK;
}

// fill a halo array ((nx+2)(ny+2)(nz+2)) from an interior array; ghosts by the copy rule
static void to_halo(const frehg_re* re, const std::vector<double>& in, double* out, bool copy_ghosts,
                    double top_ghost, bool top_fixed, double bot_ghost, bool bot_fixed) {
  const int nx = re->nx, ny = re->ny, nz = re->nz;
  const size_t hx = nx + 2, hy = ny + 2;
  memset(out, 0, sizeof(double) * hx * hy * (nz + 2));
  auto H = [&](int i, int j, int k) -> double& {
    return out[(size_t)(i + 1) + (size_t)(j + 1) * hx + (size_t)(k + 1) * hx * hy];
  };
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) H(i, j, k) = in[(size_t)i + (size_t)nx * (j + (size_t)ny * k)];
  if (!copy_ghosts) return;
  for (int k = 0; k < nz; ++k) {
    for (int j = 0; j < ny; ++j) {
      H(-1, j, k) = H(0, j, k);
      H(nx, j, k) = H(nx - 1, j, k);
    }
    for (int i = 0; i < nx; ++i) {
      H(i, -1, k) = H(i, 0, k);
      H(i, ny, k) = H(i, ny - 1, k);
    }
  }
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      H(i, j, nz) = bot_fixed ? bot_ghost : H(i, j, nz - 1);
      H(i, j, -1) = top_fixed ? top_ghost : H(i, j, 0);
    }
}

int frehg_re_get_interior(frehg_re* re, const char* name, double* out, int device_out) {
  clear_error();
  FG_ARG(re && name && out, "null argument");
  const double* src = nullptr;
  if (!strcmp(name, "h")) src = re->H[re->cur];
  else if (!strcmp(name, "wc")) src = re->W[re->cur];
  else if (!strcmp(name, "hn")) src = re->H[1 - re->cur];
  else if (!strcmp(name, "wcn")) src = re->W[1 - re->cur];
  else if (!strcmp(name, "wch")) src = re->wch;
  else if (!strcmp(name, "kr")) src = re->kr;
  FG_ARG(src != nullptr, "unknown interior field '%s'", name);
  FG_CUDA(cudaMemcpyAsync(out, src, re->n * sizeof(double),
                          device_out ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                          re->stream));
  FG_CUDA(cudaStreamSynchronize(re->stream));
  return FREHG_OK;
}

int frehg_re_get_interior_async(frehg_re* re, const char* name, double* out) {
  clear_error();
  FG_ARG(re && name && out, "null argument");
  int q = -1;
  if (!strcmp(name, "h") || !strcmp(name, "wc")) q = re->cur;
  else if (!strcmp(name, "hn") || !strcmp(name, "wcn")) q = 1 - re->cur;
  FG_ARG(q >= 0, "field '%s' has no asynchronous copy (h, wc, hn, wcn)", name);
  const double* src = name[0] == 'h' ? re->H[q] : re->W[q];
  if (!re->copy_stream) {
    FG_CUDA(cudaStreamCreateWithFlags(&re->copy_stream, cudaStreamNonBlocking));
    for (cudaEvent_t* e : {&re->copy_ev[0], &re->copy_ev[1], &re->issue_ev})
      FG_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  }
  // after the work issued so far on the handle's stream, on the copy stream
  FG_CUDA(cudaEventRecord(re->issue_ev, re->stream));
  FG_CUDA(cudaStreamWaitEvent(re->copy_stream, re->issue_ev, 0));
  FG_CUDA(cudaMemcpyAsync(out, src, re->n * sizeof(double), cudaMemcpyDeviceToHost,
                          re->copy_stream));
  FG_CUDA(cudaEventRecord(re->copy_ev[q], re->copy_stream));
  re->copy_pending[q] = true;
  return FREHG_OK;
}

int frehg_re_get_field(frehg_re* re, const char* name, double* out_halo) {
  clear_error();
  FG_ARG(re && name && out_halo, "null argument");
  const size_t n = re->n;
  std::vector<double> buf(n);
  ReArgs a = make_args(re);
  // after a step, H[cur]/W[cur] are the new state and H[1-cur]/W[1-cur] the step's start
  a.h_old = re->H[1 - re->cur];
  a.w_old = re->W[1 - re->cur];
  const double* src = nullptr;
  bool ghosts = true;
  const bool gv = re->ghosts_valid;
  if (!strcmp(name, "h")) {
    src = re->H[re->cur];
    FG_CUDA(cudaMemcpy(buf.data(), src, n * sizeof(double), cudaMemcpyDeviceToHost));
    to_halo(re, buf, out_halo, gv, re->p.htop, re->p.bc_type[5] == 1, re->p.hbot,
            re->p.bc_type[4] == 1);
    return FREHG_OK;
  }
  if (!strcmp(name, "wc") || !strcmp(name, "wcn") || !strcmp(name, "hn")) {
    src = !strcmp(name, "wc") ? re->W[re->cur]
          : !strcmp(name, "wcn") ? re->W[1 - re->cur] : re->H[1 - re->cur];
    FG_CUDA(cudaMemcpy(buf.data(), src, n * sizeof(double), cudaMemcpyDeviceToHost));
    const bool hn = !strcmp(name, "hn");
    to_halo(re, buf, out_halo, gv, re->p.htop, hn && re->p.bc_type[5] == 1, re->p.hbot,
            hn && re->p.bc_type[4] == 1);
    return FREHG_OK;
  }
  FG_CUDA(cudaStreamSynchronize(re->stream));
  const int nb = nblocks(n);
  if (!strcmp(name, "wch") || !strcmp(name, "qx") || !strcmp(name, "qy") ||
      !strcmp(name, "qz")) {
    src = !strcmp(name, "wch") ? re->wch : !strcmp(name, "qx") ? re->qx
          : !strcmp(name, "qy") ? re->qy : re->qz;
    ghosts = false;
  } else if (!strcmp(name, "ch")) {
    k_cap_of_h<<<nb, 256, 0, re->stream>>>(a, re->H[re->cur], re->scratch);
    src = re->scratch;
    ghosts = false;
  } else if (!strcmp(name, "hwc")) {
    k_h_of_theta<<<nb, 256, 0, re->stream>>>(a, re->W[re->cur], re->scratch);
    src = re->scratch;
    ghosts = false;
  } else if (!strcmp(name, "Kx") || !strcmp(name, "Ky") || !strcmp(name, "Kz")) {
    const int which = name[1] == 'x' ? 0 : name[1] == 'y' ? 1 : 2;
    k_faces_export<<<nb, 256, 0, re->stream>>>(a, re->W[1 - re->cur], which, re->scratch);
    src = re->scratch;
    ghosts = false;
  } else if (!strcmp(name, "dz3d") || !strcmp(name, "actv") || !strcmp(name, "bot3d") ||
             !strcmp(name, "room")) {
    std::vector<double> wcn;
    if (!strcmp(name, "room")) {
      wcn.resize(n);
      FG_CUDA(cudaMemcpy(wcn.data(), re->W[1 - re->cur], n * sizeof(double), cudaMemcpyDeviceToHost));
    }
    for (size_t c = 0; c < n; ++c) {
      const int k = (int)(c / re->ncol);
      if (!strcmp(name, "dz3d")) buf[c] = re->p.dz;
      else if (!strcmp(name, "actv")) buf[c] = 1.0;
      else if (!strcmp(name, "bot3d")) buf[c] = -re->p.dz * (double)(k + 1);
      else buf[c] = (re->p.soil.theta_s - wcn[c]) * re->p.dz * re->p.dx * re->p.dy;
    }
    to_halo(re, buf, out_halo, false, 0, false, 0, false);
    return FREHG_OK;
  } else {
    set_error("unknown field '%s'", name);
    return FREHG_ERR_BAD_ARG;
  }
  FG_CUDA(cudaGetLastError());
  FG_CUDA(cudaMemcpyAsync(buf.data(), src, n * sizeof(double), cudaMemcpyDeviceToHost, re->stream));
  FG_CUDA(cudaStreamSynchronize(re->stream));
  to_halo(re, buf, out_halo, ghosts, 0, false, 0, false);
  if (!strcmp(name, "qz")) {
    std::vector<double> top(re->ncol);
    FG_CUDA(cudaMemcpy(top.data(), re->qztop, re->ncol * sizeof(double), cudaMemcpyDeviceToHost));
    const size_t hx = re->nx + 2;
    for (int j = 0; j < re->ny; ++j)
      for (int i = 0; i < re->nx; ++i) out_halo[(size_t)(i + 1) + (size_t)(j + 1) * hx] = top[(size_t)i + (size_t)re->nx * j];
  }
  return FREHG_OK;
}

int frehg_re_check_staged_wait(frehg_re* re, int* err_word) {
  clear_error();
  FG_ARG(re && err_word, "null argument");
  FG_ARG(re->finalized, "check before a finalized state");
  const ReArgs a = make_args(re);
  if (re->p.scheme != 1 || !picard_ff(re) || !mixed_solve(re) || !re->fKs || (re->nx & 1)) {
    set_error("the staged assembly serves Picard handles in mixed precision with a per-cell Ks "
              "field and an even nx");
    return FREHG_ERR_UNSUPPORTED;
  }
  const size_t n = re->n;
  const StencilLaunch PL = stencil_launch(re->nx, re->ny, re->nz);
  cudaStream_t st = re->stream;
  float* f[4] = {nullptr, nullptr, nullptr, nullptr};
  double* b = nullptr;
  int rc = FREHG_OK;
  for (int q = 0; q < 4; ++q)
    if (cudaMalloc(&f[q], n * sizeof(float)) != cudaSuccess) rc = FREHG_ERR_CUDA;
  if (cudaMalloc(&b, n * sizeof(double)) != cudaSuccess) rc = FREHG_ERR_CUDA;
  if (rc != FREHG_OK) set_error("self-check allocation failed");
  if (rc == FREHG_OK) {
    Stencil32 o;
    o.n = n;
    o.a0 = f[1];
    o.a1 = f[2];
    o.a2 = f[3];
    bool staged = false;
    rc = launch_staged_assembly(re, a, PL, f[0], o, b, &staged, 1);
    o.a0 = o.a1 = o.a2 = nullptr;  // not owned
    if (rc == FREHG_OK && !staged) {
      set_error("tensor maps of the staged assembly could not be encoded");
      rc = FREHG_ERR_UNSUPPORTED;
    }
    ReScalars sh;
    if (rc == FREHG_OK && (cudaStreamSynchronize(st) != cudaSuccess ||
                           cudaMemcpy(&sh, re->sc, sizeof(sh), cudaMemcpyDeviceToHost) !=
                               cudaSuccess)) {
      set_error("staged-wait self-check failed: %s", cudaGetErrorString(cudaGetLastError()));
      rc = FREHG_ERR_CUDA;
    }
    if (rc == FREHG_OK) {
      *err_word = sh.stage_err;
      const int zero = 0;
      if (cudaMemcpy(&re->sc->stage_err, &zero, sizeof(int), cudaMemcpyHostToDevice) !=
          cudaSuccess) {
        set_error("staged-wait self-check: resetting the error word failed");
        rc = FREHG_ERR_CUDA;
      }
    }
  }
  for (int q = 0; q < 4; ++q) cudaFree(f[q]);
  cudaFree(b);
  return rc;
}

int frehg_re_check_staged_assembly(frehg_re* re, int64_t* mismatches) {
  clear_error();
  FG_ARG(re && mismatches, "null argument");
  FG_ARG(re->finalized, "check before a finalized state");
  const ReArgs a = make_args(re);
  if (re->p.scheme != 1 || !picard_ff(re) || !mixed_solve(re) || !re->fKs || (re->nx & 1)) {
    set_error("the staged assembly serves Picard handles in mixed precision with a per-cell Ks "
              "field and an even nx");
    return FREHG_ERR_UNSUPPORTED;
  }
  const size_t n = re->n;
  const StencilLaunch PL = stencil_launch(re->nx, re->ny, re->nz);
  cudaStream_t st = re->stream;
  float* f[2][4] = {{nullptr}};
  double* b[2] = {nullptr, nullptr};
  int rc = FREHG_OK;
  for (int v = 0; v < 2 && rc == FREHG_OK; ++v) {
    for (int q = 0; q < 4; ++q)
      if (cudaMalloc(&f[v][q], n * sizeof(float)) != cudaSuccess) rc = FREHG_ERR_CUDA;
    if (cudaMalloc(&b[v], n * sizeof(double)) != cudaSuccess) rc = FREHG_ERR_CUDA;
  }
  if (rc != FREHG_OK) set_error("self-check allocation failed");
  if (rc == FREHG_OK) {
    Stencil32 o;
    o.n = n;
    o.a0 = f[0][1];
    o.a1 = f[0][2];
    o.a2 = f[0][3];
    bool staged = false;
    rc = launch_staged_assembly(re, a, PL, f[0][0], o, b[0], &staged);
    o.a0 = o.a1 = o.a2 = nullptr;  // not owned
    if (rc == FREHG_OK && !staged) {
      set_error("tensor maps of the staged assembly could not be encoded");
      rc = FREHG_ERR_UNSUPPORTED;
    }
    if (rc == FREHG_OK) {
      k_pic_assemble_ff<true, false, float><<<PL.grid, PL.block, 0, st>>>(
          a, f[1][0], f[1][1], f[1][2], f[1][3], b[1], PL.planes, PL.tiles);
      if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
        set_error("assembly self-check launch failed");
        rc = FREHG_ERR_CUDA;
      }
    }
    if (rc == FREHG_OK) {
      int64_t bad = 0;
      std::vector<uint32_t> x(n), y(n);
      for (int q = 0; q < 4 && rc == FREHG_OK; ++q) {
        if (cudaMemcpy(x.data(), f[0][q], n * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(y.data(), f[1][q], n * 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
          set_error("self-check copy failed");
          rc = FREHG_ERR_CUDA;
        }
        for (size_t c = 0; c < n && rc == FREHG_OK; ++c) bad += x[c] != y[c];
      }
      std::vector<uint64_t> u(n), w(n);
      if (rc == FREHG_OK &&
          (cudaMemcpy(u.data(), b[0], n * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
           cudaMemcpy(w.data(), b[1], n * 8, cudaMemcpyDeviceToHost) != cudaSuccess)) {
        set_error("self-check copy failed");
        rc = FREHG_ERR_CUDA;
      }
      if (rc == FREHG_OK)
        for (size_t c = 0; c < n; ++c) bad += u[c] != w[c];
      *mismatches = bad;
      ReScalars sh;
      if (rc == FREHG_OK &&
          cudaMemcpy(&sh, re->sc, sizeof(sh), cudaMemcpyDeviceToHost) == cudaSuccess &&
          sh.stage_err) {
        set_error("staged Picard assembly: a bounded wait ran out (%d)", sh.stage_err);
        rc = FREHG_ERR_CUDA;
      }
    }
  }
  for (int v = 0; v < 2; ++v) {
    for (int q = 0; q < 4; ++q) cudaFree(f[v][q]);
    cudaFree(b[v]);
  }
  return rc;
}

int frehg_re_get_counters(const frehg_re* re, frehg_re_counters* c) {
  clear_error();
  FG_ARG(re && c, "null argument");
  *c = re->cnt;
  c->kernel_launches = re->prof.launches;
  FG_TRY(read_scalars(re));
  c->elastic_volume = re->sc_host->vol_elastic;
  return FREHG_OK;
}

int frehg_re_attach_unet(frehg_re* re, frehg_unet* net) {
  clear_error();
  if (re) re->constit_fresh = false;
  FG_ARG(re, "null handle");
  FG_ARG(re->nx % 4 == 0 && re->ny % 4 == 0 && re->nz % 4 == 0,
         "the learned preconditioner needs nx, ny, nz divisible by 4");
  // the time of one network application depends on the network and the grid only: keep it when
  // the same network is attached again (a restarted run), time it anew otherwise
  if (net != re->net) re->apply_ms = -1.0;
  re->net = net;
  if (net && !re->lnk_f) {
    FG_CUDA(cudaMalloc(&re->lnk_f, re->n * sizeof(float)));
    FG_CUDA(cudaMalloc(&re->cap_f, re->n * sizeof(float)));
  }
  re->plain_its_ref = 0;
  re->net_on = false;
  re->probe_pending = true;
  re->solves_since_probe = 0;
  re->last_plain_ms = 0.0;
  return FREHG_OK;
}

int frehg_re_set_assembly_staging(frehg_re* re, int on) {
  clear_error();
  FG_ARG(re, "null handle");
  re->staged = on != 0;
  return FREHG_OK;
}

int frehg_re_set_fused_iteration(frehg_re* re, int on) {
  clear_error();
  FG_ARG(re, "null handle");
  FG_ARG(on >= -1 && on <= 1, "on must be -1, 0 or 1");
  re->ksp.fused64 = on;
  return FREHG_OK;
}

int frehg_re_set_learned_policy(frehg_re* re, int probe_every, double max_ratio) {
  clear_error();
  FG_ARG(re, "null handle");
  FG_ARG(probe_every >= 0 && max_ratio > 0.0, "probe_every >= 0 and max_ratio > 0 required");
  re->probe_every = probe_every;
  re->max_ratio = max_ratio;
  re->net_on = false;
  re->probe_pending = true;
  re->solves_since_probe = 0;
  return FREHG_OK;
}

int frehg_re_training_pairs(frehg_re* re, int npairs, const int* iters, int target,
                            float* r_out, float* e_out, float* lnk_out, float* cap_out) {
  clear_error();
  if (re) re->constit_fresh = false;
  FG_ARG(re && iters && r_out && e_out && lnk_out && cap_out && npairs > 0, "bad argument");
  FG_ARG(target >= 0 && target <= 2, "target must be 0 (error), 1 (error - r) or 2 "
         "(error - line solve of r)");
  FG_ARG(re->finalized && re->attached, "training pairs need an initialised, attached solver");
  FG_ARG(re->p.scheme == 0, "training pairs are drawn from the PCA head solve");
  int kmax = 0;
  for (int q = 0; q < npairs; ++q) {
    FG_ARG(iters[q] >= 0 && (q == 0 || iters[q] > iters[q - 1]),
           "iteration numbers must be increasing");
    kmax = iters[q];
  }
  cudaStream_t st = re->stream;
  ReArgs a = make_args(re);
  const int nb = nblocks(re->n);
  const size_t n = re->n;
  // the next step's system at the current state (nothing advances)
  k_step_begin<<<1, 1, 0, st>>>(re->sc);
  k_constit<false, true><<<nb, 256, 0, st>>>(a, a.h_old, re->kr, nullptr, re->cap);
  const StencilLaunch L = stencil_launch(re->nx, re->ny, re->nz);
  re->A.scaled = false;
  re->A.s_in_r = false;
  re->A.f32_entries = false;
  k_assemble<<<L.grid, L.block, 0, st>>>(a, re->A.s, re->A.a0, re->A.a1, re->A.a2, re->A.b,
                                         L.planes, L.tiles);
  k_net_fields<<<nb, 256, 0, st>>>(a, lnk_out, cap_out);
  FG_CUDA(cudaGetLastError());
  // x~* of the scaled system, FP64 Jacobi-PCG to the handle's rtol
  frehg_solver_config cfg = re->cfg;
  cfg.precision = 0;
  CgResult res;
  KrylovSolver& K = re->ksp;
  K.net = NetPrecond();
  FG_TRY(K.solve(re->A, re->scratch, cfg, st, &res));
  double* xstar = nullptr;
  FG_CUDA(cudaMalloc(&xstar, n * sizeof(double)));
  double *zl = nullptr, *ul = nullptr;
  if (target == 2) {
    FG_CUDA(cudaMalloc(&zl, n * sizeof(double)));
    FG_CUDA(cudaMalloc(&ul, n * sizeof(double)));
  }
  const int ncol = re->nx * re->ny;
  FG_CUDA(cudaMemcpyAsync(xstar, K.x, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  // rerun the iteration and record (r~_k, x~* - x~_k)
  CgDevState init;
  memset(&init, 0, sizeof(init));
  init.rtol = 0.0;
  init.atol = 0.0;
  init.divtol = 0.0;
  init.max_it = kmax + 1;
  FG_CUDA(cudaMemcpyAsync(K.dst, &init, sizeof(init), cudaMemcpyHostToDevice, st));
  const int nbk = reduction_blocks(n, 256, 4);
  k_cg_init<<<nbk, 256, 0, st>>>(re->A.s, re->A.b, K.x, K.r, n, K.dst, K.partials);
  int q = 0;
  for (int it = 0; it <= kmax && q < npairs; ++it) {
    if (it == iters[q]) {
      const double* sub = target == 1 ? K.r : nullptr;
      if (target == 2) {
        k_line_apply64<<<(ncol + 127) / 128, 128, 0, st>>>(re->A.a2, K.r, ul, zl, ncol, re->nz);
        sub = zl;
      }
      k_pair<<<nb, 256, 0, st>>>(xstar, K.x, K.r, sub, r_out + (size_t)q * n,
                                 e_out + (size_t)q * n, n);
      ++q;
    }
    if (it == kmax) break;
    k_cg_p<<<nbk, 256, 0, st>>>(K.r, K.p, n, K.dst);
    k_cg_spmv<<<L.grid, L.block, 0, st>>>(re->A.a0, re->A.a1, re->A.a2, K.p, K.w, re->nx, re->ny,
                                          re->nz, L.planes, L.tiles, K.dst, K.partials);
    k_cg_update<<<nbk, 256, 0, st>>>(K.x, K.r, K.p, K.w, re->A.s, n, K.dst, K.partials);
  }
  FG_CUDA(cudaGetLastError());
  FG_CUDA(cudaStreamSynchronize(st));
  cudaFree(xstar);
  cudaFree(zl);
  cudaFree(ul);
  if (q < npairs) {
    set_error("training pairs: the iteration stopped before iteration %d", iters[q]);
    return FREHG_ERR_STATE;
  }
  return FREHG_OK;
}

int frehg_re_set_profiling(frehg_re* re, int on) {
  clear_error();
  FG_ARG(re, "null handle");
  FG_CUDA(cudaStreamSynchronize(re->stream));
  if (re->prof.on) FG_TRY(re->prof.flush());
  if (on) re->prof.reset();
  re->prof.on = on != 0;
  return FREHG_OK;
}

int frehg_re_kernel_stats(frehg_re* re, frehg_kernel_stat* out, int max, int* count) {
  clear_error();
  FG_ARG(re && count && (max == 0 || out), "null argument");
  FG_CUDA(cudaStreamSynchronize(re->stream));
  FG_TRY(re->prof.flush());
  const int n = (int)re->prof.stats.size();
  *count = n;
  for (int q = 0; q < n && q < max; ++q) {
    const Profiler::Stat& s = re->prof.stats[q];
    memset(&out[q], 0, sizeof(out[q]));
    strncpy(out[q].name, s.name.c_str(), sizeof(out[q].name) - 1);
    out[q].launches = s.launches;
    out[q].total_ms = s.ms;
    out[q].bytes_per_launch = s.bytes;
    out[q].idle_launches = s.idle;
  }
  return FREHG_OK;
}

int frehg_re_water_volume(frehg_re* re, double* vol) {
  clear_error();
  FG_ARG(re && vol, "null argument");
  ReArgs a = make_args(re);
  double* d_out = re->scratch;
  k_volume<<<nblocks(re->n), 256, 0, re->stream>>>(a, re->W[re->cur], d_out);
  FG_CUDA(cudaGetLastError());
  FG_CUDA(cudaMemcpyAsync(vol, d_out, sizeof(double), cudaMemcpyDeviceToHost, re->stream));
  FG_CUDA(cudaStreamSynchronize(re->stream));
  return FREHG_OK;
}

int frehg_re_boundary_volumes(frehg_re* re, double* top_in, double* bottom_in) {
  clear_error();
  FG_ARG(re && top_in && bottom_in, "null argument");
  FG_TRY(read_scalars(re));
  *top_in = re->sc_host->vol_top;
  *bottom_in = re->sc_host->vol_bot;
  return FREHG_OK;
}

int frehg_re_set_stream(frehg_re* re, void* s) {
  clear_error();
  FG_ARG(re, "null handle");
  FG_TRY(wait_copies(re, -1, true));
  FG_CUDA(cudaStreamSynchronize(re->stream));
  re->stream = s ? (cudaStream_t)s : re->own_stream;
  return FREHG_OK;
}

int frehg_re_sync(frehg_re* re) {
  clear_error();
  FG_ARG(re, "null handle");
  FG_CUDA(cudaStreamSynchronize(re->stream));
  FG_TRY(wait_copies(re, -1, true));
  return FREHG_OK;
}

}  // extern "C"
