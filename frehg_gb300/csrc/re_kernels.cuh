// Device kernels of the PCA Richards step (ReSolver::advanceStep, src/re/ReSolver.cpp:931-969).
//
// Layout: interior cells only, i fastest (c = i + nx*(j + ny*k), k = 0 the top layer).  The
// reference's halo cells are not stored; each ghost value the reference reads is produced by
// the rule that wrote it (enforceHeadBc / enforceMoistureBc copies, Dirichlet heads, or the
// zero-initialised ghosts of the first step, flagged by `ghosts_valid`).
//
// Per step:
//   k_kr            kr(h^n) per cell                             (computeKFace inputs)
//   k_assemble      C(h^n), face conductances, Gxp..Gct, Grhs    (groundwaterMatCoeff/Rhs,
//                   written as d / upper couplings / b            assembleAndSolve)
//   KrylovSolver    Jacobi-PCG head solve                         (LinearSolver::solve)
//   k_post          h^{n+1} = s x~, kr(h^{n+1}), theta(h^{n+1})   (enforceHeadBc, computeKFace,
//                                                                 updateDiagnostics)
//   k_correct       Darcy fluxes + mass-conservative corrector,   (groundwaterFlux,
//                   saturation flags, flux-imbalance max,         updateWaterContent,
//                   boundary inflow volumes                       adaptiveTimeStep dq)
//   k_realloc_sweep monotone relaxation of the reallocation sweep (reallocateWaterContent)
//   k_finalize      apply reallocation, clamp, Courant min, dt    (clampWaterContent,
//                                                                 adaptiveTimeStep)
#pragma once

#include "internal.h"
#include "reduce.cuh"
#include "vg.cuh"

namespace fg {

// flag bits of the reallocation pass
enum : uint8_t {
  F_SAT_OLD = 1,   // wc after the corrector >= theta_s
  F_WCH_SAT = 2,   // theta(h^{n+1}) >= theta_s
  F_OPEN_XP = 4,   // +x face conductance != 0
  F_OPEN_YP = 8,   // +y face conductance != 0
  F_SAT_NEW = 16,  // saturated as the reference's sequential sweep leaves it
};

// Device scalars of the step (adaptive dt state, budgets, sweep flag).
struct ReScalars {
  double dt;        // ReParams::dt
  double dtn;       // ReSolver::dtn_
  double dt_used;   // ReSolver::dt_used_
  double time;      // simulated time
  double dq_max;    // adaptiveTimeStep flux-imbalance max
  double dtco_min;  // adaptiveTimeStep Courant min
  double vol_top;   // cumulative top-face inflow volume
  double vol_bot;   // cumulative bottom-face inflow volume
  double vol_elastic;
  int changed;      // reallocation sweep changed a flag
  int stage_err;    // staged (TMA) assembly: nonzero when one of its bounded waits ran out
  unsigned int arrive[8];
};

struct ReArgs {
  int nx, ny, nz;
  size_t n, ncol;
  double dx, dy, dz;
  double htop, hbot, qtop, qbot;
  double co_max, dt_min, dt_max;
  int bc4, bc5;
  int full3d, ghosts_valid, adaptive, use_corrector, has_qtop;
  int face_mean;                   // Picard: 0 arithmetic, 1 harmonic
  double rain_rate, rain_until;    // Picard: rain pulse on the top face (no ponding)
  double picard_dh_max;            // Picard: per-iteration head change limit (0 = none)
  // ghost copies of the top layer (h, wc) taken before a surface exchange changed its cells:
  // the reference's halo keeps them until its next step re-enforces the ghosts (nullptr: the
  // ghosts follow the cells)
  const double* gh_top_h;
  const double* gh_top_w;
  // geometric factors: 1/dx, 1/dy, 1/dz; Ax/dx, Ay/dy, Az/dz; V/dz; 1/Ax, 1/Ay, 1/Az
  double inv_dx, inv_dy, inv_dz, cx, cy, cz, v_dz, inv_Ax, inv_Ay, inv_Az;
  double vol_cell;  // dx * dy * dz
  SoilView soil;
  const double* h_old;  // h^n (and hn)
  const double* w_old;  // wc^n (and wcn)
  double* h_new;
  double* w_new;
  double* kr;
  double* wch;
  double* cap;
  double* qx;
  double* qy;
  double* qz;
  double* qztop;
  const double* qtop_field;
  uint8_t* flags;
  ReScalars* sc;
  double* partials;
};

// ---- face conductance rules of computeKFace (ReSolver.cpp:217-380), one rank ---------------
// Kl = conductivity of the left (lower index) cell, Kr of the right one.

__device__ __forceinline__ double face_mean_ref(double Kp, double Km) { return 0.5 * (Kp + Km); }

// +x face of cell (i) given its conductivity Kc, the +x neighbour's Kn, the ghost conductivity
// Kg of the cell itself (K at the ghost head), the saturation of both cells (vertical-only
// closure) -- returns the Kx(c) value the reference holds after computeKFace.
__device__ __forceinline__ double face_x(const ReArgs& a, int i, double Kc, double Kn, double Kg,
                                         bool sat_c, bool sat_n) {
  if (a.full3d) return (i + 1 < a.nx) ? face_mean_ref(Kn, Kc) : 0.0;
  double K;
  if (i == 0)
    K = Kg;  // x- boundary overwrite 0.5*(Kp+Kp) with Kp = K(h ghost)
  else if (i + 1 < a.nx)
    K = face_mean_ref(Kn, Kc);
  else
    K = face_mean_ref(Kg, Kc);  // face towards the x+ ghost (a copy of this cell)
  if (!sat_c || (i + 1 < a.nx && !sat_n)) K = 0.0;
  return K;
}

__device__ __forceinline__ double face_y(const ReArgs& a, int j, double Kc, double Kn, double Kg,
                                         bool sat_c, bool sat_n) {
  if (a.full3d) return (j + 1 < a.ny) ? face_mean_ref(Kn, Kc) : 0.0;
  double K;
  if (j == 0)
    K = Kg;  // y- boundary overwrite (runs after the j == ny-1 wall)
  else if (j + 1 < a.ny)
    K = face_mean_ref(Kn, Kc);
  else
    K = 0.0;  // y+ wall (bc_type[2] == 0)
  if (!sat_c || (j + 1 < a.ny && !sat_n)) K = 0.0;
  return K;
}

// +z face (between k and k+1): mean inside, own K at the bottom unless closed.
__device__ __forceinline__ double face_z(const ReArgs& a, int k, double Kc, double Kn) {
  if (k + 1 < a.nz) return face_mean_ref(Kn, Kc);
  return a.bc4 == 0 ? 0.0 : Kc;
}

// top (k-) face of a k = 0 cell
__device__ __forceinline__ double face_top(const ReArgs& a, double Ksz, double Kc) {
  if (a.bc5 == 1) return Ksz;
  if (a.bc5 == 0) return 0.0;
  return Kc;
}

__device__ __forceinline__ bool cell_sat(const ReArgs& a, size_t c, size_t col, const double* w) {
  const CellSoil s = soil_of(a.soil, c, col);
  return w[c] >= s.ths;
}

// ---- kernels ---------------------------------------------------------------------------------

// savePreviousStepFields' scalar part: the dt this step applies (ReSolver.cpp:932)
__global__ void k_step_begin(ReScalars* sc) { sc->dt_used = sc->dt; }

// kr (and optionally theta and C) at the given head, from one set of transcendentals
template <bool THETA, bool CAP>
__global__ void k_constit(ReArgs a, const double* __restrict__ h, double* __restrict__ kr,
                          double* __restrict__ th, double* __restrict__ cap) {
  // the column index is only needed for a per-column class map; 32-bit when it fits
  const bool col_map = a.soil.cid && !a.soil.cid3d;
  const bool small = a.n <= 0xffffffffull;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < a.n;
       c += (size_t)gridDim.x * blockDim.x) {
    const size_t col = !col_map ? 0
                       : small  ? (size_t)((uint32_t)c % (uint32_t)a.ncol)
                                : c % a.ncol;
    const CellSoil s = soil_of(a.soil, c, col);
    const Constit r = vg_constit<THETA, CAP>(s, h[c]);
    kr[c] = r.kr;
    if (THETA) th[c] = r.theta;
    if (CAP) cap[c] = r.cap;
  }
}

// k_constit with the van Genuchten classes evaluated in float-float arithmetic on the FP32 pipe
// (vg_constit_ff); MVG and exponential classes take the FP64 forms.  ALL_FF: every class is
// van Genuchten (not MVG), and the FP64 forms are not compiled in.
template <bool THETA, bool CAP, bool ALL_FF>
__global__ void __launch_bounds__(256, 4) k_constit_ff(ReArgs a, const double* __restrict__ h,
                                                       double* __restrict__ kr,
                                                       double* __restrict__ th,
                                                       double* __restrict__ cap) {
  const bool col_map = a.soil.cid && !a.soil.cid3d;
  const bool small = a.n <= 0xffffffffull;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < a.n;
       c += (size_t)gridDim.x * blockDim.x) {
    const size_t col = !col_map ? 0
                       : small  ? (size_t)((uint32_t)c % (uint32_t)a.ncol)
                                : c % a.ncol;
    const int id = a.soil.cid ? (int)a.soil.cid[a.soil.cid3d ? c : col] : 0;
    const SoilClass& k = a.soil.cls[id];
    const double hc = h[c];
    Constit r;
    if (ALL_FF || (k.use_vg && !k.use_mvg)) {
      const ff alpha = a.soil.alpha ? ff_from_double_nb(a.soil.alpha[c])
                                    : ff_make(k.ff_alpha[0], k.ff_alpha[1]);
      r = vg_constit_ff<THETA, CAP>(k, alpha, a.soil.continuous_theta ? 0.0 : k.aev, hc);
    } else {
      r = vg_constit<THETA, CAP>(soil_of(a.soil, c, col), hc);
    }
    kr[c] = r.kr;
    if (THETA) th[c] = r.theta;
    if (CAP) cap[c] = r.cap;
  }
}

// groundwaterMatCoeff + groundwaterRhs + the COO rows of assembleAndSolve, written as the
// diagonal (into A.s), the +x/+y/+z couplings and b.
__global__ void __launch_bounds__(256) k_assemble(ReArgs a, double* __restrict__ dg,
                                                  double* __restrict__ a0, double* __restrict__ a1,
                                                  double* __restrict__ a2,
                                                  double* __restrict__ bvec, int planes,
                                                  int tiles) {
  const int t0 = (a.nx + 31) / 32;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
  const int i = (tile % t0) * 32 + threadIdx.x;
  const int j = (tile / t0) * 8 + threadIdx.y;
  if (i >= a.nx || j >= a.ny) continue;
  const int kb = blockIdx.y * planes, ke = min(a.nz, kb + planes);
  const size_t col = (size_t)i + (size_t)a.nx * j;
  const double dx = a.dx, dy = a.dy, dzk = a.dz;
  const double Ax = dy * dzk, Ay = dx * dzk, V = dx * dy * dzk;
  const bool gv = a.ghosts_valid;
  const double dtg = a.sc->dt_used;
  for (int k = kb; k < ke; ++k) {
    const size_t c = col + a.ncol * k;
    const CellSoil s = soil_of(a.soil, c, col);
    const double hc = a.h_old[c];
    const double krc = a.kr[c];
    const double ch = a.cap[c];
    const double wcn = a.w_old[c];
    const bool sat_c = a.full3d ? true : (wcn >= s.ths);
    // ghost conductivity of this cell: K(h ghost) = K(h_c) once ghosts exist, K(0) = Ks before
    // a top-layer ghost after a surface exchange keeps the head from before it
    const bool stale = a.gh_top_h && k == 0;
    const double krg = gv ? (stale ? vg_kr(s, a.gh_top_h[col]) : krc) : 1.0;
    // +x and -x faces
    double Kxp, Kxm = 0.0;
    {
      double Kn = 0.0;
      bool sat_n = true;
      if (i + 1 < a.nx) {
        const CellSoil sn = soil_of(a.soil, c + 1, col + 1);
        Kn = sn.Ksx * a.kr[c + 1];
        if (!a.full3d) sat_n = a.w_old[c + 1] >= sn.ths;
      }
      Kxp = face_x(a, i, s.Ksx * krc, Kn, s.Ksx * krg, sat_c, sat_n);
      if (i > 0) {
        const CellSoil sm = soil_of(a.soil, c - 1, col - 1);
        const double krm = a.kr[c - 1];
        const bool sat_m = a.full3d ? true : (a.w_old[c - 1] >= sm.ths);
        const double krmg = gv ? (stale && i - 1 == 0 ? vg_kr(sm, a.gh_top_h[col - 1]) : krm) : 1.0;
        Kxm = face_x(a, i - 1, sm.Ksx * krm, s.Ksx * krc, sm.Ksx * krmg, sat_m, sat_c);
      }
    }
    double Kyp, Kym = 0.0;
    {
      double Kn = 0.0;
      bool sat_n = true;
      if (j + 1 < a.ny) {
        const CellSoil sn = soil_of(a.soil, c + a.nx, col + a.nx);
        Kn = sn.Ksy * a.kr[c + a.nx];
        if (!a.full3d) sat_n = a.w_old[c + a.nx] >= sn.ths;
      }
      Kyp = face_y(a, j, s.Ksy * krc, Kn, s.Ksy * krg, sat_c, sat_n);
      if (j > 0) {
        const CellSoil sm = soil_of(a.soil, c - a.nx, col - a.nx);
        const double krm = a.kr[c - a.nx];
        const bool sat_m = a.full3d ? true : (a.w_old[c - a.nx] >= sm.ths);
        const double krmg =
            gv ? (stale && j - 1 == 0 ? vg_kr(sm, a.gh_top_h[col - a.nx]) : krm) : 1.0;
        Kym = face_y(a, j - 1, sm.Ksy * krm, s.Ksy * krc, sm.Ksy * krmg, sat_m, sat_c);
      }
    }
    double Kzp, Kzm;
    {
      double Kn = 0.0;
      if (k + 1 < a.nz) {
        const CellSoil sn = soil_of(a.soil, c + a.ncol, col);
        Kn = sn.Ksz * a.kr[c + a.ncol];
      }
      Kzp = face_z(a, k, s.Ksz * krc, Kn);
      if (k > 0) {
        const CellSoil sm = soil_of(a.soil, c - a.ncol, col);
        Kzm = face_z(a, k - 1, sm.Ksz * a.kr[c - a.ncol], s.Ksz * krc);
      } else {
        Kzm = face_top(a, s.Ksz, s.Ksz * krc);
      }
    }
    // groundwaterMatCoeff (ReSolver.cpp:433-468) with the geometric quotients precomputed:
    // A/d = a.cx, a.cy; V/(dz*dzf) = Az/dz (2 Az/dz for the half cell above k = 0)
    const double Gxp = -Kxp * dtg * a.cx;
    const double Gxm = -Kxm * dtg * a.cx;
    const double Gyp = -Kyp * dtg * a.cy;
    const double Gym = -Kym * dtg * a.cy;
    const double Gzp = -Kzp * dtg * a.cz;
    const double Gzm = -Kzm * dtg * ((k == 0) ? 2.0 * a.cz : a.cz);
    const double store = ch + s.Ss * wcn * s.inv_ths;
    double Gct = store;
    Gct *= V;
    Gct -= (Gxp + Gxm + Gyp + Gym);
    if (!(k == a.nz - 1 && a.bc4 != 1)) Gct -= Gzp;
    if (k == 0) {
      if (a.bc5 == 1) Gct -= Gzm;
    } else {
      Gct -= Gzm;
    }
    // groundwaterRhs (ReSolver.cpp:515-547); V/dz precomputed
    double g = store * hc * V;
    g -= dtg * a.v_dz * Kzp;
    g += dtg * a.v_dz * Kzm;
    // lateral hn ghosts are copies (or zero at step 1)
    const double hn_ghost = gv ? (stale ? a.gh_top_h[col] : hc) : 0.0;
    if (i == a.nx - 1) g -= Gxp * hn_ghost;
    if (i == 0) g -= Gxm * hn_ghost;
    if (j == a.ny - 1) g -= Gyp * hn_ghost;
    if (j == 0) g -= Gym * hn_ghost;
    if (k == a.nz - 1) {
      if (a.bc4 == 1) g += Gzp * (gv ? a.hbot : 0.0);
      if (a.bc4 == 2) g += dtg * a.v_dz * (a.qbot + Kzp);
    }
    if (k == 0 && a.bc5 == 1) g -= Gzm * a.htop;
    if (k == 0 && a.bc5 == 2) {
      const double qcol = a.has_qtop ? a.qtop_field[col] : a.qtop;
      g += -dtg * a.v_dz * (qcol + Kzm);
    }
    dg[c] = Gct;
    a0[c] = (i + 1 < a.nx) ? Gxp : 0.0;
    a1[c] = (j + 1 < a.ny) ? Gyp : 0.0;
    a2[c] = (k + 1 < a.nz) ? Gzp : 0.0;
    bvec[c] = g;
  }
  }
}

// kr(h^{n+1}) and theta(h^{n+1}) once the solve has written h^{n+1} (re_solve_unpack).
__global__ void k_post(ReArgs a) {
  const bool col_map = a.soil.cid && !a.soil.cid3d;
  const bool small = a.n <= 0xffffffffull;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < a.n;
       c += (size_t)gridDim.x * blockDim.x) {
    const size_t col = !col_map ? 0
                       : small  ? (size_t)((uint32_t)c % (uint32_t)a.ncol)
                                : c % a.ncol;
    const CellSoil so = soil_of(a.soil, c, col);
    const Constit r = vg_constit<true, false>(so, a.h_new[c]);
    a.kr[c] = r.kr;
    a.wch[c] = r.theta;
  }
}

// darcyFluxZ through the +z face of cell (k) to (k+1) inside the column
__device__ __forceinline__ double flux_z_inner(const ReArgs& a, double Kc, double Kn, double hc,
                                               double hn) {
  const double faceA = a.dx * a.dy;
  const double kface = 0.5 * (Kc + Kn);
  return faceA * kface * ((hn - hc) * a.inv_dz - 1.0);
}

// groundwaterFlux + updateWaterContent + adaptiveTimeStep's dq (ReSolver.cpp:671-786, 891-905)
__global__ void __launch_bounds__(256) k_correct(ReArgs a, int planes, int tiles) {
  const double dtg = a.sc->dt_used;
  const double dtq = a.sc->dtn;  // adaptiveTimeStep resets params_.dt = dtn_ before dq
  const int t0 = (a.nx + 31) / 32;
  double dqmax = 0.0;
  double vol[2] = {0.0, 0.0};
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int i = (tile % t0) * 32 + threadIdx.x;
    const int j = (tile / t0) * 8 + threadIdx.y;
    if (i >= a.nx || j >= a.ny) continue;
    const int kb = blockIdx.y * planes, ke = min(a.nz, kb + planes);
    const size_t col = (size_t)i + (size_t)a.nx * j;
    const double dx = a.dx, dy = a.dy, dzk = a.dz;
    const double Ax = dy * dzk, Ay = dx * dzk, Az = dx * dy, V = dx * dy * dzk;
    for (int k = kb; k < ke; ++k) {
      const size_t c = col + a.ncol * k;
      const CellSoil s = soil_of(a.soil, c, col);
      const double hc = a.h_new[c];
      const double krc = a.kr[c];
      const bool sat_c = a.full3d ? true : (a.w_old[c] >= s.ths);
      // lateral faces with the post-solve rules (ghost heads are copies: K(ghost) = K(h_c))
      double Kxp = 0.0, Kxm = 0.0, Kyp = 0.0, Kym = 0.0;
      double hxp = hc, hxm = hc, hyp = hc, hym = hc;
      {
        double Kn = 0.0;
        bool sat_n = true;
        if (i + 1 < a.nx) {
          const CellSoil sn = soil_of(a.soil, c + 1, col + 1);
          Kn = sn.Ksx * a.kr[c + 1];
          hxp = a.h_new[c + 1];
          if (!a.full3d) sat_n = a.w_old[c + 1] >= sn.ths;
        }
        Kxp = face_x(a, i, s.Ksx * krc, Kn, s.Ksx * krc, sat_c, sat_n);
        if (i > 0) {
          const CellSoil sm = soil_of(a.soil, c - 1, col - 1);
          const double Km = sm.Ksx * a.kr[c - 1];
          const bool sat_m = a.full3d ? true : (a.w_old[c - 1] >= sm.ths);
          Kxm = face_x(a, i - 1, Km, s.Ksx * krc, Km, sat_m, sat_c);
          hxm = a.h_new[c - 1];
        }
      }
      {
        double Kn = 0.0;
        bool sat_n = true;
        if (j + 1 < a.ny) {
          const CellSoil sn = soil_of(a.soil, c + a.nx, col + a.nx);
          Kn = sn.Ksy * a.kr[c + a.nx];
          hyp = a.h_new[c + a.nx];
          if (!a.full3d) sat_n = a.w_old[c + a.nx] >= sn.ths;
        }
        Kyp = face_y(a, j, s.Ksy * krc, Kn, s.Ksy * krc, sat_c, sat_n);
        if (j > 0) {
          const CellSoil sm = soil_of(a.soil, c - a.nx, col - a.nx);
          const double Km = sm.Ksy * a.kr[c - a.nx];
          const bool sat_m = a.full3d ? true : (a.w_old[c - a.nx] >= sm.ths);
          Kym = face_y(a, j - 1, Km, s.Ksy * krc, Km, sat_m, sat_c);
          hym = a.h_new[c - a.nx];
        }
      }
      double qxp = 0.0, qxm = 0.0, qyp = 0.0, qym = 0.0;
      if (a.full3d) {
        qxp = Ax * Kxp * (hxp - hc) * a.inv_dx;
        if (i > 0) qxm = Ax * Kxm * (hc - hxm) * a.inv_dx;
        qyp = Ay * Kyp * (hyp - hc) * a.inv_dy;
        if (j > 0) qym = Ay * Kym * (hc - hym) * a.inv_dy;
      }
      // vertical fluxes (upward positive): qzp through the bottom face, qzm through the top face
      const double Kc = s.Ksz * krc;
      double qzp;
      if (k + 1 < a.nz) {
        const CellSoil sn = soil_of(a.soil, c + a.ncol, col);
        qzp = flux_z_inner(a, Kc, sn.Ksz * a.kr[c + a.ncol], hc, a.h_new[c + a.ncol]);
      } else if (a.bc4 == 2) {
        qzp = a.qbot * Az;
      } else if (a.bc4 == 0) {
        qzp = 0.0;
      } else {
        const double hg = a.bc4 == 1 ? a.hbot : hc;  // enforceHeadBc bottom ghost
        const double Kg = s.Ksz * vg_kr(s, hg);
        const double kface = 0.5 * (Kc + Kg);
        qzp = Az * kface * ((hg - hc) * (2.0 * a.inv_dz) - 1.0);
      }
      double qzm;
      if (k > 0) {
        const CellSoil sm = soil_of(a.soil, c - a.ncol, col);
        qzm = flux_z_inner(a, sm.Ksz * a.kr[c - a.ncol], Kc, a.h_new[c - a.ncol], hc);
      } else if (a.bc5 == 2) {
        qzm = (a.has_qtop ? a.qtop_field[col] : a.qtop) * Az;
      } else {
        const double kface = a.bc5 == 1 ? s.Ksz : 0.0;
        const double hg = a.bc5 == 1 ? a.htop : hc;
        qzm = Az * kface * ((hc - hg) * (2.0 * a.inv_dz) - 1.0);
      }
      // updateWaterContent
      const double hn = a.h_old[c];
      const double wcn = a.w_old[c];
      double wc;
      if (a.use_corrector) {
        const double coeff = V * (1.0 + 1.0 * s.Ss * (hc - hn) * s.inv_ths);
        const double dqx = dtg * (qxp - qxm);
        const double dqy = dtg * (qyp - qym);
        const double dqz = dtg * (qzp - qzm);
        wc = (wcn * V + dqx + dqy + dqz) / coeff;
      } else {
        wc = a.wch[c];
      }
      a.w_new[c] = wc;
      a.qx[c] = qxp;
      a.qy[c] = qyp;
      a.qz[c] = qzp;
      if (k == 0) a.qztop[col] = qzm;
      uint8_t f = 0;
      if (wc >= s.ths) f |= F_SAT_OLD | F_SAT_NEW;
      if (a.wch[c] >= s.ths) f |= F_WCH_SAT;
      if (Kxp != 0.0) f |= F_OPEN_XP;
      if (Kyp != 0.0) f |= F_OPEN_YP;
      a.flags[c] = f;
      if (a.adaptive && k > 0) {
        const double qin = qxp * a.inv_Ax + qyp * a.inv_Ay + qzp * a.inv_Az;
        const double qou = qxm * a.inv_Ax + qym * a.inv_Ay + qzm * a.inv_Az;
        const double dq = fabs(qin - qou) * dtq * a.inv_dz;
        dqmax = fmax(dqmax, dq);
      }
      if (k == 0) vol[0] += -qzm * dtg;
      if (k == a.nz - 1) vol[1] += qzp * dtg;
    }
  }
  double tot[2];
  if (grid_sum<2>(vol, a.partials, &a.sc->arrive[0], tot) && flat_tid() == 0) {
    a.sc->vol_top += tot[0];
    a.sc->vol_bot += tot[1];
  }
  if (a.adaptive) {
    double m;
    if (grid_max(dqmax, a.partials + 2 * kMaxRedBlocks, &a.sc->arrive[1], &m) && flat_tid() == 0)
      a.sc->dq_max = m;
  }
}

// Saturation of the ghost cell a reallocation neighbour check reads (wc ghosts are copies of the
// previous step's final water content, zero before the first step).
__device__ __forceinline__ bool ghost_sat(const ReArgs& a, size_t c, size_t col) {
  if (!a.ghosts_valid) return false;
  if (a.gh_top_w && c < a.ncol) {  // top layer after a surface exchange: the earlier copy
    const CellSoil s = soil_of(a.soil, c, col);
    return a.gh_top_w[col] >= s.ths;
  }
  return cell_sat(a, c, col, a.w_old);
}

// One sweep of the monotone relaxation of reallocateWaterContent's k, j, i sweep
// (ReSolver.cpp:802-836).  The sequential sweep's saturation after the update obeys
//   sat_new(c) = sat_old(c) | wch_sat(c) & (pred(c) | succ(c)),
// pred = sat_new of the already-visited neighbours (k-1 or the top rule, i-1, j-1 through open
// faces), succ = sat_old of the unvisited ones (k+1 or the bottom ghost, i+1, j+1).  On this DAG
// the least fixed point is the sequential result; one thread walks a column (k order) and
// re-reads lateral predecessors, so each sweep extends every chain by at least one lateral hop.
__global__ void k_realloc_sweep(ReArgs a, int top_sat) {
  const size_t col = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (col >= a.ncol) return;
  const int i = (int)(col % a.nx), j = (int)(col / a.nx);
  bool prev = top_sat != 0;  // top rule for k = 0
  int changed = 0;
  for (int k = 0; k < a.nz; ++k) {
    const size_t c = col + a.ncol * k;
    const uint8_t f = a.flags[c];
    bool sat = (f & (F_SAT_OLD | F_SAT_NEW)) != 0;
    if (!sat && (f & F_WCH_SAT)) {
      bool adj = prev;
      if (i > 0) {
        const uint8_t g = ((volatile uint8_t*)a.flags)[c - 1];
        adj |= (g & F_OPEN_XP) && (g & F_SAT_NEW);
      }
      if (j > 0) {
        const uint8_t g = ((volatile uint8_t*)a.flags)[c - a.nx];
        adj |= (g & F_OPEN_YP) && (g & F_SAT_NEW);
      }
      if (!adj) {
        if (k + 1 < a.nz)
          adj = (a.flags[c + a.ncol] & F_SAT_OLD) != 0;
        else
          adj = ghost_sat(a, c, col);
      }
      if (!adj && (f & F_OPEN_XP))
        adj = (i + 1 < a.nx) ? (a.flags[c + 1] & F_SAT_OLD) != 0 : ghost_sat(a, c, col);
      if (!adj && (f & F_OPEN_YP))
        adj = (j + 1 < a.ny) ? (a.flags[c + a.nx] & F_SAT_OLD) != 0 : ghost_sat(a, c, col);
      if (adj) {
        sat = true;
        a.flags[c] = f | F_SAT_NEW;
        changed = 1;
      }
    }
    prev = sat;
  }
  if (changed) a.sc->changed = 1;
}

// Apply the reallocation (ReSolver.cpp:825-833), clampWaterContent (:839-853) and the
// adaptiveTimeStep Courant bound (:906-910); the last block updates dt (:921-928) and time.
// Launched on (32 x 8)-column tiles marching through `planes` levels (no index divisions).
__global__ void __launch_bounds__(256) k_finalize(ReArgs a, int top_sat, int planes, int tiles) {
  double dtco = INFINITY;
  const int t0 = (a.nx + 31) / 32;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
  const int i = (tile % t0) * 32 + threadIdx.x;
  const int j = (tile / t0) * 8 + threadIdx.y;
  if (i >= a.nx || j >= a.ny) continue;
  const size_t col = (size_t)i + (size_t)a.nx * j;
  const int kb = blockIdx.y * planes, ke = min(a.nz, kb + planes);
  for (int k = kb; k < ke; ++k) {
    const size_t c = col + a.ncol * k;
    const CellSoil s = soil_of(a.soil, c, col);
    const uint8_t f = a.flags[c];
    double wc = a.w_new[c];
    if (f & F_SAT_OLD) {
      wc = s.ths;
    } else {
      // adjacentToSat with the sequential sweep's view
      bool adj = (k == 0) ? (top_sat != 0) : (a.flags[c - a.ncol] & F_SAT_NEW) != 0;
      if (!adj && i > 0) {
        const uint8_t g = a.flags[c - 1];
        adj = (g & F_OPEN_XP) && (g & F_SAT_NEW);
      }
      if (!adj && j > 0) {
        const uint8_t g = a.flags[c - a.nx];
        adj = (g & F_OPEN_YP) && (g & F_SAT_NEW);
      }
      if (!adj) adj = (k + 1 < a.nz) ? (a.flags[c + a.ncol] & F_SAT_OLD) != 0 : ghost_sat(a, c, col);
      if (!adj && (f & F_OPEN_XP))
        adj = (i + 1 < a.nx) ? (a.flags[c + 1] & F_SAT_OLD) != 0 : ghost_sat(a, c, col);
      if (!adj && (f & F_OPEN_YP))
        adj = (j + 1 < a.ny) ? (a.flags[c + a.nx] & F_SAT_OLD) != 0 : ghost_sat(a, c, col);
      if (!adj) {
        if (wc < 0.9999 * s.ths) a.h_new[c] = vg_head(s, wc);
      } else {
        wc = a.wch[c];
      }
    }
    if (wc > s.ths)
      wc = s.ths;
    else if (wc < s.thr)
      wc = s.thr;
    a.w_new[c] = wc;
    if (a.adaptive && k > 0 && wc < s.ths) {
      const double dk = vg_dKdwc(s, wc, s.Ksz);
      const double dt_co = a.co_max * a.dz / dk;
      if (dt_co < dtco) dtco = dt_co;  // std::min(dt_Comin, dt_Co): NaN is skipped
    }
  }
  }
  // -max(-x) gives the NaN-skipping min
  double m;
  const bool last = grid_max(-dtco, a.partials + 2 * kMaxRedBlocks, &a.sc->arrive[2], &m);
  if (last && flat_tid() == 0) {
    ReScalars* sc = a.sc;
    sc->time += sc->dt_used;
    if (a.adaptive) {
      const double dt_Comin = fmin(-m, 1.0e8);
      double dt = sc->dtn;
      if (sc->dq_max > 0.02)
        dt *= 0.75;
      else if (sc->dq_max < 0.01)
        dt *= 1.25;
      if (dt > dt_Comin) dt = dt_Comin;
      if (dt > a.dt_max) dt = a.dt_max;
      if (dt < a.dt_min) dt = a.dt_min;
      sc->dt = dt;
      sc->dtn = dt;
    }
  }
}

}  // namespace fg
