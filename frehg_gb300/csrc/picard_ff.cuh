// Float-float forms of the Picard assembly and of the conservative final update (not in
// reference): the same faces, boundary closures, residual and update as k_pic_assemble /
// k_pic_final (picard.cuh), with every FP64 operation replaced by float-float arithmetic on
// the FP32 pipe (ff32.cuh; about 48 significant bits), in one tiled kernel with two modes.
// GB300 runs FP64 at 1/73 of the FP32 rate, and the FP64 forms of these kernels are bound by
// that pipe, not by memory.
//
// Doubles are read and split into float-float with integer operations; results are written
// back as doubles.  The Picard residual's storage difference (theta(h^m) - theta^n of the two
// stored doubles) and its final combination stay in FP64.  The matrix (diagonal and
// couplings) is formed from the leading floats of the float-float transmissibilities: it
// shapes each Picard update, not the fixed point the iteration converges to, and the
// mixed-precision solve rounds it to FP32 anyway.  The face fluxes are chains of the lean
// operations (no renormalisation between steps) summed in an FfSum, whose error is a few
// 2^-48 of the largest term (not of the result): the residual, which fixes the iteration's
// fixed point, needs absolute accuracy relative to its largest terms.  The face fluxes of two
// neighbouring cells are exact negatives of each other (the face mean takes its arguments in
// index order, the head difference changes sign exactly), so the water budget of the final
// update closes to rounding as in FP64.
#pragma once

#include "picard.cuh"

namespace fg {

// head and the three directional conductivities Ks * kr of one cell, float-float
struct FfCell {
  ff h, kx, ky, kz;
};

// the axis-1 / axis-2 conductivity of a cell (kx itself when one serves all axes)
template <bool ISO>
__device__ __forceinline__ ff cell_ky(const FfCell& c) { return ISO ? c.kx : c.ky; }
template <bool ISO>
__device__ __forceinline__ ff cell_kz(const FfCell& c) { return ISO ? c.kx : c.kz; }

// Cell indices are 32-bit: a handle holds fewer than 2^31 cells (frehg_re_create refuses more;
// their device state alone would exceed the GPU's memory).
using cidx = unsigned;

__device__ __forceinline__ const SoilClass& class_of(const ReArgs& a, cidx c, cidx col) {
  return a.soil.cls[a.soil.cid ? (int)a.soil.cid[a.soil.cid3d ? c : col] : 0];
}

// Ks of one cell along axis d (0 x, 1 y, 2 z)
__device__ __forceinline__ ff ff_ks(const ReArgs& a, const SoilClass& k, cidx c, int d) {
  if (a.soil.Ks) return ff_from_double(a.soil.Ks[c]);
  return ff_make(k.ff_ks[d][0], k.ff_ks[d][1]);
}

// a cell's conductivity Ks kr (lean: the face sums take it)
__device__ __forceinline__ ff ff_cond(ff ks, ff kr) { return ff_mul_lean(ks, kr); }

// ISO: one conductivity serves all three axes (a per-cell Ks field, or isotropic classes
// only); the cell then carries kx alone
// Head, kr and Ks enter as lean splits (ff_from_double_lean): only the face sums read them.
template <bool ISO = false>
__device__ __forceinline__ FfCell ff_cell(const ReArgs& a, cidx c, cidx col) {
  const ff kr = ff_from_double_nb(a.kr[c]);
  FfCell r;
  r.h = ff_from_double_nb(a.h_new[c]);
  if (ISO) {
    if (a.soil.Ks) {
      r.kx = ff_cond(ff_from_double_nb(a.soil.Ks[c]), kr);
    } else {
      const SoilClass& k = class_of(a, c, col);
      r.kx = ff_cond(ff_make(k.ff_ks[0][0], k.ff_ks[0][1]), kr);
    }
    return r;
  }
  const SoilClass& k = class_of(a, c, col);
  if (a.soil.Ks || k.ks_iso) {
    r.kx = ff_cond(a.soil.Ks ? ff_from_double_nb(a.soil.Ks[c])
                             : ff_make(k.ff_ks[0][0], k.ff_ks[0][1]), kr);
    r.ky = r.kx;
    r.kz = r.kx;
  } else {
    r.kx = ff_cond(ff_make(k.ff_ks[0][0], k.ff_ks[0][1]), kr);
    r.ky = ff_cond(ff_make(k.ff_ks[1][0], k.ff_ks[1][1]), kr);
    r.kz = ff_cond(ff_make(k.ff_ks[2][0], k.ff_ks[2][1]), kr);
  }
  return r;
}

// pic_mean of two non-negative conductivities (lower index first); lean
__device__ __forceinline__ ff ff_face_mean(int harmonic, ff lo, ff hi) {
  const ff s = ff_add_lean(lo, hi);
  if (!harmonic) return ff_scale(s, 0.5f);
  return s.h > 0.0f ? ff_scale(ff_div(ff_mul(lo, hi), s), 2.0f) : ff_make(0.0f);
}

// The flux into a cell of head h from its neighbour of head hn through a face of conductance kf
// and geometric factor g (area / distance), kf g (hn - h), lean; *t = the face's
// transmissibility kf g (leading float: the matrix entry's factor).  Antisymmetric in (hn, h).
__device__ __forceinline__ ff ff_face_flux(ff kf, ff g, ff hn, ff h, float* t) {
  const ff tt = ff_mul_lean(kf, g);
  *t = tt.h;
  // the head difference renormalised (SloppyDWPlusDW): the product keeps it to 2^-48 of itself
  return ff_mul_lean(tt, ff_add_fast(hn, ff_neg(h)));
}

// The flux into the upper cell (head hu) from the lower one (head hd) through their common z
// face, gravity included: kf cz (hd - hu) - Az kf.  The lower cell adds its exact negative.
__device__ __forceinline__ ff ff_zface_flux(ff kf, ff cz, ff Az, ff hd, ff hu, float* t) {
  return ff_dif_lean(ff_face_flux(kf, cz, hd, hu, t), ff_mul_lean(Az, kf));
}

__device__ __forceinline__ bool ff_lt(ff a, ff b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }

// a - b with SloppyDWPlusDW (absolute error a few 2^-48 (|a| + |b|)); antisymmetric:
// ff_dif(a, b) = -ff_dif(b, a) exactly, so the two cells of a face see opposite fluxes
__device__ __forceinline__ ff ff_dif(ff a, ff b) { return ff_add_fast(a, ff_neg(b)); }

// geometric factors and boundary values of a launch, float-float
struct FfConst {
  ff cx, cy, cz, cz2, Az, V, dt, htop, hbot, qbot;
};

__device__ __forceinline__ FfConst ff_consts(const ReArgs& a, double dt) {
  FfConst k;
  k.cx = ff_from_double(a.cx);
  k.cy = ff_from_double(a.cy);
  k.cz = ff_from_double(a.cz);
  k.cz2 = ff_scale(k.cz, 2.0f);
  k.Az = ff_from_double(a.dx * a.dy);
  k.V = ff_from_double(a.dx * a.dy * a.dz);
  k.dt = ff_from_double(dt);
  k.htop = ff_from_double(a.htop);
  k.hbot = ff_from_double(a.hbot);
  k.qbot = ff_from_double(a.qbot);
  return k;
}

// the top-face closure of one cell: flux into the cell and the transmissibility it adds to the
// diagonal (pic_row's k = 0 branch)
__device__ __forceinline__ void ff_top_face(const ReArgs& a, const FfConst& K, const FfCell& cell,
                                            const SoilClass& kc, cidx c, cidx col, ff* flux,
                                            ff* trans) {
  *flux = ff_make(0.0f);
  *trans = ff_make(0.0f);
  if (a.bc5 == 1) {
    const ff kf = ff_ks(a, kc, c, 2);
    const ff t = ff_mul(kf, K.cz2);
    *flux = ff_add(ff_mul(t, ff_sub(K.htop, cell.h)), ff_mul(K.Az, kf));
    *trans = t;
  } else if (a.bc5 == 2) {
    const ff qin = ff_neg(ff_mul(ff_from_double(pic_qtop(a, col)), K.Az));
    const ff ksz = ff_ks(a, kc, c, 2);
    const ff tD = ff_mul(ksz, K.cz2);
    const ff fD = ff_add(ff_neg(ff_mul(tD, cell.h)), ff_mul(K.Az, ksz));
    if (a.rain_rate != 0.0 && qin.h > 0.0f && ff_lt(fD, qin)) {
      *flux = fD;  // no ponding: Dirichlet h = 0 face for this iterate
      *trans = tD;
    } else {
      *flux = qin;
    }
  }
}

// the bottom-face closure (pic_row's k = nz-1 branch)
template <bool ISO = false>
__device__ __forceinline__ void ff_bottom_face(const ReArgs& a, const FfConst& K,
                                               const FfCell& cell, cidx c, cidx col, ff* flux,
                                               ff* trans) {
  *flux = ff_make(0.0f);
  *trans = ff_make(0.0f);
  if (a.bc4 == 1) {
    const CellSoil s = soil_of(a.soil, c, col);
    const ff kb = ff_from_double(s.Ksz * vg_kr(s, a.hbot));
    const ff kf = ff_face_mean(a.face_mean, cell_kz<ISO>(cell), kb);
    const ff t = ff_mul(kf, K.cz2);
    *flux = ff_sub(ff_mul(t, ff_sub(K.hbot, cell.h)), ff_mul(K.Az, kf));
    *trans = t;
  } else if (a.bc4 == 2) {
    *flux = ff_mul(K.qbot, K.Az);
  } else if (a.bc4 == 3) {
    *flux = ff_neg(ff_mul(cell_kz<ISO>(cell), K.Az));
  }
}

// The Picard update and the next iteration's constitutive relations in one pass:
// h += s x~ with the limiter and |d|_inf exactly as k_pic_update<true>, then theta, K/Ks and C at
// the new head exactly as k_constit_ff, into kr, th, cap (the caller's second set of arrays:
// the current ones still hold the values at the previous head, which the final update of a
// converged step uses).  Same bits as the two kernels; one read of the head instead of two.
template <bool ALL_FF>
__global__ void __launch_bounds__(256, 4) k_pic_update_constit_ff(
    ReArgs a, const double* __restrict__ d, const double* __restrict__ s,
    double* __restrict__ kr, double* __restrict__ th, double* __restrict__ cap) {
  const long long kAbs = 0x7fffffffffffffffll;
  long long m = 0;
  const double lim = a.picard_dh_max;
  const long long lim_bits = lim > 0.0 ? __double_as_longlong(lim) : kAbs;
  const bool col_map = a.soil.cid && !a.soil.cid3d;
  const bool small = a.n <= 0xffffffffull;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < a.n;
       c += (size_t)gridDim.x * blockDim.x) {
    const size_t col = !col_map ? 0
                       : small  ? (size_t)((uint32_t)c % (uint32_t)a.ncol)
                                : c % a.ncol;
    const int id = a.soil.cid ? (int)a.soil.cid[a.soil.cid3d ? c : col] : 0;
    double dc = d[c];
    dc *= s[c];
    const double hc = a.h_new[c] + pic_limited(dc, lim_bits, m);
    a.h_new[c] = hc;
    const SoilClass& k = a.soil.cls[id];
    Constit r;
    if (ALL_FF || (k.use_vg && !k.use_mvg)) {
      const ff alpha = a.soil.alpha ? ff_from_double_nb(a.soil.alpha[c])
                                    : ff_make(k.ff_alpha[0], k.ff_alpha[1]);
      r = vg_constit_ff<true, true>(k, alpha, a.soil.continuous_theta ? 0.0 : k.aev, hc);
    } else {
      r = vg_constit<true, true>(soil_of(a.soil, c, col), hc);
    }
    kr[c] = r.kr;
    th[c] = r.theta;
    cap[c] = r.cap;
  }
  m = m > 0x7ff0000000000000ll ? 0x7ff0000000000000ll : m;  // NaN -> inf
  double tot;
  if (grid_max(__longlong_as_double(m), a.partials + 2 * kMaxRedBlocks, &a.sc->arrive[1], &tot) &&
      flat_tid() == 0)
    a.sc->dq_max = tot;
}

// The Picard residual's float-float part V Ss (wcn/ths) (h - h_old) - dt q, renormalised (the
// storage difference and the final combination are FP64)
__device__ __forceinline__ ff ff_residual_rest(ff V, ff dt, ff st, ff h, double h_old, ff q) {
  const ff dh = ff_add_fast(h, ff_neg(ff_from_double_nb(h_old)));  // renormalised, as in faces
  FfSum r = ff_sum_of(ff_mul_lean(V, ff_mul_lean(st, dh)));
  ff_sum_add(r, ff_neg(ff_mul_lean(dt, q)));
  return ff_sum_value(r);
}

// One level of a (32 x 8)-column tile plus the rows above and below it: the head and the
// axis-1 conductivity of each cell, float-float (the y faces read their neighbours here).
struct FfYPlane {
  float hh[10][32], hl[10][32], kh[10][32], kl[10][32];
  // the cells left (0) and right (1) of each tile row: head and axis-0 conductivity
  float xhh[8][2], xhl[8][2], xkh[8][2], xkl[8][2];
};

// k_pic_assemble in float-float as a tiled stencil: a (32 x 8)-thread block marches its column
// tile down `planes` levels.  Per level each thread stages its own cell's (h, K_y) in shared
// memory (threads 0-63 also stage the rows above and below the tile, threads 64-79 the cells
// left and right of its rows), then, after one barrier, forms the faces: x from the adjacent
// lanes (warp shuffles; lanes 0 and 31 read their outer neighbour from shared memory), y from
// shared memory, z with the cell below, which it loads while the others stage and carries to
// the next level as its own cell.  The level buffers alternate, so one
// barrier per level suffices: a buffer is rewritten two levels later, after every thread has
// passed the barrier that follows its last read.
//
// FINAL: the same faces at h^{n+1} with the last frozen K form the conservative update
// th^{n+1} = th^n + (dt Q - V Ss (th^n/ths)(h^{n+1} - h^n)) / V (k_pic_final's job) instead of
// the system, with the top / bottom / elastic volumes summed across the grid (FP64) and the
// time advanced.
// T: the type of the diagonal and couplings written (FP32 values either way; float when the
// mixed-precision solve's preparation reads them, which halves their traffic).
template <bool ISO, bool FINAL = false, typename T = double>
__global__ void __launch_bounds__(256, 4) k_pic_assemble_ff(ReArgs a, T* __restrict__ dg,
                                                           T* __restrict__ a0,
                                                           T* __restrict__ a1,
                                                           T* __restrict__ a2,
                                                           double* __restrict__ bvec, int planes,
                                                           int tiles) {
  __shared__ FfYPlane ys[2];
  // the launch's constants in shared memory rather than in 20 registers per thread
  __shared__ FfConst K;
  __shared__ ff inv_V;
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    K = ff_consts(a, a.sc->dt_used);
    inv_V = ff_div(ff_make(1.0f), K.V);
  }
  __syncthreads();
  double vol[3] = {0.0, 0.0, 0.0};  // FINAL: top, bottom, elastic volumes
  const int hm = a.face_mean;
  const int t0 = (a.nx + 31) / 32;
  const int lane = threadIdx.x, row = threadIdx.y;
  const int tid = row * 32 + lane;
  const unsigned full = 0xffffffffu;
  const ff zero = ff_make(0.0f);
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int i = (tile % t0) * 32 + lane;
    const int j0 = (tile / t0) * 8, j = j0 + row;
    const bool act = i < a.nx && j < a.ny;
    const cidx ncol = (cidx)a.ncol;
    const cidx col = act ? (cidx)i + (cidx)a.nx * j : 0u;
    // halo rows of the tile: threads 0-31 stage row j0 - 1, threads 32-63 row j0 + 8
    const int jh = tid < 32 ? j0 - 1 : j0 + 8;
    const bool act_h = tid < 64 && i < a.nx && jh >= 0 && jh < a.ny;
    const cidx colh = act_h ? (cidx)i + (cidx)a.nx * jh : 0u;
    const int hrow = tid < 32 ? 0 : 9;
    const int kb = blockIdx.y * planes, ke = min(a.nz, kb + planes);
    FfCell cur = {zero, zero, zero, zero};
    ff fzm = zero;     // flux into the current cell through its top face
    float tzm = 0.0f;  // and that face's transmissibility (leading float)
    if (act && kb < ke) {
      cur = ff_cell<ISO>(a, col + ncol * kb, col);
      if (kb > 0) {  // the face above the slab, as the slab above forms it (negated)
        const FfCell up = ff_cell<ISO>(a, col + ncol * (kb - 1), col);
        const ff kf = ff_face_mean(hm, cell_kz<ISO>(up), cell_kz<ISO>(cur));
        fzm = ff_neg(ff_zface_flux(kf, K.cz, K.Az, cur.h, up.h, &tzm));
      }
    }
    for (int k = kb; k < ke; ++k) {
      FfYPlane& P = ys[k & 1];
      const cidx c = col + ncol * k;
      // stage this level: the own cell and the halo rows
      P.hh[row + 1][lane] = cur.h.h;
      P.hl[row + 1][lane] = cur.h.l;
      P.kh[row + 1][lane] = cell_ky<ISO>(cur).h;
      P.kl[row + 1][lane] = cell_ky<ISO>(cur).l;
      if (tid < 64) {
        FfCell hc = {zero, zero, zero, zero};
        if (act_h) hc = ff_cell<ISO>(a, colh + ncol * k, colh);
        P.hh[hrow][lane] = hc.h.h;
        P.hl[hrow][lane] = hc.h.l;
        P.kh[hrow][lane] = cell_ky<ISO>(hc).h;
        P.kl[hrow][lane] = cell_ky<ISO>(hc).l;
      } else if (tid < 80) {
        const int xr = (tid - 64) >> 1, side = (tid - 64) & 1;
        const int ix = (tile % t0) * 32 + (side ? 32 : -1), jx = j0 + xr;
        FfCell xc = {zero, zero, zero, zero};
        if (ix >= 0 && ix < a.nx && jx < a.ny) {
          const cidx colx = (cidx)ix + (cidx)a.nx * jx;
          xc = ff_cell<ISO>(a, colx + ncol * k, colx);
        }
        P.xhh[xr][side] = xc.h.h;
        P.xhl[xr][side] = xc.h.l;
        P.xkh[xr][side] = xc.kx.h;
        P.xkl[xr][side] = xc.kx.l;
      }
      // This cell's residual values are read after the faces, from L1: their lines are
      // prefetched one level earlier (below), which keeps no registers of loads in flight during
      // the face sums.  The cell below (z face, carried to the next level) is loaded before the
      // barrier and converted after it.
      const bool has_below = act && k + 1 < a.nz;
      if (act) {
        if (has_below) {
          const cidx cn = c + ncol;
          asm volatile("prefetch.global.L1 [%0];" ::"l"(a.w_old + cn));
          asm volatile("prefetch.global.L1 [%0];" ::"l"(a.h_old + cn));
          if (!FINAL) {
            asm volatile("prefetch.global.L1 [%0];" ::"l"(a.wch + cn));
            asm volatile("prefetch.global.L1 [%0];" ::"l"(a.cap + cn));
          }
        }
      }
      // the halo cells of the next level (their rows are not the tile's own)
      if (k + 1 < ke) {
        if (tid < 64) {
          if (act_h) {
            const cidx ch = colh + ncol * (k + 1);
            asm volatile("prefetch.global.L1 [%0];" ::"l"(a.h_new + ch));
            asm volatile("prefetch.global.L1 [%0];" ::"l"(a.kr + ch));
            if (a.soil.Ks) asm volatile("prefetch.global.L1 [%0];" ::"l"(a.soil.Ks + ch));
          }
        } else if (tid < 80) {
          const int xr = (tid - 64) >> 1, side = (tid - 64) & 1;
          const int ix = (tile % t0) * 32 + (side ? 32 : -1), jx = j0 + xr;
          if (ix >= 0 && ix < a.nx && jx < a.ny) {
            const cidx cx = (cidx)ix + (cidx)a.nx * jx + ncol * (k + 1);
            asm volatile("prefetch.global.L1 [%0];" ::"l"(a.h_new + cx));
            asm volatile("prefetch.global.L1 [%0];" ::"l"(a.kr + cx));
            if (a.soil.Ks) asm volatile("prefetch.global.L1 [%0];" ::"l"(a.soil.Ks + cx));
          }
        }
      }
      const cidx cb = has_below ? c + ncol : c;
      double rb_h = 0.0, rb_kr = 0.0, rb_ks = 0.0;
      int rb_id = 0;
      if (act) {
        rb_h = a.h_new[cb];
        rb_kr = a.kr[cb];
        if (a.soil.Ks) rb_ks = a.soil.Ks[cb];
        if (a.soil.cid) rb_id = a.soil.cid[a.soil.cid3d ? cb : col];
      }
      __syncthreads();
      // +x face from the next lane's cell (lane 31 loads its neighbour)
      ff Kxn = ff_make(__shfl_down_sync(full, cur.kx.h, 1), __shfl_down_sync(full, cur.kx.l, 1));
      ff hxn = ff_make(__shfl_down_sync(full, cur.h.h, 1), __shfl_down_sync(full, cur.h.l, 1));
      float tx = 0.0f;
      ff fxp = zero;
      if (act && i + 1 < a.nx) {
        if (lane == 31) {
          Kxn = ff_make(P.xkh[row][1], P.xkl[row][1]);
          hxn = ff_make(P.xhh[row][1], P.xhl[row][1]);
        }
        fxp = ff_face_flux(ff_face_mean(hm, cur.kx, Kxn), K.cx, hxn, cur.h, &tx);
      }
      // -x face: the previous lane's +x face (lane 0 evaluates its own)
      float txm = __shfl_up_sync(full, tx, 1);
      ff fxm = ff_neg(ff_make(__shfl_up_sync(full, fxp.h, 1), __shfl_up_sync(full, fxp.l, 1)));
      FfCell below = cur;
      if (act) {
        if (i == 0) {
          txm = 0.0f;
          fxm = zero;
        } else if (lane == 0) {
          const ff kxm = ff_make(P.xkh[row][0], P.xkl[row][0]);
          const ff hxm = ff_make(P.xhh[row][0], P.xhl[row][0]);
          fxm = ff_face_flux(ff_face_mean(hm, kxm, cur.kx), K.cx, hxm, cur.h, &txm);
        }
        FfSum q = ff_sum_of(fxm);
        ff_sum_add(q, fxp);
        float tsum = txm + tx;
        // y faces from the staged neighbours
        float ty = 0.0f;
        if (j > 0) {
          const ff hn = ff_make(P.hh[row][lane], P.hl[row][lane]);
          const ff kn = ff_make(P.kh[row][lane], P.kl[row][lane]);
          float t;
          const ff kf = ff_face_mean(hm, kn, cell_ky<ISO>(cur));
          ff_sum_add(q, ff_face_flux(kf, K.cy, hn, cur.h, &t));
          tsum += t;
        }
        if (j + 1 < a.ny) {
          const ff hn = ff_make(P.hh[row + 2][lane], P.hl[row + 2][lane]);
          const ff kn = ff_make(P.kh[row + 2][lane], P.kl[row + 2][lane]);
          const ff kf = ff_face_mean(hm, cell_ky<ISO>(cur), kn);
          ff_sum_add(q, ff_face_flux(kf, K.cy, hn, cur.h, &ty));
          tsum += ty;
        }
        const SoilClass& kc = class_of(a, c, col);
        // face above: carried, or the top boundary
        if (k > 0) {
          ff_sum_add(q, fzm);
          tsum += tzm;
        } else {
          ff f, t;
          ff_top_face(a, K, cur, kc, c, col, &f, &t);
          ff_sum_add(q, f);
          tsum += t.h;
          if (FINAL) vol[0] += ff_to_double(ff_mul(f, K.dt));
        }
        // face below, carried to the next level
        float tz = 0.0f;
        if (has_below) {
          const SoilClass& kb = a.soil.cls[rb_id];
          const ff kr = ff_from_double_nb(rb_kr);
          below.h = ff_from_double_nb(rb_h);
          if (ISO || a.soil.Ks || kb.ks_iso) {
            below.kx = ff_cond(a.soil.Ks ? ff_from_double_nb(rb_ks)
                                         : ff_make(kb.ff_ks[0][0], kb.ff_ks[0][1]), kr);
            if (!ISO) {
              below.ky = below.kx;
              below.kz = below.kx;
            }
          } else {
            below.kx = ff_cond(ff_make(kb.ff_ks[0][0], kb.ff_ks[0][1]), kr);
            below.ky = ff_cond(ff_make(kb.ff_ks[1][0], kb.ff_ks[1][1]), kr);
            below.kz = ff_cond(ff_make(kb.ff_ks[2][0], kb.ff_ks[2][1]), kr);
          }
          const ff kf = ff_face_mean(hm, cell_kz<ISO>(cur), cell_kz<ISO>(below));
          const ff fz = ff_zface_flux(kf, K.cz, K.Az, below.h, cur.h, &tz);
          ff_sum_add(q, fz);
          tsum += tz;
          tzm = tz;
          fzm = ff_neg(fz);
        } else {
          ff f, t;
          ff_bottom_face<ISO>(a, K, cur, c, col, &f, &t);
          ff_sum_add(q, f);
          tsum += t.h;
          if (FINAL && k + 1 == a.nz) vol[1] += ff_to_double(ff_mul(f, K.dt));
        }
        const ff qv = ff_sum_value(q);
        const double r_wo = a.w_old[c], r_ho = a.h_old[c];
        const double r_wch = FINAL ? 0.0 : a.wch[c], r_cap = FINAL ? 0.0 : a.cap[c];
        const ff wcn = ff_from_double_nb(r_wo);
        const ff st = ff_mul(ff_make(kc.ff_ss_ths[0], kc.ff_ss_ths[1]), wcn);  // Ss wcn / ths
        if (FINAL) {
          const ff el = ff_mul(ff_mul(K.V, st), ff_dif(cur.h, ff_from_double_nb(r_ho)));
          const ff dw = ff_mul(ff_dif(ff_mul(K.dt, qv), el), inv_V);
          a.w_new[c] = ff_to_double_nb(ff_add_fast(wcn, dw));
          vol[2] += ff_to_double_nb(el);
          cur = below;
          continue;
        }
        // diagonal V (C + Ss wcn/ths) + dt sum T and couplings -dt T (FP32), rhs -Rdt with
        // Rdt = V (wch - wcn) + V Ss (wcn/ths) (h - h_old) - dt q (float-float)
        const float dtf = K.dt.h;
        dg[c] = (T)fmaf(dtf, tsum, K.V.h * (ff_hi_of_nb(r_cap) + st.h));
        a0[c] = (T)(-dtf * tx);
        a1[c] = (T)(-dtf * ty);
        a2[c] = (T)(-dtf * tz);
        // the storage difference wch - wcn of the two stored doubles and the residual's last
        // combination in FP64 (the difference is exact where the values are close, Sterbenz);
        // the elastic term and the face-flux sum in float-float
        const double dth = r_wch - r_wo;
        bvec[c] = -fma(a.vol_cell, dth, ff_to_double_nb(ff_residual_rest(K.V, K.dt, st, cur.h,
                                                                         r_ho, qv)));
      }
      cur = below;
    }
    __syncthreads();  // the next tile restages both buffers
  }
  if (FINAL) {
    double tot[3];
    if (grid_sum<3>(vol, a.partials, &a.sc->arrive[0], tot) && flat_tid() == 0) {
      a.sc->vol_top += tot[0];
      a.sc->vol_bot += tot[1];
      a.sc->vol_elastic += tot[2];
      a.sc->time += a.sc->dt_used;
    }
  }
}

}  // namespace fg
