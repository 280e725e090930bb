// Mixed-form modified Picard step on the device (not in reference: the reference only has the
// PCA scheme).  A rain pulse (rain_rate) enters through the top face up to what the face
// admits with the surface held at h = 0 (Dirichlet branch for that iterate, the excess runs
// off); a fixed qtop is forced as in the PCA step.  Optionally the head change of one
// iteration is limited to +-picard_dh_max.  The same scheme as the oracle's FP64 statement (Celia, Bouloutas & Zarba 1990):
//   per iterate h^m, with K and C frozen at h^m,
//   [V(C + Ss th^n/ths) + dt sum T] d_c - dt sum_nb T d_nb = -Rdt_c,
//   Rdt_c = V(th(h^m) - th^n) + V Ss (th^n/ths)(h^m - h^n) - dt Q_c(h^m)   (FP64 residual),
//   h^{m+1} = h^m + d until |d|_inf < picard_tol;
// then the conservative update th^{n+1} = th^n + [dt Q_c(h^{n+1}) - V Ss (th^n/ths)(h^{n+1}-h^n)]/V
// with the last frozen K, so the water budget closes to rounding.
#pragma once

#include "re_kernels.cuh"

namespace fg {

__device__ __forceinline__ double pic_mean(int harmonic, double a, double b) {
  if (!harmonic) return 0.5 * (a + b);
  const double s = a + b;
  return s > 0.0 ? 2.0 * a * b / s : 0.0;
}

__device__ __forceinline__ double pic_qtop(const ReArgs& a, size_t col) {
  // rain pulse: the per-column top flux field, when set, distributes it over the columns
  const double q = a.has_qtop ? a.qtop_field[col] : (a.rain_rate != 0.0 ? a.rain_rate : a.qtop);
  if (a.rain_rate != 0.0) return a.sc->time < a.rain_until ? q : 0.0;
  return q;
}

// Net inflow Q_c of cell (i,j,k) at the current iterate (a.h_new) with the frozen cell
// conductivities Ks*kr; optionally the transmissibility sum and the +x/+y/+z couplings, and the
// part of Q_c through the top / bottom domain faces.
struct PicRow {
  double q, tsum, tx, ty, tz, top, bot;
};

__device__ __forceinline__ PicRow pic_row(const ReArgs& a, const CellSoil& s, size_t c,
                                          size_t col, int i, int j, int k) {
  const int hm = a.face_mean;
  const double dz = a.dz;
  const double Az = a.dx * a.dy;
  const double hc = a.h_new[c];
  const double krc = a.kr[c];
  const double Kxc = s.Ksx * krc, Kyc = s.Ksy * krc, Kzc = s.Ksz * krc;
  PicRow r = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  double t;
  if (i > 0) {
    const CellSoil sm = soil_of(a.soil, c - 1, col - 1);
    t = pic_mean(hm, sm.Ksx * a.kr[c - 1], Kxc) * a.cx;
    r.q += t * (a.h_new[c - 1] - hc);
    r.tsum += t;
  }
  if (i + 1 < a.nx) {
    const CellSoil sp = soil_of(a.soil, c + 1, col + 1);
    t = pic_mean(hm, Kxc, sp.Ksx * a.kr[c + 1]) * a.cx;
    r.q += t * (a.h_new[c + 1] - hc);
    r.tsum += t;
    r.tx = t;
  }
  if (j > 0) {
    const CellSoil sm = soil_of(a.soil, c - a.nx, col - a.nx);
    t = pic_mean(hm, sm.Ksy * a.kr[c - a.nx], Kyc) * a.cy;
    r.q += t * (a.h_new[c - a.nx] - hc);
    r.tsum += t;
  }
  if (j + 1 < a.ny) {
    const CellSoil sp = soil_of(a.soil, c + a.nx, col + a.nx);
    t = pic_mean(hm, Kyc, sp.Ksy * a.kr[c + a.nx]) * a.cy;
    r.q += t * (a.h_new[c + a.nx] - hc);
    r.tsum += t;
    r.ty = t;
  }
  // face above
  if (k > 0) {
    const CellSoil sm = soil_of(a.soil, c - a.ncol, col);
    const double kf = pic_mean(hm, sm.Ksz * a.kr[c - a.ncol], Kzc);
    t = kf * a.cz;
    r.q += t * (a.h_new[c - a.ncol] - hc) + Az * kf;
    r.tsum += t;
  } else if (a.bc5 == 1) {
    const double kf = s.Ksz;
    t = kf * (2.0 * a.cz);
    r.top = t * (a.htop - hc) + Az * kf;
    r.q += r.top;
    r.tsum += t;
  } else if (a.bc5 == 2) {
    const double qin = -pic_qtop(a, col) * Az;
    const double tD = s.Ksz * (2.0 * a.cz);
    const double fD = tD * (0.0 - hc) + Az * s.Ksz;
    if (a.rain_rate != 0.0 && qin > 0.0 && fD < qin) {
      // rain beyond what the face admits with the surface at h = 0: the top face is a
      // Dirichlet h = 0 face for this iterate and the excess runs off (no ponding)
      r.top = fD;
      r.tsum += tD;
    } else {
      r.top = qin;
    }
    r.q += r.top;
  }
  // face below
  if (k + 1 < a.nz) {
    const CellSoil sp = soil_of(a.soil, c + a.ncol, col);
    const double kf = pic_mean(hm, Kzc, sp.Ksz * a.kr[c + a.ncol]);
    t = kf * a.cz;
    r.q += t * (a.h_new[c + a.ncol] - hc) - Az * kf;
    r.tsum += t;
    r.tz = t;
  } else if (a.bc4 == 1) {
    const double kb = s.Ksz * vg_kr(s, a.hbot);
    const double kf = pic_mean(hm, Kzc, kb);
    t = kf * (2.0 * a.cz);
    r.bot = t * (a.hbot - hc) - Az * kf;
    r.q += r.bot;
    r.tsum += t;
  } else if (a.bc4 == 2) {
    r.bot = a.qbot * Az;
    r.q += r.bot;
  } else if (a.bc4 == 3) {
    r.bot = -Kzc * Az;
    r.q += r.bot;
  }
  return r;
}

// Linearised system of one Picard iteration (diagonal into dg, +x/+y/+z couplings, rhs), with
// the same face values as pic_row but each x and z face evaluated once: a thread marches down
// its column and carries the face below a level to the next level as that level's face above,
// and takes a cell's -x face from the lane to its left (warp shuffle; lane 0 evaluates its own).
// Launched on (32 x 8)-column tiles marching through `planes` levels: a warp is one tile row.
__global__ void __launch_bounds__(256) k_pic_assemble(ReArgs a, double* __restrict__ dg,
                                                      double* __restrict__ a0,
                                                      double* __restrict__ a1,
                                                      double* __restrict__ a2,
                                                      double* __restrict__ bvec, int planes,
                                                      int tiles) {
  const double dt = a.sc->dt_used;
  const double V = a.dx * a.dy * a.dz;
  const double Az = a.dx * a.dy;
  const int hm = a.face_mean;
  const int t0 = (a.nx + 31) / 32;
  const int lane = threadIdx.x;
  const unsigned full = 0xffffffffu;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int i = (tile % t0) * 32 + lane;
    const int j = (tile / t0) * 8 + threadIdx.y;
    const bool act = i < a.nx && j < a.ny;
    const size_t col = act ? (size_t)i + (size_t)a.nx * j : 0;
    const int kb = blockIdx.y * planes, ke = min(a.nz, kb + planes);
    // face above the current level: transmissibility and flux into the current cell
    double tzm = 0.0, fzm = 0.0;
    if (act && kb > 0) {
      const size_t c = col + a.ncol * kb;
      const CellSoil s0 = soil_of(a.soil, c, col);
      const CellSoil sm = soil_of(a.soil, c - a.ncol, col);
      const double kf = pic_mean(hm, sm.Ksz * a.kr[c - a.ncol], s0.Ksz * a.kr[c]);
      tzm = kf * a.cz;
      fzm = tzm * (a.h_new[c - a.ncol] - a.h_new[c]) + Az * kf;
    }
    for (int k = kb; k < ke; ++k) {
      const size_t c = col + a.ncol * k;
      CellSoil s;
      double hc = 0.0, krc = 0.0, Kxc = 0.0;
      if (act) {
        s = soil_of(a.soil, c, col);
        hc = a.h_new[c];
        krc = a.kr[c];
        Kxc = s.Ksx * krc;
      }
      // +x face, the neighbour's K and h from the next lane (lane 31 loads them)
      double Kxn = __shfl_down_sync(full, Kxc, 1);
      double hxn = __shfl_down_sync(full, hc, 1);
      double tx = 0.0, fxp = 0.0;
      if (act && i + 1 < a.nx) {
        if (lane == 31) {
          const CellSoil sp = soil_of(a.soil, c + 1, col + 1);
          Kxn = sp.Ksx * a.kr[c + 1];
          hxn = a.h_new[c + 1];
        }
        tx = pic_mean(hm, Kxc, Kxn) * a.cx;
        fxp = tx * (hxn - hc);
      }
      // -x face: the +x face of the previous lane (lane 0 evaluates it)
      double txm = __shfl_up_sync(full, tx, 1);
      double fxm = -__shfl_up_sync(full, fxp, 1);
      if (!act) continue;  // after the shuffles: every lane took part in them
      if (i == 0) {
        txm = 0.0;
        fxm = 0.0;
      } else if (lane == 0) {
        const CellSoil sm = soil_of(a.soil, c - 1, col - 1);
        txm = pic_mean(hm, sm.Ksx * a.kr[c - 1], Kxc) * a.cx;
        fxm = txm * (a.h_new[c - 1] - hc);
      }
      double q = fxm + fxp;
      double tsum = txm + tx;
      // y faces
      const double Kyc = s.Ksy * krc, Kzc = s.Ksz * krc;
      double ty = 0.0;
      if (j > 0) {
        const CellSoil sm = soil_of(a.soil, c - a.nx, col - a.nx);
        const double t = pic_mean(hm, sm.Ksy * a.kr[c - a.nx], Kyc) * a.cy;
        q += t * (a.h_new[c - a.nx] - hc);
        tsum += t;
      }
      if (j + 1 < a.ny) {
        const CellSoil sp = soil_of(a.soil, c + a.nx, col + a.nx);
        ty = pic_mean(hm, Kyc, sp.Ksy * a.kr[c + a.nx]) * a.cy;
        q += ty * (a.h_new[c + a.nx] - hc);
        tsum += ty;
      }
      // face above: carried, or the top boundary
      if (k > 0) {
        q += fzm;
        tsum += tzm;
      } else if (a.bc5 == 1) {
        const double kf = s.Ksz;
        const double t = kf * (2.0 * a.cz);
        q += t * (a.htop - hc) + Az * kf;
        tsum += t;
      } else if (a.bc5 == 2) {
        const double qin = -pic_qtop(a, col) * Az;
        const double tD = s.Ksz * (2.0 * a.cz);
        const double fD = tD * (0.0 - hc) + Az * s.Ksz;
        if (a.rain_rate != 0.0 && qin > 0.0 && fD < qin) {
          q += fD;  // no ponding: Dirichlet h = 0 face for this iterate
          tsum += tD;
        } else {
          q += qin;
        }
      }
      // face below: evaluated here and carried to the next level, or the bottom boundary
      double tz = 0.0;
      if (k + 1 < a.nz) {
        const CellSoil sp = soil_of(a.soil, c + a.ncol, col);
        const double kf = pic_mean(hm, Kzc, sp.Ksz * a.kr[c + a.ncol]);
        tz = kf * a.cz;
        const double fz = tz * (a.h_new[c + a.ncol] - hc) - Az * kf;
        q += fz;
        tsum += tz;
        tzm = tz;
        fzm = -fz;
      } else if (a.bc4 == 1) {
        const double kbv = s.Ksz * vg_kr(s, a.hbot);
        const double kf = pic_mean(hm, Kzc, kbv);
        const double t = kf * (2.0 * a.cz);
        q += t * (a.hbot - hc) - Az * kf;
        tsum += t;
      } else if (a.bc4 == 2) {
        q += a.qbot * Az;
      } else if (a.bc4 == 3) {
        q += -Kzc * Az;
      }
      const double wcn = a.w_old[c];
      dg[c] = V * (a.cap[c] + s.Ss * wcn * s.inv_ths) + dt * tsum;
      a0[c] = -dt * tx;
      a1[c] = -dt * ty;
      a2[c] = -dt * tz;
      const double rdt =
          V * (a.wch[c] - wcn) + V * s.Ss * (wcn * s.inv_ths) * (hc - a.h_old[c]) - dt * q;
      bvec[c] = -rdt;
    }
  }
}

// h^{m+1} = h^m + d (d limited to +-picard_dh_max when set) and |d|_inf.  The limit and the
// maximum compare bit patterns (non-negative doubles order like their 64-bit integers), which
// keeps them off the FP64 pipe; a NaN in d counts as an infinite change, which fails the
// convergence test.
// SCALED: the solver left its solution scaled, d = s x~ is formed here (k_unscale fused)
// Two cells per step with 16-byte accesses (whole cudaMalloc allocations: 256-byte aligned).
__device__ __forceinline__ double pic_limited(double dc, long long lim_bits, long long& m) {
  const long long kAbs = 0x7fffffffffffffffll;
  const long long b = __double_as_longlong(dc);
  long long ab = b & kAbs;
  if (ab > lim_bits) {
    ab = lim_bits;
    dc = __longlong_as_double((b & ~kAbs) | lim_bits);
  }
  m = ab > m ? ab : m;
  return dc;
}

template <bool SCALED = false>
__global__ void k_pic_update(ReArgs a, const double* __restrict__ d,
                             const double* __restrict__ s = nullptr) {
  const long long kAbs = 0x7fffffffffffffffll;
  long long m = 0;
  const double lim = a.picard_dh_max;
  const long long lim_bits = lim > 0.0 ? __double_as_longlong(lim) : kAbs;
  const size_t gid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const double2* d2 = reinterpret_cast<const double2*>(d);
  const double2* s2 = reinterpret_cast<const double2*>(s);
  double2* h2 = reinterpret_cast<double2*>(a.h_new);
  for (size_t q = gid; q < a.n / 2; q += stride) {
    double2 dv = d2[q];
    if (SCALED) {
      const double2 sv = s2[q];
      dv.x *= sv.x;
      dv.y *= sv.y;
    }
    double2 hv = h2[q];
    hv.x += pic_limited(dv.x, lim_bits, m);
    hv.y += pic_limited(dv.y, lim_bits, m);
    h2[q] = hv;
  }
  if ((a.n & 1) && gid == 0) {
    const size_t c = a.n - 1;
    a.h_new[c] += pic_limited(SCALED ? s[c] * d[c] : d[c], lim_bits, m);
  }
  m = m > 0x7ff0000000000000ll ? 0x7ff0000000000000ll : m;  // NaN -> inf
  double tot;
  if (grid_max(__longlong_as_double(m), a.partials + 2 * kMaxRedBlocks, &a.sc->arrive[1], &tot) &&
      flat_tid() == 0)
    a.sc->dq_max = tot;
}

// conservative water-content update + boundary / elastic volumes + time
__global__ void __launch_bounds__(256) k_pic_final(ReArgs a, int planes, int tiles) {
  const double dt = a.sc->dt_used;
  const double V = a.dx * a.dy * a.dz;
  const double inv_V = 1.0 / V;
  double v[3] = {0.0, 0.0, 0.0};
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
    const double wcn = a.w_old[c];
    const PicRow r = pic_row(a, s, c, col, i, j, k);
    const double el = V * s.Ss * (wcn * s.inv_ths) * (a.h_new[c] - a.h_old[c]);
    a.w_new[c] = wcn + (dt * r.q - el) * inv_V;
    v[0] += r.top * dt;
    v[1] += r.bot * dt;
    v[2] += el;
  }
  }
  double tot[3];
  if (grid_sum<3>(v, a.partials, &a.sc->arrive[0], tot) && flat_tid() == 0) {
    a.sc->vol_top += tot[0];
    a.sc->vol_bot += tot[1];
    a.sc->vol_elastic += tot[2];
    a.sc->time += dt;
  }
}

__global__ void k_copy64(double* __restrict__ dst, const double* __restrict__ src, size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n;
       c += (size_t)gridDim.x * blockDim.x)
    dst[c] = src[c];
}

}  // namespace fg
