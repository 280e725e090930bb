// The float-float Picard assembly (k_pic_assemble_ff, mixed-precision form) with its inputs
// staged through the Tensor Memory Accelerator (not in reference).
//
// Same faces, closures, residual and matrix entries as k_pic_assemble_ff<ISO, false, float>
// (picard_ff.cuh), in the same arithmetic order, so both write identical bits.  What changes is
// how the data arrive: a (32 x 8)-column tile marches down its levels, and one producer warp
// copies every level's inputs into a three-stage shared-memory ring with
// cp.async.bulk.tensor.3d (this GPU's own memory only, no cluster multicast), signalling a
// "full" mbarrier per stage; the eight consumer warps wait on it, form their cell's faces and
// residual from shared memory, and arrive on the stage's "empty" mbarrier, which the producer
// waits on before it refills the stage.  Per stage and level:
//   h, kr, Ks     a 36 x 10 box (the tile, one row either side, two columns either side so the
//                 box starts on a 16-byte boundary: x0 - 2 with x0 a multiple of 32);
//   wc^n, h^n, theta(h), C   a 32 x 8 box (the tile's own cells).
// The loads of the next levels are in flight while a level is computed and no thread holds raw
// loads in registers; each cell's head and conductivity are split into float-float once per
// level into a shared plane that the neighbours read (one barrier over the consumer warps per
// level).  Out-of-range box elements (domain edges) read as zero and are never used.  The grid
// is persistent (three blocks per SM), so a block's pipeline runs on from one tile into the
// next.
//
// Every wait is bounded: a wait that runs out sets the block's abort flag and the caller's error
// word; the producer then stops issuing, waits (bounded) for the copies it has in flight, and
// the block returns.  Used for the isotropic case with a per-cell Ks field and an even nx (the
// tensor's row stride must be a multiple of 16 bytes); other cases take k_pic_assemble_ff.
#pragma once

#include <cuda.h>

#include "picard_ff.cuh"

namespace fg {

constexpr int kPtStages = 3;
constexpr int kPtWideX = 36, kPtWideY = 10;
constexpr int kPtWideBytes = kPtWideX * kPtWideY * 8;  // 2880
constexpr int kPtWideStride = 2944;                    // 128-byte multiple
constexpr int kPtNarrowBytes = 32 * 8 * 8;             // 2048
// stage layout: h, kr, Ks (wide boxes), then wc^n, h^n, theta(h), C (narrow boxes)
constexpr int kPtStageBytes = 3 * kPtWideStride + 4 * kPtNarrowBytes;  // 17024
constexpr int kPtSmemBytes = kPtStages * kPtStageBytes;               // 51072
constexpr uint32_t kPtTxBytes = 3u * kPtWideBytes + 4u * kPtNarrowBytes;
// a waiting thread is suspended in try_wait for up to kPtSuspendNs per poll (it resumes when the
// phase completes); kPtSpinLimit polls (at most about 1.3 s) before a wait counts as failed
constexpr uint32_t kPtSuspendNs = 10000;
constexpr long kPtSpinLimit = 1L << 17;

struct PicTmaMaps {
  CUtensorMap h, kr, ks, wo, ho, wch, cap;
};

// ---- mbarrier and bulk-tensor primitives (PTX) ----------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(kPtSuspendNs)
      : "memory");
  return ok != 0;
}
// bounded wait for the phase of `parity`; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (long q = 0; q < kPtSpinLimit; ++q)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

struct PtStage {
  const double* h;    // [10][36]
  const double* kr;
  const double* ks;
  const double* wo;   // [8][32]
  const double* ho;
  const double* wch;
  const double* cap;
};

__device__ __forceinline__ PtStage pt_stage(const unsigned char* base, int slot) {
  const unsigned char* s = base + (size_t)slot * kPtStageBytes;
  PtStage p;
  p.h = reinterpret_cast<const double*>(s);
  p.kr = reinterpret_cast<const double*>(s + kPtWideStride);
  p.ks = reinterpret_cast<const double*>(s + 2 * kPtWideStride);
  p.wo = reinterpret_cast<const double*>(s + 3 * kPtWideStride);
  p.ho = reinterpret_cast<const double*>(s + 3 * kPtWideStride + kPtNarrowBytes);
  p.wch = reinterpret_cast<const double*>(s + 3 * kPtWideStride + 2 * kPtNarrowBytes);
  p.cap = reinterpret_cast<const double*>(s + 3 * kPtWideStride + 3 * kPtNarrowBytes);
  return p;
}

// head and conductivity of the cell at box position (r, x) of a stage (ff_cell<true> with a
// per-cell Ks field: K = Ks * kr, both split from their doubles)
__device__ __forceinline__ FfCell pt_cell(const PtStage& s, int r, int x) {
  const int q = r * kPtWideX + x;
  FfCell c;
  c.h = ff_from_double_nb(s.h[q]);
  c.kx = ff_cond(ff_from_double_nb(s.ks[q]), ff_from_double_nb(s.kr[q]));
  return c;
}

// levels a slab [kb, ke) stages: the level above it (its first face) and the level below it
// (its last face) when they exist
__device__ __forceinline__ void pt_levels(int kb, int ke, int nz, int* lo, int* hi) {
  *lo = kb > 0 ? kb - 1 : kb;
  *hi = ke < nz ? ke : ke - 1;
}

__global__ void __launch_bounds__(288, 3) k_pic_assemble_tma(
    ReArgs a, const __grid_constant__ PicTmaMaps m, float* __restrict__ dg,
    float* __restrict__ a0, float* __restrict__ a1, float* __restrict__ a2,
    double* __restrict__ bvec, int planes, int tiles, int* err, int stall_producer = 0) {
  extern __shared__ __align__(128) unsigned char pt_dyn[];
  // the stages start on a 128-byte boundary (the launch adds 128 bytes of slack)
  unsigned char* pt_smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(pt_dyn) + 127) & ~static_cast<uintptr_t>(127));
  __shared__ __align__(8) uint64_t full_bar[kPtStages];
  __shared__ __align__(8) uint64_t empty_bar[kPtStages];
  __shared__ FfConst K;
  __shared__ int abort_word;
  volatile int& abort_flag = abort_word;
  const int lane = threadIdx.x, row = threadIdx.y;
  const bool producer = row == 8;
  if (row == 0 && lane == 0) {
    K = ff_consts(a, a.sc->dt_used);
    abort_word = 0;
    for (int s = 0; s < kPtStages; ++s) {
      mbar_init(&full_bar[s], 1);   // the producer's arrive.expect_tx
      mbar_init(&empty_bar[s], 8);  // one arrival per consumer warp
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int t0 = (a.nx + 31) / 32;
  const int kb = blockIdx.y * planes, ke = min(a.nz, kb + planes);
  int lo, hi;
  pt_levels(kb, ke, a.nz, &lo, &hi);

  if (producer) {
    // ---- producer warp: lane 0 issues every level's copies in the consumers' order ----------
    // (stall_producer, the self-check of the bounded waits: nothing is issued, so the
    // consumers' first waits run out and the block finishes without reading a stage)
    if (lane == 0 && !stall_producer) {
      uint32_t seq = 0;
      for (int tile = blockIdx.x; tile < tiles && !abort_flag; tile += gridDim.x) {
        const int x0 = (tile % t0) * 32, y0 = (tile / t0) * 8;
        for (int L = lo; L <= hi; ++L, ++seq) {
          const int slot = seq % kPtStages;
          const uint32_t use = seq / kPtStages;
          if (!mbar_wait(&empty_bar[slot], (use & 1u) ^ 1u)) {
            abort_flag = 1;
            atomicExch(err, 1);
            break;
          }
          unsigned char* s = pt_smem + (size_t)slot * kPtStageBytes;
          mbar_arrive_tx(&full_bar[slot], kPtTxBytes);
          tma_load_3d(s, &m.h, x0 - 2, y0 - 1, L, &full_bar[slot]);
          tma_load_3d(s + kPtWideStride, &m.kr, x0 - 2, y0 - 1, L, &full_bar[slot]);
          tma_load_3d(s + 2 * kPtWideStride, &m.ks, x0 - 2, y0 - 1, L, &full_bar[slot]);
          unsigned char* nr = s + 3 * kPtWideStride;
          tma_load_3d(nr, &m.wo, x0, y0, L, &full_bar[slot]);
          tma_load_3d(nr + kPtNarrowBytes, &m.ho, x0, y0, L, &full_bar[slot]);
          tma_load_3d(nr + 2 * kPtNarrowBytes, &m.wch, x0, y0, L, &full_bar[slot]);
          tma_load_3d(nr + 3 * kPtNarrowBytes, &m.cap, x0, y0, L, &full_bar[slot]);
        }
      }
      if (abort_flag) {
        // copies still in flight land before the block's shared memory goes away: wait
        // (bounded) for the last use of every stage
        for (int q = 0; q < kPtStages; ++q) {
          if (seq < (uint32_t)(q + 1)) break;
          const uint32_t sq = seq - 1 - q;
          (void)mbar_wait(&full_bar[sq % kPtStages], (sq / kPtStages) & 1u);
        }
      }
    }
    return;
  }

  // ---- consumer warps: one cell per thread and level ---------------------------------------
  // Each level, every cell's head and conductivity are split into float-float once: a thread
  // writes its own cell into the level's plane (double-buffered), threads 0-63 the rows above
  // and below the tile and threads 64-79 the cells left and right of its rows, all from the
  // staged boxes; one barrier over the 256 consumer threads (named barrier 1, the producer does
  // not take part) makes the plane readable.  A plane is rewritten two levels later, after every
  // consumer has passed the barrier that follows its last read.
  __shared__ float ph[2][10][34], pl[2][10][34], pkh[2][10][34], pkl[2][10][34];
  const int hm = a.face_mean;
  const unsigned full = 0xffffffffu;
  const ff zero = ff_make(0.0f);
  const int tid = row * 32 + lane;
  uint32_t seq = 0;
  // wait until the stage of sequence number sq is full; false on abort (warp-uniform: every
  // lane of a warp takes the same branch afterwards)
  auto ready = [&](uint32_t sq) -> bool {
    bool ok = !abort_flag && mbar_wait(&full_bar[sq % kPtStages], (sq / kPtStages) & 1u);
    ok = __all_sync(full, ok);
    if (!ok && lane == 0) {
      abort_flag = 1;
      atomicExch(err, 2);
    }
    return ok;
  };
  auto release = [&](uint32_t sq) {
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty_bar[sq % kPtStages]);
  };
  auto put = [&](int b, int r, int x, const FfCell& v) {
    ph[b][r][x] = v.h.h;
    pl[b][r][x] = v.h.l;
    pkh[b][r][x] = v.kx.h;
    pkl[b][r][x] = v.kx.l;
  };
  auto get = [&](int b, int r, int x) -> FfCell {
    FfCell v;
    v.h = ff_make(ph[b][r][x], pl[b][r][x]);
    v.kx = ff_make(pkh[b][r][x], pkl[b][r][x]);
    return v;
  };
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int i = (tile % t0) * 32 + lane;
    const int j0 = (tile / t0) * 8, j = j0 + row;
    const bool act = i < a.nx && j < a.ny;
    const cidx col = act ? (cidx)i + (cidx)a.nx * j : 0u;
    const uint32_t seq0 = seq;  // sequence number of level lo
    seq += (uint32_t)(hi - lo + 1);
    const int bx = lane + 2, br = row + 1;  // this cell's position in the wide boxes
    FfCell cur = {zero, zero, zero, zero};
    ff fzm = zero;
    float tzm = 0.0f;
    // after a failed wait a warp keeps stepping through the levels (it still takes every
    // barrier, so no other warp waits on it) but reads and writes nothing
    bool live = ready(seq0 + (uint32_t)(kb - lo));
    {
      const uint32_t sk = seq0 + (uint32_t)(kb - lo);
      if (live) cur = pt_cell(pt_stage(pt_smem, sk % kPtStages), br, bx);
      if (kb > 0 && live && ready(seq0)) {  // the face above the slab, level kb - 1
        const FfCell up = pt_cell(pt_stage(pt_smem, seq0 % kPtStages), br, bx);
        const ff kf = ff_face_mean(hm, up.kx, cur.kx);
        fzm = ff_neg(ff_zface_flux(kf, K.cz, K.Az, cur.h, up.h, &tzm));
      }
      if (kb > 0) release(seq0);
      live = __all_sync(full, live && !abort_flag);
    }
    for (int k = kb; k < ke; ++k) {
      const uint32_t sk = seq0 + (uint32_t)(k - lo);
      const cidx c = col + (cidx)a.ncol * k;
      const bool has_below = k + 1 < a.nz;
      const int b = k & 1;
      // the class id for the residual's Ss / theta_s (direct load, issued before the waits)
      int cid = 0;
      if (live && act && a.soil.cid) cid = a.soil.cid[a.soil.cid3d ? c : col];
      const PtStage S = pt_stage(pt_smem, sk % kPtStages);
      // this level's plane: own cell, halo rows, halo columns
      if (live) {
        put(b, br, lane + 1, cur);
        if (tid < 64) {
          const int r = tid < 32 ? 0 : 9;
          put(b, r, lane + 1, pt_cell(S, r, bx));
        } else if (tid < 80) {
          const int r = 1 + ((tid - 64) >> 1), side = (tid - 64) & 1;
          put(b, r, side ? 33 : 0, pt_cell(S, r, side ? 34 : 1));
        }
      }
      if (live && has_below) live = ready(sk + 1);
      asm volatile("bar.sync 1, 256;" ::: "memory");
      if (!live) {
        release(sk);
        continue;
      }
      // +x face from the next lane's cell (lane 31 reads its neighbour from the plane)
      ff Kxn = ff_make(__shfl_down_sync(full, cur.kx.h, 1), __shfl_down_sync(full, cur.kx.l, 1));
      ff hxn = ff_make(__shfl_down_sync(full, cur.h.h, 1), __shfl_down_sync(full, cur.h.l, 1));
      float tx = 0.0f;
      ff fxp = zero;
      if (act && i + 1 < a.nx) {
        if (lane == 31) {
          const FfCell xn = get(b, br, 33);
          Kxn = xn.kx;
          hxn = xn.h;
        }
        fxp = ff_face_flux(ff_face_mean(hm, cur.kx, Kxn), K.cx, hxn, cur.h, &tx);
      }
      float txm = __shfl_up_sync(full, tx, 1);
      ff fxm = ff_neg(ff_make(__shfl_up_sync(full, fxp.h, 1), __shfl_up_sync(full, fxp.l, 1)));
      FfCell below = cur;
      if (act) {
        if (i == 0) {
          txm = 0.0f;
          fxm = zero;
        } else if (lane == 0) {
          const FfCell xm = get(b, br, 0);
          fxm = ff_face_flux(ff_face_mean(hm, xm.kx, cur.kx), K.cx, xm.h, cur.h, &txm);
        }
        FfSum q = ff_sum_of(fxm);
        ff_sum_add(q, fxp);
        float tsum = txm + tx;
        float ty = 0.0f;
        if (j > 0) {
          const FfCell yn = get(b, br - 1, lane + 1);
          float t;
          ff_sum_add(q, ff_face_flux(ff_face_mean(hm, yn.kx, cur.kx), K.cy, yn.h, cur.h, &t));
          tsum += t;
        }
        if (j + 1 < a.ny) {
          const FfCell yn = get(b, br + 1, lane + 1);
          ff_sum_add(q, ff_face_flux(ff_face_mean(hm, cur.kx, yn.kx), K.cy, yn.h, cur.h, &ty));
          tsum += ty;
        }
        const SoilClass& kc = a.soil.cls[cid];
        if (k > 0) {
          ff_sum_add(q, fzm);
          tsum += tzm;
        } else {
          ff f, t;
          ff_top_face(a, K, cur, kc, c, col, &f, &t);
          ff_sum_add(q, f);
          tsum += t.h;
        }
        float tz = 0.0f;
        if (has_below) {
          below = pt_cell(pt_stage(pt_smem, (sk + 1) % kPtStages), br, bx);
          const ff kf = ff_face_mean(hm, cur.kx, below.kx);
          const ff fz = ff_zface_flux(kf, K.cz, K.Az, below.h, cur.h, &tz);
          ff_sum_add(q, fz);
          tsum += tz;
          tzm = tz;
          fzm = ff_neg(fz);
        } else {
          ff f, t;
          ff_bottom_face<true>(a, K, cur, c, col, &f, &t);
          ff_sum_add(q, f);
          tsum += t.h;
        }
        const ff qv = ff_sum_value(q);
        const int nq = row * 32 + lane;  // this cell in the narrow boxes
        const double r_wo = S.wo[nq], r_ho = S.ho[nq];
        const ff wcn = ff_from_double_nb(r_wo);
        const ff st = ff_mul(ff_make(kc.ff_ss_ths[0], kc.ff_ss_ths[1]), wcn);  // Ss wcn / ths
        const float dtf = K.dt.h;
        dg[c] = fmaf(dtf, tsum, K.V.h * (ff_hi_of_nb(S.cap[nq]) + st.h));
        a0[c] = -dtf * tx;
        a1[c] = -dtf * ty;
        a2[c] = -dtf * tz;
        const double dth = S.wch[nq] - r_wo;
        bvec[c] = -fma(a.vol_cell, dth, ff_to_double_nb(ff_residual_rest(K.V, K.dt, st, cur.h,
                                                                         r_ho, qv)));
      } else if (has_below) {
        below = pt_cell(pt_stage(pt_smem, (sk + 1) % kPtStages), br, bx);
      }
      cur = below;
      release(sk);
    }
    if (ke < a.nz) release(seq0 + (uint32_t)(ke - lo));  // the level below the slab
  }
}

}  // namespace fg
