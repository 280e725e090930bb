// The U-Net's 3x3x3 convolutions on the fifth-generation tensor cores (tcgen05, accumulators in
// tensor memory).  Not in reference.
//
// Implicit GEMM per tile of 8 x 16 pixels (x, y) of one z plane: D[128 x COUT] (FP32, in TMEM;
// row r = 8 py + px) = sum over the 27 taps and the input channels of A[128 x 16] . B[16 x COUT],
// one tcgen05.mma.cta_group::1.kind::f16 (BF16 operands, FP32 accumulation, M = 128, N = COUT,
// K = 16) per tap and 16-channel slice.  Operands sit in shared memory in the no-swizzle
// K-major core-matrix layout, which the channels-last activations reach by splitting the
// channels into 8-channel chunks:
//   input patch [chunk][hy][hx][8]  (the 10 x 18 pixels x0-1 .. x0+8, y0-1 .. y0+16 of a plane,
//               zero outside the grid): a tap (dx, dy) is the view starting at pixel
//               (dx, dy); its M-adjacent core matrices (eight pixels of one patch row) are one
//               patch row (160 bytes) apart, its K-adjacent ones one chunk plane (2880 bytes);
//   weights     [tap][chunk][o][8]:  N-adjacent core matrices 128 bytes apart, K-adjacent ones
//               COUT x 16 bytes.
// Two-dimensional tiles stage 180 pixels per plane where a 128-pixel row tile needs three rows of
// 130, which leaves shared memory for more resident blocks and deeper copy pipelines.
// k_conv3_tc: a block (one warpgroup) walks its tiles; per z plane it loads the plane's patch and
// the nine taps' weights of that plane with 16-byte cp.async copies, one thread issues the plane's
// MMAs and commits them to an mbarrier, and the block waits for them before the next plane's
// copies reuse the buffers.  The four warps then read the accumulator lanes (tcgen05.ld 32x32b:
// warp w owns lanes 32w .. 32w+31 = rows), add the bias, apply the ReLU and store BF16.  Several
// blocks per SM (shared memory, tensor-memory columns permitting) overlap one block's copies with
// another's MMAs.
//
// Every wait is bounded: a wait that runs out records an error word and the block stops
// issuing work, waits (bounded) for its MMAs in flight, frees its tensor memory and returns.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

namespace fg {
namespace unet {

constexpr int kTcM = 128;                       // pixels per tile (the MMA's M)
constexpr int kTcTX = 8, kTcTY = 16;             // the tile: 8 x 16 pixels, row r = 8 py + px
constexpr int kTcHX = kTcTX + 2, kTcHY = kTcTY + 2;  // with the halo
constexpr int kTcHP = kTcHX * kTcHY;             // 180 staged pixels per plane
constexpr long kTcSpin = 1L << 24;

// tiles of an nx x ny plane
__host__ __device__ inline int tc_tiles_x(int nx) { return (nx + kTcTX - 1) / kTcTX; }
__host__ __device__ inline int tc_tiles_y(int ny) { return (ny + kTcTY - 1) / kTcTY; }

template <int CIN, int COUT>
struct TcShape {
  static_assert(CIN % 16 == 0 && COUT % 16 == 0 && COUT <= 128, "channel counts");
  static constexpr int CH = CIN / 8;
  static constexpr int PLANE = kTcHP * 16;             // one chunk plane of a patch
  static constexpr int ROWS = CH * PLANE;              // one z plane's patch
  static constexpr int WTS = 9 * CH * COUT * 16;       // the nine taps of one z plane
  static constexpr int SMEM = ROWS + WTS + 128;        // + alignment slack
  static constexpr int TMEM_COLS = COUT <= 32 ? 32 : (COUT <= 64 ? 64 : 128);
};

__device__ __forceinline__ uint32_t tc_smem(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: start, leading (K) and stride (M / N) byte offsets, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of the fifth-generation tensor cores
  return d;                // base offset 0, absolute leading offset, layout: no swizzle
}

// instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major, M = 128, N = n
__host__ __device__ constexpr uint32_t tc_idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(kTcM >> 4) << 24);
}

// 16-byte copy global -> shared with zero fill past `bytes`, through L1: a thread's chunks of one
// pixel share 32-byte sectors, which L1 then serves once
__device__ __forceinline__ void tc_cp16(void* dst, const void* src, int bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(tc_smem(dst)), "l"(src),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity) {
  for (long q = 0; q < kTcSpin; ++q) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(tc_smem(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// Copies of the patch of plane zz (pixels x0-1 .. x0+8, y0-1 .. y0+16) into dst,
// [chunk][hy][hx][8], with zero fill outside the grid: thread t copies patch pixel t (threads
// 0-51 also pixel 128 + t), every chunk, so the index arithmetic is per pixel, not per copy.
template <int CH>
__device__ __forceinline__ void tc_load_patch(unsigned char* dst, const __nv_bfloat16* in,
                                              int in_stride, int in_off, int x0, int y0, int zz,
                                              int nx, int ny, int nz, int tid) {
  const bool zok = zz >= 0 && zz < nz;
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    const int p = half ? kTcM + tid : tid;
    if (half && p >= kTcHP) break;
    const int xx = x0 + p % kTcHX - 1, yy = y0 + p / kTcHX - 1;
    const bool ok = zok && xx >= 0 && xx < nx && yy >= 0 && yy < ny;
    const __nv_bfloat16* src =
        ok ? in + ((size_t)xx + (size_t)nx * ((size_t)yy + (size_t)ny * zz)) * in_stride + in_off
           : in;
    unsigned char* d = dst + p * 16;
#pragma unroll
    for (int c = 0; c < CH; ++c) tc_cp16(d + c * kTcHP * 16, ok ? src + 8 * c : in, ok ? 16 : 0);
  }
}

// byte offset of tap (dx, dy)'s view and of 16-channel slice kc in a patch
template <int CH>
__host__ __device__ constexpr uint32_t tc_tap_offset(int dx, int dy, int kc) {
  return (uint32_t)(((2 * kc) * kTcHP + dy * kTcHX + dx) * 16);
}

// A descriptor advanced by a byte offset (a multiple of 16): the start address is the low
// 14-bit field in 16-byte units, and shared-memory addresses stay below 2^18 bytes, so the sum
// does not carry out of the field.
__device__ __forceinline__ uint64_t tc_desc_at(uint64_t d, uint32_t bytes) {
  return d + (uint64_t)(bytes >> 4);
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv3_tc(const __nv_bfloat16* __restrict__ in,
                                                  int in_stride, int in_off,
                                                  const __nv_bfloat16* __restrict__ W,
                                                  const float* __restrict__ bias,
                                                  __nv_bfloat16* __restrict__ out, int out_stride,
                                                  int out_off, int nx, int ny, int nz, int relu,
                                                  int* err) {
  using S = TcShape<CIN, COUT>;
  extern __shared__ __align__(128) unsigned char tc_dyn[];
  unsigned char* rows = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(tc_dyn) + 127) & ~static_cast<uintptr_t>(127));
  unsigned char* wts = rows + S::ROWS;
  __shared__ __align__(8) uint64_t mma_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_word;
  volatile int& abort_flag = abort_word;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     tc_smem(&tmem_slot)),
                 "r"(S::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&mma_bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_word = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const uint32_t rows_s = tc_smem(rows), wts_s = tc_smem(wts);
  constexpr uint32_t idesc = tc_idesc(COUT);
  uint32_t phase = 0;
  int pending = 0;  // MMAs committed and not yet waited for

  const int xt = tc_tiles_x(nx), yt = tc_tiles_y(ny);
  const long tiles = (long)xt * yt * nz;
  for (long tile = blockIdx.x; tile < tiles && !abort_flag; tile += gridDim.x) {
    const int x0 = (int)(tile % xt) * kTcTX;
    const long yz = tile / xt;
    const int y0 = (int)(yz % yt) * kTcTY, z = (int)(yz / yt);
    bool first = true;
    for (int dz = -1; dz <= 1 && !abort_flag; ++dz) {
      const int zz = z + dz;
      if (zz < 0 || zz >= nz) continue;  // zero padding: the plane adds nothing
      // the plane's patch, [chunk][hy][hx][8]
      tc_load_patch<S::CH>(rows, in, in_stride, in_off, x0, y0, zz, nx, ny, nz, tid);
      // the plane's nine taps of W[tap][o][i], [tap][chunk][o][8]
      for (int q = tid; q < 9 * S::CH * COUT; q += 128) {
        const int o = q % COUT, c = (q / COUT) % S::CH, t9 = q / (COUT * S::CH);
        const int tap = (dz + 1) * 9 + t9;
        tc_cp16(wts + ((t9 * S::CH + c) * COUT + o) * 16,
                W + ((size_t)tap * COUT + o) * CIN + 8 * c, 16);
      }
      asm volatile("cp.async.wait_all;" ::: "memory");
      // the copies are generic-proxy writes the tensor cores read through the async proxy
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (tid == 0) {
        const uint64_t a0 = tc_desc(rows_s, S::PLANE, kTcHX * 16);
        const uint64_t b0 = tc_desc(wts_s, COUT * 16, 128);
#pragma unroll
        for (int t9 = 0; t9 < 9; ++t9) {
          const int dy = t9 / 3, dx = t9 % 3;
#pragma unroll
          for (int kc = 0; kc < CIN / 16; ++kc) {
            const uint64_t a = tc_desc_at(a0, tc_tap_offset<S::CH>(dx, dy, kc));
            const uint64_t b = tc_desc_at(b0, (t9 * S::CH + 2 * kc) * COUT * 16);
            const uint32_t acc = first ? 0u : 1u;
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
                "l"(a), "l"(b), "r"(idesc), "r"(acc)
                : "memory");
            first = false;
          }
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                tc_smem(&mma_bar))
            : "memory");
      }
      first = false;
      pending = 1;
      // the plane's MMAs read the buffers the next plane's copies overwrite (the outcome of the
      // wait is made block-uniform, so every thread takes the same path)
      const bool late = __syncthreads_or(!tc_wait(&mma_bar, phase));
      if (late) {
        if (tid == 0) atomicExch(err, 1);
        abort_flag = 1;
        break;
      }
      pending = 0;
      phase ^= 1u;
    }
    if (abort_flag) break;
    // epilogue: warp w reads TMEM lanes 32w .. 32w+31 (its 32 pixels), 16 columns at a time
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int r = warp * 32 + lane, px = x0 + (r & 7), py = y0 + (r >> 3);
    __nv_bfloat16* dst =
        out + ((size_t)px + (size_t)nx * ((size_t)py + (size_t)ny * z)) * out_stride + out_off;
#pragma unroll
    for (int cb = 0; cb < COUT; cb += 16) {
      uint32_t r[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
          "%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
            "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
            "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cb));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      uint32_t packed[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        float v0 = __uint_as_float(r[2 * q]) + (bias ? bias[cb + 2 * q] : 0.f);
        float v1 = __uint_as_float(r[2 * q + 1]) + (bias ? bias[cb + 2 * q + 1] : 0.f);
        if (relu) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        __nv_bfloat162 h = __floats2bfloat162_rn(v0, v1);
        packed[q] = *reinterpret_cast<uint32_t*>(&h);
      }
      if (px < nx && py < ny) {
        uint4* d4 = reinterpret_cast<uint4*>(dst + cb);
        d4[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
        d4[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
      }
    }
  }
  // MMAs still in flight (a wait that ran out) finish before the tensor memory is freed
  if (pending) (void)tc_wait(&mma_bar, phase);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(S::TMEM_COLS)
                 : "memory");
}


// ---------------------------------------------------------------------------------------------
// Per-output-plane pipelined form, for the 16-channel-input layers: their patches and weights
// are small, and small tensor-memory accumulators (COUT columns, two of them) let six blocks
// share an SM, which beats the dz-stacked form below for them (2.0 against 2.6 ms per
// 16-to-16-channel layer at 768 x 768 x 96).  The 27 taps of weights stay resident in shared
// memory (27 x CIN x COUT x 2 bytes <= 64 KB).
// A block walks columns of ZC tiles along z at one (x, y) tile: a ring of four slots holds
// input planes (one patch each, [slot][chunk][hy][hx][8]); each tile needs one new plane,
// loaded one tile ahead with cp.async while the previous tile's MMAs run, and two tensor-memory
// accumulators let the epilogue of tile z-1 overlap the MMAs of tile z:
//   wait for plane z+1, barrier; issue MMA(z) -> acc[z&1], commit;
//   wait MMA(z-1); load plane z+2 into the slot of plane z-2 (free: MMA(z-1) was its last
//   reader); epilogue(z-1) from acc[(z-1)&1] while those copies land.
// The MMA issue is unrolled over the taps and channel slices with the descriptors advanced by
// constant offsets.
constexpr int kTcZC = 16;  // output planes of one z column

template <int CIN, int COUT>
struct TcPShape {
  static_assert(CIN % 16 == 0 && COUT % 16 == 0, "channel counts");
  static constexpr int CH = CIN / 8;
  static constexpr int PLANE = kTcHP * 16;
  static constexpr int SLOT = CH * PLANE;              // one input plane's patch
  static constexpr int WTS = 27 * CH * COUT * 16;      // all taps, [tap][chunk][o][8]
  static constexpr int SMEM = WTS + 4 * SLOT + 128;
  static constexpr int ACC_COLS = COUT <= 16 ? 16 : (COUT <= 32 ? 32 : 64);
  static constexpr int TMEM_COLS = 2 * ACC_COLS < 32 ? 32 : 2 * ACC_COLS;
  static constexpr bool FITS = WTS <= 64 * 1024 && COUT <= 64;
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv3_tcp(const __nv_bfloat16* __restrict__ in,
                                                   int in_stride, int in_off,
                                                   const __nv_bfloat16* __restrict__ W,
                                                   const float* __restrict__ bias,
                                                   __nv_bfloat16* __restrict__ out,
                                                   int out_stride, int out_off, int nx, int ny,
                                                   int nz, int relu, int* err) {
  using S = TcPShape<CIN, COUT>;
  extern __shared__ __align__(128) unsigned char tcp_dyn[];
  unsigned char* wts = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(tcp_dyn) + 127) & ~static_cast<uintptr_t>(127));
  unsigned char* ring = wts + S::WTS;
  __shared__ __align__(8) uint64_t mma_bar[2];
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     tc_smem(&tmem_slot)),
                 "r"(S::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&mma_bar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&mma_bar[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // all 27 taps of the weights, once per block
  for (int q = tid; q < 27 * S::CH * COUT; q += 128) {
    const int o = q % COUT, c = (q / COUT) % S::CH, tap = q / (COUT * S::CH);
    tc_cp16(wts + ((tap * S::CH + c) * COUT + o) * 16, W + ((size_t)tap * COUT + o) * CIN + 8 * c,
            16);
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const uint32_t wts_s = tc_smem(wts), ring_s = tc_smem(ring);
  constexpr uint32_t idesc = tc_idesc(COUT);
  uint32_t phase[2] = {0u, 0u};
  int outstanding[2] = {0, 0};  // MMAs committed to mma_bar[b] and not yet waited for
  bool failed = false;

  // copies of input plane zz's patch into ring slot zz & 3, zero outside the grid
  auto load_plane = [&](int x0, int y0, int zz) {
    tc_load_patch<S::CH>(ring + (zz & 3) * S::SLOT, in, in_stride, in_off, x0, y0, zz, nx, ny, nz,
                         tid);
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  // bias + ReLU + BF16 store of tile (x0, y0, z) from accumulator b
  auto epilogue = [&](int x0, int y0, int z, int b) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int r = warp * 32 + lane, px = x0 + (r & 7), py = y0 + (r >> 3);
    __nv_bfloat16* dst =
        out + ((size_t)px + (size_t)nx * ((size_t)py + (size_t)ny * z)) * out_stride + out_off;
#pragma unroll
    for (int cb = 0; cb < COUT; cb += 16) {
      uint32_t r[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
          "%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
            "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
            "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(b * S::ACC_COLS + cb)));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      uint32_t packed[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        float v0 = __uint_as_float(r[2 * q]) + (bias ? bias[cb + 2 * q] : 0.f);
        float v1 = __uint_as_float(r[2 * q + 1]) + (bias ? bias[cb + 2 * q + 1] : 0.f);
        if (relu) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        __nv_bfloat162 h = __floats2bfloat162_rn(v0, v1);
        packed[q] = *reinterpret_cast<uint32_t*>(&h);
      }
      if (px < nx && py < ny) {
        uint4* d4 = reinterpret_cast<uint4*>(dst + cb);
        d4[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
        d4[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  };
  // block-uniform bounded wait for the MMAs committed to mma_bar[b]
  auto wait_mma = [&](int b) -> bool {
    const bool late = __syncthreads_or(!tc_wait(&mma_bar[b], phase[b]));
    if (late) {
      if (tid == 0) atomicExch(err, 2);
      return false;
    }
    phase[b] ^= 1u;
    outstanding[b] = 0;
    return true;
  };

  const int xt = tc_tiles_x(nx), yt = tc_tiles_y(ny);
  const int zcols = (nz + kTcZC - 1) / kTcZC;
  const long items = (long)xt * yt * zcols;
  for (long item = blockIdx.x; item < items && !failed; item += gridDim.x) {
    const int x0 = (int)(item % xt) * kTcTX;
    const long rest = item / xt;
    const int y0 = (int)(rest % yt) * kTcTY;
    const int zb = (int)(rest / yt) * kTcZC, ze = min(nz, zb + kTcZC);
    load_plane(x0, y0, zb - 1);
    load_plane(x0, y0, zb);
    load_plane(x0, y0, zb + 1);
    for (int z = zb; z < ze; ++z) {
      const int b = z & 1;
      // planes z-1, z, z+1 (and, the first time, the weights) have landed
      asm volatile("cp.async.wait_all;" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (tid == 0) {
        bool first = true;
        const uint64_t b0 = tc_desc(wts_s, COUT * 16, 128);
        const uint32_t d_tmem = tmem + (uint32_t)(b * S::ACC_COLS);
#pragma unroll
        for (int dz = 0; dz < 3; ++dz) {
          const int zz = z + dz - 1;
          if (zz < 0 || zz >= nz) continue;  // zero padding
          const uint64_t a0 =
              tc_desc(ring_s + (uint32_t)((zz & 3) * S::SLOT), S::PLANE, kTcHX * 16);
#pragma unroll
          for (int t9 = 0; t9 < 9; ++t9) {
            const int dy = t9 / 3, dx = t9 % 3, t = dz * 9 + t9;
#pragma unroll
            for (int kc = 0; kc < CIN / 16; ++kc) {
              const uint64_t a = tc_desc_at(a0, tc_tap_offset<S::CH>(dx, dy, kc));
              const uint64_t bd = tc_desc_at(b0, (t * S::CH + 2 * kc) * COUT * 16);
              const uint32_t acc = first ? 0u : 1u;
              asm volatile(
                  "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                  " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
                  "l"(a), "l"(bd), "r"(idesc), "r"(acc)
                  : "memory");
              first = false;
            }
          }
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                tc_smem(&mma_bar[b]))
            : "memory");
      }
      outstanding[b] = 1;
      if (z > zb) {  // the previous tile: its MMAs were the last readers of plane z-2's slot
        if (!wait_mma(b ^ 1)) {
          failed = true;
          break;
        }
        // the next plane's copies first, so that they run during the epilogue
        if (z + 1 < ze) load_plane(x0, y0, z + 2);
        epilogue(x0, y0, z - 1, b ^ 1);
      } else if (z + 1 < ze) {
        load_plane(x0, y0, z + 2);
      }
    }
    if (failed) break;
    if (!wait_mma((ze - 1) & 1)) {
      failed = true;
      break;
    }
    epilogue(x0, y0, ze - 1, (ze - 1) & 1);
    __syncthreads();  // the next column's first copies reuse slots the last epilogue's MMAs read
  }
  // MMAs still in flight after a wait that ran out finish before the tensor memory is freed
  for (int b = 0; b < 2; ++b)
    if (outstanding[b]) (void)tc_wait(&mma_bar[b], phase[b]);
  asm volatile("cp.async.wait_all;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(S::TMEM_COLS)
                 : "memory");
}

// ---------------------------------------------------------------------------------------------
// dz-stacked pipelined form, for the layers with 32 or more input channels whose 27 taps of
// weights stay resident in shared memory (27 x CIN x COUT x 2 bytes <= 64 KB).  The three dz
// taps are stacked along N: the weights sit as [t9][chunk][rb * COUT + o][8] with
// row block rb = 2 - dz, so one group of MMAs per INPUT plane z' (9 taps x CIN/16 slices, N =
// 3 COUT) adds W(dz=2) In(z') to out(z'-1), W(1) In(z') to out(z') and W(0) In(z') to out(z'+1)
// at once: a third of the MMAs of one group per output plane over the three input planes, and
// each input patch is read by one group only.  The accumulators of a column of ZC output planes
// and of the planes on either side lie side by side in tensor memory (COUT columns each, zeroed
// when the column starts); the input planes just outside the column add their one relevant
// third (N = COUT).
// A block walks columns of ZC output planes along z at one (x, y) tile with a ring of three
// input patches; per input plane z' of the column (zb-1 .. ze):
//   wait for plane z' (copied two planes ahead), barrier; issue MMAs(z'), commit;
//   wait MMAs(z'-1), the last reader of plane z'-1's slot: copy plane z'+2 into it, then the
//   epilogue of out(z'-2), complete with MMAs(z'-1), while MMAs(z') run.
// The MMA issue is unrolled over the taps and channel slices with the descriptors advanced by
// constant offsets.
template <int CIN, int COUT>
struct TcZShape {
  static_assert(CIN % 16 == 0 && COUT % 16 == 0, "channel counts");
  static constexpr int CH = CIN / 8;
  static constexpr int N3 = 3 * COUT;                  // the stacked N
  static constexpr int PLANE = kTcHP * 16;
  static constexpr int SLOT = CH * PLANE;              // one input plane's patch
  static constexpr int WTS = 9 * CH * N3 * 16;         // all taps, [t9][chunk][rb COUT + o][8]
  static constexpr int SMEM = WTS + 3 * SLOT + 128;
  static constexpr int TMEM_COLS = 256;
  static constexpr int ZC = TMEM_COLS / COUT - 2;      // output planes per z column
  static constexpr bool FITS = WTS <= 64 * 1024 && N3 <= 256;
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv3_tcz(const __nv_bfloat16* __restrict__ in,
                                                   int in_stride, int in_off,
                                                   const __nv_bfloat16* __restrict__ W,
                                                   const float* __restrict__ bias,
                                                   __nv_bfloat16* __restrict__ out,
                                                   int out_stride, int out_off, int nx, int ny,
                                                   int nz, int relu, int* err) {
  using S = TcZShape<CIN, COUT>;
  extern __shared__ __align__(128) unsigned char tcz_dyn[];
  unsigned char* wts = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(tcz_dyn) + 127) & ~static_cast<uintptr_t>(127));
  unsigned char* ring = wts + S::WTS;
  __shared__ __align__(8) uint64_t mma_bar[2];
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     tc_smem(&tmem_slot)),
                 "r"(S::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&mma_bar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&mma_bar[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // all 27 taps of the weights, once per block, the dz taps stacked along N
  for (int q = tid; q < 9 * S::CH * S::N3; q += 128) {
    const int orow = q % S::N3, c = (q / S::N3) % S::CH, t9 = q / (S::N3 * S::CH);
    const int rb = orow / COUT, o = orow % COUT, tap = (2 - rb) * 9 + t9;
    tc_cp16(wts + ((t9 * S::CH + c) * S::N3 + orow) * 16,
            W + ((size_t)tap * COUT + o) * CIN + 8 * c, 16);
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
  const uint32_t wts_s = tc_smem(wts), ring_s = tc_smem(ring);
  constexpr uint32_t idesc3 = tc_idesc(S::N3), idesc1 = tc_idesc(COUT);
  uint32_t phase[2] = {0u, 0u};
  int outstanding[2] = {0, 0};  // MMAs committed to mma_bar[b] and not yet waited for
  bool failed = false;

  // copies of input plane zz's patch into ring slot (zz + 3) % 3, zero outside the grid; a
  // commit group every call (empty past the column), so each wait leaves exactly one pending
  auto load_plane = [&](int x0, int y0, int zz, bool copy) {
    if (copy)
      tc_load_patch<S::CH>(ring + ((zz + 3) % 3) * S::SLOT, in, in_stride, in_off, x0, y0, zz,
                           nx, ny, nz, tid);
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  // bias + ReLU + BF16 store of tile (x0, y0, z) from its accumulator (column col)
  auto epilogue = [&](int x0, int y0, int z, uint32_t col) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int r = warp * 32 + lane, px = x0 + (r & 7), py = y0 + (r >> 3);
    __nv_bfloat16* dst =
        out + ((size_t)px + (size_t)nx * ((size_t)py + (size_t)ny * z)) * out_stride + out_off;
#pragma unroll
    for (int cb = 0; cb < COUT; cb += 16) {
      uint32_t v[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
          "%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
            "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
            "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(lane_base + col + (uint32_t)cb));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      uint32_t packed[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        float v0 = __uint_as_float(v[2 * q]) + (bias ? bias[cb + 2 * q] : 0.f);
        float v1 = __uint_as_float(v[2 * q + 1]) + (bias ? bias[cb + 2 * q + 1] : 0.f);
        if (relu) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        __nv_bfloat162 h = __floats2bfloat162_rn(v0, v1);
        packed[q] = *reinterpret_cast<uint32_t*>(&h);
      }
      if (px < nx && py < ny) {
        uint4* d4 = reinterpret_cast<uint4*>(dst + cb);
        d4[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
        d4[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  };
  // block-uniform bounded wait for the MMAs committed to mma_bar[b]
  auto wait_mma = [&](int b) -> bool {
    const bool late = __syncthreads_or(!tc_wait(&mma_bar[b], phase[b]));
    if (late) {
      if (tid == 0) atomicExch(err, 2);
      return false;
    }
    phase[b] ^= 1u;
    outstanding[b] = 0;
    return true;
  };

  const int xt = tc_tiles_x(nx), yt = tc_tiles_y(ny);
  const int zcols = (nz + S::ZC - 1) / S::ZC;
  const long items = (long)xt * yt * zcols;
  for (long item = blockIdx.x; item < items && !failed; item += gridDim.x) {
    const int x0 = (int)(item % xt) * kTcTX;
    const long rest = item / xt;
    const int y0 = (int)(rest % yt) * kTcTY;
    const int zb = (int)(rest / yt) * S::ZC, ze = min(nz, zb + S::ZC);
    // accumulator of output plane z (zb-1 .. ze) at column (z - zb + 1) COUT
    auto col = [&](int z) { return (uint32_t)((z - zb + 1) * COUT); };
    // zero the column's accumulators (the previous column's epilogues have read theirs)
    {
      const uint32_t zero[16] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
      for (int c0 = 0; c0 < (ze - zb + 2) * COUT; c0 += 16)
        asm volatile(
            "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
            "%13,%14,%15,%16};" ::"r"(lane_base + (uint32_t)c0),
            "r"(zero[0]), "r"(zero[1]), "r"(zero[2]), "r"(zero[3]), "r"(zero[4]), "r"(zero[5]),
            "r"(zero[6]), "r"(zero[7]), "r"(zero[8]), "r"(zero[9]), "r"(zero[10]),
            "r"(zero[11]), "r"(zero[12]), "r"(zero[13]), "r"(zero[14]), "r"(zero[15])
            : "memory");
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    load_plane(x0, y0, zb - 1, true);
    load_plane(x0, y0, zb, true);
    for (int zp = zb - 1; zp <= ze; ++zp) {
      const int b = (zp + 1) & 1;
      // plane zp (and, the first time, the weights) has landed; plane zp+1 may be in flight
      asm volatile("cp.async.wait_group 1;" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (tid == 0) {
        if (zp >= 0 && zp < nz) {  // zero padding outside the grid adds nothing
          // the stacked row blocks this plane adds: rb = 2 - dz adds to out(zp - 1 + rb)
          const int rb0 = zp < zb ? 2 : 0, rbn = (zp < zb || zp >= ze) ? 1 : 3;
          const uint64_t a0 =
              tc_desc(ring_s + (uint32_t)(((zp + 3) % 3) * S::SLOT), S::PLANE, kTcHX * 16);
          const uint64_t b0 = tc_desc(wts_s + (uint32_t)(rb0 * COUT * 16), S::N3 * 16, 128);
          const uint32_t d_tmem = tmem + col(zp - 1 + rb0);
          const uint32_t idesc = rbn == 3 ? idesc3 : idesc1;
#pragma unroll
          for (int t9 = 0; t9 < 9; ++t9) {
            const int dy = t9 / 3, dx = t9 % 3;
#pragma unroll
            for (int kc = 0; kc < CIN / 16; ++kc) {
              const uint64_t a = tc_desc_at(a0, tc_tap_offset<S::CH>(dx, dy, kc));
              const uint64_t bd = tc_desc_at(b0, (t9 * S::CH + 2 * kc) * S::N3 * 16);
              asm volatile(
                  "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                  " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
                  "l"(a), "l"(bd), "r"(idesc), "r"(1u)
                  : "memory");
            }
          }
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                tc_smem(&mma_bar[b]))
            : "memory");
      }
      outstanding[b] = 1;
      if (zp > zb - 1) {  // MMAs(zp-1) were the last readers of plane zp-1's slot
        if (!wait_mma(b ^ 1)) {
          failed = true;
          break;
        }
        load_plane(x0, y0, zp + 2, zp + 2 <= ze);
        if (zp - 2 >= zb) epilogue(x0, y0, zp - 2, col(zp - 2));
      } else {
        load_plane(x0, y0, zp + 2, zp + 2 <= ze);
      }
    }
    if (failed) break;
    if (!wait_mma((ze + 1) & 1)) {  // MMAs(ze)
      failed = true;
      break;
    }
    epilogue(x0, y0, ze - 1, col(ze - 1));
    // the next column zeroes accumulators and overwrites slots this column's last reads used
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
  }
  // MMAs still in flight after a wait that ran out finish before the tensor memory is freed
  for (int b = 0; b < 2; ++b)
    if (outstanding[b]) (void)tc_wait(&mma_bar[b], phase[b]);
  asm volatile("cp.async.wait_all;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(S::TMEM_COLS)
                 : "memory");
}

}  // namespace unet
}  // namespace fg
