// Learned preconditioner (not in reference): a 3-level 3D U-Net, BF16 activations and weights
// on the tensor cores with FP32 accumulation, with its own forward, backward and Adam kernels.
//
// Architecture (channels 16 / 32 / 64, 3x3x3 convolutions, ReLU, 2x2x2 average pooling,
// nearest 2x upsampling, skip connections by channel concatenation):
//   x0  (r~, ln K, C, zero padding: 16 ch)            level 1 (full grid)
//   e1 = relu(c1b(relu(c1a(x0))))                     16 -> 16 -> 16
//   e2 = relu(c2b(relu(c2a(pool(e1)))))               level 2: 16 -> 32 -> 32
//   e3 = relu(c3b(relu(c3a(pool(e2)))))               level 3: 32 -> 64 -> 64
//   d2 = relu(d2b(relu(d2a([up(e3) | e2]))))          level 2: 96 -> 32 -> 32
//   d1 = relu(d1b(relu(d1a([up(d2) | e1]))))          level 1: 48 -> 16 -> 16
//   y  = w_o . d1 + b_o                               1x1 output, FP32
// 354,145 trained parameters: 353,808 weights (1,296 + 6,912 + 13,824 + 27,648 + 55,296 +
// 110,592 + 82,944 + 27,648 + 20,736 + 6,912, with 3 live input channels in c1a), 320 biases and
// the 17 of the output layer.
//
// Layout: activations channels-last, BF16, pixel p = x + nx (y + ny z); a layer may read or
// write a channel slice of a wider buffer (the concatenations).  Convolutions are implicit GEMMs
// (M = 16 pixels of an x-row per warp, N = output channels, K = 27 taps x input channels) on
// mma.sync.m16n8k16 BF16 -> FP32; the data gradient is the same kernel with the weights
// mirrored in space and transposed in channels; weight gradients accumulate in FP32.
#include "internal.h"
#include "reduce.cuh"

#include <cuda_bf16.h>

#include "unet_tc.cuh"

#include <cmath>
#include <algorithm>
#include <cstring>
#include <vector>

namespace fg {
namespace unet {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ uint32_t ld32(const bf16* p) {
  return __ldg(reinterpret_cast<const unsigned int*>(p));
}
__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// out[p][o] = act( sum_{t,i} in[p + off(t)][i] * W[t][o][i] + b[o] ), zero padding.
// Block = 4 warps = 4 consecutive y rows of 16 x pixels at one z.
template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv3(const bf16* __restrict__ in, int in_stride,
                                               int in_off, const bf16* __restrict__ W,
                                               const float* __restrict__ bias,
                                               bf16* __restrict__ out, int out_stride,
                                               int out_off, int nx, int ny, int nz, int relu) {
  static_assert(CIN % 16 == 0 && COUT % 8 == 0, "channel counts");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t4 = lane & 3;
  const int x0 = blockIdx.x * 16;
  const int y = blockIdx.y * 4 + warp;
  const int z = blockIdx.z;
  if (y >= ny) return;
  float acc[COUT / 8][4];
#pragma unroll
  for (int q = 0; q < COUT / 8; ++q) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.f;
  for (int dz = -1; dz <= 1; ++dz) {
    const int zz = z + dz;
    if (zz < 0 || zz >= nz) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int yy = y + dy;
      if (yy < 0 || yy >= ny) continue;
      const size_t rowbase = (size_t)nx * ((size_t)yy + (size_t)ny * zz);
#pragma unroll
      for (int dx = -1; dx <= 1; ++dx) {
        const int tap = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1);
        const int xa = x0 + g + dx, xb = xa + 8;
        const bool oka = xa >= 0 && xa < nx, okb = xb >= 0 && xb < nx;
        const size_t ia = (rowbase + (size_t)(oka ? xa : 0)) * in_stride + in_off + 2 * t4;
        const size_t ib = (rowbase + (size_t)(okb ? xb : 0)) * in_stride + in_off + 2 * t4;
        const bf16* wb = W + ((size_t)tap * COUT + g) * CIN + 2 * t4;
#pragma unroll
        for (int kc = 0; kc < CIN / 16; ++kc) {
          uint32_t a[4];
          a[0] = oka ? ld32(in + ia + kc * 16) : 0u;
          a[1] = okb ? ld32(in + ib + kc * 16) : 0u;
          a[2] = oka ? ld32(in + ia + kc * 16 + 8) : 0u;
          a[3] = okb ? ld32(in + ib + kc * 16 + 8) : 0u;
#pragma unroll
          for (int nt = 0; nt < COUT / 8; ++nt) {
            const bf16* w = wb + (size_t)nt * 8 * CIN + kc * 16;
            mma_bf16(acc[nt], a, ld32(w), ld32(w + 8));
          }
        }
      }
    }
  }
  const size_t orow = (size_t)nx * ((size_t)y + (size_t)ny * z);
  const int xa = x0 + g, xb = xa + 8;
#pragma unroll
  for (int nt = 0; nt < COUT / 8; ++nt) {
    const int o = nt * 8 + 2 * t4;
    const float b0 = bias ? bias[o] : 0.f, b1 = bias ? bias[o + 1] : 0.f;
    float v0 = acc[nt][0] + b0, v1 = acc[nt][1] + b1, v2 = acc[nt][2] + b0, v3 = acc[nt][3] + b1;
    if (relu) {
      v0 = fmaxf(v0, 0.f);
      v1 = fmaxf(v1, 0.f);
      v2 = fmaxf(v2, 0.f);
      v3 = fmaxf(v3, 0.f);
    }
    if (xa < nx)
      *reinterpret_cast<uint32_t*>(out + (orow + xa) * out_stride + out_off + o) = pack2(v0, v1);
    if (xb < nx)
      *reinterpret_cast<uint32_t*>(out + (orow + xb) * out_stride + out_off + o) = pack2(v2, v3);
  }
}

// dW[t][o][i] += sum_p g[p][o] * in[p + off(t)][i]  (FP32; one tap per block row)
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_conv3_dw(const bf16* __restrict__ in, int in_stride,
                                                  int in_off, const bf16* __restrict__ gout,
                                                  int g_stride, int g_off, float* __restrict__ dW,
                                                  int nx, int ny, int nz, size_t chunk) {
  constexpr int TP = 32;
  __shared__ float gs[TP][COUT];
  __shared__ float is[TP][CIN];
  const int tap = blockIdx.x;
  const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
  const size_t n = (size_t)nx * ny * nz;
  const size_t p0 = blockIdx.y * chunk, p1 = min(n, p0 + chunk);
  constexpr int NOUT = COUT * CIN;
  constexpr int PER = (NOUT + 255) / 256;
  float acc[PER];
#pragma unroll
  for (int q = 0; q < PER; ++q) acc[q] = 0.f;
  for (size_t pt = p0; pt < p1; pt += TP) {
    for (int e = threadIdx.x; e < TP * COUT; e += 256) {
      const int pp = e / COUT, o = e % COUT;
      const size_t p = pt + pp;
      gs[pp][o] = p < p1 ? __bfloat162float(gout[p * g_stride + g_off + o]) : 0.f;
    }
    for (int e = threadIdx.x; e < TP * CIN; e += 256) {
      const int pp = e / CIN, i = e % CIN;
      const size_t p = pt + pp;
      float v = 0.f;
      if (p < p1) {
        const int x = (int)(p % nx), y = (int)((p / nx) % ny), z = (int)(p / ((size_t)nx * ny));
        const int xx = x + dx, yy = y + dy, zz = z + dz;
        if (xx >= 0 && xx < nx && yy >= 0 && yy < ny && zz >= 0 && zz < nz)
          v = __bfloat162float(in[((size_t)xx + (size_t)nx * ((size_t)yy + (size_t)ny * zz)) *
                                      in_stride + in_off + i]);
      }
      is[pp][i] = v;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int e = threadIdx.x + q * 256;
      if (e < NOUT) {
        const int o = e / CIN, i = e % CIN;
        float s = acc[q];
#pragma unroll 8
        for (int pp = 0; pp < TP; ++pp) s = fmaf(gs[pp][o], is[pp][i], s);
        acc[q] = s;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int e = threadIdx.x + q * 256;
    if (e < NOUT) atomicAdd(&dW[(size_t)tap * NOUT + e], acc[q]);
  }
}

// db[o] += sum_p g[p][o]
__global__ void k_bias_grad(const bf16* __restrict__ g, int g_stride, int g_off, int cout,
                            size_t n, float* __restrict__ db) {
  __shared__ float s[64];
  if (threadIdx.x < 64) s[threadIdx.x] = 0.f;
  __syncthreads();
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n;
       p += (size_t)gridDim.x * blockDim.x)
    for (int o = 0; o < cout; ++o) atomicAdd(&s[o], __bfloat162float(g[p * g_stride + g_off + o]));
  __syncthreads();
  if (threadIdx.x < cout) atomicAdd(&db[threadIdx.x], s[threadIdx.x]);
}

// grad *= (act > 0)
__global__ void k_relu_bwd(bf16* __restrict__ g, int g_stride, int g_off,
                           const bf16* __restrict__ act, int a_stride, int a_off, int c, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n * c;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t p = e / c;
    const int ch = (int)(e % c);
    if (!(__bfloat162float(act[p * a_stride + a_off + ch]) > 0.f))
      g[p * g_stride + g_off + ch] = __float2bfloat16(0.f);
  }
}

// 2x2x2 average pooling: out (coarse, stride C) from a channel slice of in (fine)
// 2x2x2 mean pooling of a channel slice: one thread per coarse cell and group of 8 channels
// (16-byte loads of the eight children, one 16-byte store); c, in_stride and in_off are
// multiples of 8, and the network's cell counts stay below 2^32
__global__ void k_pool(const bf16* __restrict__ in, int in_stride, int in_off, bf16* __restrict__ out,
                       int c, int nx, int ny, int nz) {
  const uint32_t cx = nx / 2, cy = ny / 2, cz = nz / 2;
  const uint32_t g = (uint32_t)c / 8;
  const uint64_t tot = (uint64_t)cx * cy * cz * g;
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < tot;
       e += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t q = (uint32_t)(e / g), cg = (uint32_t)(e - (uint64_t)q * g);
    const uint32_t x = q % cx, yz = q / cx, y = yz % cy, z = yz / cy;
    float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const uint32_t p = (2 * x + (k & 1)) + (uint32_t)nx * ((2 * y + ((k >> 1) & 1)) +
                                                             (uint32_t)ny * (2 * z + (k >> 2)));
      const uint4 v = *reinterpret_cast<const uint4*>(in + (size_t)p * in_stride + in_off + 8 * cg);
      const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float2 f = __bfloat1622float2(h[u]);
        s[2 * u] += f.x;
        s[2 * u + 1] += f.y;
      }
    }
    uint4 o;
    uint32_t* ow = reinterpret_cast<uint32_t*>(&o);
#pragma unroll
    for (int u = 0; u < 4; ++u) ow[u] = pack2(0.125f * s[2 * u], 0.125f * s[2 * u + 1]);
    *reinterpret_cast<uint4*>(out + (size_t)q * c + 8 * cg) = o;
  }
}

// gradient of pooling, added to an existing gradient slice: gin[p] += gout[pool(p)] / 8
__global__ void k_pool_bwd_add(const bf16* __restrict__ gout, bf16* __restrict__ gin,
                               int gin_stride, int gin_off, int c, int nx, int ny, int nz) {
  const size_t n = (size_t)nx * ny * nz;
  const int cx = nx / 2, cy = ny / 2;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n * c;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t p = e / c;
    const int ch = (int)(e % c);
    const int x = (int)(p % nx), y = (int)((p / nx) % ny), z = (int)(p / ((size_t)nx * ny));
    const size_t q = (size_t)(x / 2) + (size_t)cx * ((size_t)(y / 2) + (size_t)cy * (z / 2));
    bf16* d = gin + p * gin_stride + gin_off + ch;
    *d = __float2bfloat16(__bfloat162float(*d) + 0.125f * __bfloat162float(gout[q * c + ch]));
  }
}

// nearest 2x upsampling of a coarse field (stride c) into a channel slice of a fine buffer
__global__ void k_up(const bf16* __restrict__ in, bf16* __restrict__ out, int out_stride,
                     int out_off, int c, int nx, int ny, int nz) {
  // one thread per fine cell and group of 8 channels (16-byte copies); c, out_stride and
  // out_off are multiples of 8.  Cell counts of the network's grids stay below 2^32.
  const uint32_t n = (uint32_t)nx * ny * nz;
  const uint32_t g = (uint32_t)c / 8;
  const uint32_t cx = nx / 2, cy = ny / 2;
  const uint64_t tot = (uint64_t)n * g;
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < tot;
       e += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t p = (uint32_t)(e / g), cg = (uint32_t)(e - (uint64_t)p * g);
    const uint32_t x = p % nx, yz = p / nx, y = yz % ny, z = yz / ny;
    const uint32_t q = (x >> 1) + cx * ((y >> 1) + cy * (z >> 1));
    const uint4 v = *reinterpret_cast<const uint4*>(in + (size_t)q * c + 8 * cg);
    *reinterpret_cast<uint4*>(out + (size_t)p * out_stride + out_off + 8 * cg) = v;
  }
}

// gradient of upsampling: gin[q] = sum of the 8 children of a fine gradient slice
__global__ void k_up_bwd(const bf16* __restrict__ gout, int g_stride, int g_off,
                         bf16* __restrict__ gin, int c, int nx, int ny, int nz) {
  const int cx = nx / 2, cy = ny / 2, cz = nz / 2;
  const size_t nc = (size_t)cx * cy * cz;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nc * c;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t q = e / c;
    const int ch = (int)(e % c);
    const int x = (int)(q % cx), y = (int)((q / cx) % cy), z = (int)(q / ((size_t)cx * cy));
    float s = 0.f;
    for (int k = 0; k < 8; ++k) {
      const size_t p = (size_t)(2 * x + (k & 1)) + (size_t)nx * ((size_t)(2 * y + ((k >> 1) & 1)) +
                                                                   (size_t)ny * (2 * z + (k >> 2)));
      s += __bfloat162float(gout[p * g_stride + g_off + ch]);
    }
    gin[q * c + ch] = __float2bfloat16(s);
  }
}

// network input: [r * rscale, (lnK - mean) * kscale, cap * cscale, 0 ...] in 16 channels
__global__ void k_pack_input(const float* __restrict__ r, const float* __restrict__ lnk,
                             const float* __restrict__ cap, const float* __restrict__ rscale,
                             float kmean, float kscale, float cscale, bf16* __restrict__ x,
                             size_t n) {
  const float rs = *rscale;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n;
       p += (size_t)gridDim.x * blockDim.x) {
    uint4* o = reinterpret_cast<uint4*>(x + p * 16);  // two 16-byte stores per cell
    o[0] = make_uint4(pack2(r[p] * rs, (lnk[p] - kmean) * kscale), pack2(cap[p] * cscale, 0.f),
                      0u, 0u);
    o[1] = make_uint4(0u, 0u, 0u, 0u);
  }
}

// 1 / rms of r (zero -> 1) in two deterministic passes: per-block partial sums of r^2, then one
// block adds the partials in a fixed order.
constexpr int kRmsBlocks = 1024;
__global__ void k_rms_partial(const float* __restrict__ r, size_t n, double* __restrict__ part) {
  double s = 0.0;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n;
       p += (size_t)gridDim.x * blockDim.x)
    s += (double)r[p] * r[p];
  __shared__ double sh[32];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sh[q];
    part[blockIdx.x] = t;
  }
}

__global__ void k_rms_scale(const double* __restrict__ part, int nparts, size_t n,
                            float* __restrict__ scale, float* __restrict__ inv) {
  double s = 0.0;
  for (int q = threadIdx.x; q < nparts; q += blockDim.x) s += part[q];
  __shared__ double sh[32];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sh[q];
    const double rms = sqrt(t / (double)n);
    *scale = rms > 0.0 ? (float)(1.0 / rms) : 1.0f;
    *inv = rms > 0.0 ? (float)rms : 1.0f;
  }
}

// y[p] = (w_o . d1[p] + b_o) * outscale
__global__ void k_out(const bf16* __restrict__ d1, const float* __restrict__ wo,
                      const float* __restrict__ outscale, float* __restrict__ y, size_t n) {
  const float s = outscale ? *outscale : 1.0f;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n;
       p += (size_t)gridDim.x * blockDim.x) {
    float v = wo[16];
    const uint4* dv = reinterpret_cast<const uint4*>(d1 + p * 16);  // two 16-byte loads
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const uint4 w = dv[half];
      const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&w);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float2 f = __bfloat1622float2(h[u]);
        v = fmaf(wo[8 * half + 2 * u], f.x, v);
        v = fmaf(wo[8 * half + 2 * u + 1], f.y, v);
      }
    }
    y[p] = v * s;
  }
}

// loss = mean((y - t)^2); gy = 2 (y - t) / n; plus the output-layer gradients and dL/dd1
__global__ void k_out_bwd(const bf16* __restrict__ d1, const float* __restrict__ wo,
                          const float* __restrict__ y, const float* __restrict__ tgt,
                          const float* __restrict__ tscale, size_t n, float weight,
                          bf16* __restrict__ gd1, float* __restrict__ gwo,
                          double* __restrict__ loss) {
  const float ts = *tscale;
  float lw[17];
#pragma unroll
  for (int c = 0; c < 17; ++c) lw[c] = 0.f;
  double ls = 0.0;
  const float inv_n = 1.0f / (float)n;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n;
       p += (size_t)gridDim.x * blockDim.x) {
    const float e = y[p] - tgt[p] * ts;
    ls += (double)weight * e * e;
    const float gy = 2.0f * weight * e * inv_n;
    uint32_t* o = reinterpret_cast<uint32_t*>(gd1 + p * 16);
#pragma unroll
    for (int c = 0; c < 16; c += 2) {
      const float a = __bfloat162float(d1[p * 16 + c]), b = __bfloat162float(d1[p * 16 + c + 1]);
      lw[c] = fmaf(gy, a, lw[c]);
      lw[c + 1] = fmaf(gy, b, lw[c + 1]);
      o[c / 2] = pack2(gy * wo[c], gy * wo[c + 1]);
    }
    lw[16] += gy;
  }
#pragma unroll
  for (int c = 0; c < 17; ++c) {
    float v = lw[c];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(&gwo[c], v);
  }
  ls = warp_sum(ls);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, ls / (double)n);
}

// mirrored-and-transposed weights for the data gradient: Wt[t'][i][o] = W[26-t'][o][i]
__global__ void k_transpose_w(const bf16* __restrict__ W, bf16* __restrict__ Wt, int cin,
                              int cout) {
  const int tot = 27 * cin * cout;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
    const int t = e / (cin * cout), rem = e % (cin * cout);
    const int i = rem / cout, o = rem % cout;
    Wt[e] = W[((size_t)(26 - t) * cout + o) * cin + i];
  }
}

// Adam on the FP32 master parameters, then the BF16 copies of the convolution weights
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, size_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2, const uint8_t* __restrict__ frozen) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    if (frozen && frozen[e]) continue;
    const float gg = g[e];
    const float mm = b1 * m[e] + (1.f - b1) * gg;
    const float vv = b2 * v[e] + (1.f - b2) * gg * gg;
    m[e] = mm;
    v[e] = vv;
    w[e] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
  }
}

__global__ void k_to_bf16(const float* __restrict__ a, bf16* __restrict__ b, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x)
    b[e] = __float2bfloat16(a[e]);
}

}  // namespace unet
}  // namespace fg

// ============================================================================================
// The network object

namespace fg {
namespace unet {

struct ConvSpec {
  int cin, cout, level, cin_live;
};
// c1a c1b c2a c2b c3a c3b d2a d2b d1a d1b
static const ConvSpec kConv[10] = {{16, 16, 0, 3},  {16, 16, 0, 16}, {16, 32, 1, 16},
                                   {32, 32, 1, 32}, {32, 64, 2, 32}, {64, 64, 2, 64},
                                   {96, 32, 1, 96}, {32, 32, 1, 32}, {48, 16, 0, 48},
                                   {16, 16, 0, 16}};

static int blocks_for(size_t n) {
  size_t b = (n + 255) / 256;
  if (b > (size_t)kNumSMs * 16) b = (size_t)kNumSMs * 16;
  return (int)(b < 1 ? 1 : b);
}

// the error word of the tensor-core convolutions (a bounded wait ran out), one per process
int* tc_error_word() {
  static int* w = nullptr;
  if (!w && cudaMalloc(&w, sizeof(int)) == cudaSuccess) cudaMemset(w, 0, sizeof(int));
  return w;
}

// The convolutions of the network (forward and data gradient) run on the tcgen05 kernel.
// resident blocks per SM of a kernel with `smem` dynamic bytes and `tmem_cols` tensor-memory
// columns: shared memory (1 KB reserved per block), 16 blocks of 128 threads, and the SM's 512
// tensor-memory columns shared by its blocks
static int tc_blocks_per_sm(int smem, int tmem_cols) {
  int dev = 0, smem_sm = 228 * 1024;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  return std::max(1, std::min({smem_sm / (smem + 128 + 1024), 16, 512 / tmem_cols}));
}

template <int CIN, int COUT>
static void conv(const bf16* in, int in_stride, int in_off, const bf16* W, const float* bias,
                 bf16* out, int out_stride, int out_off, int nx, int ny, int nz, bool relu,
                 cudaStream_t st) {
  if constexpr (CIN <= 16 && TcPShape<CIN, COUT>::FITS) {
    // weights resident, one MMA group per output plane (16-channel inputs)
    using Z = TcPShape<CIN, COUT>;
    static int per_sm = 0;
    if (per_sm == 0) {
      cudaFuncSetAttribute(k_conv3_tcp<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           Z::SMEM);
      per_sm = tc_blocks_per_sm(Z::SMEM, Z::TMEM_COLS);
    }
    const long items = (long)tc_tiles_x(nx) * tc_tiles_y(ny) * ((nz + kTcZC - 1) / kTcZC);
    const int grid = (int)std::min<long>(items, (long)kNumSMs * per_sm);
    k_conv3_tcp<CIN, COUT><<<grid, 128, Z::SMEM, st>>>(in, in_stride, in_off, W, bias, out,
                                                       out_stride, out_off, nx, ny, nz,
                                                       relu ? 1 : 0, tc_error_word());
    return;
  } else if constexpr (TcZShape<CIN, COUT>::FITS) {
    // weights resident, z columns pipelined
    using Z = TcZShape<CIN, COUT>;
    static int per_sm = 0;
    if (per_sm == 0) {
      cudaFuncSetAttribute(k_conv3_tcz<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           Z::SMEM);
      per_sm = tc_blocks_per_sm(Z::SMEM, Z::TMEM_COLS);
    }
    const long items = (long)tc_tiles_x(nx) * tc_tiles_y(ny) * ((nz + Z::ZC - 1) / Z::ZC);
    const int grid = (int)std::min<long>(items, (long)kNumSMs * per_sm);
    k_conv3_tcz<CIN, COUT><<<grid, 128, Z::SMEM, st>>>(in, in_stride, in_off, W, bias, out,
                                                       out_stride, out_off, nx, ny, nz,
                                                       relu ? 1 : 0, tc_error_word());
    return;
  }
  using S = TcShape<CIN, COUT>;
  static int per_sm = 0;
  if (per_sm == 0) {
    cudaFuncSetAttribute(k_conv3_tc<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         S::SMEM);
    per_sm = tc_blocks_per_sm(S::SMEM, S::TMEM_COLS);
  }
  const long tiles = (long)tc_tiles_x(nx) * tc_tiles_y(ny) * nz;
  const int grid = (int)std::min<long>(tiles, (long)kNumSMs * per_sm);
  k_conv3_tc<CIN, COUT><<<grid, 128, S::SMEM, st>>>(in, in_stride, in_off, W, bias, out,
                                                    out_stride, out_off, nx, ny, nz,
                                                    relu ? 1 : 0, tc_error_word());
}

// the same convolution on the mma.sync kernel (the self-check's comparison)
template <int CIN, int COUT>
static void conv_sync(const bf16* in, int in_stride, int in_off, const bf16* W,
                      const float* bias, bf16* out, int out_stride, int out_off, int nx, int ny,
                      int nz, bool relu, cudaStream_t st) {
  dim3 grid((nx + 15) / 16, (ny + 3) / 4, nz);
  k_conv3<CIN, COUT><<<grid, 128, 0, st>>>(in, in_stride, in_off, W, bias, out, out_stride,
                                           out_off, nx, ny, nz, relu ? 1 : 0);
}

template <int CIN, int COUT>
static void conv_dw(const bf16* in, int in_stride, int in_off, const bf16* g, int g_stride,
                    int g_off, float* dW, int nx, int ny, int nz, cudaStream_t st) {
  const size_t n = (size_t)nx * ny * nz;
  const int chunks = (int)std::max<size_t>(1, std::min<size_t>(64, n / 256));
  const size_t chunk = (n + chunks - 1) / chunks;
  dim3 grid(27, chunks);
  k_conv3_dw<CIN, COUT><<<grid, 256, 0, st>>>(in, in_stride, in_off, g, g_stride, g_off, dW, nx,
                                               ny, nz, chunk);
}

}  // namespace unet
}  // namespace fg

using namespace fg;
using namespace fg::unet;

struct frehg_unet {
  // parameters: per conv W[27][cout][cin] then b[cout]; then output w[16], b
  size_t woff[10], boff[10], ooff = 0, nparam = 0;
  size_t wboff[10], nwb = 0;  // bf16 weight offsets
  float* master = nullptr;    // device FP32
  float* grad = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  uint8_t* frozen = nullptr;
  bf16* wb = nullptr;   // BF16 weights
  bf16* wt = nullptr;   // mirrored/transposed BF16 weights (data gradient)
  int adam_t = 0;
  float kmean = 0.f, kscale = 1.f, cscale = 1.f;
  float loss_weight = 1.f;  // multiplies the loss and its gradients
  // activations
  int nx = 0, ny = 0, nz = 0;
  size_t cap1 = 0;
  bf16 *x0 = nullptr, *a1 = nullptr, *cat1 = nullptr, *d1a = nullptr, *d1 = nullptr;
  bf16 *p1 = nullptr, *a2 = nullptr, *cat2 = nullptr, *d2a = nullptr, *d2 = nullptr;
  bf16 *p2 = nullptr, *a3 = nullptr, *e3 = nullptr;
  bf16 *g_d1 = nullptr, *g_d1a = nullptr, *g_cat1 = nullptr, *g_a1 = nullptr;
  bf16 *g_d2 = nullptr, *g_d2a = nullptr, *g_cat2 = nullptr, *g_p1 = nullptr, *g_a2 = nullptr;
  bf16 *g_e3 = nullptr, *g_a3 = nullptr, *g_p2 = nullptr;
  float* y = nullptr;
  float* scal = nullptr;  // [0] 1/rms(r), [1] rms(r)
  double* rms_part = nullptr;  // per-block partial sums of r^2
  double* loss = nullptr;
  std::vector<void*> bufs;
  ~frehg_unet() {
    for (void* b : bufs) cudaFree(b);
    cudaFree(master);
    cudaFree(grad);
    cudaFree(m);
    cudaFree(v);
    cudaFree(frozen);
    cudaFree(wb);
    cudaFree(wt);
    cudaFree(scal);
    cudaFree(rms_part);
    cudaFree(loss);
  }
};

namespace {

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double gauss(uint64_t& s) {
  const double u1 = ((splitmix(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  const double u2 = ((splitmix(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

int refresh_bf16(frehg_unet* net, cudaStream_t st) {
  for (int l = 0; l < 10; ++l) {
    const size_t nw = (size_t)27 * kConv[l].cin * kConv[l].cout;
    k_to_bf16<<<blocks_for(nw), 256, 0, st>>>(net->master + net->woff[l], net->wb + net->wboff[l],
                                              nw);
    k_transpose_w<<<blocks_for(nw), 256, 0, st>>>(net->wb + net->wboff[l], net->wt + net->wboff[l],
                                                  kConv[l].cin, kConv[l].cout);
  }
  FG_CUDA(cudaGetLastError());
  return FREHG_OK;
}

int ensure_acts(frehg_unet* net, int nx, int ny, int nz) {
  FG_ARG(nx % 4 == 0 && ny % 4 == 0 && nz % 4 == 0,
         "U-Net grids need nx, ny, nz divisible by 4 (two 2x2x2 poolings), got %dx%dx%d", nx, ny,
         nz);
  net->nx = nx;
  net->ny = ny;
  net->nz = nz;
  const size_t n1 = (size_t)nx * ny * nz;
  if (n1 <= net->cap1) return FREHG_OK;
  for (void* b : net->bufs) cudaFree(b);
  net->bufs.clear();
  const size_t n2 = n1 / 8, n3 = n1 / 64;
  auto A = [&](bf16** p, size_t elems) -> int {
    FG_CUDA(cudaMalloc(p, elems * sizeof(bf16)));
    net->bufs.push_back(*p);
    return FREHG_OK;
  };
  FG_TRY(A(&net->x0, n1 * 16));
  FG_TRY(A(&net->a1, n1 * 16));
  FG_TRY(A(&net->cat1, n1 * 48));
  FG_TRY(A(&net->d1a, n1 * 16));
  FG_TRY(A(&net->d1, n1 * 16));
  FG_TRY(A(&net->p1, n2 * 16));
  FG_TRY(A(&net->a2, n2 * 32));
  FG_TRY(A(&net->cat2, n2 * 96));
  FG_TRY(A(&net->d2a, n2 * 32));
  FG_TRY(A(&net->d2, n2 * 32));
  FG_TRY(A(&net->p2, n3 * 32));
  FG_TRY(A(&net->a3, n3 * 64));
  FG_TRY(A(&net->e3, n3 * 64));
  FG_TRY(A(&net->g_d1, n1 * 16));
  FG_TRY(A(&net->g_d1a, n1 * 16));
  FG_TRY(A(&net->g_cat1, n1 * 48));
  FG_TRY(A(&net->g_a1, n1 * 16));
  FG_TRY(A(&net->g_d2, n2 * 32));
  FG_TRY(A(&net->g_d2a, n2 * 32));
  FG_TRY(A(&net->g_cat2, n2 * 96));
  FG_TRY(A(&net->g_p1, n2 * 16));
  FG_TRY(A(&net->g_a2, n2 * 32));
  FG_TRY(A(&net->g_e3, n3 * 64));
  FG_TRY(A(&net->g_a3, n3 * 64));
  FG_TRY(A(&net->g_p2, n3 * 32));
  FG_CUDA(cudaMalloc(&net->y, n1 * sizeof(float)));
  net->bufs.push_back(net->y);
  net->cap1 = n1;
  return FREHG_OK;
}

// forward pass; y = network output times `outscale` (rms of r) when scaled_out
int forward(frehg_unet* net, const float* r, const float* lnk, const float* cap, float* y,
            bool scaled_out, cudaStream_t st) {
  const int nx = net->nx, ny = net->ny, nz = net->nz;
  const int x2 = nx / 2, y2 = ny / 2, z2 = nz / 2, x3 = nx / 4, y3 = ny / 4, z3 = nz / 4;
  const size_t n1 = (size_t)nx * ny * nz, n2 = n1 / 8, n3 = n1 / 64;
  const float* M = net->master;
  const bf16* W = net->wb;
  {
    const int nb = (int)std::min<size_t>((n1 + 255) / 256, (size_t)kRmsBlocks);
    k_rms_partial<<<nb, 256, 0, st>>>(r, n1, net->rms_part);
    k_rms_scale<<<1, 256, 0, st>>>(net->rms_part, nb, n1, net->scal, net->scal + 1);
  }
  k_pack_input<<<blocks_for(n1), 256, 0, st>>>(r, lnk, cap, net->scal, net->kmean, net->kscale,
                                               net->cscale, net->x0, n1);
  conv<16, 16>(net->x0, 16, 0, W + net->wboff[0], M + net->boff[0], net->a1, 16, 0, nx, ny, nz, true, st);
  conv<16, 16>(net->a1, 16, 0, W + net->wboff[1], M + net->boff[1], net->cat1, 48, 32, nx, ny, nz, true, st);
  k_pool<<<blocks_for(n2 * 2), 256, 0, st>>>(net->cat1, 48, 32, net->p1, 16, nx, ny, nz);
  conv<16, 32>(net->p1, 16, 0, W + net->wboff[2], M + net->boff[2], net->a2, 32, 0, x2, y2, z2, true, st);
  conv<32, 32>(net->a2, 32, 0, W + net->wboff[3], M + net->boff[3], net->cat2, 96, 64, x2, y2, z2, true, st);
  k_pool<<<blocks_for(n3 * 4), 256, 0, st>>>(net->cat2, 96, 64, net->p2, 32, x2, y2, z2);
  conv<32, 64>(net->p2, 32, 0, W + net->wboff[4], M + net->boff[4], net->a3, 64, 0, x3, y3, z3, true, st);
  conv<64, 64>(net->a3, 64, 0, W + net->wboff[5], M + net->boff[5], net->e3, 64, 0, x3, y3, z3, true, st);
  k_up<<<blocks_for(n2 * 64), 256, 0, st>>>(net->e3, net->cat2, 96, 0, 64, x2, y2, z2);
  conv<96, 32>(net->cat2, 96, 0, W + net->wboff[6], M + net->boff[6], net->d2a, 32, 0, x2, y2, z2, true, st);
  conv<32, 32>(net->d2a, 32, 0, W + net->wboff[7], M + net->boff[7], net->d2, 32, 0, x2, y2, z2, true, st);
  k_up<<<blocks_for(n1 * 32), 256, 0, st>>>(net->d2, net->cat1, 48, 0, 32, nx, ny, nz);
  conv<48, 16>(net->cat1, 48, 0, W + net->wboff[8], M + net->boff[8], net->d1a, 16, 0, nx, ny, nz, true, st);
  conv<16, 16>(net->d1a, 16, 0, W + net->wboff[9], M + net->boff[9], net->d1, 16, 0, nx, ny, nz, true, st);
  k_out<<<blocks_for(n1), 256, 0, st>>>(net->d1, M + net->ooff, scaled_out ? net->scal + 1 : nullptr,
                                        y, n1);
  (void)n3;
  FG_CUDA(cudaGetLastError());
  return FREHG_OK;
}

// loss = mean((NN(r) - target / rms(r))^2) and all parameter gradients (into net->grad)
int backward(frehg_unet* net, const float* target, cudaStream_t st) {
  const int nx = net->nx, ny = net->ny, nz = net->nz;
  const int x2 = nx / 2, y2 = ny / 2, z2 = nz / 2, x3 = nx / 4, y3 = ny / 4, z3 = nz / 4;
  const size_t n1 = (size_t)nx * ny * nz, n2 = n1 / 8, n3 = n1 / 64;
  const float* M = net->master;
  const bf16* T = net->wt;
  float* G = net->grad;
  FG_CUDA(cudaMemsetAsync(G, 0, net->nparam * sizeof(float), st));
  FG_CUDA(cudaMemsetAsync(net->loss, 0, sizeof(double), st));
  // normalised target: t * (1/rms r); y holds the unscaled network output
  k_out_bwd<<<blocks_for(n1), 256, 0, st>>>(net->d1, M + net->ooff, net->y, target, net->scal,
                                            n1, net->loss_weight, net->g_d1, G + net->ooff,
                                            net->loss);
  auto relu_b = [&](bf16* g, int gs, int go, const bf16* a, int as, int ao, int c, size_t n) {
    k_relu_bwd<<<blocks_for(n * c), 256, 0, st>>>(g, gs, go, a, as, ao, c, n);
  };
  auto bias_g = [&](const bf16* g, int gs, int go, int c, size_t n, int l) {
    k_bias_grad<<<blocks_for(n), 256, 0, st>>>(g, gs, go, c, n, G + net->boff[l]);
  };
  // level 1 decoder
  relu_b(net->g_d1, 16, 0, net->d1, 16, 0, 16, n1);
  conv_dw<16, 16>(net->d1a, 16, 0, net->g_d1, 16, 0, G + net->woff[9], nx, ny, nz, st);
  bias_g(net->g_d1, 16, 0, 16, n1, 9);
  conv<16, 16>(net->g_d1, 16, 0, T + net->wboff[9], nullptr, net->g_d1a, 16, 0, nx, ny, nz, false, st);
  relu_b(net->g_d1a, 16, 0, net->d1a, 16, 0, 16, n1);
  conv_dw<48, 16>(net->cat1, 48, 0, net->g_d1a, 16, 0, G + net->woff[8], nx, ny, nz, st);
  bias_g(net->g_d1a, 16, 0, 16, n1, 8);
  conv<16, 48>(net->g_d1a, 16, 0, T + net->wboff[8], nullptr, net->g_cat1, 48, 0, nx, ny, nz, false, st);
  // level 2 decoder
  k_up_bwd<<<blocks_for(n2 * 32), 256, 0, st>>>(net->g_cat1, 48, 0, net->g_d2, 32, nx, ny, nz);
  relu_b(net->g_d2, 32, 0, net->d2, 32, 0, 32, n2);
  conv_dw<32, 32>(net->d2a, 32, 0, net->g_d2, 32, 0, G + net->woff[7], x2, y2, z2, st);
  bias_g(net->g_d2, 32, 0, 32, n2, 7);
  conv<32, 32>(net->g_d2, 32, 0, T + net->wboff[7], nullptr, net->g_d2a, 32, 0, x2, y2, z2, false, st);
  relu_b(net->g_d2a, 32, 0, net->d2a, 32, 0, 32, n2);
  conv_dw<96, 32>(net->cat2, 96, 0, net->g_d2a, 32, 0, G + net->woff[6], x2, y2, z2, st);
  bias_g(net->g_d2a, 32, 0, 32, n2, 6);
  conv<32, 96>(net->g_d2a, 32, 0, T + net->wboff[6], nullptr, net->g_cat2, 96, 0, x2, y2, z2, false, st);
  // level 3
  k_up_bwd<<<blocks_for(n3 * 64), 256, 0, st>>>(net->g_cat2, 96, 0, net->g_e3, 64, x2, y2, z2);
  relu_b(net->g_e3, 64, 0, net->e3, 64, 0, 64, n3);
  conv_dw<64, 64>(net->a3, 64, 0, net->g_e3, 64, 0, G + net->woff[5], x3, y3, z3, st);
  bias_g(net->g_e3, 64, 0, 64, n3, 5);
  conv<64, 64>(net->g_e3, 64, 0, T + net->wboff[5], nullptr, net->g_a3, 64, 0, x3, y3, z3, false, st);
  relu_b(net->g_a3, 64, 0, net->a3, 64, 0, 64, n3);
  conv_dw<32, 64>(net->p2, 32, 0, net->g_a3, 64, 0, G + net->woff[4], x3, y3, z3, st);
  bias_g(net->g_a3, 64, 0, 64, n3, 4);
  conv<64, 32>(net->g_a3, 64, 0, T + net->wboff[4], nullptr, net->g_p2, 32, 0, x3, y3, z3, false, st);
  // level 2 encoder: e2 gradient = skip part + pooling part
  k_pool_bwd_add<<<blocks_for(n2 * 32), 256, 0, st>>>(net->g_p2, net->g_cat2, 96, 64, 32, x2, y2, z2);
  relu_b(net->g_cat2, 96, 64, net->cat2, 96, 64, 32, n2);
  conv_dw<32, 32>(net->a2, 32, 0, net->g_cat2, 96, 64, G + net->woff[3], x2, y2, z2, st);
  bias_g(net->g_cat2, 96, 64, 32, n2, 3);
  conv<32, 32>(net->g_cat2, 96, 64, T + net->wboff[3], nullptr, net->g_a2, 32, 0, x2, y2, z2, false, st);
  relu_b(net->g_a2, 32, 0, net->a2, 32, 0, 32, n2);
  conv_dw<16, 32>(net->p1, 16, 0, net->g_a2, 32, 0, G + net->woff[2], x2, y2, z2, st);
  bias_g(net->g_a2, 32, 0, 32, n2, 2);
  conv<32, 16>(net->g_a2, 32, 0, T + net->wboff[2], nullptr, net->g_p1, 16, 0, x2, y2, z2, false, st);
  // level 1 encoder: e1 gradient = skip part + pooling part
  k_pool_bwd_add<<<blocks_for(n1 * 16), 256, 0, st>>>(net->g_p1, net->g_cat1, 48, 32, 16, nx, ny, nz);
  relu_b(net->g_cat1, 48, 32, net->cat1, 48, 32, 16, n1);
  conv_dw<16, 16>(net->a1, 16, 0, net->g_cat1, 48, 32, G + net->woff[1], nx, ny, nz, st);
  bias_g(net->g_cat1, 48, 32, 16, n1, 1);
  conv<16, 16>(net->g_cat1, 48, 32, T + net->wboff[1], nullptr, net->g_a1, 16, 0, nx, ny, nz, false, st);
  relu_b(net->g_a1, 16, 0, net->a1, 16, 0, 16, n1);
  conv_dw<16, 16>(net->x0, 16, 0, net->g_a1, 16, 0, G + net->woff[0], nx, ny, nz, st);
  bias_g(net->g_a1, 16, 0, 16, n1, 0);
  FG_CUDA(cudaGetLastError());
  return FREHG_OK;
}

}  // namespace

namespace fg {
// used by the Krylov solver: z = NN(r) scaled back by rms(r)
int unet_apply(frehg_unet* net, int nx, int ny, int nz, const float* r, const float* lnk,
               const float* cap, float* z, cudaStream_t st) {
  FG_TRY(ensure_acts(net, nx, ny, nz));
  return forward(net, r, lnk, cap, z, true, st);
}
}  // namespace fg

// tensor-core convolution against the mma.sync one on seeded random inputs (a self-check)
template <int CIN, int COUT>
static int conv_check_shape(int in_stride, int in_off, int out_stride, int out_off, int nx,
                            int ny, int nz, int relu, uint64_t seed, double* max_diff,
                            double* max_ref) {
  const size_t n = (size_t)nx * ny * nz;
  const size_t nin = n * in_stride, nout = n * out_stride, nw = (size_t)27 * CIN * COUT;
  std::vector<bf16> hin(nin), hw(nw);
  std::vector<float> hb(COUT);
  uint64_t s = seed * 0x9E3779B97F4A7C15ull + 7u;
  for (auto& v : hin) v = __float2bfloat16((float)gauss(s));
  for (auto& v : hw) v = __float2bfloat16((float)(0.1 * gauss(s)));
  for (auto& v : hb) v = (float)(0.1 * gauss(s));
  bf16 *din = nullptr, *dw = nullptr, *o1 = nullptr, *o2 = nullptr;
  float* db = nullptr;
  int rc = FREHG_OK;
  if (cudaMalloc(&din, nin * 2) || cudaMalloc(&dw, nw * 2) || cudaMalloc(&o1, nout * 2) ||
      cudaMalloc(&o2, nout * 2) || cudaMalloc(&db, COUT * 4)) {
    set_error("conv check: device allocation");
    rc = FREHG_ERR_CUDA;
  }
  if (rc == FREHG_OK) {
    cudaMemcpy(din, hin.data(), nin * 2, cudaMemcpyHostToDevice);
    cudaMemcpy(dw, hw.data(), nw * 2, cudaMemcpyHostToDevice);
    cudaMemcpy(db, hb.data(), COUT * 4, cudaMemcpyHostToDevice);
    cudaMemset(o1, 0, nout * 2);
    cudaMemset(o2, 0, nout * 2);
    conv<CIN, COUT>(din, in_stride, in_off, dw, db, o1, out_stride, out_off, nx, ny, nz,
                    relu != 0, 0);
    conv_sync<CIN, COUT>(din, in_stride, in_off, dw, db, o2, out_stride, out_off, nx, ny, nz,
                         relu != 0, 0);
    const cudaError_t e = cudaDeviceSynchronize();
    int tc_err = 0;
    cudaMemcpy(&tc_err, tc_error_word(), sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess || tc_err) {
      set_error("conv check: %s (tensor-core error word %d)", cudaGetErrorString(e), tc_err);
      rc = FREHG_ERR_CUDA;
    }
  }
  if (rc == FREHG_OK) {
    std::vector<bf16> a(nout), b(nout);
    cudaMemcpy(a.data(), o1, nout * 2, cudaMemcpyDeviceToHost);
    cudaMemcpy(b.data(), o2, nout * 2, cudaMemcpyDeviceToHost);
    double md = 0.0, mr = 0.0;
    for (size_t q = 0; q < nout; ++q) {
      const double x = __bfloat162float(a[q]), y = __bfloat162float(b[q]);
      md = std::max(md, std::fabs(x - y));
      mr = std::max(mr, std::fabs(y));
    }
    *max_diff = md;
    *max_ref = mr;
  }
  cudaFree(din);
  cudaFree(dw);
  cudaFree(o1);
  cudaFree(o2);
  cudaFree(db);
  return rc;
}

// the tensor-core convolutions' error word (a bounded wait ran out); checked where the host
// synchronises anyway
static int check_tc_error() {
  int e = 0;
  FG_CUDA(cudaMemcpy(&e, tc_error_word(), sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    set_error("tensor-core convolution: a bounded wait ran out (%d)", e);
    return FREHG_ERR_CUDA;
  }
  return FREHG_OK;
}

extern "C" {

int frehg_unet_create(uint64_t seed, frehg_unet** out) {
  clear_error();
  FG_ARG(out, "null argument");
  frehg_unet* net = new frehg_unet();
  size_t off = 0, boff = 0;
  for (int l = 0; l < 10; ++l) {
    net->woff[l] = off;
    off += (size_t)27 * kConv[l].cin * kConv[l].cout;
    net->boff[l] = off;
    off += kConv[l].cout;
    net->wboff[l] = boff;
    boff += (size_t)27 * kConv[l].cin * kConv[l].cout;
  }
  net->ooff = off;
  off += 17;
  net->nparam = off;
  net->nwb = boff;
  std::vector<float> h(off, 0.0f);
  std::vector<uint8_t> fz(off, 0);
  uint64_t s = seed * 0x2545F4914F6CDD1Dull + 12345u;
  for (int l = 0; l < 10; ++l) {
    const ConvSpec& c = kConv[l];
    const double sd = sqrt(2.0 / (27.0 * c.cin_live));
    for (int t = 0; t < 27; ++t)
      for (int o = 0; o < c.cout; ++o)
        for (int i = 0; i < c.cin; ++i) {
          const size_t e = net->woff[l] + ((size_t)t * c.cout + o) * c.cin + i;
          if (i < c.cin_live) {
            h[e] = (float)(sd * gauss(s));
          } else {
            h[e] = 0.0f;
            fz[e] = 1;  // padding channels of the input layer stay zero
          }
        }
  }
  for (int c = 0; c < 16; ++c) h[net->ooff + c] = (float)(0.1 / 4.0 * gauss(s));
  auto fail = [&](const char* what) {
    set_error("frehg_unet_create: %s", what);
    delete net;
    return FREHG_ERR_CUDA;
  };
  if (cudaMalloc(&net->master, off * 4) || cudaMalloc(&net->grad, off * 4) ||
      cudaMalloc(&net->m, off * 4) || cudaMalloc(&net->v, off * 4) ||
      cudaMalloc(&net->frozen, off) || cudaMalloc(&net->wb, boff * 2) ||
      cudaMalloc(&net->wt, boff * 2) || cudaMalloc(&net->scal, 2 * sizeof(float)) ||
      cudaMalloc(&net->rms_part, kRmsBlocks * sizeof(double)) ||
      cudaMalloc(&net->loss, sizeof(double)))
    return fail("device allocation");
  cudaMemcpy(net->master, h.data(), off * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(net->frozen, fz.data(), off, cudaMemcpyHostToDevice);
  cudaMemset(net->m, 0, off * 4);
  cudaMemset(net->v, 0, off * 4);
  cudaMemset(net->grad, 0, off * 4);
  if (refresh_bf16(net, 0) != FREHG_OK) return fail("weight conversion");
  if (cudaDeviceSynchronize() != cudaSuccess) return fail("initialisation");
  *out = net;
  return FREHG_OK;
}

int frehg_unet_destroy(frehg_unet* net) {
  clear_error();
  if (net) {
    cudaDeviceSynchronize();
    delete net;
  }
  return FREHG_OK;
}

int frehg_unet_num_params(const frehg_unet* net, int64_t* n) {
  clear_error();
  FG_ARG(net && n, "null argument");
  *n = (int64_t)net->nparam;
  return FREHG_OK;
}

int frehg_unet_get_params(frehg_unet* net, float* host) {
  clear_error();
  FG_ARG(net && host, "null argument");
  FG_CUDA(cudaDeviceSynchronize());
  FG_CUDA(cudaMemcpy(host, net->master, net->nparam * 4, cudaMemcpyDeviceToHost));
  return FREHG_OK;
}

int frehg_unet_set_params(frehg_unet* net, const float* host) {
  clear_error();
  FG_ARG(net && host, "null argument");
  FG_CUDA(cudaDeviceSynchronize());
  FG_CUDA(cudaMemcpy(net->master, host, net->nparam * 4, cudaMemcpyHostToDevice));
  FG_TRY(refresh_bf16(net, 0));
  FG_CUDA(cudaDeviceSynchronize());
  return FREHG_OK;
}

int frehg_unet_set_input_scaling(frehg_unet* net, float lnk_mean, float lnk_scale,
                                 float cap_scale) {
  clear_error();
  FG_ARG(net, "null handle");
  net->kmean = lnk_mean;
  net->kscale = lnk_scale;
  net->cscale = cap_scale;
  return FREHG_OK;
}

int frehg_unet_conv_check(int cin, int cout, int in_stride, int in_off, int out_stride,
                          int out_off, int nx, int ny, int nz, int relu, uint64_t seed,
                          double* max_diff, double* max_ref) {
  clear_error();
  FG_ARG(max_diff && max_ref, "null argument");
  FG_ARG(nx > 0 && ny > 0 && nz > 0 && in_off + cin <= in_stride && out_off + cout <= out_stride &&
             in_stride % 8 == 0 && in_off % 8 == 0 && out_stride % 8 == 0 && out_off % 8 == 0,
         "conv check: bad sizes or channel slices");
#define FG_CONV_CASE(CI, CO)                                                                  \
  if (cin == CI && cout == CO)                                                                \
    return conv_check_shape<CI, CO>(in_stride, in_off, out_stride, out_off, nx, ny, nz, relu, \
                                    seed, max_diff, max_ref);
  FG_CONV_CASE(16, 16)
  FG_CONV_CASE(16, 32)
  FG_CONV_CASE(32, 32)
  FG_CONV_CASE(32, 64)
  FG_CONV_CASE(64, 64)
  FG_CONV_CASE(96, 32)
  FG_CONV_CASE(48, 16)
  FG_CONV_CASE(16, 48)
  FG_CONV_CASE(32, 96)
  FG_CONV_CASE(64, 32)
  FG_CONV_CASE(32, 16)
#undef FG_CONV_CASE
  set_error("conv check: no convolution of the network has %d -> %d channels", cin, cout);
  return FREHG_ERR_UNSUPPORTED;
}

int frehg_unet_forward(frehg_unet* net, int nx, int ny, int nz, const float* r, const float* lnk,
                       const float* cap, float* y, void* stream) {
  clear_error();
  FG_ARG(net && r && lnk && cap && y, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  FG_TRY(ensure_acts(net, nx, ny, nz));
  FG_TRY(forward(net, r, lnk, cap, y, true, st));
  FG_CUDA(cudaStreamSynchronize(st));
  return check_tc_error();
}

int frehg_unet_loss_grad(frehg_unet* net, int nx, int ny, int nz, const float* r,
                         const float* lnk, const float* cap, const float* target, double* loss,
                         float* grad_host, void* stream) {
  clear_error();
  FG_ARG(net && r && lnk && cap && target, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  FG_TRY(ensure_acts(net, nx, ny, nz));
  FG_TRY(forward(net, r, lnk, cap, net->y, false, st));
  FG_TRY(backward(net, target, st));
  if (loss) FG_CUDA(cudaMemcpyAsync(loss, net->loss, sizeof(double), cudaMemcpyDeviceToHost, st));
  if (grad_host)
    FG_CUDA(cudaMemcpyAsync(grad_host, net->grad, net->nparam * 4, cudaMemcpyDeviceToHost, st));
  FG_CUDA(cudaStreamSynchronize(st));
  return check_tc_error();
}

int frehg_unet_set_loss_weight(frehg_unet* net, float weight) {
  clear_error();
  FG_ARG(net && weight > 0.f, "positive weight required");
  net->loss_weight = weight;
  return FREHG_OK;
}

int frehg_unet_adam_step(frehg_unet* net, float lr, float beta1, float beta2, float eps,
                         void* stream) {
  clear_error();
  FG_ARG(net, "null handle");
  cudaStream_t st = (cudaStream_t)stream;
  net->adam_t += 1;
  const float c1 = 1.0f - powf(beta1, (float)net->adam_t);
  const float c2 = 1.0f - powf(beta2, (float)net->adam_t);
  k_adam<<<blocks_for(net->nparam), 256, 0, st>>>(net->master, net->grad, net->m, net->v,
                                                  net->nparam, lr, beta1, beta2, eps, c1, c2,
                                                  net->frozen);
  FG_TRY(refresh_bf16(net, st));
  return FREHG_OK;
}

int frehg_unet_flops(int nx, int ny, int nz, double* flops) {
  clear_error();
  FG_ARG(flops, "null argument");
  const double n1 = (double)nx * ny * nz;
  double macs = 0.0;
  for (int l = 0; l < 10; ++l) {
    const double px = n1 / (kConv[l].level == 0 ? 1.0 : kConv[l].level == 1 ? 8.0 : 64.0);
    macs += px * 27.0 * kConv[l].cin * kConv[l].cout;  // as executed (padded channels included)
  }
  macs += n1 * 16.0;
  *flops = 2.0 * macs;
  return FREHG_OK;
}

}  // extern "C"
