// Deterministic block / grid reductions shared by the kernels (last-arriving-block pattern:
// no grid barrier, no spin-wait), and the bounded grid barrier of cooperative launches.
#pragma once

#include "internal.h"

namespace fg {

// per-thread compensated FP32 sum (Kahan); the FP32 Krylov kernels combine these in FP64
struct Kahan32 {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ int flat_tid() { return threadIdx.x + threadIdx.y * blockDim.x; }
__device__ __forceinline__ int flat_nthreads() { return blockDim.x * blockDim.y; }
__device__ __forceinline__ int flat_bid() { return blockIdx.x + blockIdx.y * gridDim.x; }
__device__ __forceinline__ int flat_nblocks() { return gridDim.x * gridDim.y; }

// Sum NV values over the block; the result is valid in thread 0.  Uses sh[NV*32].
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* sh) {
  const int tid = flat_tid(), lane = tid & 31, wid = tid >> 5, nw = flat_nthreads() >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = warp_sum(v[q]);
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) sh[q * 32 + wid] = v[q];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double t = lane < nw ? sh[q * 32 + lane] : 0.0;
      v[q] = warp_sum(t);
    }
  }
  __syncthreads();
}

// Grid-wide sum through per-block partials; returns true in every thread of the last block
// to arrive, where tot[] (valid in thread 0) holds the deterministic grid total.
template <int NV>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], double* partials, unsigned int* arrive,
                         double (&tot)[NV]) {
  __shared__ double sh[NV * 32];
  __shared__ unsigned int ticket;
  const int tid = flat_tid(), bid = flat_bid(), nb = flat_nblocks();
  block_sum<NV>(v, sh);
  if (tid == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) partials[q * kMaxRedBlocks + bid] = v[q];
    __threadfence();
    ticket = atomicAdd(arrive, 1u);
  }
  __syncthreads();
  if (ticket != (unsigned)(nb - 1)) return false;
  __threadfence();
  double acc[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    acc[q] = 0.0;
    for (int b = tid; b < nb; b += flat_nthreads()) acc[q] += __ldcg(&partials[q * kMaxRedBlocks + b]);
  }
  block_sum<NV>(acc, sh);
#pragma unroll
  for (int q = 0; q < NV; ++q) tot[q] = acc[q];
  if (tid == 0) *arrive = 0u;
  return true;
}

// Grid barrier for cooperative launches (every block resident at once): an arrival counter
// and a generation word in device memory, both 0 before the first use; the last block to
// arrive resets the counter and advances the generation, so consecutive barriers and launches
// reuse them.  The wait is bounded (kGridBarrierPolls polls, about two seconds); a block whose
// wait runs out sets *timeout and gets false, and the caller stops (its launch then reports
// the timeout instead of a result).
constexpr long kGridBarrierPolls = 1L << 24;
__device__ __forceinline__ bool grid_barrier(unsigned int* count, unsigned int* gen,
                                             int* timeout, long max_polls = kGridBarrierPolls) {
  __shared__ int ok;
  __syncthreads();
  if (flat_tid() == 0) {
    volatile unsigned int* vgen = gen;
    const unsigned int g = *vgen;
    __threadfence();
    int good = 1;
    if (atomicAdd(count, 1u) + 1u == (unsigned int)flat_nblocks()) {
      atomicExch(count, 0u);
      __threadfence();
      atomicAdd(gen, 1u);
    } else {
      for (long q = 0; *vgen == g; ++q) {
        if (q >= max_polls) {
          good = 0;
          atomicExch(timeout, 1);
          break;
        }
        if (q >= 256) __nanosleep(100);  // poll at once first: most waits are short
      }
      __threadfence();
    }
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// Grid-wide max through per-block partials (NaN-ignoring, as std::max/std::min with a NaN
// second argument keep the first).  Same last-block contract as grid_sum.
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ bool grid_max(double v, double* partials, unsigned int* arrive, double* tot) {
  __shared__ double sh[32];
  __shared__ unsigned int ticket;
  const int tid = flat_tid(), lane = tid & 31, wid = tid >> 5, nw = flat_nthreads() >> 5;
  const int bid = flat_bid(), nb = flat_nblocks();
  v = warp_max(v);
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    double t = lane < nw ? sh[lane] : -INFINITY;
    t = warp_max(t);
    if (lane == 0) {
      partials[bid] = t;
      __threadfence();
      ticket = atomicAdd(arrive, 1u);
    }
  }
  __syncthreads();
  if (ticket != (unsigned)(nb - 1)) return false;
  __threadfence();
  double acc = -INFINITY;
  for (int b = tid; b < nb; b += flat_nthreads()) acc = fmax(acc, __ldcg(&partials[b]));
  acc = warp_max(acc);
  __syncthreads();
  if (lane == 0) sh[wid] = acc;
  __syncthreads();
  if (tid == 0) {
    double t = -INFINITY;
    for (int q = 0; q < nw; ++q) t = fmax(t, sh[q]);
    *tot = t;
    *arrive = 0u;
  }
  return true;
}

}  // namespace fg
