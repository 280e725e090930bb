// Self-check entry points of the elementary functions (fastmath64.cuh, ff32.cuh) and of the
// constitutive evaluations (vg.cuh) (not in reference): they evaluate on host arrays so that a
// test can compare the variants on the device that runs the kernels.
#include "internal.h"
#include "vg.cuh"

#include <cmath>

namespace fg {
namespace {
__device__ __forceinline__ double ff_eval(int fn, double v) {
  const ff x = ff_from_double(v);
  switch (fn) {
    case 8: return ff_to_double(ff_exp(x));
    case 9: return ff_to_double(ff_log(x));
    case 10: return ff_to_double(ff_log1p(x));
    case 11: return ff_to_double(ff_expm1(x));
    case 12: return ff_to_double(x);  // the double -> float-float split and back
    default: return ff_to_double(ff_div(ff_make(1.0f), x));
  }
}

__global__ void k_fastmath_eval(int fn, const double* __restrict__ x, double* __restrict__ y,
                                size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const double v = x[i];
    double r;
    switch (fn) {
      case 0: r = fexp(v); break;
      case 1: r = flog(v); break;
      case 2: r = flog1p(v); break;
      case 3: r = fexpm1(v); break;
      case 4: r = exp(v); break;
      case 5: r = log(v); break;
      case 6: r = log1p(v); break;
      case 7: r = expm1(v); break;
      default: r = ff_eval(fn, v); break;
    }
    y[i] = r;
  }
}

__global__ void k_constit_eval(SoilClass k, int arith, int continuous, const double* __restrict__ h,
                               size_t n, double* __restrict__ kr, double* __restrict__ wc,
                               double* __restrict__ cap) {
  SoilClass* cls = &k;
  SoilView v;
  v.cls = cls;
  v.continuous_theta = continuous;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    Constit r;
    if (arith == 1 && k.use_vg && !k.use_mvg)
      r = vg_constit_ff<true, true>(k, ff_make(k.ff_alpha[0], k.ff_alpha[1]),
                                    continuous ? 0.0 : k.aev, h[i]);
    else
      r = vg_constit<true, true>(soil_of(v, i, 0), h[i]);
    kr[i] = r.kr;
    wc[i] = r.theta;
    cap[i] = r.cap;
  }
}
}  // namespace
}  // namespace fg

extern "C" int frehg_fastmath_eval(int fn, const double* x, double* y, int64_t n) {
  using namespace fg;
  clear_error();
  FG_ARG(x && y && n > 0 && fn >= 0 && fn <= 13, "bad argument");
  double *dx = nullptr, *dy = nullptr;
  const size_t bytes = (size_t)n * sizeof(double);
  int rc = FREHG_OK;
  if (cudaMalloc(&dx, bytes) != cudaSuccess || cudaMalloc(&dy, bytes) != cudaSuccess ||
      cudaMemcpy(dx, x, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = FREHG_ERR_CUDA;
  } else {
    k_fastmath_eval<<<1216, 256>>>(fn, dx, dy, (size_t)n);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpy(y, dy, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = FREHG_ERR_CUDA;
  }
  if (rc != FREHG_OK) set_error("frehg_fastmath_eval: %s", cudaGetErrorString(cudaGetLastError()));
  cudaFree(dx);
  cudaFree(dy);
  return rc;
}

extern "C" int frehg_constit_eval(const frehg_soil_params* soil, int arith, int continuous_theta,
                                  const double* h, int64_t n, double* kr, double* wc,
                                  double* cap) {
  using namespace fg;
  clear_error();
  FG_ARG(soil && h && kr && wc && cap && n > 0 && (arith == 0 || arith == 1), "bad argument");
  const SoilClass k = make_soil_class(*soil);
  double* d = nullptr;
  const size_t bytes = (size_t)n * sizeof(double);
  int rc = FREHG_OK;
  if (cudaMalloc(&d, 4 * bytes) != cudaSuccess ||
      cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = FREHG_ERR_CUDA;
  } else {
    k_constit_eval<<<1216, 256>>>(k, arith, continuous_theta, d, (size_t)n, d + n, d + 2 * n,
                                  d + 3 * n);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpy(kr, d + n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(wc, d + 2 * n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(cap, d + 3 * n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = FREHG_ERR_CUDA;
  }
  if (rc != FREHG_OK) set_error("frehg_constit_eval: %s", cudaGetErrorString(cudaGetLastError()));
  cudaFree(d);
  return rc;
}
