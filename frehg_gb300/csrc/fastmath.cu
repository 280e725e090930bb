// Self-check entry point of the FP64 elementary functions in fastmath64.cuh (not in reference):
// evaluates one of them, or the CUDA math library's counterpart, on host arrays so that a test
// can compare the two on the device that runs the kernels.
#include "fastmath64.cuh"
#include "internal.h"

#include <cmath>

namespace fg {
namespace {
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
      default: r = expm1(v); break;
    }
    y[i] = r;
  }
}
}  // namespace
}  // namespace fg

extern "C" int frehg_fastmath_eval(int fn, const double* x, double* y, int64_t n) {
  using namespace fg;
  clear_error();
  FG_ARG(x && y && n > 0 && fn >= 0 && fn <= 7, "bad argument");
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
