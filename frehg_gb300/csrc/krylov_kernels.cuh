// Declarations of the Krylov kernels defined in krylov.cu, for launches from other files.
#pragma once

#include "internal.h"

namespace fg {
__global__ void k_diag_rsqrt(double* __restrict__ s, size_t n);
__global__ void k_scale_offdiag(double* __restrict__ a0, double* __restrict__ a1,
                                double* __restrict__ a2, const double* __restrict__ s, int n0,
                                int n1, int n2, int planes, int tiles);
__global__ void k_cg_init(const double* __restrict__ s, const double* __restrict__ b,
                          double* __restrict__ x, double* __restrict__ r, size_t n,
                          CgDevState* st, double* partials);
__global__ void k_cg_p(const double* __restrict__ r, double* __restrict__ p, size_t n,
                       const CgDevState* st);
__global__ void __launch_bounds__(256) k_cg_spmv(const double* __restrict__ a0,
                                                 const double* __restrict__ a1,
                                                 const double* __restrict__ a2,
                                                 const double* __restrict__ p,
                                                 double* __restrict__ w, int n0, int n1, int n2,
                                                 int planes, int tiles, CgDevState* st,
                                                 double* partials);
__global__ void k_cg_update(double* __restrict__ x, double* __restrict__ r,
                            const double* __restrict__ p, const double* __restrict__ w,
                            const double* __restrict__ s, size_t n, CgDevState* st,
                            double* partials);
__global__ void k_unscale(const double* __restrict__ s, const double* __restrict__ xs,
                          double* __restrict__ x, size_t n);
}  // namespace fg
