// post.h -- launch interface of the element-wise kernels in post.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bem_types.h"

namespace bemgpu {
int launch_gather(const double2* in, double2* out, const int64_t* perm, int64_t N, int R,
                  cudaStream_t s);
int launch_backsub(const double2* x, const double2* g, const double2* a, const double2* b,
                   const BcCoef* bc, const int64_t* perm, int64_t N, int R, double2 pfac, double2* phi,
                   double2* dphi, double2* p, cudaStream_t s);
int launch_finite_check(const double2* v, int64_t n, int* bad, cudaStream_t s);
}  // namespace bemgpu
