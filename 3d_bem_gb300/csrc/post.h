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
// rhs (N x R, cluster order) += the point sources' source term at every
// collocation point (src: nsrc x 5 doubles on the device)
int launch_source_rhs(const Elem* E, int64_t N, const double* src, int nsrc, double k,
                      double2 alpha, double2* rhs, int R, cudaStream_t s);
}  // namespace bemgpu
