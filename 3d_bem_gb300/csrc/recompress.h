// recompress.h -- launch interface of the truncating SVD recompression kernel.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bem_types.h"

namespace bemgpu {

struct RecompressArgs {
  int precision;            // 0: complex FP64 pools, 1: complex FP32 pools
  const FarBlock* far;
  const int32_t* order;     // far blocks, largest first (may be null)
  int64_t nfar;
  void *U, *V, *S;          // the block pools, rewritten in place
  int32_t* rank;            // per far block, rewritten
  void *wa, *wb;            // scratch with the U / V pool layouts
  void* wc;                 // scratch: 2 k^2 complex per block at coff
  const int64_t* coff;      // complex-element offsets into wc
  int64_t max_rank;         // preconditionerRank-style cap (0: none)
  double tol;               // relative Frobenius tail
};

// Returns the number of kernels launched.
int launch_recompress(const RecompressArgs& a, cudaStream_t s);

}  // namespace bemgpu
