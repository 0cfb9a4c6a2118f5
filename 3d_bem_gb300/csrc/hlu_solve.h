// hlu_solve.h -- launch interface of the H-LU block-triangular solve kernel.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace bemgpu {

constexpr int HLU_MAX_RANK = 512;  // largest low-rank leaf of a factor
constexpr int HLU_MAX_LEAF = 512;  // largest diagonal leaf (leaf_size - 1)

// One sweep over a flattened factor: upper = 0 applies L^{-1} (y = Q^H w on
// diagonal leaves), upper = 1 applies U^{-1}. data holds the factor in complex
// FP64 (precision 0) or complex FP32 (precision 1, FP32 arithmetic). w (R x N,
// complex FP64) is consumed, x gets the result. Returns the kernels launched.
int launch_hlu_sweep(const int32_t* sched, int nops, const int64_t* leaves, const void* data,
                     int precision, double2* w, double2* x, int64_t N, int R, int upper,
                     cudaStream_t s);

}  // namespace bemgpu
