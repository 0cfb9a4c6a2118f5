// hlu_solve.cu -- K7: the H-LU preconditioner's forward and backward
// block-triangular solves, x = U^{-1} L^{-1} b, for R right-hand sides.
//
// Reference: HArithm::forwardSubstitution / backwardSubstitution
// (HMatrix/harithm.cpp:1314-1340, :1386-1412), called twice per GMRES
// iteration by LUPrecondidionedHMatrixWrapper (HMatrix/gmres.h:134-147). The
// recursion is flattened on the host into a schedule of leaf operations in
// exactly the reference's order: a diagonal leaf (QR leaf: y = Q^H w forward,
// R x = w backward) or an off-diagonal leaf (w_rows -= B x_cols, B full or
// low rank). Each diagonal leaf depends on every earlier one, so one CTA per
// right-hand side walks the schedule; the 16 warps share each operation.
// Complex FP64 throughout (the pivot blocks of the preconditioner).
#include "bem_kernels.h"
#include "hlu_solve.h"
#include "quadrature.cuh"

namespace bemgpu {
namespace {

constexpr int HT = 512;
constexpr int HW = HT / 32;

__device__ __forceinline__ double2 warp_sum2(double2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}

// w: right-hand sides (consumed), x: solution, both R x N
__global__ void __launch_bounds__(HT) hlu_sweep_kernel(const int32_t* __restrict__ sched,
                                                       int nops, const int64_t* __restrict__ lv,
                                                       const double2* __restrict__ data,
                                                       double2* __restrict__ w,
                                                       double2* __restrict__ x, int64_t N,
                                                       int upper) {
  __shared__ double2 tk[HLU_MAX_RANK];
  __shared__ double2 xs[HLU_MAX_LEAF];
  double2* wr = w + (int64_t)blockIdx.x * N;
  double2* xr = x + (int64_t)blockIdx.x * N;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int o = 0; o < nops; o++) {
    const int op = sched[o];
    if (op >= 0) {  // diagonal leaf
      const int64_t* L = lv + 7 * (int64_t)op;
      const int64_t r0 = L[0];
      const int m = (int)L[1];
      const double2* D = data + L[6];
      if (!upper) {  // y = Q^H w (Q column-major m x m)
        for (int i = tid; i < m; i += HT) {
          double2 s = make_double2(0, 0);
          const double2* q = D + (int64_t)i * m;  // column i of Q
          for (int t = 0; t < m; t++) {
            const double2 a = q[t], b = wr[r0 + t];  // conj(a) * b
            s.x += a.x * b.x + a.y * b.y;
            s.y += a.x * b.y - a.y * b.x;
          }
          xr[r0 + i] = s;
        }
      } else {  // R x = w, R upper triangular: back substitution by warp 0
        if (warp == 0) {
          for (int i = lane; i < m; i += 32) xs[i] = wr[r0 + i];
          __syncwarp();
          for (int i = m - 1; i >= 0; i--) {
            double2 s = make_double2(0, 0);
            for (int t = i + 1 + lane; t < m; t += 32) s = cadd(s, cmul(D[(int64_t)t * m + i], xs[t]));
            s = warp_sum2(s);
            if (lane == 0) xs[i] = cdiv(csub(xs[i], s), D[(int64_t)i * m + i]);
            __syncwarp();
          }
          for (int i = lane; i < m; i += 32) xr[r0 + i] = xs[i];
        }
      }
    } else {  // off-diagonal leaf: w_rows -= B x_cols
      const int64_t* L = lv + 7 * (int64_t)(-op - 1);
      const int64_t r0 = L[0], c0 = L[2];
      const int m = (int)L[1], n = (int)L[3], kind = (int)L[4], k = (int)L[5];
      const double2* D = data + L[6];
      if (kind == 0) {  // full, column-major m x n: one warp per row, lanes over columns
        for (int i = warp; i < m; i += HW) {
          double2 s = make_double2(0, 0);
          for (int j = lane; j < n; j += 32) s = cadd(s, cmul(D[(int64_t)j * m + i], xr[c0 + j]));
          s = warp_sum2(s);
          if (lane == 0) wr[r0 + i] = csub(wr[r0 + i], s);
        }
      } else {  // low rank: U (m x k col-major), V (k x n row-major)
        const double2* U = D;
        const double2* V = D + (int64_t)m * k;
        for (int l = warp; l < k; l += HW) {
          double2 s = make_double2(0, 0);
          for (int j = lane; j < n; j += 32) s = cadd(s, cmul(V[(int64_t)l * n + j], xr[c0 + j]));
          s = warp_sum2(s);
          if (lane == 0) tk[l] = s;
        }
        __syncthreads();
        for (int i = tid; i < m; i += HT) {
          double2 s = make_double2(0, 0);
          for (int l = 0; l < k; l++) s = cadd(s, cmul(U[(int64_t)l * m + i], tk[l]));
          wr[r0 + i] = csub(wr[r0 + i], s);
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace

int launch_hlu_sweep(const int32_t* sched, int nops, const int64_t* leaves, const double2* data,
                     double2* w, double2* x, int64_t N, int R, int upper, cudaStream_t s) {
  if (nops <= 0 || R <= 0) return 0;
  hlu_sweep_kernel<<<(unsigned)R, HT, 0, s>>>(sched, nops, leaves, data, w, x, N, upper);
  return 1;
}

}  // namespace bemgpu
