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
// right-hand side walks the schedule; its 16 warps share each operation with
// coalesced reads of the leaf (warp per Q column / V row, lanes over
// contiguous entries; threads over rows of column-major full and U blocks).
//
// Precision follows the factors' storage: complex FP64 factors (plain
// method) in FP64, complex FP32 factors (mixed method: the preconditioner
// only steers GMRES, the FP64 refinement residual keeps the accuracy) in
// FP32 arithmetic, which is what GB300 runs fast -- its FP64 rate would make
// each 32 x 32 leaf cost ~1 us on one SM. The vectors stay complex FP64.
#include "bem_kernels.h"
#include "hlu_solve.h"
#include "quadrature.cuh"

namespace bemgpu {
namespace {

constexpr int HT = 512;
constexpr int HW = HT / 32;

template <typename T2> struct HC;
template <> struct HC<double2> {
  using R = double;
  static __device__ __forceinline__ double2 ld(const double2* p) { return *p; }
};
template <> struct HC<float2> {
  using R = float;
  static __device__ __forceinline__ float2 ld(const float2* p) { return __ldg(p); }
};

template <typename R>
__device__ __forceinline__ R wsum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// w: right-hand sides (consumed), x: solution, both R x N, complex FP64
template <typename T2>
__global__ void __launch_bounds__(HT) hlu_sweep_kernel(const int32_t* __restrict__ sched,
                                                       int nops, const int64_t* __restrict__ lv,
                                                       const T2* __restrict__ data,
                                                       double2* __restrict__ w,
                                                       double2* __restrict__ x, int64_t N,
                                                       int upper) {
  using R = typename HC<T2>::R;
  __shared__ R tkx[HLU_MAX_RANK], tky[HLU_MAX_RANK];
  __shared__ R xsx[HLU_MAX_LEAF], xsy[HLU_MAX_LEAF];
  __shared__ R px[HW][32], py[HW][32];
  double2* wr = w + (int64_t)blockIdx.x * N;
  double2* xr = x + (int64_t)blockIdx.x * N;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int o = 0; o < nops; o++) {
    const int op = sched[o];
    if (op >= 0) {  // diagonal leaf
      const int64_t* L = lv + 7 * (int64_t)op;
      const int64_t r0 = L[0];
      const int m = (int)L[1];
      const T2* D = data + L[6];
      if (!upper) {  // x_i = (Q^H w)_i = sum_t conj(Q[t, i]) w_t: warp per i, lanes over t
        for (int i = warp; i < m; i += HW) {
          const T2* q = D + (int64_t)i * m;
          R sx = 0, sy = 0;
          for (int t = lane; t < m; t += 32) {
            const T2 a = HC<T2>::ld(q + t);
            const double2 b = wr[r0 + t];
            sx += a.x * (R)b.x + a.y * (R)b.y;
            sy += a.x * (R)b.y - a.y * (R)b.x;
          }
          sx = wsum(sx);
          sy = wsum(sy);
          if (lane == 0) xr[r0 + i] = make_double2((double)sx, (double)sy);
        }
      } else if (warp == 0) {  // R x = w by columns: x_i = w_i / R_ii, then w_t -= R_ti x_i
        for (int i = lane; i < m; i += 32) {
          xsx[i] = (R)wr[r0 + i].x;
          xsy[i] = (R)wr[r0 + i].y;
        }
        __syncwarp();
        for (int i = m - 1; i >= 0; i--) {
          const T2 d = HC<T2>::ld(D + (int64_t)i * m + i);
          // x_i = xs_i / d (all lanes compute the same value)
          const R den = d.x * d.x + d.y * d.y;
          const R ax = xsx[i], ay = xsy[i];
          const R xi = (ax * d.x + ay * d.y) / den, yi = (ay * d.x - ax * d.y) / den;
          __syncwarp();
          const T2* col = D + (int64_t)i * m;
          for (int t = lane; t < i; t += 32) {
            const T2 c = HC<T2>::ld(col + t);
            xsx[t] -= c.x * xi - c.y * yi;
            xsy[t] -= c.x * yi + c.y * xi;
          }
          if (lane == 0) {
            xsx[i] = xi;
            xsy[i] = yi;
          }
          __syncwarp();
        }
        for (int i = lane; i < m; i += 32) xr[r0 + i] = make_double2((double)xsx[i], (double)xsy[i]);
      }
    } else {  // off-diagonal leaf: w_rows -= B x_cols
      const int64_t* L = lv + 7 * (int64_t)(-op - 1);
      const int64_t r0 = L[0], c0 = L[2];
      const int m = (int)L[1], n = (int)L[3], kind = (int)L[4], k = (int)L[5];
      const T2* D = data + L[6];
      if (kind == 0) {
        // full, column-major m x n: 32-row panels; warp w takes columns
        // w, w + 16, ..., lane = row; the 16 partials meet in shared memory
        for (int i0 = 0; i0 < m; i0 += 32) {
          const int i = i0 + lane;
          R sx = 0, sy = 0;
          if (i < m)
            for (int j = warp; j < n; j += HW) {
              const T2 f = HC<T2>::ld(D + (int64_t)j * m + i);
              const double2 xv = xr[c0 + j];
              sx += f.x * (R)xv.x - f.y * (R)xv.y;
              sy += f.x * (R)xv.y + f.y * (R)xv.x;
            }
          px[warp][lane] = sx;
          py[warp][lane] = sy;
          __syncthreads();
          if (warp == 0 && i < m) {
            R ax = 0, ay = 0;
#pragma unroll
            for (int q = 0; q < HW; q++) {
              ax += px[q][lane];
              ay += py[q][lane];
            }
            double2 v = wr[r0 + i];
            v.x -= (double)ax;
            v.y -= (double)ay;
            wr[r0 + i] = v;
          }
          __syncthreads();
        }
      } else {  // low rank: U (m x k col-major), V (k x n row-major)
        const T2* U = D;
        const T2* V = D + (int64_t)m * k;
        for (int l = warp; l < k; l += HW) {
          R sx = 0, sy = 0;
          for (int j = lane; j < n; j += 32) {
            const T2 v = HC<T2>::ld(V + (int64_t)l * n + j);
            const double2 xv = xr[c0 + j];
            sx += v.x * (R)xv.x - v.y * (R)xv.y;
            sy += v.x * (R)xv.y + v.y * (R)xv.x;
          }
          sx = wsum(sx);
          sy = wsum(sy);
          if (lane == 0) {
            tkx[l] = sx;
            tky[l] = sy;
          }
        }
        __syncthreads();
        for (int i = tid; i < m; i += HT) {
          R sx = 0, sy = 0;
          for (int l = 0; l < k; l++) {
            const T2 u = HC<T2>::ld(U + (int64_t)l * m + i);
            sx += u.x * tkx[l] - u.y * tky[l];
            sy += u.x * tky[l] + u.y * tkx[l];
          }
          double2 v = wr[r0 + i];
          v.x -= (double)sx;
          v.y -= (double)sy;
          wr[r0 + i] = v;
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace

int launch_hlu_sweep(const int32_t* sched, int nops, const int64_t* leaves, const void* data,
                     int precision, double2* w, double2* x, int64_t N, int R, int upper,
                     cudaStream_t s) {
  if (nops <= 0 || R <= 0) return 0;
  if (precision == 0)
    hlu_sweep_kernel<double2><<<(unsigned)R, HT, 0, s>>>(sched, nops, leaves, (const double2*)data,
                                                         w, x, N, upper);
  else
    hlu_sweep_kernel<float2><<<(unsigned)R, HT, 0, s>>>(sched, nops, leaves, (const float2*)data,
                                                        w, x, N, upper);
  return 1;
}

}  // namespace bemgpu
