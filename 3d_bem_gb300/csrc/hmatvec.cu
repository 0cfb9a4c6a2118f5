// hmatvec.cu -- K5: H-matrix times a block of R vectors, y = beta*y + H x.
//
// Reference: HArithm::MVM (HMatrix/harithm.cpp:3-28) loops over the partition
// and scatters each block's U(s o (V^T x)) or F x into y under an omp critical.
// Here the product runs in two passes with no atomics and a fixed summation
// order:
//   pass V: t_b = s_b o (V_b x_C) for every admissible block (one CTA each);
//   pass U: one CTA per leaf row cluster sums, for its rows, every block whose
//           row range contains them (U_b rows . t_b and dense F_b rows . x_C).
// Every stored matrix entry is read once per call for all R vectors.
//
// Arithmetic variants (GB300's FP64 rate is far below what HBM can feed):
//   double2 storage, FP64 math  -- the plain complex-FP64 method;
//   float2 storage,  FP64 math  -- exact products of the stored operator, used
//                                  for the iterative-refinement residual;
//   float2 storage,  FP32 math  -- FP32 products inside a block, FP64 sums
//                                  across blocks; the inner GMRES operator.
#include <mutex>

#include "bem_kernels.h"
#include "quadrature.cuh"

namespace bemgpu {
namespace {

constexpr int VT = 128;  // threads of a pass-V CTA
constexpr int UT = 512;  // threads of a pass-U CTA (16 warps split a leaf's block list)
// The FP32 U pass has two launch shapes. With many leaves (at least 4 per SM)
// 256-thread CTAs capped at 40 registers (6 per SM, 48 warps) stream faster:
// 20,480 elements 0.241 -> 0.222 ms per product against 512-thread CTAs with 60
// registers (2 per SM); 128-thread CTAs (0.291 ms) and a 32-register cap
// (0.226 ms, more spills) were slower. With few leaves the 512-thread CTAs
// keep more warps busy: 5,120 elements 0.074 against 0.107 ms, 1,280 elements
// 0.030 against 0.038 ms.
constexpr int UT32_NARROW = 256, UT32_NARROW_MIN_CTAS = 6;
constexpr int UT32_NARROW_LEAVES_PER_SM = 4;
constexpr int UT32_WIDE_R = 256, UT32_WIDE_R_MIN_CTAS = 2;  // R >= 4: up to 128 registers
constexpr int VROWS = 16;  // rows of V per pass-V work item (4 warps x 4 rows)

template <typename T, bool F32> struct Acc;
// FP64 accumulation
template <typename T> struct Acc<T, false> {
  double x = 0, y = 0;
  __device__ __forceinline__ void fma(double2 a, double2 b) {
    x += a.x * b.x - a.y * b.y;
    y += a.x * b.y + a.y * b.x;
  }
};
// FP32 accumulation
template <typename T> struct Acc<T, true> {
  float x = 0, y = 0;
  __device__ __forceinline__ void fma(float2 a, float2 b) {
    x += a.x * b.x - a.y * b.y;
    y += a.x * b.y + a.y * b.x;
  }
};

__device__ __forceinline__ float2 ld32(const float2* p) { return __ldg(p); }

// The block and row range of a pass-V CTA: with a work list, item
// (block, first row) covers up to VROWS rows of V, so the largest blocks are
// spread over many CTAs; without one, a CTA takes a whole block.
__device__ __forceinline__ void vrange(const int2* __restrict__ vwork,
                                       const int32_t* __restrict__ rank, int& b, int& lbeg,
                                       int& lend) {
  if (vwork) {
    const int2 wi = vwork[blockIdx.x];
    b = wi.x;
    lbeg = wi.y;
    lend = min(wi.y + VROWS, rank[b]);
  } else {
    b = blockIdx.x;
    lbeg = 0;
    lend = rank[b];
  }
}
__device__ __forceinline__ float2 tof(double2 v) { return make_float2((float)v.x, (float)v.y); }

// t[r][soff + l] = s_l * sum_j V[l, j] x[c0 + j, r]
template <typename T, bool F32, int R>
__global__ void __launch_bounds__(VT) hmv_vpass(const FarBlock* __restrict__ far,
                                                const int32_t* __restrict__ rank,
                                                const T* __restrict__ Vp,
                                                const T* __restrict__ Sp,
                                                const double2* __restrict__ x, int64_t ldx,
                                                double2* __restrict__ t, int64_t ldt,
                                                const int2* __restrict__ vwork, HmvGate gate) {
  int bi, lbeg, lend;
  vrange(vwork, rank, bi, lbeg, lend);
  if (gate_closed(gate)) lend = lbeg;  // an empty range, not an early return: the
                                       // kernel keeps its load scheduling
  const FarBlock fb = far[bi];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int l = lbeg + w; l < lend; l += VT / 32) {
    const T* Vl = Vp + fb.voff + (int64_t)l * fb.n;
    double ax[R], ay[R];
#pragma unroll
    for (int r = 0; r < R; r++) ax[r] = ay[r] = 0.0;
    if constexpr (F32) {
      float fx[R], fy[R];
#pragma unroll
      for (int r = 0; r < R; r++) fx[r] = fy[r] = 0.0f;
#pragma unroll 4
      for (int j = lane; j < fb.n; j += 32) {
        const float2 v = ld32((const float2*)(Vl + j));
#pragma unroll
        for (int r = 0; r < R; r++) {
          const float2 xv = tof(x[r * ldx + fb.c0 + j]);
          fx[r] += v.x * xv.x - v.y * xv.y;
          fy[r] += v.x * xv.y + v.y * xv.x;
        }
      }
#pragma unroll
      for (int r = 0; r < R; r++) {
        ax[r] = fx[r];
        ay[r] = fy[r];
      }
    } else {
#pragma unroll 4
      for (int j = lane; j < fb.n; j += 32) {
        const double2 v = load_c(Vl + j);
#pragma unroll
        for (int r = 0; r < R; r++) {
          const double2 xv = x[r * ldx + fb.c0 + j];
          ax[r] += v.x * xv.x - v.y * xv.y;
          ay[r] += v.x * xv.y + v.y * xv.x;
        }
      }
    }
#pragma unroll
    for (int r = 0; r < R; r++) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        ax[r] += __shfl_xor_sync(0xffffffffu, ax[r], o);
        ay[r] += __shfl_xor_sync(0xffffffffu, ay[r], o);
      }
    }
    if (lane == 0) {
      const double2 s = load_c(Sp + fb.soff + l);
#pragma unroll
      for (int r = 0; r < R; r++) t[r * ldt + fb.soff + l] = cmul(s, make_double2(ax[r], ay[r]));
    }
  }
}

// One CTA per leaf row cluster; warps split the leaf's block list, lanes own
// rows (32 rows per pass).
template <typename T, bool F32, int R>
__global__ void __launch_bounds__(UT) hmv_upass(
    const LeafRows* __restrict__ leaves, const int32_t* __restrict__ list_off,
    const int32_t* __restrict__ list, const FarBlock* __restrict__ far,
    const int32_t* __restrict__ rank, const NearBlock* __restrict__ nearb,
    const T* __restrict__ Up, const T* __restrict__ F, const double2* __restrict__ x,
    int64_t ldx, const double2* __restrict__ t, int64_t ldt, double2* __restrict__ y,
    int64_t ldy, int accumulate, HmvGate gate) {
  __shared__ double2 part[UT / 32][32];
  LeafRows lf = leaves[blockIdx.x];
  if (gate_closed(gate)) lf.size = 0;  // no rows (see the V pass)
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int beg = list_off[blockIdx.x], end = list_off[blockIdx.x + 1];
  for (int base = 0; base < lf.size; base += 32) {
    const int ri = base + lane;  // row inside the leaf
    const bool active = ri < lf.size;
    const int64_t grow = lf.start + ri;
    double ax[R], ay[R];
#pragma unroll
    for (int r = 0; r < R; r++) ax[r] = ay[r] = 0.0;
    for (int e = beg + w; e < end; e += UT / 32) {
      const int32_t code = list[e];
      Acc<T, F32> acc[R];
      if (code >= 0) {  // admissible block: U rows . t
        const FarBlock fb = far[code];
        const int k = rank[code];
        const T* U = Up + fb.uoff + (grow - fb.r0);
        if (active) {
#pragma unroll 4
          for (int l = 0; l < k; l++) {
            if constexpr (F32) {
              const float2 u = ld32((const float2*)(U + (int64_t)l * fb.m));
#pragma unroll
              for (int r = 0; r < R; r++)
                acc[r].fma(u, tof(t[r * ldt + fb.soff + l]));
            } else {
              const double2 u = load_c(U + (int64_t)l * fb.m);
#pragma unroll
              for (int r = 0; r < R; r++)
                acc[r].fma(u, t[r * ldt + fb.soff + l]);
            }
          }
        }
      } else {  // dense near-field block: F rows . x
        const NearBlock nb = nearb[-code - 1];
        const T* Fb = F + nb.off + (grow - nb.r0);
        if (active) {
#pragma unroll 4
          for (int j = 0; j < nb.n; j++) {
            if constexpr (F32) {
              const float2 f = ld32((const float2*)(Fb + (int64_t)j * nb.m));
#pragma unroll
              for (int r = 0; r < R; r++)
                acc[r].fma(f, tof(x[r * ldx + nb.c0 + j]));
            } else {
              const double2 f = load_c(Fb + (int64_t)j * nb.m);
#pragma unroll
              for (int r = 0; r < R; r++)
                acc[r].fma(f, x[r * ldx + nb.c0 + j]);
            }
          }
        }
      }
#pragma unroll
      for (int r = 0; r < R; r++) {  // block partial into the FP64 row sum
        ax[r] += (double)acc[r].x;
        ay[r] += (double)acc[r].y;
      }
    }
#pragma unroll
    for (int r = 0; r < R; r++) {
      part[w][lane] = make_double2(ax[r], ay[r]);
      __syncthreads();
      if (w == 0 && active) {
        double2 s = part[0][lane];
#pragma unroll
        for (int q = 1; q < UT / 32; q++) s = cadd(s, part[q][lane]);
        double2* yp = y + r * ldy + grow;
        *yp = accumulate ? cadd(*yp, s) : s;
      }
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------
// FP32-arithmetic variant (complex-FP32 storage): x and t travel as FP32, the
// block partials are added across blocks with a compensated (two-sum) FP32
// accumulator, so no instruction of the inner loops touches the FP64 pipe.
// ---------------------------------------------------------------------------
struct TwoSum {
  float hi = 0, lo = 0;
  __device__ __forceinline__ void add(float v) {
    const float s = hi + v;
    const float bp = s - hi;
    lo += (hi - (s - bp)) + (v - bp);
    hi = s;
  }
};

template <int R>
__global__ void __launch_bounds__(VT) hmv32_vpass(const FarBlock* __restrict__ far,
                                                  const int32_t* __restrict__ rank,
                                                  const float2* __restrict__ Vp,
                                                  const float2* __restrict__ Sp,
                                                  const float2* __restrict__ x, int64_t ldx,
                                                  float2* __restrict__ t, int64_t ldt,
                                                  const int2* __restrict__ vwork, HmvGate gate) {
  int bi, lbeg, lend;
  vrange(vwork, rank, bi, lbeg, lend);
  if (gate_closed(gate)) lend = lbeg;  // an empty range, not an early return: the
                                       // kernel keeps its load scheduling
  const FarBlock fb = far[bi];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // each warp streams G rows of V at once (G independent loads in flight per
  // lane; short rows would otherwise leave one load per reduction chain)
  constexpr int G = 4;
  for (int l0 = lbeg + w * G; l0 < lend; l0 += (VT / 32) * G) {
    const int ng = min(G, lend - l0);
    const float2* V0 = Vp + fb.voff + (int64_t)l0 * fb.n;
    float fx[G][R], fy[G][R];
#pragma unroll
    for (int g = 0; g < G; g++)
#pragma unroll
      for (int r = 0; r < R; r++) fx[g][r] = fy[g][r] = 0.0f;
    for (int j = lane; j < fb.n; j += 32) {
      float2 v[G];
#pragma unroll
      for (int g = 0; g < G; g++) v[g] = g < ng ? __ldg(V0 + (int64_t)g * fb.n + j) : make_float2(0, 0);
#pragma unroll
      for (int r = 0; r < R; r++) {
        const float2 xv = __ldg(x + r * ldx + fb.c0 + j);
#pragma unroll
        for (int g = 0; g < G; g++) {
          fx[g][r] += v[g].x * xv.x - v[g].y * xv.y;
          fy[g][r] += v[g].x * xv.y + v[g].y * xv.x;
        }
      }
    }
#pragma unroll
    for (int g = 0; g < G; g++)
#pragma unroll
      for (int r = 0; r < R; r++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          fx[g][r] += __shfl_xor_sync(0xffffffffu, fx[g][r], o);
          fy[g][r] += __shfl_xor_sync(0xffffffffu, fy[g][r], o);
        }
      }
    if (lane < ng) {
#pragma unroll
      for (int g = 0; g < G; g++) {
        if (g != lane) continue;  // lane g writes row l0 + g
        const float2 s = __ldg(Sp + fb.soff + l0 + g);
#pragma unroll
        for (int r = 0; r < R; r++)
          t[r * ldt + fb.soff + l0 + g] = fmul(s, make_float2(fx[g][r], fy[g][r]));
      }
    }
  }
}

template <int R, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) hmv32_upass(
    const LeafRows* __restrict__ leaves, const int32_t* __restrict__ list_off,
    const int32_t* __restrict__ list, const FarBlock* __restrict__ far,
    const int32_t* __restrict__ rank, const NearBlock* __restrict__ nearb,
    const float2* __restrict__ Up, const float2* __restrict__ F, const float2* __restrict__ x,
    int64_t ldx, const float2* __restrict__ t, int64_t ldt, double2* __restrict__ y,
    int64_t ldy, int accumulate, HmvGate gate) {
  __shared__ float4 part[NT / 32][32];
  LeafRows lf = leaves[blockIdx.x];
  if (gate_closed(gate)) lf.size = 0;  // no rows (see the V pass)
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int beg = list_off[blockIdx.x], end = list_off[blockIdx.x + 1];
  for (int base = 0; base < lf.size; base += 32) {
    const int ri = base + lane;
    const bool active = ri < lf.size;
    const int64_t grow = lf.start + ri;
    TwoSum sx[R], sy[R];
    for (int e = beg + w; e < end; e += NT / 32) {
      const int32_t code = list[e];
      float ax[R], ay[R];
#pragma unroll
      for (int r = 0; r < R; r++) ax[r] = ay[r] = 0.0f;
      if (code >= 0) {
        const FarBlock fb = far[code];
        const int k = rank[code];
        const float2* U = Up + fb.uoff + (grow - fb.r0);
        if (active) {
#pragma unroll 4
          for (int l = 0; l < k; l++) {
            const float2 u = __ldg(U + (int64_t)l * fb.m);
#pragma unroll
            for (int r = 0; r < R; r++) {
              const float2 tv = __ldg(t + r * ldt + fb.soff + l);
              ax[r] += u.x * tv.x - u.y * tv.y;
              ay[r] += u.x * tv.y + u.y * tv.x;
            }
          }
        }
      } else {
        const NearBlock nb = nearb[-code - 1];
        const float2* Fb = F + nb.off + (grow - nb.r0);
        if (active) {
#pragma unroll 4
          for (int j = 0; j < nb.n; j++) {
            const float2 f = __ldg(Fb + (int64_t)j * nb.m);
#pragma unroll
            for (int r = 0; r < R; r++) {
              const float2 xv = __ldg(x + r * ldx + nb.c0 + j);
              ax[r] += f.x * xv.x - f.y * xv.y;
              ay[r] += f.x * xv.y + f.y * xv.x;
            }
          }
        }
      }
#pragma unroll
      for (int r = 0; r < R; r++) {
        sx[r].add(ax[r]);
        sy[r].add(ay[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < R; r++) {
      part[w][lane] = make_float4(sx[r].hi, sx[r].lo, sy[r].hi, sy[r].lo);
      __syncthreads();
      if (w == 0 && active) {
        TwoSum ux, uy;  // combine the warps' partials in FP32, then one FP64 add
#pragma unroll
        for (int q = 0; q < NT / 32; q++) {
          const float4 p = part[q][lane];
          ux.add(p.x);
          ux.add(p.y);
          uy.add(p.z);
          uy.add(p.w);
        }
        const double2 v = make_double2((double)ux.hi + (double)ux.lo, (double)uy.hi + (double)uy.lo);
        double2* yp = y + r * ldy + grow;
        *yp = accumulate ? cadd(*yp, v) : v;
      }
      __syncthreads();
    }
  }
}

__global__ void to_float_kernel(const double2* __restrict__ x, float2* __restrict__ xf,
                                int64_t n, HmvGate gate) {
  const int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x;
  if (i < n && !gate_closed(gate)) xf[i] = make_float2((float)x[i].x, (float)x[i].y);
}

// streaming multiprocessors of the current device (cached per device)
int sm_count() {
  static int cached[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (!cached[dev]) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 152;
    cached[dev] = n;
  }
  return cached[dev];
}

template <int R>
void launch32_r(const HmvArgs& a, cudaStream_t s) {
  to_float_kernel<<<(unsigned)((a.ldx * R + 255) / 256), 256, 0, s>>>(a.x, a.xf, a.ldx * R,
                                                                      a.gate);
  const int64_t nv = a.vwork ? a.nvwork : a.nfar;
  if (nv > 0)
    hmv32_vpass<R><<<(unsigned)nv, VT, 0, s>>>(a.far, a.rank, (const float2*)a.V,
                                               (const float2*)a.S, a.xf, a.ldx, a.tf, a.ldt,
                                               a.vwork, a.gate);
  if (a.nleaves > 0) {
    if (R >= 4)  // many right-hand sides: their accumulators need the registers
                 // (the 40-register narrow shape spilled ~0.9 KB a thread at R = 8)
      hmv32_upass<R, UT32_WIDE_R, UT32_WIDE_R_MIN_CTAS><<<(unsigned)a.nleaves, UT32_WIDE_R, 0, s>>>(
          a.leaves, a.list_off, a.list, a.far, a.rank, a.nearb, (const float2*)a.U,
          (const float2*)a.F, a.xf, a.ldx, a.tf, a.ldt, a.y, a.ldy, a.accumulate, a.gate);
    else if (a.nleaves >= (int64_t)UT32_NARROW_LEAVES_PER_SM * sm_count())
      hmv32_upass<R, UT32_NARROW, UT32_NARROW_MIN_CTAS><<<(unsigned)a.nleaves, UT32_NARROW, 0, s>>>(
          a.leaves, a.list_off, a.list, a.far, a.rank, a.nearb, (const float2*)a.U,
          (const float2*)a.F, a.xf, a.ldx, a.tf, a.ldt, a.y, a.ldy, a.accumulate, a.gate);
    else
      hmv32_upass<R, UT, 2><<<(unsigned)a.nleaves, UT, 0, s>>>(
          a.leaves, a.list_off, a.list, a.far, a.rank, a.nearb, (const float2*)a.U,
          (const float2*)a.F, a.xf, a.ldx, a.tf, a.ldt, a.y, a.ldy, a.accumulate, a.gate);
  }
}

void launch32(const HmvArgs& a, cudaStream_t s) {
  switch (a.nrhs) {
    case 1: launch32_r<1>(a, s); break;
    case 2: launch32_r<2>(a, s); break;
    case 3: launch32_r<3>(a, s); break;
    case 4: launch32_r<4>(a, s); break;
    case 5: launch32_r<5>(a, s); break;
    case 6: launch32_r<6>(a, s); break;
    case 7: launch32_r<7>(a, s); break;
    default: launch32_r<8>(a, s); break;
  }
}

template <typename T, bool F32, int R>
void launch_r(const HmvArgs& a, cudaStream_t s) {
  const int64_t nv = a.vwork ? a.nvwork : a.nfar;
  if (nv > 0)
    hmv_vpass<T, F32, R><<<(unsigned)nv, VT, 0, s>>>(a.far, a.rank, (const T*)a.V,
                                                     (const T*)a.S, a.x, a.ldx, a.t, a.ldt,
                                                     a.vwork, a.gate);
  if (a.nleaves > 0)
    hmv_upass<T, F32, R><<<(unsigned)a.nleaves, UT, 0, s>>>(
        a.leaves, a.list_off, a.list, a.far, a.rank, a.nearb, (const T*)a.U, (const T*)a.F, a.x,
        a.ldx, a.t, a.ldt, a.y, a.ldy, a.accumulate, a.gate);
}

template <typename T, bool F32>
void launch_t(const HmvArgs& a, cudaStream_t s) {
  switch (a.nrhs) {
    case 1: launch_r<T, F32, 1>(a, s); break;
    case 2: launch_r<T, F32, 2>(a, s); break;
    case 3: launch_r<T, F32, 3>(a, s); break;
    case 4: launch_r<T, F32, 4>(a, s); break;
    case 5: launch_r<T, F32, 5>(a, s); break;
    case 6: launch_r<T, F32, 6>(a, s); break;
    case 7: launch_r<T, F32, 7>(a, s); break;
    default: launch_r<T, F32, 8>(a, s); break;  // the runtime splits R > 8 into chunks of 8
  }
}
}  // namespace

// ---------------------------------------------------------------------------
// Double-float variant (complex-FP32 storage): FP64-accurate products of the
// stored operator computed on the FP32 units. x and t are unevaluated sums
// hi + lo of two floats; each stored entry a (exact in FP32) times hi is
// split exactly with an FMA (p + e = a * hi), and sums run in two-float
// precision (~2^-48). Used for the iterative-refinement residual b - A x,
// which needs ~1e-14 relative accuracy but would be FP64-pipe-bound in
// native FP64 on GB300.
// ---------------------------------------------------------------------------
struct DF {
  float hi = 0, lo = 0;
  // this += a * (yh + yl), a exact
  __device__ __forceinline__ void fma(float a, float yh, float yl) {
    const float p = a * yh;
    const float ep = fmaf(a, yh, -p);
    const float s = hi + p;
    const float bb = s - hi;
    const float e = (hi - (s - bb)) + (p - bb);
    lo += e + ep + a * yl;
    hi = s;
  }
  __device__ __forceinline__ void add(float h2, float l2) {
    const float s = hi + h2;
    const float bb = s - hi;
    const float e = (hi - (s - bb)) + (h2 - bb);
    lo += e + l2;
    hi = s;
  }
  __device__ __forceinline__ void shfl_reduce() {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float h2 = __shfl_xor_sync(0xffffffffu, hi, o);
      const float l2 = __shfl_xor_sync(0xffffffffu, lo, o);
      add(h2, l2);
    }
  }
};

// complex df accumulator: re + i im
struct CDF {
  DF re, im;
  // += a * y, a = (ax, ay) exact floats, y = (yrh + yrl) + i (yih + yil)
  __device__ __forceinline__ void fma(float2 a, float4 y) {
    re.fma(a.x, y.x, y.y);
    re.fma(-a.y, y.z, y.w);
    im.fma(a.x, y.z, y.w);
    im.fma(a.y, y.x, y.y);
  }
};

__global__ void to_df_kernel(const double2* __restrict__ x, float4* __restrict__ xd, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  const double2 v = x[i];
  const float rh = (float)v.x, ih = (float)v.y;
  xd[i] = make_float4(rh, (float)(v.x - (double)rh), ih, (float)(v.y - (double)ih));
}

// t[r][soff + l] = s_l * sum_j V[l, j] x[c0 + j, r], all in two-float
template <int R>
__global__ void __launch_bounds__(VT) hmvdf_vpass(const FarBlock* __restrict__ far,
                                                  const int32_t* __restrict__ rank,
                                                  const float2* __restrict__ Vp,
                                                  const float2* __restrict__ Sp,
                                                  const float4* __restrict__ x, int64_t ldx,
                                                  float4* __restrict__ t, int64_t ldt,
                                                  const int2* __restrict__ vwork) {
  int bi, lbeg, lend;
  vrange(vwork, rank, bi, lbeg, lend);
  const FarBlock fb = far[bi];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int l = lbeg + w; l < lend; l += VT / 32) {
    const float2* Vl = Vp + fb.voff + (int64_t)l * fb.n;
    CDF acc[R];
#pragma unroll 2
    for (int j = lane; j < fb.n; j += 32) {
      const float2 v = __ldg(Vl + j);
#pragma unroll
      for (int r = 0; r < R; r++) acc[r].fma(v, __ldg(x + r * ldx + fb.c0 + j));
    }
    const float2 s = __ldg(Sp + fb.soff + l);
#pragma unroll
    for (int r = 0; r < R; r++) {
      acc[r].re.shfl_reduce();
      acc[r].im.shfl_reduce();
      if (lane == 0) {
        // (s) * (re + i im): s exact floats
        CDF o;
        o.fma(s, make_float4(acc[r].re.hi, acc[r].re.lo, acc[r].im.hi, acc[r].im.lo));
        t[r * ldt + fb.soff + l] = make_float4(o.re.hi, o.re.lo, o.im.hi, o.im.lo);
      }
    }
  }
}

template <int R>
__global__ void __launch_bounds__(UT) hmvdf_upass(
    const LeafRows* __restrict__ leaves, const int32_t* __restrict__ list_off,
    const int32_t* __restrict__ list, const FarBlock* __restrict__ far,
    const int32_t* __restrict__ rank, const NearBlock* __restrict__ nearb,
    const float2* __restrict__ Up, const float2* __restrict__ F, const float2* __restrict__ Flo,
    const float4* __restrict__ x, int64_t ldx, const float4* __restrict__ t, int64_t ldt,
    double2* __restrict__ y, int64_t ldy, int accumulate) {
  __shared__ float4 part[UT / 32][32];
  const LeafRows lf = leaves[blockIdx.x];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int beg = list_off[blockIdx.x], end = list_off[blockIdx.x + 1];
  for (int base = 0; base < lf.size; base += 32) {
    const int ri = base + lane;
    const bool active = ri < lf.size;
    const int64_t grow = lf.start + ri;
    CDF acc[R];
    for (int e = beg + w; e < end; e += UT / 32) {
      const int32_t code = list[e];
      if (!active) continue;
      if (code >= 0) {
        const FarBlock fb = far[code];
        const int k = rank[code];
        const float2* U = Up + fb.uoff + (grow - fb.r0);
#pragma unroll 2
        for (int l = 0; l < k; l++) {
          const float2 u = __ldg(U + (int64_t)l * fb.m);
#pragma unroll
          for (int r = 0; r < R; r++) acc[r].fma(u, __ldg(t + r * ldt + fb.soff + l));
        }
      } else {
        const NearBlock nb = nearb[-code - 1];
        const float2* Fb = F + nb.off + (grow - nb.r0);
        if (Flo) {  // FP64 entries as hi + lo
          const float2* Lb = Flo + nb.off + (grow - nb.r0);
          for (int j = 0; j < nb.n; j++) {
            const float2 f = __ldg(Fb + (int64_t)j * nb.m), fl = __ldg(Lb + (int64_t)j * nb.m);
#pragma unroll
            for (int r = 0; r < R; r++) {
              const float4 xv = __ldg(x + r * ldx + nb.c0 + j);
              acc[r].fma(f, xv);
              acc[r].fma(fl, xv);
            }
          }
        } else {
#pragma unroll 2
          for (int j = 0; j < nb.n; j++) {
            const float2 f = __ldg(Fb + (int64_t)j * nb.m);
#pragma unroll
            for (int r = 0; r < R; r++) acc[r].fma(f, __ldg(x + r * ldx + nb.c0 + j));
          }
        }
      }
    }
#pragma unroll
    for (int r = 0; r < R; r++) {
      part[w][lane] = make_float4(acc[r].re.hi, acc[r].re.lo, acc[r].im.hi, acc[r].im.lo);
      __syncthreads();
      if (w == 0 && active) {
        CDF sum;
#pragma unroll
        for (int q = 0; q < UT / 32; q++) {
          const float4 p = part[q][lane];
          sum.re.add(p.x, p.y);
          sum.im.add(p.z, p.w);
        }
        const double2 v = make_double2((double)sum.re.hi + (double)sum.re.lo,
                                       (double)sum.im.hi + (double)sum.im.lo);
        double2* yp = y + r * ldy + grow;
        *yp = accumulate ? cadd(*yp, v) : v;
      }
      __syncthreads();
    }
  }
}

template <int R>
void launchdf_r(const HmvArgs& a, cudaStream_t s) {
  float4* xd = (float4*)a.xf;
  float4* td = (float4*)a.tf;
  to_df_kernel<<<(unsigned)((a.ldx * R + 255) / 256), 256, 0, s>>>(a.x, xd, a.ldx * R);
  const int64_t nv = a.vwork ? a.nvwork : a.nfar;
  if (nv > 0)
    hmvdf_vpass<R><<<(unsigned)nv, VT, 0, s>>>(a.far, a.rank, (const float2*)a.V,
                                               (const float2*)a.S, xd, a.ldx, td, a.ldt,
                                               a.vwork);
  if (a.nleaves > 0)
    hmvdf_upass<R><<<(unsigned)a.nleaves, UT, 0, s>>>(
        a.leaves, a.list_off, a.list, a.far, a.rank, a.nearb, (const float2*)a.U,
        (const float2*)a.F, (const float2*)a.Flo, xd, a.ldx, td, a.ldt, a.y, a.ldy, a.accumulate);
}

void launchdf(const HmvArgs& a, cudaStream_t s) {
  switch (a.nrhs) {
    case 1: launchdf_r<1>(a, s); break;
    case 2: launchdf_r<2>(a, s); break;
    case 3: launchdf_r<3>(a, s); break;
    case 4: launchdf_r<4>(a, s); break;
    default: launchdf_r<4>(a, s); break;  // the runtime passes at most 4 per pass
  }
}

// ---------------------------------------------------------------------------
// Fixed scratch for bem_hmatvec_noalloc: the per-block projections t = s o (V x)
// of one pass (ldt x nrhs complex FP64 values) live in this file-scope device
// array instead of a cudaMalloc'd buffer. Every GPU that loads the library
// holds it (32 MiB) until the process exits; all calls share it, so calls that
// overlap on the GPU race. Nothing in it needs clearing: pass V writes every
// entry pass U reads.
// ---------------------------------------------------------------------------
static __device__ __align__(256) double2 g_noalloc_t[HMV_NOALLOC_SCRATCH];

int64_t hmatvec_noalloc_capacity() { return HMV_NOALLOC_SCRATCH; }

// Device address of the scratch array on the current device. The first call
// on each device looks it up (cudaGetSymbolAddress, with that device current);
// later calls reuse the cached address. The cache is keyed by device ordinal,
// i.e. it assumes the device's primary context (the one the CUDA runtime
// uses): after cudaDeviceReset, or under a driver-API context of its own, the
// cached address no longer belongs to the current context.
cudaError_t hmatvec_noalloc_scratch(double2** out) {
  static std::mutex mu;
  static void* addr[256] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 256) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_t);
    if (e != cudaSuccess) return e;
    addr[dev] = p;
  }
  *out = static_cast<double2*>(addr[dev]);
  return cudaSuccess;
}

int launch_hmatvec(const HmvArgs& a, cudaStream_t s) {
  if (a.precision == 0) launch_t<double2, false>(a, s);
  else if (a.fp32_math == 1) {
    launch32(a, s);
    return 1 + (a.nfar > 0) + (a.nleaves > 0);
  } else if (a.fp32_math == 2) {
    launchdf(a, s);
    return 1 + (a.nfar > 0) + (a.nleaves > 0);
  } else launch_t<float2, false>(a, s);
  return (a.nfar > 0) + (a.nleaves > 0);
}

}  // namespace bemgpu
