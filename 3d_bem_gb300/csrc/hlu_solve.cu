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

#include <algorithm>
#include <stdexcept>
#include <string>

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


// ---------------------------------------------------------------------------
// Dataflow sweep. Block 0 (the driver) walks the diagonal leaves in solve
// order: s = w(i) - acc(i) - corner(i) x, x(i) = M(i) s with M = Q^H (L) or
// R^{-1} (U), then publishes progress = i + 1. Its inputs for the next step
// (M, the corner leaf's rows and the corner's already solved columns) are
// copied to shared memory with cp.async while the current step runs. A
// low-rank corner's t = V x takes the prefix over the columns before chunk
// i - 2 (pre) and adds chunks i - 2 and i - 1 from the driver's own last two
// results, so no item solved after x(i - 2) sits between two driver steps.
// Blocks 1.. (helpers) claim items in a fixed order, three per level
// L = 0, 1, ...: C(L - 1), E(L + LAG - 1), R(L + 1), where
//   C(j): t partials of the low-rank leaves over cols(j) into pre (through
//         the third-to-last column chunk of a leaf), pre2 (through the
//         second-to-last) or fin (complete), one warp per (leaf, row of V),
//         lanes over the columns; ready when x(j) is solved and C(j - 1) is
//         done;
//   E(i): eacc(i), the contributions of the early leaves to rows(i), one warp
//         per leaf; ready when x(i - LAG) is solved and C(i - LAG) is done,
//         LAG - 2 steps before the driver needs it;
//   R(i): acc(i) = eacc(i) + the late leaves (at most LAG - 2, one warp each,
//         their constants staged in shared memory before the wait); ready
//         when x(i - 2) is solved and C(i - 3) and E(i) are done.
// Every item waits only on progress up to its level and on items earlier in
// the order. Roles follow the order in which blocks start: the first one
// drives, the others claim items in order, so every wait is on a block that
// is already running and the chain advances with any number of resident
// blocks; the launch needs no co-residency and starts on the SMs that are
// free, beside other streams' kernels. Each sum has one fixed order: results do not depend
// on which block ran an item or on the number of helpers. Every wait is
// bounded: after DfArgs::wait_ns the block sets the sticky error word and
// returns.
// All arithmetic and every vector inside the sweep (x, acc, partial sums,
// staging) is in the factor's type T2: complex FP32 for the mixed method,
// whose FP64 rate on GB300 would otherwise bound the sweep through FP64
// conversions and sums; only w is read and x written in complex FP64.
// ---------------------------------------------------------------------------
namespace {

constexpr int DT = 512;  // threads per block
constexpr int NW = DT / 32;
constexpr int DM = HLU_DF_MAX_M, DR = HLU_DF_MAX_R, DK = HLU_DF_MAX_RANK;
constexpr int LAG = HLU_DF_LAG, NLATE = HLU_DF_NLATE;
constexpr int PS = 4;  // column pairs per warp and round in C(j)
constexpr int MS_ELEMS = DM * (DM + 1);  // apply matrix, rows padded
constexpr int CS_ELEMS = 3 * DK * DM;    // corner: F (<= 64 cols x rows) or U rows + V over
                                         // the columns of chunks i - 1 and i - 2
constexpr int BUF_ELEMS = MS_ELEMS + CS_ELEMS;
constexpr int WCOLS = 2 * DM;            // widest staged full leaf (corner, late entries)

#define CUDA_OK(x)                                                                     \
  do {                                                                                 \
    const cudaError_t e_ = (x);                                                        \
    if (e_ != cudaSuccess)                                                             \
      throw std::runtime_error(std::string(#x) + ": " + cudaGetErrorString(e_));      \
  } while (0)

template <typename T2> struct DfT;
template <> struct DfT<double2> { using R = double; };
template <> struct DfT<float2> { using R = float; };

template <typename T2> __device__ __forceinline__ T2 mk(typename DfT<T2>::R x, typename DfT<T2>::R y) {
  T2 t;
  t.x = x;
  t.y = y;
  return t;
}
template <typename T2> __device__ __forceinline__ T2 from_d2(double2 v) {
  return mk<T2>((typename DfT<T2>::R)v.x, (typename DfT<T2>::R)v.y);
}
// s += a b (complex)
template <typename T2> __device__ __forceinline__ void cmac(T2& s, T2 a, T2 b) {
  s.x += a.x * b.x - a.y * b.y;
  s.y += a.x * b.y + a.y * b.x;
}

// dynamic shared memory of one block: the driver's staging (two buffers of M,
// corner data and corner columns), x, s, t and the chunk ring; E's per-warp
// partial sums; R's partials, vectors and constants
template <typename T2>
constexpr size_t df_smem() {
  constexpr size_t drv = 2 * BUF_ELEMS * sizeof(T2) + 2 * WCOLS * DR * sizeof(T2) +
                         3 * DM * DR * sizeof(T2) + DK * DR * sizeof(T2) + 4 * sizeof(HluDfChunk) +
                         NW * 32 * sizeof(T2);
  constexpr size_t ei = NW * DR * 32 * sizeof(T2);
  constexpr size_t ri = NW * DR * 32 * sizeof(T2) + NLATE * WCOLS * DR * sizeof(T2) +
                        NLATE * DK * DR * sizeof(T2) + HLU_DF_STAGE_BYTES;
  return drv > ei ? (drv > ri ? drv : ri) : (ei > ri ? ei : ri);
}

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// 8- or 16-byte asynchronous copy global -> shared
template <typename T>
__device__ __forceinline__ void cp_async(T* dst, const T* src) {
  static_assert(sizeof(T) == 8 || sizeof(T) == 16, "cp.async of 8 or 16 bytes");
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if (sizeof(T) == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}
// loads of vectors written during the launch: L2 only (no stale L1 lines)
__device__ __forceinline__ float2 ldv(const float2* p) { return __ldcg(p); }
__device__ __forceinline__ double2 ldv(const double2* p) { return __ldcg(p); }

// thread 0 only: wait until *p >= v; false (and the error word set) after the
// time limit or when another block already gave up
__device__ bool df_wait(const int* p, int v, int* err, unsigned long long lim) {
  if (ld_acquire(p) >= v) return true;
  const unsigned long long t0 = gtimer();
  for (unsigned it = 1;; it++) {
    if (ld_acquire(p) >= v) return true;
    if ((it & 63) == 1) {  // after the first failed poll, then every 64
      if (ld_acquire(err)) return false;
      if (gtimer() - t0 > lim) {
        atomicCAS(err, 0, 1);
        return false;
      }
    }
  }
}

// thread 0 only: wait until chunks 0 .. v - 1 are solved
struct DfArgs;
__device__ bool df_wait_progress(const DfArgs& a, int v);

// publish: every thread's global writes of this block, then the flag (the
// barrier orders them before thread 0's release store)
__device__ __forceinline__ void df_publish(int* p, int v) {
  __syncthreads();
  if (threadIdx.x == 0) st_release(p, v);
}

template <typename R>
__device__ __forceinline__ R wred(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

struct DfArgs {
  HluDfDev p;
  const int64_t* lv;
  const void* data;
  const double2* w;  // right-hand sides (complex FP64)
  double2* x;        // result (complex FP64)
  void* xi;          // result in the factor type, read by the helpers (== x for FP64)
  void* acc;         // factor type
  void* eacc;
  void* pre;
  void* fin;
  int* ctrl;  // [0] item counter, [1] progress, [2] arrival ticket, then R, C and E done (D each)
  int* err;
  unsigned long long wait_ns;  // bound of one wait
  int64_t N;
  int R;
  HmvGate gate;
  unsigned long long* trace;  // optional: per chunk the driver's phase times (ns)
  __device__ int* flagR(int i) const { return ctrl + 4 + i; }
  __device__ int* flagC(int j) const { return ctrl + 4 + p.D + j; }
  __device__ int* flagE(int i) const { return ctrl + 4 + 2 * p.D + i; }
  // chunk i solved (x(i) published): one flag per chunk, so the items that
  // wait for different chunks poll different lines instead of one counter
  __device__ int* flagX(int i) const { return ctrl + 4 + 3 * p.D + i; }
};

__device__ bool df_wait_progress(const DfArgs& a, int v) {
  return v <= 0 || df_wait(a.flagX(v - 1), 1, a.err, a.wait_ns);
}


// cp.async of step i's inputs: M(i) into Ms (row-major, padded rows); the
// corner leaf's F[rows(i), :] as Cs[c * DM + row] (full, <= WCOLS columns)
// with its solved columns outside chunk i - 1 as xc[c * DR + r], or
// U[rows(i), :] as Cs[l * DM + row] and V[:, cols(i - 1)] as Cs[DK * DM + l * DM + c].
// Issued during step i - 1: the columns outside chunk i - 1 belong to chunks
// <= i - 2, already solved. c and cp are chunks i and i - 1 (shared-memory ring).
template <typename T2>
__device__ void df_stage(const DfArgs& a, const HluDfChunk& c, const HluDfChunk& cp, T2* buf,
                         T2* xc) {
  const int tid = threadIdx.x;
  const int m = c.m;
  const T2* diag = (const T2*)a.p.diag + c.moff;
  for (int e = tid; e < m * m; e += DT) cp_async(buf + (e / m) * (DM + 1) + e % m, diag + e);
  if (c.corner < 0) return;
  const int64_t mL = c.cm, nL = c.cn;
  const int k = c.ck;
  const T2* Dd = (const T2*)a.data + c.cdata;
  T2* Cs = buf + MS_ELEMS;
  if (!(c.cflags & 1)) {
    if (nL > WCOLS) return;
    for (int e = tid; e < m * (int)nL; e += DT) {
      const int row = e % m, cc = e / m;
      cp_async(Cs + cc * DM + row, Dd + c.cro + row + cc * mL);
    }
    if (!(c.cflags & 4))
      for (int e = tid; e < (int)nL * a.R; e += DT) {
        const int cc = e / a.R, r = e % a.R;
        if (cc < c.cco || cc >= c.cco + cp.m)
          cp_async(xc + cc * DR + r, (const T2*)a.xi + (int64_t)r * a.N + c.cc0 + cc);
      }
  } else {
    const int pw = cp.m;
    for (int e = tid; e < m * k; e += DT) {
      const int row = e % m, l = e / m;
      cp_async(Cs + l * DM + row, Dd + c.cro + row + l * mL);
    }
    const T2* V = Dd + mL * k + c.cco;
    for (int e = tid; e < k * pw; e += DT) {
      const int l = e / pw, cc = e % pw;
      cp_async(Cs + DK * DM + l * DM + cc, V + l * nL + cc);
    }
    if (c.cflags & 2) {  // and over cols(i - 2)
      const int w2 = c.cw2;
      const T2* V2 = Dd + mL * k + c.cco2;
      for (int e = tid; e < k * w2; e += DT) {
        const int l = e / w2, cc = e % w2;
        cp_async(Cs + 2 * DK * DM + l * DM + cc, V2 + l * nL + cc);
      }
    }
  }
}

// chunk j of the plan into ring slot j & 3 (five 16-byte copies)
__device__ __forceinline__ void df_ring_load(const DfArgs& a, HluDfChunk* ring, int j) {
  if (threadIdx.x < 5)
    cp_async((int4*)(ring + (j & 3)) + threadIdx.x, (const int4*)(a.p.chunks + j) + threadIdx.x);
}

template <typename T2>
__device__ void df_driver(const DfArgs& a, unsigned char* sm) {
  T2* bufs = (T2*)sm;
  T2* xcs = bufs + 2 * BUF_ELEMS;            // corner columns, 2 buffers [c][r]
  T2* xs2 = xcs + 2 * WCOLS * DR;            // x of the last two chunks, [chunk & 1][c][r]
  T2* ss = xs2 + 2 * DM * DR;                // s, [t][r]
  T2* tks = ss + DM * DR;                    // corner t, [l][r]
  HluDfChunk* ring = (HluDfChunk*)(tks + DK * DR);  // chunks, slot = index & 3
  T2* red = (T2*)(ring + 4);                 // partial sums, [part][r][row]
  // thread = (row, r, part): the P parts split the column loops of the corner
  // and of M(i) s; part 0 adds the P partial sums in part order
  const int tid = threadIdx.x, row = tid & 31;
  const int P = DT / (32 * a.R);
  const int r = (tid >> 5) % a.R, part = (tid >> 5) / a.R;
  const bool lanes = part < P;
  const int D = a.p.D;
  const int64_t N = a.N;
  T2* xi = (T2*)a.xi;
  df_ring_load(a, ring, 0);
  df_ring_load(a, ring, 1);  // D + 1 chunks (sentinel)
  cp_async_commit();
  cp_async_wait_all();
  __syncthreads();
  df_stage<T2>(a, ring[0], ring[0], bufs, xcs);
  cp_async_commit();
  double2 wn = make_double2(0.0, 0.0);
  if (row < ring[0].m && part == 0) wn = a.w[(int64_t)r * N + ring[0].r0 + row];
  unsigned long long* tr = a.trace;
  for (int i = 0; i < D; i++) {
    cp_async_wait_all();
    __syncthreads();  // M(i), corner(i) and chunk i + 1 have landed
    if (tr && tid == 0) tr[4 * (int64_t)i] = gtimer();
    const HluDfChunk& c = ring[i & 3];
    const int m = c.m;
    const bool act = row < m && lanes;  // this thread holds partial sums
    const bool own = row < m && part == 0;  // this thread owns s(row, r) and x(row, r)
    T2 sv = from_d2<T2>(wn);
    if (i + 1 < D) {  // next step's inputs and the chunk after, in flight during this one
      const HluDfChunk& cn = ring[(i + 1) & 3];
      df_stage<T2>(a, cn, c, bufs + ((i + 1) & 1) * BUF_ELEMS, xcs + ((i + 1) & 1) * WCOLS * DR);
      df_ring_load(a, ring, i + 2);
      cp_async_commit();
      if (row < cn.m && part == 0) wn = a.w[(int64_t)r * N + cn.r0 + row];
    }
    const T2* Ms = bufs + (i & 1) * BUF_ELEMS;
    const T2* Cs = Ms + MS_ELEMS;
    const T2* xc = xcs + (i & 1) * WCOLS * DR;
    bool ok = true;
    if (tid == 0 && i >= 1) ok = df_wait(a.flagR(i), 1, a.err, a.wait_ns);
    if (!__syncthreads_and(ok)) {
      cp_async_wait_all();  // no copy in flight at exit
      return;
    }
    if (tr && tid == 0) tr[4 * (int64_t)i + 1] = gtimer();
    T2 accv = mk<T2>(0, 0);
    if (i >= 1 && own) accv = ldv((const T2*)a.acc + (int64_t)r * N + c.r0 + row);
    T2 cs = mk<T2>(0, 0);  // this thread's part of the corner contribution
    const T2* xs = xs2 + ((i - 1) & 1) * DM * DR;  // x(i - 1)
    if (c.corner >= 0) {
      const int64_t mL = c.cm, nL = c.cn;
      const int k = c.ck;
      const int pw = ring[(i - 1) & 3].m;
      if (!(c.cflags & 1)) {  // full leaf
        if (act) {
          if (nL <= WCOLS) {  // staged: F and the columns outside chunk i - 1
            for (int cc = part; cc < (int)nL; cc += P) {
              const int q = cc - c.cco;
              cmac(cs, Cs[cc * DM + row], (q >= 0 && q < pw) ? xs[q * DR + r] : xc[cc * DR + r]);
            }
          } else {
            const T2* xr = xi + (int64_t)r * N + c.cc0;
            const T2* fg = (const T2*)a.data + c.cdata + c.cro + row;
            for (int cc = part; cc < (int)nL; cc += P)
              cmac(cs, HC<T2>::ld(fg + (int64_t)cc * mL), ldv(xr + cc));
          }
        }
      } else {  // low rank: t = pre + V[:, cols(i - 2)] x(i - 2) + V[:, cols(i - 1)] x(i - 1),
                // then U[rows(i), :] t; pre (the columns before chunk i - 2) is
                // complete: R(i) waited for C(i - 3) before publishing
        const T2* pre = (const T2*)a.pre + (a.p.slot[c.corner] >= 0 ? a.p.slot[c.corner] : 0);
        const T2* xp = xs2 + (i & 1) * DM * DR;  // x(i - 2)
        const int w2 = c.cw2;
        for (int q = tid; q < k * a.R; q += DT) {
          const int l = q / a.R, rr = q % a.R;
          T2 t = mk<T2>(0, 0);
          const T2* v = Cs + DK * DM + l * DM;
          for (int cc = 0; cc < pw; cc++) cmac(t, v[cc], xs[cc * DR + rr]);
          if (c.cflags & 2) {
            const T2* v2 = Cs + 2 * DK * DM + l * DM;
            for (int cc = 0; cc < w2; cc++) cmac(t, v2[cc], xp[cc * DR + rr]);
          }
          if (c.cflags & 8) {
            const T2 p = ldv(pre + l * DR + rr);
            t.x = p.x + t.x;
            t.y = p.y + t.y;
          }
          tks[l * DR + rr] = t;
        }
        __syncthreads();
        if (act)
          for (int l = part; l < k; l += P) cmac(cs, Cs[l * DM + row], tks[l * DR + r]);
      }
      if (act) red[(part * a.R + r) * 32 + row] = cs;
    }
    __syncthreads();  // corner partials complete; x(i - 2) no longer read
    if (tr && tid == 0) tr[4 * (int64_t)i + 2] = gtimer();
    if (own) {
      if (c.corner >= 0) {
        cs = red[r * 32 + row];
        for (int q = 1; q < P; q++) {
          const T2 v = red[(q * a.R + r) * 32 + row];
          cs.x += v.x;
          cs.y += v.y;
        }
      }
      sv.x -= accv.x + cs.x;
      sv.y -= accv.y + cs.y;
      ss[row * DR + r] = sv;
    }
    __syncthreads();
    if (act) {
      T2 y = mk<T2>(0, 0);
      const T2* mr = Ms + row * (DM + 1);
      for (int t = part; t < m; t += P) cmac(y, mr[t], ss[t * DR + r]);
      red[(part * a.R + r) * 32 + row] = y;
    }
    __syncthreads();
    if (own) {
      T2 y = red[r * 32 + row];
      for (int q = 1; q < P; q++) {
        const T2 v = red[(q * a.R + r) * 32 + row];
        y.x += v.x;
        y.y += v.y;
      }
      xs2[(i & 1) * DM * DR + row * DR + r] = y;  // x(i), over x(i - 2)
      xi[(int64_t)r * N + c.r0 + row] = y;
      if ((void*)xi != (void*)a.x) a.x[(int64_t)r * N + c.r0 + row] = make_double2(y.x, y.y);
    }
    if (tr && tid == 0) tr[4 * (int64_t)i + 3] = gtimer();
    df_publish(a.ctrl + 1, i + 1);
    if (tid == 0) st_release(a.flagX(i), 1);
  }
  cp_async_wait_all();
}

// E(i): eacc(i) = contributions of the early leaves to rows(i) (full, or low
// rank with t = fin). Warp w takes entries w, w + NW, ... (lane = row); the NW
// partial sums meet in shared memory in warp order.
template <typename T2>
__device__ bool df_early_item(const DfArgs& a, int i, unsigned char* sm) {
  T2* part = (T2*)sm;  // [warp][r][row]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t N = a.N;
  const HluDfChunk c = a.p.chunks[i];
  const int e1 = a.p.chunks[i + 1].ebeg;
  bool ok = true;
  if (tid == 0) {
    ok = df_wait_progress(a, i - LAG + 1);
    if (ok && i >= LAG) ok = df_wait(a.flagC(i - LAG), 1, a.err, a.wait_ns);
  }
  if (!__syncthreads_and(ok)) return false;
  const int m = c.m, RR = a.R;
  const int row = lane < m ? lane : 0;
  const T2* data = (const T2*)a.data;
  const T2* xi = (const T2*)a.xi;
  T2 acc[DR];
#pragma unroll
  for (int r = 0; r < DR; r++) acc[r] = mk<T2>(0, 0);
  for (int e = c.ebeg + warp; e < e1; e += NW) {
    const HluDfRow en = a.p.erows[e];
    const int64_t* L = a.lv + 7 * (int64_t)en.leaf;
    const int64_t mL = L[1], nL = L[3];
    const T2* Dd = data + L[6];
    T2 s[DR];
#pragma unroll
    for (int r = 0; r < DR; r++) s[r] = mk<T2>(0, 0);
    if (L[4] == 0) {  // full: loop over columns, x broadcast
      const T2* f = Dd + en.ro + row;
      const T2* xr = xi + L[2];
#pragma unroll 4
      for (int cc = 0; cc < (int)nL; cc++) {
        const T2 v = HC<T2>::ld(f + (int64_t)cc * mL);
#pragma unroll
        for (int r = 0; r < DR; r++)
          if (r < RR) cmac(s[r], v, ldv(xr + (int64_t)r * N + cc));
      }
    } else {  // low rank, t = fin (broadcast)
      const int k = (int)L[5];
      const T2* u = Dd + en.ro + row;
      const T2* fin = (const T2*)a.fin + a.p.slot[en.leaf];
      for (int l = 0; l < k; l++) {
        const T2 uv = HC<T2>::ld(u + (int64_t)l * mL);
#pragma unroll
        for (int r = 0; r < DR; r++)
          if (r < RR) cmac(s[r], uv, ldv(fin + l * DR + r));
      }
    }
#pragma unroll
    for (int r = 0; r < DR; r++) {
      acc[r].x += s[r].x;
      acc[r].y += s[r].y;
    }
  }
#pragma unroll
  for (int r = 0; r < DR; r++)
    if (r < RR) part[(warp * DR + r) * 32 + lane] = acc[r];
  __syncthreads();
  if (tid < 32 * RR) {
    const int rw = tid & 31, r = tid >> 5;
    if (rw < m) {
      T2 v = mk<T2>(0, 0);
      for (int q = 0; q < NW; q++) {
        const T2 p = part[(q * DR + r) * 32 + rw];
        v.x += p.x;
        v.y += p.y;
      }
      ((T2*)a.eacc)[(int64_t)r * N + c.r0 + rw] = v;
    }
  }
  df_publish(a.flagE(i), 1);
  return true;
}

// R(i): acc(i) = eacc(i) + the late leaves' contributions, warp e on late
// entry e (lane = row); constants staged before the wait, vectors after it
template <typename T2>
__device__ bool df_late_item(const DfArgs& a, int i, unsigned char* sm) {
  constexpr int XE = WCOLS * DR;                // vector staging per entry
  T2* part = (T2*)sm;                           // [NW][DR][32]
  T2* xst = part + NW * DR * 32;                // [NLATE][WCOLS][DR]
  T2* tst = xst + NLATE * XE;                   // [NLATE][DK][DR]: fin / pre, then t
  T2* cst = tst + NLATE * DK * DR;              // constants, HLU_DF_STAGE_BYTES
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t N = a.N;
  const HluDfChunk c = a.p.chunks[i];
  const int e0 = c.rbeg, ne = a.p.chunks[i + 1].rbeg - e0;
  const int m = c.m, RR = a.R;
  const int row = lane < m ? lane : 0;
  const T2* data = (const T2*)a.data;
  const T2* xi = (const T2*)a.xi;
  const int w2 = i >= 2 ? a.p.chunks[i - 2].m : 0;
  const int c02 = i >= 2 ? a.p.chunks[i - 2].r0 : 0;
  // warp w works on entry w % ne as part w / ne of its P warps: a full
  // entry's columns are split over the parts, a low-rank entry is done by
  // part 0; part 0 (warp ew < ne) also stages the entry
  const bool mine = warp < ne;
  const int ew = ne > 0 ? warp % ne : 0, pw = ne > 0 ? warp / ne : 0;
  const int P = ne > 0 ? (NW - 1 - ew) / ne + 1 : 1;
  HluDfRow en{};
  int64_t mL = 0, nL = 0, c0 = 0, kind = 0, so = 0;
  int k = 0;
  const T2* Dd = data;
  if (ne > 0) {
    en = a.p.rows[e0 + ew];
    const int64_t* L = a.lv + 7 * (int64_t)en.leaf;
    mL = L[1];
    nL = L[3];
    c0 = L[2];
    kind = L[4];
    k = (int)L[5];
    Dd = data + L[6];
    so = a.p.slot[en.leaf];
  }
  if (mine) {
    if (en.soff >= 0) {  // constants (in flight during the wait)
      T2* cs = cst + en.soff;
      if (lane < m) {
        if (kind == 0)
          for (int cc = 0; cc < (int)nL; cc++) cp_async(cs + cc * 32 + lane, Dd + en.ro + lane + cc * mL);
        else
          for (int l = 0; l < k; l++) cp_async(cs + l * 32 + lane, Dd + en.ro + lane + l * mL);
      }
      if (kind != 0 && en.mode >= 2 && lane < w2)
        for (int l = 0; l < k; l++)
          cp_async(cs + 32 * k + l * 32 + lane, Dd + mL * k + l * nL + en.co2 + lane);
    }
  }
  cp_async_commit();
  bool ok = true;
  if (tid == 0) {
    ok = df_wait_progress(a, i - 1);
    const int cdep = i - 3;  // pre (corner) and pre2 (mode 2) are complete after C(i - 3)
    if (ok && cdep >= 0) ok = df_wait(a.flagC(cdep), 1, a.err, a.wait_ns);
    if (ok && i >= LAG - 1) ok = df_wait(a.flagE(i), 1, a.err, a.wait_ns);
  }
  if (!__syncthreads_and(ok)) {
    cp_async_wait_all();
    return false;
  }
  T2 ev = mk<T2>(0, 0);  // eacc, in flight during the staging
  if (tid < 32 * RR && lane < m && i >= LAG - 1) ev = ldv((const T2*)a.eacc + (int64_t)(tid >> 5) * N + c.r0 + lane);
  if (mine) {  // solved vectors, fin / pre
    T2* xs = xst + warp * XE;
    T2* ts = tst + warp * DK * DR;
    if (kind == 0) {
      if (nL <= WCOLS)
        for (int cc = lane; cc < (int)nL; cc += 32)
          for (int r = 0; r < RR; r++) cp_async(xs + cc * DR + r, xi + (int64_t)r * N + c0 + cc);
    } else if (en.mode == 1) {
      const T2* fin = (const T2*)a.fin + so;
      for (int q = lane; q < k * DR; q += 32)
        if (q % DR < RR) cp_async(ts + q, fin + q);
    } else {
      if (lane < w2)
        for (int r = 0; r < RR; r++) cp_async(xs + lane * DR + r, xi + (int64_t)r * N + c02 + lane);
      if (en.mode == 2) {
        const T2* pre = (const T2*)a.pre + a.p.nslot + so;  // pre2
        for (int q = lane; q < k * DR; q += 32)
          if (q % DR < RR) cp_async(ts + q, pre + q);
      }
    }
  }
  cp_async_commit();
  cp_async_wait_all();
  __syncthreads();
  if (ne > 0) {
    T2 s[DR];
#pragma unroll
    for (int r = 0; r < DR; r++) s[r] = mk<T2>(0, 0);
    const T2* xs = xst + ew * XE;
    const T2* cs = cst + (en.soff >= 0 ? en.soff : 0);
    if (kind == 0) {
      const bool sf = en.soff >= 0, sxs = nL <= WCOLS;
      const T2* fg = Dd + en.ro + row;
      const T2* xg = xi + c0;
      for (int cc = pw; cc < (int)nL; cc += P) {
        const T2 v = sf ? cs[cc * 32 + row] : HC<T2>::ld(fg + (int64_t)cc * mL);
#pragma unroll
        for (int r = 0; r < DR; r++)
          if (r < RR) cmac(s[r], v, sxs ? xs[cc * DR + r] : ldv(xg + (int64_t)r * N + cc));
      }
    } else if (pw == 0) {
      T2* ts = tst + warp * DK * DR;
      if (en.mode >= 2) {  // t(l, r) = (pre) + V[l, cols(i - 2)] x(i - 2), lanes over (l, r)
        for (int q = lane; q < k * DR; q += 32) {
          const int l = q / DR, r = q % DR;
          if (r >= RR) continue;
          T2 t = mk<T2>(0, 0);
          const T2* vg = Dd + mL * k + l * nL + en.co2;
          for (int cc = 0; cc < w2; cc++)
            cmac(t, en.soff >= 0 ? cs[32 * k + l * 32 + cc] : HC<T2>::ld(vg + cc), xs[cc * DR + r]);
          if (en.mode == 2) {
            const T2 p = ts[q];
            t.x = p.x + t.x;
            t.y = p.y + t.y;
          }
          ts[q] = t;
        }
        __syncwarp();
      }
      const T2* ug = Dd + en.ro + row;
      for (int l = 0; l < k; l++) {
        const T2 u = en.soff >= 0 ? cs[l * 32 + row] : HC<T2>::ld(ug + (int64_t)l * mL);
#pragma unroll
        for (int r = 0; r < DR; r++)
          if (r < RR) cmac(s[r], u, ts[l * DR + r]);
      }
    }
#pragma unroll
    for (int r = 0; r < DR; r++)
      if (r < RR) part[(warp * DR + r) * 32 + lane] = s[r];
  }
  __syncthreads();
  if (tid < 32 * RR) {
    const int rw = tid & 31, r = tid >> 5;
    if (rw < m) {
      T2 v = ev;
      for (int q = 0; q < (ne > 0 ? NW : 0); q++) {
        const T2 p = part[(q * DR + r) * 32 + rw];
        v.x += p.x;
        v.y += p.y;
      }
      ((T2*)a.acc)[(int64_t)r * N + c.r0 + rw] = v;
    }
  }
  df_publish(a.flagR(i), 1);
  return true;
}

// C(j): t partials of the low-rank leaves over cols(j), into pre / fin. One
// warp per (leaf, row l of V), lanes over the columns; V is loaded before the
// wait, x(j) right after it (both one coalesced load per lane).
template <typename T2>
__device__ bool df_col_item(const DfArgs& a, int j) {
  using R = typename DfT<T2>::R;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t N = a.N;
  const HluDfChunk c = a.p.chunks[j];
  const int p0 = c.cbeg, P = a.p.chunks[j + 1].cbeg - p0;
  const int w = c.m, RR = a.R;
  const bool cok = lane < w;
  const T2* data = (const T2*)a.data;
  T2 v[PS];
  int64_t so[PS];
  int fl[PS];
  auto load = [&](int base) {
#pragma unroll
    for (int s = 0; s < PS; s++) {
      const int p = base + warp + NW * s;
      v[s] = mk<T2>(0, 0);
      so[s] = 0;
      fl[s] = -1;
      if (p < P) {
        const HluDfCol en = a.p.cols[p0 + p];
        const int64_t* L = a.lv + 7 * (int64_t)en.leaf;
        if (cok) v[s] = HC<T2>::ld(data + L[6] + L[1] * L[5] + (int64_t)en.l * L[3] + en.co + lane);
        so[s] = a.p.slot[en.leaf] + (int64_t)en.l * DR;
        fl[s] = en.flags;
      }
    }
  };
  load(0);
  bool ok = true;
  if (tid == 0) {
    ok = df_wait_progress(a, j + 1);
    if (ok && j >= 1) ok = df_wait(a.flagC(j - 1), 1, a.err, a.wait_ns);
  }
  if (!__syncthreads_and(ok)) return false;
  T2 xr[DR];
#pragma unroll
  for (int r = 0; r < DR; r++)
    xr[r] = (r < RR && cok) ? ldv((const T2*)a.xi + (int64_t)r * N + c.r0 + lane) : mk<T2>(0, 0);
  for (int base = 0; base < P; base += NW * PS) {
    if (base > 0) load(base);
    T2 pr[PS];
#pragma unroll
    for (int s = 0; s < PS; s++) {
      pr[s] = mk<T2>(0, 0);
      if (fl[s] >= 0 && !(fl[s] & 1) && lane < RR)
        pr[s] = ldv((const T2*)a.pre + ((fl[s] & 8) ? a.p.nslot : 0) + so[s] + lane);
    }
#pragma unroll
    for (int s = 0; s < PS; s++) {
      if (fl[s] < 0) continue;  // warp-uniform
      T2 res = mk<T2>(0, 0);
#pragma unroll
      for (int r = 0; r < DR; r++)
        if (r < RR) {
          const R tx = wred<R>(v[s].x * xr[r].x - v[s].y * xr[r].y);
          const R ty = wred<R>(v[s].x * xr[r].y + v[s].y * xr[r].x);
          if (lane == r) res = mk<T2>(tx, ty);
        }
      if (lane < RR) {
        res.x = pr[s].x + res.x;
        res.y = pr[s].y + res.y;
        T2* dst = (fl[s] & 2) ? (T2*)a.fin : (T2*)a.pre + ((fl[s] & 4) ? a.p.nslot : 0);
        dst[so[s] + lane] = res;
      }
    }
  }
  df_publish(a.flagC(j), 1);
  return true;
}

template <typename T2>
__device__ void df_helper(const DfArgs& a, unsigned char* sm, int* sq) {
  const int D = a.p.D;
  const int nitems = 3 * (D + 1);
  while (true) {
    if (threadIdx.x == 0) *sq = atomicAdd(a.ctrl, 1);
    __syncthreads();
    const int q = *sq;
    __syncthreads();
    if (q >= nitems) return;
    const int L = q / 3, t = q % 3;
    bool ok = true;
    if (t == 0) {
      if (L - 1 >= 0 && L - 1 <= D - 2) ok = df_col_item<T2>(a, L - 1);
    } else if (t == 1) {
      const int i = L + LAG - 1;
      if (i >= 1 && i <= D - 1) ok = df_early_item<T2>(a, i, sm);
    } else {
      const int i = L + 1;
      if (i <= D - 1) ok = df_late_item<T2>(a, i, sm);
    }
    if (!ok) return;
  }
}

template <typename T2>
__global__ void __launch_bounds__(DT, 1) hlu_df_kernel(DfArgs a) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ int sq;
  if (gate_closed(a.gate)) return;  // every block reads the same flags
  if (threadIdx.x == 0) sq = atomicAdd(a.ctrl + 2, 1);  // arrival order
  __syncthreads();
  const bool driver = sq == 0;
  __syncthreads();  // sq is the helpers' claim slot from here on
  if (driver)
    df_driver<T2>(a, sm);
  else
    df_helper<T2>(a, sm, &sq);
}

template <typename T2>
int df_prepare() {  // max resident blocks, after raising the shared-memory limit
  static int cached[64] = {0};
  int dev = 0;
  CUDA_OK(cudaGetDevice(&dev));
  if (dev < 64 && cached[dev]) return cached[dev];
  CUDA_OK(cudaFuncSetAttribute(hlu_df_kernel<T2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)df_smem<T2>()));
  int nb = 0, sms = 0;
  CUDA_OK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, hlu_df_kernel<T2>, DT, df_smem<T2>()));
  CUDA_OK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int v = std::max(1, nb * sms);
  if (dev < 64) cached[dev] = v;
  return v;
}

}  // namespace

int launch_hlu_df(const HluDfDev& p, const int64_t* leaves, const void* data, int precision,
                  const double2* w, double2* x, int64_t N, int R, const HluDfWork& ws, int helpers,
                  cudaStream_t s, HmvGate gate) {
  if (p.D <= 0 || R <= 0) return 0;
  if (R > HLU_DF_MAX_R) throw std::runtime_error("launch_hlu_df: more than 8 right-hand sides");
  CUDA_OK(cudaMemsetAsync(ws.ctrl, 0, (size_t)(4 + 4 * p.D) * sizeof(int), s));
  DfArgs a;
  a.p = p;
  a.lv = leaves;
  a.data = data;
  a.w = w;
  a.x = x;
  a.xi = precision == 0 ? (void*)x : ws.xi;
  a.acc = ws.acc;
  a.eacc = ws.eacc;
  a.pre = ws.pre;
  a.fin = ws.fin;
  a.ctrl = ws.ctrl;
  a.err = ws.err;
  a.N = N;
  a.R = R;
  a.gate = gate;
  a.trace = ws.trace;
  a.wait_ns = ws.wait_ns;
  void* args[] = {&a};
  const int cap = precision == 0 ? df_prepare<double2>() : df_prepare<float2>();
  const int grid = std::max(2, std::min(1 + std::max(1, helpers), cap));
  if (precision == 0)
    CUDA_OK(cudaLaunchKernel((const void*)hlu_df_kernel<double2>, dim3(grid), dim3(DT), args,
                             df_smem<double2>(), s));
  else
    CUDA_OK(cudaLaunchKernel((const void*)hlu_df_kernel<float2>, dim3(grid), dim3(DT), args,
                             df_smem<float2>(), s));
  return 2;
}

}  // namespace bemgpu
