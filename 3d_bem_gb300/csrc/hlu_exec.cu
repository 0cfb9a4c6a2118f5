// hlu_exec.cu -- executor of the H-LU task program (hlu_gpu.h): one persistent
// kernel over a ready queue. A CTA takes the next queue slot, waits (bounded)
// until a task is pushed into it, runs the task with all its threads, then
// releases the task's successors; the release that completes a successor's
// dependencies pushes it. Only CTAs that are running hold slots and tasks, so
// the queue advances with any number of resident CTAs: the launch needs no
// co-residency and starts on the SMs that are free (beside other streams'
// kernels) instead of waiting for a whole idle GPU.
//
// Data that other CTAs wrote during the launch is read through L2
// (ld.global.cg) and written with st.global.cg, so no SM reads a stale L1
// line of the arena. The arithmetic is the storage type's: complex FP32
// factors are computed in FP32, complex FP64 factors in FP64.
#include <cuda_runtime.h>

#include "hlu_gpu.h"

namespace bemgpu {

namespace {

constexpr int HX_THREADS = 256;
constexpr int HX_WARPS = HX_THREADS / 32;
constexpr int HX_MAX_PAIRS = 64;  // truncation inputs per task (checked on the host)

template <typename T2>
struct Cx;
template <>
struct Cx<float2> {
  using R = float;
  static constexpr int SMEM = 6144;  // complex elements of dynamic shared memory
  __device__ static float2 mk(float a, float b) { return make_float2(a, b); }
  __device__ static float sq(float x) { return sqrtf(x); }
  __device__ static float rsq(float x) { return rsqrtf(x); }
  __device__ static float div(float a, float b) { return __fdividef(a, b); }
  // orthogonality target of the FP32 rotations: one decade above FP32
  // rounding, where the relative test would otherwise oscillate
  __device__ static float jacobi_thr() { return 1e-5f; }
  // columns below this fraction of the squared Frobenius norm are rounding
  // noise: they take no rotations (their relative test never settles)
  __device__ static float jacobi_floor() { return 1e-14f; }
  static constexpr int JACOBI_SWEEPS = 15;
};
template <>
struct Cx<double2> {
  using R = double;
  static constexpr int SMEM = 6144;
  __device__ static double2 mk(double a, double b) { return make_double2(a, b); }
  __device__ static double sq(double x) { return sqrt(x); }
  __device__ static double rsq(double x) { return rsqrt(x); }
  __device__ static double div(double a, double b) { return a / b; }
  __device__ static double jacobi_thr() { return 1e-15; }
  __device__ static double jacobi_floor() { return 1e-30; }
  static constexpr int JACOBI_SWEEPS = 60;
};

template <typename T2>
__device__ __forceinline__ T2 cz() {
  return Cx<T2>::mk(0, 0);
}
template <typename T2>
__device__ __forceinline__ T2 cadd(T2 a, T2 b) {
  return Cx<T2>::mk(a.x + b.x, a.y + b.y);
}
template <typename T2>
__device__ __forceinline__ T2 csub(T2 a, T2 b) {
  return Cx<T2>::mk(a.x - b.x, a.y - b.y);
}
template <typename T2>
__device__ __forceinline__ T2 cmul(T2 a, T2 b) {
  return Cx<T2>::mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) b
template <typename T2>
__device__ __forceinline__ T2 cmulc(T2 a, T2 b) {
  return Cx<T2>::mk(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
template <typename T2>
__device__ __forceinline__ T2 cconj(T2 a) {
  return Cx<T2>::mk(a.x, -a.y);
}
template <typename T2, typename R>
__device__ __forceinline__ T2 cscale(T2 a, R s) {
  return Cx<T2>::mk(a.x * s, a.y * s);
}
template <typename T2>
__device__ __forceinline__ T2 cneg(T2 a) {
  return Cx<T2>::mk(-a.x, -a.y);
}
template <typename T2>
__device__ __forceinline__ typename Cx<T2>::R cabs2(T2 a) {
  return a.x * a.x + a.y * a.y;
}

// arena: written by other CTAs during the launch -> L2 only
template <typename T2>
__device__ __forceinline__ T2 ldA(const T2* p) {
  return __ldcg(p);
}
template <typename T2>
__device__ __forceinline__ void stA(T2* p, T2 v) {
  __stcg(p, v);
}

template <typename R>
__device__ __forceinline__ R warp_sum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// CTA-wide sum of one value per thread; red: >= HX_WARPS + 1 values
template <typename R>
__device__ R block_sum(R v, R* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    R x = l < HX_WARPS ? red[l] : R(0);
    x = warp_sum(x);
    if (l == 0) red[HX_WARPS] = x;
  }
  __syncthreads();
  const R r = red[HX_WARPS];
  __syncthreads();
  return r;
}

// op(A)(i, l) of a column-major matrix with leading dimension ld
template <typename T2>
__device__ __forceinline__ T2 opget(const T2* A, int op, int64_t i, int64_t l, int64_t ld) {
  if (op == HOP_N) return ldA(A + i + l * ld);
  const T2 v = ldA(A + l + i * ld);
  return op == HOP_C ? cconj(v) : v;
}

// ---------------------------------------------------------------- GEMM
template <typename T2>
__device__ void task_gemm(const HluTask& t, T2* arena, T2* sm) {
  using R = typename Cx<T2>::R;
  const int m = t.m, n = t.n, q = t.q;
  const int opa = t.flags & 3, opb = (t.flags >> 2) & 3;
  const bool accu = t.flags & HF_ACC, neg = t.flags & HF_NEG;
  const T2* A = arena + t.a;
  const T2* B = arena + t.b;
  T2* C = arena + t.c;
  const int tid = threadIdx.x;
  if ((int64_t)m * n <= 64 && q >= 64) {  // few long dot products: a warp each
    const int w = tid >> 5, ln = tid & 31;
    for (int o = w; o < m * n; o += HX_WARPS) {
      const int i = o % m, j = o / m;
      R sr = 0, si = 0;
      for (int l = ln; l < q; l += 32) {
        const T2 p = cmul(opget(A, opa, i, l, t.lda), opget(B, opb, l, j, t.ldb));
        sr += p.x;
        si += p.y;
      }
      sr = warp_sum(sr);
      si = warp_sum(si);
      if (ln == 0) {
        T2 v = Cx<T2>::mk(neg ? -sr : sr, neg ? -si : si);
        T2* c = C + i + (int64_t)j * t.ldc;
        if (accu) v = cadd(ldA(c), v);
        stA(c, v);
      }
    }
    return;
  }
  const int ldb_s = q | 1;  // odd: threads on different columns of B hit distinct banks
  if (m * n <= 4 * HX_THREADS && (int64_t)m * q + (int64_t)ldb_s * n <= Cx<T2>::SMEM) {
    // small product: both operands staged whole (one round of loads, C's
    // old values fetched alongside), then up to four outputs per thread
    T2* sa = sm;          // m x q
    T2* sb = sm + m * q;  // q x n, leading dimension ldb_s
    for (int e = tid; e < m * q; e += HX_THREADS) sa[e] = opget(A, opa, e % m, e / m, t.lda);
    for (int e = tid; e < q * n; e += HX_THREADS) {
      const int l = e % q, j = e / q;
      sb[l + j * ldb_s] = opget(B, opb, l, j, t.ldb);
    }
    T2 cv[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int o = tid + k * HX_THREADS;
      cv[k] = (accu && o < m * n) ? ldA(C + o % m + (int64_t)(o / m) * t.ldc) : cz<T2>();
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int o = tid + k * HX_THREADS;
      if (o < m * n) {
        const int i = o % m, j = o / m;
        R ar = 0, ai = 0;
        for (int l = 0; l < q; l++) {
          const T2 av = sa[i + l * m], bv = sb[l + j * ldb_s];
          ar += av.x * bv.x - av.y * bv.y;
          ai += av.x * bv.y + av.y * bv.x;
        }
        const T2 v = Cx<T2>::mk(neg ? cv[k].x - ar : cv[k].x + ar, neg ? cv[k].y - ai : cv[k].y + ai);
        stA(C + i + (int64_t)j * t.ldc, v);
      }
    }
    return;
  }
  // tiles of TM x TN outputs (4 per thread), q in chunks of 16 staged in
  // shared memory
  const int TM = n <= 4 ? 256 : (n <= 16 ? 64 : 32);
  const int TN = 1024 / TM;
  const int QC = 16;
  T2* sa = sm;             // TM x QC
  T2* sb = sm + TM * QC;   // QC x TN
  const int ti = tid % TM, tj0 = tid / TM, tjs = HX_THREADS / TM;
  for (int i0 = 0; i0 < m; i0 += TM)
    for (int j0 = 0; j0 < n; j0 += TN) {
      T2 acc[4];
#pragma unroll
      for (int k = 0; k < 4; k++) acc[k] = cz<T2>();
      for (int l0 = 0; l0 < q; l0 += QC) {
        for (int e = tid; e < TM * QC; e += HX_THREADS) {
          const int ii = e % TM, ll = e / TM;
          const int gi = i0 + ii, gl = l0 + ll;
          sa[e] = (gi < m && gl < q) ? opget(A, opa, gi, gl, t.lda) : cz<T2>();
        }
        for (int e = tid; e < QC * TN; e += HX_THREADS) {
          const int ll = e % QC, jj = e / QC;
          const int gl = l0 + ll, gj = j0 + jj;
          sb[e] = (gl < q && gj < n) ? opget(B, opb, gl, gj, t.ldb) : cz<T2>();
        }
        __syncthreads();
#pragma unroll 4
        for (int ll = 0; ll < QC; ll++) {
          const T2 av = sa[ti + ll * TM];
#pragma unroll
          for (int k = 0; k < 4; k++) {
            const T2 bv = sb[ll + (tj0 + k * tjs) * QC];
            acc[k].x += av.x * bv.x - av.y * bv.y;
            acc[k].y += av.x * bv.y + av.y * bv.x;
          }
        }
        __syncthreads();
      }
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const int gi = i0 + ti, gj = j0 + tj0 + k * tjs;
        if (gi < m && gj < n) {
          T2 v = neg ? cneg(acc[k]) : acc[k];
          T2* c = C + gi + (int64_t)gj * t.ldc;
          if (accu) v = cadd(ldA(c), v);
          stA(c, v);
        }
      }
    }
}

// ---------------------------------------------------------------- LMUL / RMUL
// X (m x n) := op(M) X, M m x m
template <typename T2>
__device__ void task_lmul(const HluTask& t, T2* arena, T2* sm) {
  const int m = t.m, n = t.n, op = t.flags & 3;
  const T2* M = arena + t.a;
  T2* X = arena + t.c;
  T2* sM = sm;           // op(M), m x m column-major
  T2* sX = sm + m * m;   // m x cw
  const int cw = max(1, min(n, (Cx<T2>::SMEM - m * m) / m));
  for (int e = threadIdx.x; e < m * m; e += HX_THREADS) sM[e] = opget(M, op, e % m, e / m, t.lda);
  for (int j0 = 0; j0 < n; j0 += cw) {
    const int w = min(cw, n - j0);
    __syncthreads();
    for (int e = threadIdx.x; e < m * w; e += HX_THREADS)
      sX[e] = ldA(X + (e % m) + (int64_t)(j0 + e / m) * t.ldc);
    __syncthreads();
    for (int e = threadIdx.x; e < m * w; e += HX_THREADS) {
      const int i = e % m, j = e / m;
      T2 acc = cz<T2>();
      for (int l = 0; l < m; l++) acc = cadd(acc, cmul(sM[i + l * m], sX[l + j * m]));
      stA(X + i + (int64_t)(j0 + j) * t.ldc, acc);
    }
  }
}

// X (m x n) := X op(M), M n x n
template <typename T2>
__device__ void task_rmul(const HluTask& t, T2* arena, T2* sm) {
  const int m = t.m, n = t.n, op = t.flags & 3;
  const T2* M = arena + t.a;
  T2* X = arena + t.c;
  T2* sM = sm;          // op(M), n x n column-major
  T2* sX = sm + n * n;  // rw x n
  const int rw = max(1, min(m, (Cx<T2>::SMEM - n * n) / n));
  for (int e = threadIdx.x; e < n * n; e += HX_THREADS) sM[e] = opget(M, op, e % n, e / n, t.lda);
  for (int i0 = 0; i0 < m; i0 += rw) {
    const int h = min(rw, m - i0);
    __syncthreads();
    for (int e = threadIdx.x; e < h * n; e += HX_THREADS)
      sX[e] = ldA(X + (i0 + e % h) + (int64_t)(e / h) * t.ldc);
    __syncthreads();
    for (int e = threadIdx.x; e < h * n; e += HX_THREADS) {
      const int i = e % h, j = e / h;
      T2 acc = cz<T2>();
      for (int l = 0; l < n; l++) acc = cadd(acc, cmul(sX[i + l * h], sM[l + j * n]));
      stA(X + (i0 + i) + (int64_t)j * t.ldc, acc);
    }
  }
}

// ---------------------------------------------------------------- COPY / ZERO
template <typename T2>
__device__ void task_copy(const HluTask& t, T2* arena, const T2* F) {
  const int src = (t.flags >> HF_SRC_SHIFT) & 7;
  const bool accu = t.flags & HF_ACC, neg = t.flags & HF_NEG;
  T2* C = arena + t.c;
  const int64_t tot = (int64_t)t.m * t.n;
  for (int64_t e = threadIdx.x; e < tot; e += HX_THREADS) {
    const int64_t i = e % t.m, j = e / t.m;
    T2 v = src == 1 ? __ldg(F + t.a + i + j * t.lda) : ldA(arena + t.a + i + j * t.lda);
    if (neg) v = cneg(v);
    T2* c = C + i + j * t.ldc;
    if (accu) v = cadd(ldA(c), v);
    stA(c, v);
  }
}

template <typename T2>
__device__ void task_zero(const HluTask& t, T2* arena) {
  T2* C = arena + t.c;
  const int64_t tot = (int64_t)t.m * t.n;
  for (int64_t e = threadIdx.x; e < tot; e += HX_THREADS)
    stA(C + e % t.m + (e / t.m) * t.ldc, cz<T2>());
}

// ---------------------------------------------------------------- QR of a diagonal leaf
// Householder reflectors H_j = I - 2 v v^H (|v| = 1) as in the host H-LU:
// H_{m-1} .. H_0 A = R, Q = H_0 .. H_{m-1}. W accumulates Q^H = H_{m-1} .. H_0
// alongside. Outputs: Q, R (column-major), Q^H and R^{-1} (row-major).
template <typename T2>
__device__ void task_qr(const HluTask& t, const HluExecArgs& a, T2* arena, T2* sm) {
  using R = typename Cx<T2>::R;
  const int m = t.m, ld = m + 1;  // odd leading dimension
  T2* sA = sm;               // m x m
  T2* sW = sA + m * ld;      // m x m
  T2* sv = sW + m * ld;      // reflectors of steps j (even / odd), 2 x m
  T2* sd = sv + 2 * m;       // 1 / R(r, r), m
  __shared__ R s_r[4];
  for (int e = threadIdx.x; e < m * m; e += HX_THREADS) {
    const int i = e % m, j = e / m;
    sA[i + j * ld] = ldA(arena + t.a + i + (int64_t)j * t.lda);
    sW[i + j * ld] = i == j ? Cx<T2>::mk(1, 0) : cz<T2>();
  }
  if (threadIdx.x == 0) s_r[0] = 0;
  __syncthreads();
  // tpc threads per column (consecutive lanes): rows i = j + sub, j + sub + tpc, ..
  const int tpc = m <= 32 ? 4 : 2;
  const int c = threadIdx.x / tpc, sub = threadIdx.x % tpc;
  const unsigned gmask = ((1u << tpc) - 1u) << ((threadIdx.x & 31) & ~(tpc - 1));  // the group's lanes
  // reflector of column j from the group holding it (only its lanes call):
  // v = (x + ph |x| e_j) / |.|
  auto reflector = [&](int j) {
    const T2* x = sA + j * ld;
    R xn2 = 0;
    for (int i = j + sub; i < m; i += tpc) xn2 += cabs2(x[i]);
    for (int o = tpc / 2; o > 0; o >>= 1) xn2 += __shfl_xor_sync(gmask, xn2, o, tpc);
    const T2 x0 = x[j];
    const R ax2 = cabs2(x0);
    const R xn = Cx<T2>::sq(xn2);
    const T2 ph = ax2 > 0 ? cscale(x0, Cx<T2>::rsq(ax2)) : Cx<T2>::mk(1, 0);
    const T2 v0 = cadd(x0, cscale(ph, xn));
    const R vn2 = xn2 - ax2 + cabs2(v0);
    const R inv = vn2 > 0 ? Cx<T2>::rsq(vn2) : R(0);
    T2* v = sv + (j & 1) * m;
    for (int i = j + sub; i < m; i += tpc) v[i] = cscale(i == j ? v0 : x[i], inv);
  };
  if (c == 0) reflector(0);
  __syncthreads();
  for (int j = 0; j < m; j++) {
    // H_j = I - 2 v v^H on columns j.. of A and all columns of W (rows j..);
    // the group of A's column j + 1 then forms the next reflector
    const T2* v = sv + (j & 1) * m;
    const bool act = c < 2 * m - j;
    T2* y = c < m - j ? sA + (j + c) * ld : sW + (c - (m - j)) * ld;
    R dr = 0, di = 0;
    if (act)
      for (int i = j + sub; i < m; i += tpc) {
        const T2 p = cmulc(v[i], y[i]);
        dr += p.x;
        di += p.y;
      }
    for (int o = tpc / 2; o > 0; o >>= 1) {
      dr += __shfl_xor_sync(0xffffffffu, dr, o, tpc);
      di += __shfl_xor_sync(0xffffffffu, di, o, tpc);
    }
    if (act) {
      const T2 d2 = Cx<T2>::mk(2 * dr, 2 * di);
      for (int i = j + sub; i < m; i += tpc) y[i] = csub(y[i], cmul(v[i], d2));
    }
    __syncwarp();
    if (c == 1 && j + 1 < m) reflector(j + 1);
    __syncthreads();
  }
  const HluQrOut o = a.qr[t.x0];
  // Q = W^H, Q^H row-major = W column-major read by rows: Qh[r m + c] = W(r, c)
  for (int e = threadIdx.x; e < m * m; e += HX_THREADS) {
    const int i = e % m, j = e / m;
    stA(arena + o.q + e, cconj(sW[j + i * ld]));          // Q(i, j) = conj(W(j, i))
    stA(arena + o.qh + (int64_t)i * m + j, sW[i + j * ld]);  // Q^H(i, j) = W(i, j)
    stA(arena + o.r + e, i <= j ? sA[i + j * ld] : cz<T2>());
  }
  if (threadIdx.x < m) {  // 1 / R(r, r); a zero or non-finite pivot is flagged
    const int r = threadIdx.x;
    const T2 d = sA[r + r * ld];
    const R dd = cabs2(d);
    if (!(dd > 0) || !isfinite(dd)) {
      s_r[0] = 1;
      sd[r] = cz<T2>();
    } else {
      sd[r] = cscale(cconj(d), Cx<T2>::div(R(1), dd));
    }
  }
  __syncthreads();
  // R^{-1} row-major, a warp per column tc (lanes over rows, two rows a lane
  // up to 64): y = R^{-1} e_tc by column-oriented back substitution
  {
    const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
    for (int tc = w; tc < m; tc += HX_WARPS) {
      T2 acc0 = ln == tc ? Cx<T2>::mk(1, 0) : cz<T2>();
      T2 acc1 = ln + 32 == tc ? Cx<T2>::mk(1, 0) : cz<T2>();
      for (int r = tc; r >= 0; r--) {
        // y_r = acc_r / R(r, r) from the lane holding row r, to every lane
        const T2 mine = r < 32 ? acc0 : acc1;
        T2 yr = cmul(mine, sd[r]);
        yr.x = __shfl_sync(0xffffffffu, yr.x, r & 31);
        yr.y = __shfl_sync(0xffffffffu, yr.y, r & 31);
        if (ln == (r & 31)) {
          if (r < 32) acc0 = yr;
          else acc1 = yr;
        }
        if (ln < r) acc0 = csub(acc0, cmul(sA[ln + r * ld], yr));
        if (ln + 32 < r) acc1 = csub(acc1, cmul(sA[ln + 32 + r * ld], yr));
      }
      if (ln < m) stA(arena + o.rinv + (int64_t)ln * m + tc, ln <= tc ? acc0 : cz<T2>());
      if (ln + 32 < m) stA(arena + o.rinv + (int64_t)(ln + 32) * m + tc, ln + 32 <= tc ? acc1 : cz<T2>());
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_r[0] != 0) atomicAdd(&a.ctrl[2], 1);
}

// ---------------------------------------------------------------- truncation
// Householder QR of X (rows x cols, column-major, ld = rows) in place: R in
// the upper triangle, reflector j (unit norm) as head[j] at row j and X rows
// below the diagonal; p = min(rows, cols) reflectors. Every pass runs over the
// rows with all threads and carries up to HQ_G columns in registers, so a
// tall panel is streamed a few times per column instead of once per column
// pair by a single warp.
constexpr int HQ_G = 8;

// CTA-wide sums of nv values per thread (nv <= 2 HQ_G); thread t < nv gets
// sum t in out[t] (shared), the rest unchanged; ends with a barrier
template <typename R>
__device__ void block_sums(R* v, int nv, R (*part)[2 * HQ_G], R* out) {
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
  for (int q = 0; q < nv; q++) {
    const R x = warp_sum(v[q]);
    if (ln == 0) part[w][q] = x;
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    R x = 0;
    for (int q = 0; q < HX_WARPS; q++) x += part[q][threadIdx.x];
    out[threadIdx.x] = x;
  }
  __syncthreads();
}

template <typename T2>
__device__ void house_qr(T2* X, int64_t rows, int cols, T2* head) {
  using R = typename Cx<T2>::R;
  const int p = (int)(rows < cols ? rows : (int64_t)cols);
  __shared__ R part[HX_WARPS][2 * HQ_G];
  __shared__ R sums[2 * HQ_G];
  __shared__ T2 s_v0, s_ph, s_c[HQ_G];
  __shared__ R s_inv, s_xn;
  for (int j = 0; j < p; j++) {
    T2* x = X + (int64_t)j * rows;
    R nrm = 0;
    for (int64_t i = j + threadIdx.x; i < rows; i += HX_THREADS) nrm += cabs2(x[i]);
    block_sums(&nrm, 1, part, sums);
    if (threadIdx.x == 0) {
      const R xn2 = sums[0];
      const R xn = Cx<T2>::sq(xn2);
      const T2 x0 = x[j];
      const R ax0 = Cx<T2>::sq(cabs2(x0));
      const T2 ph = ax0 > 0 ? cscale(x0, R(1) / ax0) : Cx<T2>::mk(1, 0);
      const T2 v0 = cadd(x0, cscale(ph, xn));
      const R vn2 = xn2 - cabs2(x0) + cabs2(v0);
      s_inv = vn2 > 0 ? R(1) / Cx<T2>::sq(vn2) : R(0);
      s_v0 = v0;
      s_ph = ph;
      s_xn = -xn;
    }
    __syncthreads();
    const R inv = s_inv;
    const T2 v0 = cscale(s_v0, inv);  // the unit reflector is v = inv (v0, x_{j+1}, ...)
    // columns j + 1 .. in groups: c_g = 2 v^H y, y -= c_g v
    for (int c0 = j + 1; c0 < cols; c0 += HQ_G) {
      const int nc = min(HQ_G, cols - c0);
      R acc[2 * HQ_G];
#pragma unroll
      for (int g = 0; g < 2 * HQ_G; g++) acc[g] = 0;
      for (int64_t i = j + 1 + threadIdx.x; i < rows; i += HX_THREADS) {
        const T2 xi = cscale(x[i], inv);
#pragma unroll
        for (int g = 0; g < HQ_G; g++)
          if (g < nc) {
            const T2 pr = cmulc(xi, X[i + (int64_t)(c0 + g) * rows]);
            acc[2 * g] += pr.x;
            acc[2 * g + 1] += pr.y;
          }
      }
      block_sums(acc, 2 * nc, part, sums);
      if (threadIdx.x < nc) {
        const T2 yj = X[j + (int64_t)(c0 + threadIdx.x) * rows];
        const T2 d = cadd(cmulc(v0, yj), Cx<T2>::mk(sums[2 * threadIdx.x], sums[2 * threadIdx.x + 1]));
        s_c[threadIdx.x] = cscale(d, R(2));
      }
      __syncthreads();
      for (int64_t i = j + threadIdx.x; i < rows; i += HX_THREADS) {
        const T2 vi = i == j ? v0 : cscale(x[i], inv);
#pragma unroll
        for (int g = 0; g < HQ_G; g++)
          if (g < nc) {
            T2* y = X + i + (int64_t)(c0 + g) * rows;
            *y = csub(*y, cmul(s_c[g], vi));
          }
      }
      __syncthreads();
    }
    // normalise the reflector below the diagonal, R(j, j) on the diagonal
    for (int64_t i = j + 1 + threadIdx.x; i < rows; i += HX_THREADS) x[i] = cscale(x[i], inv);
    if (threadIdx.x == 0) {
      head[j] = v0;
      x[j] = cscale(s_ph, s_xn);
    }
    __syncthreads();
  }
}

// Y (rows x nc, column-major, ld, in the arena) := H_0 .. H_{p-1} Y with the
// reflectors of house_qr
template <typename T2, bool ARENA = true>
__device__ void house_apply(const T2* X, int64_t rows, int p, const T2* head, T2* Y, int64_t ld,
                            int nc) {
  using R = typename Cx<T2>::R;
  __shared__ R part[HX_WARPS][2 * HQ_G];
  __shared__ R sums[2 * HQ_G];
  __shared__ T2 s_c[HQ_G];
  for (int j = p - 1; j >= 0; j--) {
    const T2* x = X + (int64_t)j * rows;
    const T2 v0 = head[j];
    for (int c0 = 0; c0 < nc; c0 += HQ_G) {
      const int ng = min(HQ_G, nc - c0);
      R acc[2 * HQ_G];
#pragma unroll
      for (int g = 0; g < 2 * HQ_G; g++) acc[g] = 0;
      for (int64_t i = j + threadIdx.x; i < rows; i += HX_THREADS) {
        const T2 vi = i == j ? v0 : x[i];
#pragma unroll
        for (int g = 0; g < HQ_G; g++)
          if (g < ng) {
            const T2* yp = Y + i + (int64_t)(c0 + g) * ld;
            const T2 pr = cmulc(vi, ARENA ? ldA(yp) : *yp);
            acc[2 * g] += pr.x;
            acc[2 * g + 1] += pr.y;
          }
      }
      block_sums(acc, 2 * ng, part, sums);
      if (threadIdx.x < ng)
        s_c[threadIdx.x] = Cx<T2>::mk(2 * sums[2 * threadIdx.x], 2 * sums[2 * threadIdx.x + 1]);
      __syncthreads();
      for (int64_t i = j + threadIdx.x; i < rows; i += HX_THREADS) {
        const T2 vi = i == j ? v0 : x[i];
#pragma unroll
        for (int g = 0; g < HQ_G; g++)
          if (g < ng) {
            T2* y = Y + i + (int64_t)(c0 + g) * ld;
            if (ARENA) stA(y, csub(ldA(y), cmul(vi, s_c[g])));
            else *y = csub(*y, cmul(vi, s_c[g]));
          }
      }
      __syncthreads();
    }
  }
}

// element (r, l) of a truncation piece (kinds 0, 2, 3; identity handled by the caller)
template <typename T2>
__device__ __forceinline__ T2 piece_get(const HluExecArgs& a, int kind, int64_t off, int64_t soff,
                                        int rs, int cs, int64_t r, int l) {
  if (kind == 0) return ldA(reinterpret_cast<const T2*>(a.arena) + off + r * rs + (int64_t)l * cs);
  if (kind == 2) {
    const T2 u = __ldg(reinterpret_cast<const T2*>(a.U) + off + r * rs + (int64_t)l * cs);
    const T2 s = __ldg(reinterpret_cast<const T2*>(a.S) + soff + l);
    return cmul(u, s);
  }
  return __ldg(reinterpret_cast<const T2*>(a.V) + off + r * rs + (int64_t)l * cs);
}

// One-sided Jacobi on the q columns of X (p x q, column-major): X V = U diag(s),
// V (q x q) accumulates the rotations (set to I here). Round-robin pairs, a
// warp per pair. Rotations keep the Frobenius norm, so one floor decides
// which columns are rounding noise: those take no rotations (between two of
// them the relative test never settles).
template <typename T2>
__device__ void jacobi_cols(T2* X, int p, int q, T2* V, typename Cx<T2>::R* red) {
  using R = typename Cx<T2>::R;
  __shared__ unsigned s_off;
  for (int e = threadIdx.x; e < q * q; e += HX_THREADS)
    V[e] = (e % q == e / q) ? Cx<T2>::mk(1, 0) : cz<T2>();
  R fro = 0;
  for (int e = threadIdx.x; e < p * q; e += HX_THREADS) fro += cabs2(X[e]);
  const R floor2 = block_sum(fro, red) * Cx<T2>::jacobi_floor();
  const int qq = q + (q & 1);
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
  for (int sweep = 0; sweep < Cx<T2>::JACOBI_SWEEPS && q > 1; sweep++) {
    if (threadIdx.x == 0) s_off = 0u;
    __syncthreads();
    for (int rd = 0; rd < qq - 1; rd++) {
      for (int k = w; k < qq / 2; k += HX_WARPS) {
        int i1, i2;
        if (k == 0) {
          i1 = rd;
          i2 = qq - 1;
        } else {
          i1 = (rd + k) % (qq - 1);
          i2 = (rd - k + (qq - 1)) % (qq - 1);
        }
        if (i1 > i2) {
          const int tt = i1;
          i1 = i2;
          i2 = tt;
        }
        if (i2 >= q) continue;
        T2* xa = X + (int64_t)i1 * p;
        T2* xb = X + (int64_t)i2 * p;
        R na = 0, nb = 0, gr = 0, gi = 0;
        for (int i = ln; i < p; i += 32) {
          na += cabs2(xa[i]);
          nb += cabs2(xb[i]);
          const T2 g = cmulc(xa[i], xb[i]);
          gr += g.x;
          gi += g.y;
        }
        na = warp_sum(na);
        nb = warp_sum(nb);
        gr = warp_sum(gr);
        gi = warp_sum(gi);
        if (!(na > floor2) || !(nb > floor2)) continue;
        const R g2 = gr * gr + gi * gi;
        if (g2 == R(0)) continue;
        const R iga = Cx<T2>::rsq(g2);  // 1 / |g|
        const R rel = g2 * iga * Cx<T2>::rsq(na * nb);
        if (!(rel > Cx<T2>::jacobi_thr())) continue;
        if (ln == 0) atomicMax(&s_off, __float_as_uint((float)rel));
        const R er = gr * iga, ei = gi * iga;
        const R zeta = (nb - na) * (R(0.5) * iga);
        const R tt = Cx<T2>::div(zeta >= 0 ? R(1) : R(-1),
                                 fabs(zeta) + Cx<T2>::sq(1 + zeta * zeta));
        const R cs = Cx<T2>::rsq(1 + tt * tt), sn = cs * tt;
        // x' = c x - s (y conj(e)), y' = s x + c (y conj(e))
        for (int i = ln; i < p; i += 32) {
          const T2 x = xa[i], y = xb[i];
          const T2 ye = Cx<T2>::mk(y.x * er + y.y * ei, y.y * er - y.x * ei);
          xa[i] = Cx<T2>::mk(cs * x.x - sn * ye.x, cs * x.y - sn * ye.y);
          xb[i] = Cx<T2>::mk(sn * x.x + cs * ye.x, sn * x.y + cs * ye.y);
        }
        T2* va = V + (int64_t)i1 * q;
        T2* vb = V + (int64_t)i2 * q;
        for (int i = ln; i < q; i += 32) {
          const T2 x = va[i], y = vb[i];
          const T2 ye = Cx<T2>::mk(y.x * er + y.y * ei, y.y * er - y.x * ei);
          va[i] = Cx<T2>::mk(cs * x.x - sn * ye.x, cs * x.y - sn * ye.y);
          vb[i] = Cx<T2>::mk(sn * x.x + cs * ye.x, sn * x.y + cs * ye.y);
        }
      }
      __syncthreads();
    }
    const bool done = __uint_as_float(s_off) == 0.0f;
    __syncthreads();
    if (done) break;
  }
}

// Singular values of the rotated columns (sig, q values) and the kept ones,
// largest first (idx, returned count): minRankforError with the cap kc and,
// for tol > 0, the tail relative to the sum of the squared singular values
template <typename T2>
__device__ int pick_rank(const T2* X, int p, int q, typename Cx<T2>::R* sig,
                         typename Cx<T2>::R* mark, int kc, double tol, int* idx) {
  using R = typename Cx<T2>::R;
  __shared__ int s_r;
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
  for (int j = w; j < q; j += HX_WARPS) {
    R s2 = 0;
    for (int i = ln; i < p; i += 32) s2 += cabs2(X[i + (int64_t)j * p]);
    s2 = warp_sum(s2);
    if (ln == 0) {
      sig[j] = Cx<T2>::sq(s2);
      mark[j] = 0;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    R full = 0;
    for (int j = 0; j < q; j++) full += sig[j] * sig[j];
    const int rmax = min(kc, q);
    int r = 0;
    R kept = 0;
    while (r < rmax) {
      int bj = -1;
      for (int j = 0; j < q; j++)
        if (mark[j] == R(0) && (bj < 0 || sig[j] > sig[bj])) bj = j;
      if (bj < 0 || !(sig[bj] > 0)) break;
      mark[bj] = 1;
      idx[r++] = bj;
      kept += sig[bj] * sig[bj];
      if (tol > 0 && full > 0 && (full - kept) / full < R(tol * tol)) break;
    }
    s_r = r;
  }
  __syncthreads();
  const int r = s_r;
  __syncthreads();
  return r;
}

// seeded value in [-1, 1] of the randomized range finder's test matrix
__device__ __forceinline__ float rnd_pm1(int64_t j, int c) {
  const uint64_t h = pivot_hash(0x5DEECE66Dull, (uint64_t)j, (uint64_t)c);
  return (float)((double)(h >> 11) * (2.0 / 9007199254740992.0) - 1.0);
}

// T (kt x L) = op(S)^T Y with S (rows x kt), Y (rows x L) in scratch
// (column-major); conj_s: conj(S); omega: Y is the seeded test matrix. A warp
// per entry, lanes over the rows.
template <typename T2>
__device__ void mm_ty(const T2* S, int64_t rows, int kt, const T2* Y, int L, T2* T, bool conj_s,
                      bool omega) {
  using R = typename Cx<T2>::R;
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
  for (int o = w; o < kt * L; o += HX_WARPS) {
    const int l = o % kt, c = o / kt;
    const T2* sc = S + (int64_t)l * rows;
    R sr = 0, si = 0;
    for (int64_t i = ln; i < rows; i += 32) {
      const T2 sv = conj_s ? cconj(sc[i]) : sc[i];
      const T2 yv = omega ? Cx<T2>::mk((R)rnd_pm1(i, c), 0) : Y[i + (int64_t)c * rows];
      const T2 pr = cmul(sv, yv);
      sr += pr.x;
      si += pr.y;
    }
    sr = warp_sum(sr);
    si = warp_sum(si);
    if (ln == 0) T[l + (int64_t)c * kt] = Cx<T2>::mk(sr, si);
  }
  __syncthreads();
}
// Y (rows x L) = op(S) T with S (rows x kt), T (kt x L)
template <typename T2>
__device__ void mm_st(const T2* S, int64_t rows, int kt, const T2* T, int L, T2* Y, bool conj_s) {
  for (int64_t e = threadIdx.x; e < rows * L; e += HX_THREADS) {
    const int64_t i = e % rows;
    const int c = (int)(e / rows);
    T2 acc = cz<T2>();
    for (int l = 0; l < kt; l++) {
      const T2 sv = S[i + (int64_t)l * rows];
      acc = cadd(acc, cmul(conj_s ? cconj(sv) : sv, T[l + (int64_t)c * kt]));
    }
    Y[e] = acc;
  }
  __syncthreads();
}
// Q (rows x L) := orthonormal basis of the columns of Y (Householder; Y is
// overwritten by the reflectors)
template <typename T2>
__device__ void orth(T2* Y, int64_t rows, int L, T2* head, T2* Q) {
  house_qr(Y, rows, L, head);
  for (int64_t e = threadIdx.x; e < rows * L; e += HX_THREADS)
    Q[e] = (e % rows == e / rows) ? Cx<T2>::mk(1, 0) : cz<T2>();
  __syncthreads();
  house_apply<T2, false>(Y, rows, L, head, Q, rows, L);
}

// ---------------------------------------------------------------- subspace truncation
// For ranks kc <= 2 without a tolerance (the preconditioner's default) every
// truncation works through a basis of at most HS_L columns held in shared
// memory: small matrices, a warp per long reduction, no CTA-wide sweeps over
// L2-resident panels.
constexpr int HS_L = HLU_SUB_L;
static_assert(Cx<float2>::SMEM == HLU_SMEM_ELEMS && Cx<double2>::SMEM == HLU_SMEM_ELEMS,
              "the planner's shared-memory size");

// One side of a truncation (A: m x kt or B: n x kt, column-major, leading
// dimension ld): in shared memory (odd ld: a warp reading one row of
// consecutive columns hits distinct banks), or in the CTA's scratch, where
// the products stage it in chunks of rows.
template <typename T2>
struct Side {
  const T2* p;
  int ld;
  bool glob;
};
// Staging area of the products: up to rc rows of a side, leading dimension
// rc | 1.
template <typename T2>
struct Stage {
  T2* p;
  int rc;
};

// rows i0 .. i0 + h of side S (all kt columns) as a shared-memory matrix
// (returns its pointer and leading dimension)
template <typename T2>
__device__ const T2* stage_rows(const Side<T2>& S, int i0, int h, int kt, const Stage<T2>& st,
                                int& ld) {
  if (!S.glob) {
    ld = S.ld;
    return S.p + i0;
  }
  const int ldp = st.rc | 1;
  __syncthreads();  // the previous chunk's readers are done
  for (int e = threadIdx.x; e < h * kt; e += HX_THREADS)
    st.p[e % h + (e / h) * ldp] = S.p[i0 + e % h + (int64_t)(e / h) * S.ld];
  __syncthreads();
  ld = ldp;
  return st.p;
}

// T (kt x lq, shared) = op(S)^T Y, Y (rows x lq, shared); a thread per entry
// of T, summed chunk by chunk
template <typename T2>
__device__ void sub_mm_ty(const Side<T2>& S, int rows, int kt, const T2* Y, int lq, T2* T,
                          bool conj_s, bool conj_out, const Stage<T2>& st) {
  using R = typename Cx<T2>::R;
  const int nout = kt * lq;
  for (int o = threadIdx.x; o < nout; o += HX_THREADS) T[o] = cz<T2>();
  const int rc = S.glob ? st.rc : rows;
  for (int i0 = 0; i0 < rows; i0 += rc) {
    const int h = min(rc, rows - i0);
    int ld;
    const T2* Sc = stage_rows(S, i0, h, kt, st, ld);
    for (int o = threadIdx.x; o < nout; o += HX_THREADS) {
      const int l = o % kt, c = o / kt;
      const T2* sc = Sc + l * ld;
      const T2* yc = Y + i0 + c * rows;
      R ar = 0, ai = 0;
#pragma unroll 4
      for (int i = 0; i < h; i++) {
        T2 sv = sc[i];
        if (conj_s) sv.y = -sv.y;
        const T2 y = yc[i];
        ar += sv.x * y.x - sv.y * y.y;
        ai += sv.x * y.y + sv.y * y.x;
      }
      const T2 t0 = T[o];
      T[o] = Cx<T2>::mk(t0.x + ar, t0.y + ai);
    }
  }
  if (conj_out) {
    __syncthreads();
    for (int o = threadIdx.x; o < nout; o += HX_THREADS) T[o] = cconj(T[o]);
  }
  __syncthreads();
}

// Y (rows x lq, shared) = op(S) T, T (kt x lq, shared); a thread per entry of
// Y, chunk by chunk
template <typename T2>
__device__ void sub_mm_st(const Side<T2>& S, int rows, int kt, const T2* T, int lq, T2* Y,
                          bool conj_s, const Stage<T2>& st) {
  using R = typename Cx<T2>::R;
  const int rc = S.glob ? st.rc : rows;
  for (int i0 = 0; i0 < rows; i0 += rc) {
    const int h = min(rc, rows - i0);
    int ld;
    const T2* Sc = stage_rows(S, i0, h, kt, st, ld);
    for (int o = threadIdx.x; o < h * lq; o += HX_THREADS) {
      const int i = o % h, c = o / h;
      const T2* tc = T + c * kt;
      R ar = 0, ai = 0;
#pragma unroll 4
      for (int l = 0; l < kt; l++) {
        T2 sv = Sc[i + l * ld];
        if (conj_s) sv.y = -sv.y;
        const T2 tv = tc[l];
        ar += sv.x * tv.x - sv.y * tv.y;
        ai += sv.x * tv.y + sv.y * tv.x;
      }
      Y[i0 + i + c * rows] = Cx<T2>::mk(ar, ai);
    }
  }
  __syncthreads();
}

// Orthonormal columns of Y (rows x lq, shared) in place by modified
// Gram-Schmidt with a second pass (one warp, lanes over the rows). A column
// whose remainder falls below drop x its own norm lies in the span of the
// earlier ones (rank deficiency) and becomes zero: it adds no direction, and
// a zero column of the basis carries no singular value.
template <typename T2>
__device__ void sub_orth(T2* Y, int rows, int lq, T2* Rz = nullptr) {
  using R = typename Cx<T2>::R;
  const R drop = sizeof(R) == 4 ? R(1e-10) : R(1e-26);
  if (threadIdx.x < 32) {
    const int ln = threadIdx.x;
    if (Rz) {
      for (int e = ln; e < HS_L * HS_L; e += 32) Rz[e] = cz<T2>();
      __syncwarp();
    }
    R n0 = 0;  // |y_j|^2 before the projections
    for (int i = ln; i < rows; i += 32) n0 += cabs2(Y[i]);
    for (int j = 0; j < lq; j++) {
      T2* y = Y + j * rows;
      R nn = 0;
      for (int pass = 0; pass < 2; pass++) {
        // d_k = q_k^H y (k < j) and, in the first pass, |y|^2: one butterfly
        // over all the sums at once
        R d[2 * HS_L + 1];
#pragma unroll
        for (int k = 0; k < 2 * HS_L + 1; k++) d[k] = 0;
        if (j > 0) {
          for (int i = ln; i < rows; i += 32) {
            const T2 yi = y[i];
#pragma unroll
            for (int k = 0; k < HS_L; k++)
              if (k < j) {
                const T2 q = Y[i + k * rows];  // conj(q) y
                d[2 * k] += q.x * yi.x + q.y * yi.y;
                d[2 * k + 1] += q.x * yi.y - q.y * yi.x;
              }
          }
        }
        if (pass == 0) d[2 * HS_L] = n0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
          for (int k = 0; k < 2 * HS_L + 1; k++) d[k] += __shfl_xor_sync(0xffffffffu, d[k], o);
        }
        if (pass == 0) n0 = d[2 * HS_L];
        if (Rz && ln < j) {  // R(k, j) = the two passes' coefficients
#pragma unroll
          for (int k = 0; k < HS_L; k++)
            if (k == ln) {
              const T2 o = Rz[k + j * HS_L];
              Rz[k + j * HS_L] = Cx<T2>::mk(o.x + d[2 * k], o.y + d[2 * k + 1]);
            }
        }
        // y -= sum_k d_k q_k, and the new |y|^2
        R part = 0;
        for (int i = ln; i < rows; i += 32) {
          T2 yi = y[i];
#pragma unroll
          for (int k = 0; k < HS_L; k++)
            if (k < j) {
              const T2 q = Y[i + k * rows];
              yi.x -= q.x * d[2 * k] - q.y * d[2 * k + 1];
              yi.y -= q.x * d[2 * k + 1] + q.y * d[2 * k];
            }
          y[i] = yi;
          part += cabs2(yi);
        }
        nn = warp_sum(part);
        __syncwarp();
        if (j == 0) break;  // nothing to project on
      }
      const R s = (nn > 0 && nn > drop * n0) ? Cx<T2>::rsq(nn) : R(0);
      if (Rz && ln == 0) Rz[j + j * HS_L] = Cx<T2>::mk(s > 0 ? nn * s : R(0), 0);
      R nx = 0;  // |y_{j+1}|^2 for the next column
      for (int i = ln; i < rows; i += 32) {
        y[i] = cscale(y[i], s);
        if (j + 1 < lq) nx += cabs2(y[i + rows]);
      }
      n0 = nx;  // reduced with the next column's first pass
      __syncwarp();
    }
  }
  __syncthreads();
}

// One-sided Jacobi on X (q x q, q <= 8, column-major, leading dimension 8,
// shared) by one warp: X V = U diag(s), V (q x q, leading dimension 8)
// accumulates the rotations. Lane = 8 x pair + row: the four pairs of a
// round rotate at once, each reduced over its 8 lanes; the same noise floor
// and threshold as jacobi_cols.
template <typename T2>
__device__ void jacobi_small(T2* X, int q, T2* V) {
  using R = typename Cx<T2>::R;
  if (threadIdx.x < 32) {
    const int ln = threadIdx.x, g = ln >> 3, r = ln & 7;
    for (int e = ln; e < HS_L * HS_L; e += 32)
      V[e] = (e % HS_L == e / HS_L && e % HS_L < q) ? Cx<T2>::mk(1, 0) : cz<T2>();
    R fro = 0;
    if (g == 0 && r < q)
      for (int c = 0; c < q; c++) fro += cabs2(X[r + c * HS_L]);
    const R floor2 = warp_sum(fro) * Cx<T2>::jacobi_floor();
    __syncwarp();
    const int qq = q + (q & 1);
    for (int sweep = 0; sweep < Cx<T2>::JACOBI_SWEEPS && q > 1; sweep++) {
      unsigned off = 0u;
      for (int rd = 0; rd < qq - 1; rd++) {
        int i1, i2;
        if (g == 0) {
          i1 = rd;
          i2 = qq - 1;
        } else {
          i1 = (rd + g) % (qq - 1);
          i2 = (rd - g + (qq - 1)) % (qq - 1);
        }
        if (i1 > i2) {
          const int tt = i1;
          i1 = i2;
          i2 = tt;
        }
        const bool pair = g < qq / 2 && i2 < q;
        T2 xa = cz<T2>(), xb = cz<T2>();
        if (pair && r < q) {
          xa = X[r + i1 * HS_L];
          xb = X[r + i2 * HS_L];
        }
        R na = cabs2(xa), nb = cabs2(xb);
        const T2 gp = cmulc(xa, xb);
        R gr = gp.x, gi = gp.y;
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) {
          na += __shfl_xor_sync(0xffffffffu, na, o, 8);
          nb += __shfl_xor_sync(0xffffffffu, nb, o, 8);
          gr += __shfl_xor_sync(0xffffffffu, gr, o, 8);
          gi += __shfl_xor_sync(0xffffffffu, gi, o, 8);
        }
        const R g2 = gr * gr + gi * gi;
        bool rot = pair && na > floor2 && nb > floor2 && g2 > R(0);
        R rel = 0, iga = 0;
        if (rot) {
          iga = Cx<T2>::rsq(g2);
          rel = g2 * iga * Cx<T2>::rsq(na * nb);
          rot = rel > Cx<T2>::jacobi_thr();
        }
        if (rot) {
          const unsigned rb = __float_as_uint((float)rel);
          off = rb > off ? rb : off;
          const R er = gr * iga, ei = gi * iga;
          const R zeta = (nb - na) * (R(0.5) * iga);
          const R tt = Cx<T2>::div(zeta >= 0 ? R(1) : R(-1),
                                   fabs(zeta) + Cx<T2>::sq(1 + zeta * zeta));
          const R cs = Cx<T2>::rsq(1 + tt * tt), sn = cs * tt;
          if (r < q) {
            const T2 ye = Cx<T2>::mk(xb.x * er + xb.y * ei, xb.y * er - xb.x * ei);
            X[r + i1 * HS_L] = Cx<T2>::mk(cs * xa.x - sn * ye.x, cs * xa.y - sn * ye.y);
            X[r + i2 * HS_L] = Cx<T2>::mk(sn * xa.x + cs * ye.x, sn * xa.y + cs * ye.y);
            const T2 va = V[r + i1 * HS_L], vb = V[r + i2 * HS_L];
            const T2 we = Cx<T2>::mk(vb.x * er + vb.y * ei, vb.y * er - vb.x * ei);
            V[r + i1 * HS_L] = Cx<T2>::mk(cs * va.x - sn * we.x, cs * va.y - sn * we.y);
            V[r + i2 * HS_L] = Cx<T2>::mk(sn * va.x + cs * we.x, sn * va.y + cs * we.y);
          }
        }
        __syncwarp();
      }
      if (__reduce_max_sync(0xffffffffu, off) == 0u) break;
    }
  }
  __syncthreads();
}

// A' (m x kc) B'^T (n x kc) = the rank-kc truncated SVD of A B^T with
// A = SA (m x kt), B = SB (n x kt); the buffers in shared memory at sm.
template <typename T2>
__device__ void trunc_subspace(const Side<T2>& SA, const Side<T2>& SB, int m, int n, int kt,
                               int kc, int power, T2* sm, const Stage<T2>& st, T2* Ao, T2* Bo,
                               int* s_idx) {
  using R = typename Cx<T2>::R;
  T2* Q = sm;               // m x lq
  T2* Z = Q + m * HS_L;     // n x lq
  T2* T = Z + n * HS_L;     // kt x lq
  T2* V = T + kt * HS_L;    // lq x lq (leading dimension 8)
  T2* Rz = V + HS_L * HS_L;  // lq x lq (leading dimension 8)
  R* sig = reinterpret_cast<R*>(Rz + HS_L * HS_L);
  R* mark = sig + HS_L;
  const bool ident = m <= HS_L;  // Q = I_m
  int lq;
  if (ident) {
    lq = m;
  } else if (kt <= HS_L) {  // range(M) inside range(A): Q = orth(A), exact
    lq = kt;
    for (int e = threadIdx.x; e < m * kt; e += HX_THREADS)
      Q[e] = SA.p[e % m + (int64_t)(e / m) * SA.ld];
    __syncthreads();
    sub_orth(Q, m, lq);
  } else if (n <= HS_L) {  // Q = orth(M), M = A B^T formed (m x n), exact
    lq = n;
    for (int e = threadIdx.x; e < kt * n; e += HX_THREADS) {
      const int l = e % kt, c = e / kt;
      T[e] = SB.p[c + (int64_t)l * SB.ld];  // T = B^T
    }
    __syncthreads();
    sub_mm_st(SA, m, kt, T, lq, Q, false, st);
    sub_orth(Q, m, lq);
  } else {
    // seeded randomized range finder with power iterations q = power (0 or
    // 1; Halko, Martinsson, Tropp, SIAM Review 53(2), 2011: algorithm 4.4)
    lq = kc + 6 < HS_L ? kc + 6 : HS_L;
    for (int e = threadIdx.x; e < n * lq; e += HX_THREADS)
      Z[e] = Cx<T2>::mk((R)rnd_pm1(e % n, e / n), 0);
    __syncthreads();
    sub_mm_ty(SB, n, kt, Z, lq, T, false, false, st);  // T = B^T Omega
    sub_mm_st(SA, m, kt, T, lq, Q, false, st);         // Q = A T = M Omega
    sub_orth(Q, m, lq);
    if (power) {
      sub_mm_ty(SA, m, kt, Q, lq, T, true, false, st);   // T = A^H Q
      sub_mm_st(SB, n, kt, T, lq, Z, true, st);          // Z = conj(B) T = M^H Q
      sub_orth(Z, n, lq);
      sub_mm_ty(SB, n, kt, Z, lq, T, false, false, st);  // T = B^T Z
      sub_mm_st(SA, m, kt, T, lq, Q, false, st);         // Q = M Z
      sub_orth(Q, m, lq);
    }
  }
  // the projection's transpose (Q^H M)^T = B conj(A^H Q) (n x lq); its SVD
  // Z V = U S gives M ~ Q conj(V) S U^T
  if (ident) {
    for (int e = threadIdx.x; e < kt * m; e += HX_THREADS) {
      const int l = e % kt, c = e / kt;
      T[e] = SA.p[c + (int64_t)l * SA.ld];  // conj(A^H I) = A^T
    }
    __syncthreads();
  } else {
    sub_mm_ty(SA, m, kt, Q, lq, T, true, true, st);
  }
  sub_mm_st(SB, n, kt, T, lq, Z, false, st);
  // Z = Qz Rz, then Rz V = Ur S (Jacobi on the small factor): Z V = Qz Ur S
  sub_orth(Z, n, lq, Rz);
  jacobi_small(Rz, lq, V);
  const int r = pick_rank(Rz, HS_L, lq, sig, mark, kc, 0.0, s_idx);
  for (int e = threadIdx.x; e < m * kc; e += HX_THREADS) {  // A' = Q conj(V) S
    const int i = e % m, l = e / m;
    T2 v = cz<T2>();
    if (l < r) {
      const int j = s_idx[l];
      if (ident) {
        v = cconj(V[i + j * HS_L]);
      } else {
        for (int c = 0; c < lq; c++) v = cadd(v, cmul(Q[i + c * m], cconj(V[c + j * HS_L])));
      }
      v = cscale(v, sig[j]);
    }
    stA(Ao + e, v);
  }
  for (int e = threadIdx.x; e < n * kc; e += HX_THREADS) {  // B' = U = Qz Ur
    const int i = e % n, l = e / n;
    T2 v = cz<T2>();
    if (l < r) {
      const int j = s_idx[l];
      for (int c = 0; c < lq; c++) v = cadd(v, cmul(Z[i + c * n], Rz[c + j * HS_L]));
      v = cscale(v, Cx<T2>::div(R(1), sig[j]));
    }
    stA(Bo + e, v);
  }
}

template <typename T2>
__device__ void task_trunc(const HluTask& t, const HluExecArgs& a, T2* arena, T2* slot, T2* sm) {
  using R = typename Cx<T2>::R;
  __shared__ int s_cb[HX_MAX_PAIRS + 1];
  __shared__ R red[HX_WARPS + 8];
  __shared__ int s_idx[64];
  const int64_t m = t.m, n = t.n;
  const int kc = a.kc;
  const HluTruncPair* P = a.pairs + t.x0;
  const int np = t.x1;
  if (threadIdx.x == 0) {
    int c = 0;
    for (int p = 0; p < np; p++) {
      s_cb[p] = c;
      int w = P[p].cols;
      if (P[p].rank_idx >= 0) w = min(w, max(0, __ldg(a.rank + P[p].rank_idx)));
      c += w;
    }
    s_cb[np] = c;
  }
  __syncthreads();
  const int kt = s_cb[np];
  T2* Ao = arena + t.c;
  T2* Bo = arena + t.b;
  if (kt == 0 || m == 0 || n == 0) {
    for (int64_t e = threadIdx.x; e < m * kc; e += HX_THREADS) stA(Ao + e, cz<T2>());
    for (int64_t e = threadIdx.x; e < n * kc; e += HX_THREADS) stA(Bo + e, cz<T2>());
    return;
  }
  // Three ways to the truncated SVD of A B^T (A = [A_1 ..], B = [B_1 ..]):
  //  small  -- both sides <= 32 (the common leaf-level update): the dense
  //            m x n sum in shared memory, Jacobi on it directly;
  //  range  -- a small rank (kc <= 8, no tolerance) of a wide sum: a seeded
  //            randomized range finder with one power iteration on L = kc + 6
  //            columns (Halko, Martinsson, Tropp 2011), then the SVD of the
  //            L x n projection;
  //  qr     -- otherwise: Householder QR of both sides, Jacobi on the core
  //            R_A R_B^T, the reflectors applied to the kept vectors.
  const int K2 = kt > 32 ? kt : 32;
  // subspace path (kc <= 2, no tolerance) when its buffers and a staging
  // area of at least 8 rows fit in shared memory; the two sides go there too
  // when they fit beside the buffers (odd leading dimensions)
  const int64_t subb = hlu_sub_buffers(m, n, kt);
  const int64_t mp = m | 1, np1 = n | 1;
  const bool sub = kc <= 2 && !(a.tol > 0) && subb + 9 * kt <= Cx<T2>::SMEM;
  const bool sub_sides = sub && subb + (mp + np1) * kt <= Cx<T2>::SMEM;
  const bool small = !sub && m <= 32 && n <= 32 &&
                     (m + n) * kt + m * n + 32 * 32 + 4 * K2 <= Cx<T2>::SMEM;
  const int L = kc + 6;
  const bool range = !sub && !small && kc <= 8 && !(a.tol > 0) && kt > L && m > L && n > L;
  T2* S = small ? sm
                : (sub_sides ? sm + subb
                             : (t.a >= 0 ? reinterpret_cast<T2*>(a.big_scratch) + t.a : slot));
  const int lda = (int)(sub_sides ? mp : m), ldb = (int)(sub_sides ? np1 : n);
  T2* SA = S;
  T2* SB = S + (int64_t)lda * kt;
  T2* W = SB + (int64_t)ldb * kt;  // work area of the chosen path
  // gather both sides (placements, zeros elsewhere), four loads in flight
  // per thread
  for (int p = 0; p < np; p++) {
    const HluTruncPair pp = P[p];
    const int c0 = s_cb[p], w = s_cb[p + 1] - c0;
    const bool na = pp.neg & 1, nb = pp.neg & 2;
    for (int side = 0; side < 2; side++) {
      const int rows = (int)(side ? n : m), ld = side ? ldb : lda;
      const int64_t r0 = side ? pp.rb : pp.ra, mr = side ? pp.mb : pp.ma;
      const int kind = side ? pp.bkind : pp.akind;
      const int64_t off = side ? pp.boff : pp.aoff, soff = side ? 0 : pp.soff;
      const int rs = side ? pp.brs : pp.ars, cs = side ? pp.bcs : pp.acs;
      const bool ng = side ? nb : na;
      T2* D = side ? SB : SA;
      for (int e0 = threadIdx.x; e0 < rows * w; e0 += 4 * HX_THREADS) {
        T2 v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int e = e0 + u * HX_THREADS;
          v[u] = cz<T2>();
          if (e < rows * w) {
            const int r = e % rows, l = e / rows;
            const int64_t rr = r - r0;
            if (rr >= 0 && rr < mr) {
              if (kind == 1) v[u] = rr == l ? Cx<T2>::mk(1, 0) : cz<T2>();
              else v[u] = piece_get<T2>(a, kind, off, soff, rs, cs, rr, l);
              if (ng) v[u] = cneg(v[u]);
            }
          }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int e = e0 + u * HX_THREADS;
          if (e < rows * w) D[e % rows + (int64_t)(c0 + e / rows) * ld] = v[u];
        }
      }
    }
  }
  __syncthreads();

  if (sub) {
    const Side<T2> sa{SA, lda, !sub_sides}, sb{SB, ldb, !sub_sides};
    int rc = (int)((Cx<T2>::SMEM - subb) / kt) - 1;  // (rc | 1) * kt elements fit
    rc = rc > 256 ? 256 : rc;
    const Stage<T2> st{sm + subb, rc};
    trunc_subspace(sa, sb, (int)m, (int)n, kt, kc, a.range_power, sm, st, Ao, Bo, s_idx);
    return;
  }
  if (range) {
    T2* Y = W;            // m x L
    T2* Q = Y + m * L;    // m x L
    T2* Z = Q + m * L;    // n x L
    T2* Zq = Z + n * L;   // n x L
    T2* T = Zq + n * L;   // kt x L
    T2* V = T + (int64_t)kt * L;  // L x L
    T2* hd = V + L * L;   // L
    R* sig = reinterpret_cast<R*>(hd + L);
    R* mark = sig + L;
    // Y = M Omega with M = A B^T, then one power iteration Y = M M^H Y
    mm_ty(SB, n, kt, (const T2*)nullptr, L, T, false, true);  // T = B^T Omega
    mm_st(SA, m, kt, T, L, Y, false);                         // Y = A T
    orth(Y, m, L, hd, Q);
    mm_ty(SA, m, kt, Q, L, T, true, false);                   // T = A^H Q
    mm_st(SB, n, kt, T, L, Z, true);                          // Z = conj(B) T = M^H Q
    orth(Z, n, L, hd, Zq);
    mm_ty(SB, n, kt, Zq, L, T, false, false);                 // T = B^T Zq
    mm_st(SA, m, kt, T, L, Y, false);                         // Y = M Zq
    orth(Y, m, L, hd, Q);
    // the projection's transpose (Q^H M)^T = M^T conj(Q) = B conj(A^H Q)
    // (n x L); its SVD Z V = U S gives M ~ Q conj(V) S U^T
    mm_ty(SA, m, kt, Q, L, T, true, false);
    for (int o = threadIdx.x; o < kt * L; o += HX_THREADS) T[o] = cconj(T[o]);
    __syncthreads();
    mm_st(SB, n, kt, T, L, Z, false);
    jacobi_cols(Z, (int)n, L, V, red);
    const int r = pick_rank(Z, (int)n, L, sig, mark, kc, 0.0, s_idx);
    for (int64_t e = threadIdx.x; e < m * kc; e += HX_THREADS) {  // A' = Q conj(V) S
      const int64_t i = e % m;
      const int l = (int)(e / m);
      T2 v = cz<T2>();
      if (l < r) {
        const int j = s_idx[l];
        for (int c = 0; c < L; c++) v = cadd(v, cmul(Q[i + (int64_t)c * m], cconj(V[c + j * L])));
        v = cscale(v, sig[j]);
      }
      stA(Ao + e, v);
    }
    for (int64_t e = threadIdx.x; e < n * kc; e += HX_THREADS) {  // B' = U
      const int64_t i = e % n;
      const int l = (int)(e / n);
      T2 v = cz<T2>();
      if (l < r) {
        const int j = s_idx[l];
        v = cscale(Z[i + (int64_t)j * n], R(1) / sig[j]);
      }
      stA(Bo + e, v);
    }
    return;
  }

  T2* hA = W;
  T2* hB = hA + K2;
  R* sig = reinterpret_cast<R*>(hB + K2);  // K2 singular values, then K2 marks
  R* mark = sig + K2;
  T2* C = hB + 2 * K2;  // the Jacobi matrix X (p x q): the core, or the dense sum
  T2* V = C + (small ? m * n : (int64_t)kt * kt);  // q x q
  if (!small) {
    house_qr(SA, m, kt, hA);
    house_qr(SB, n, kt, hB);
  }
  // core = R_A R_B^T (pa x pb; R entries (r, l) with r <= l), or for small
  // targets the whole sum A B^T (m x n)
  const int pa = small ? (int)m : (int)(m < kt ? m : (int64_t)kt);
  const int pb = small ? (int)n : (int)(n < kt ? n : (int64_t)kt);
  const bool tr = pa < pb;  // Jacobi on the orientation with fewer columns
  const int p = tr ? pb : pa, q = tr ? pa : pb;
  T2* X = C;  // p x q
  for (int e = threadIdx.x; e < pa * pb; e += HX_THREADS) {
    const int r = e % pa, c = e / pa;
    T2 acc = cz<T2>();
    for (int l = small ? 0 : max(r, c); l < kt; l++)
      acc = cadd(acc, cmul(SA[r + (int64_t)l * m], SB[c + (int64_t)l * n]));
    if (tr) X[c + r * p] = acc;  // X = core^T
    else X[r + c * p] = acc;
  }
  __syncthreads();
  jacobi_cols(X, p, q, V, red);
  const int r = pick_rank(X, p, q, sig, mark, kc, a.tol, s_idx);
  // top rows of the outputs: A' = [W S; 0], B' = [conj(Z); 0] (hlu rk_truncate)
  for (int64_t e = threadIdx.x; e < m * kc; e += HX_THREADS) {
    const int64_t i = e % m;
    const int l = (int)(e / m);
    T2 v = cz<T2>();
    if (l < r && i < pa) {
      const int j = s_idx[l];
      v = tr ? cscale(cconj(V[i + (int64_t)j * q]), sig[j]) : X[i + (int64_t)j * p];
    }
    stA(Ao + e, v);
  }
  for (int64_t e = threadIdx.x; e < n * kc; e += HX_THREADS) {
    const int64_t i = e % n;
    const int l = (int)(e / n);
    T2 v = cz<T2>();
    if (l < r && i < pb) {
      const int j = s_idx[l];
      v = tr ? cscale(X[i + (int64_t)j * p], R(1) / sig[j]) : cconj(V[i + (int64_t)j * q]);
    }
    stA(Bo + e, v);
  }
  __syncthreads();
  if (!small) {
    house_apply(SA, m, pa, hA, Ao, m, r);
    house_apply(SB, n, pb, hB, Bo, n, r);
  }
}

// ---------------------------------------------------------------- the executor
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// the ready task in queue slot q (-1 until pushed); -1 when the error word is
// set or the wait ran out (a bounded wait)
__device__ int wait_slot(const int* q, int* ctrl, int64_t limit) {
  int v = ld_acquire(q);
  if (v >= 0) return v;
  const long long t0 = clock64();
  unsigned ns = 32;
  for (;;) {
    __nanosleep(ns);
    if (ns < 512) ns <<= 1;
    v = ld_acquire(q);
    if (v >= 0) return v;
    if (ld_relaxed(ctrl + 1)) return -1;
    if (clock64() - t0 > limit) {
      atomicCAS(ctrl + 1, 0, 1);  // 1: a wait ran out of time
      return -1;
    }
  }
}

// *p -= 1 with acquire-release ordering (the last predecessor to finish
// sees every earlier one's results); returns the old value
__device__ __forceinline__ int dec_acq_rel(int* p) {
  int old;
  asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], -1;" : "=r"(old) : "l"(p) : "memory");
  return old;
}

// The executor pops ready tasks in the order they became ready: thread 0
// takes the next queue slot and waits (bounded) until a task is pushed into
// it; the CTA runs the task; then its threads release the successors, each
// decrementing a successor's pending count, and the one that reaches zero
// pushes it. Every task is pushed once, so the queue has one slot per task.
template <typename T2>
__global__ void __launch_bounds__(HX_THREADS, sizeof(T2) == 8 ? 4 : 2) hlu_exec_kernel(HluExecArgs a) {
  extern __shared__ __align__(16) unsigned char hx_smem[];
  T2* sm = reinterpret_cast<T2*>(hx_smem);
  __shared__ int s_task;
  T2* arena = reinterpret_cast<T2*>(a.arena);
  T2* slot = reinterpret_cast<T2*>(a.scratch) + (int64_t)blockIdx.x * a.scratch_per_cta;
  for (;;) {
    if (threadIdx.x == 0) {
      int t = -1;
      if (ld_relaxed(a.ctrl + 1) == 0) {
        const int h = atomicAdd(a.ctrl, 1);
        if (h < a.ntasks) {
          const unsigned long long tc = a.trace ? globaltimer() : 0ull;
          t = wait_slot(a.queue + h, a.ctrl, a.wait_cycles);
          if (t >= 0 && a.trace) {
            a.trace[3 * (int64_t)t] = tc;
            a.trace[3 * (int64_t)t + 1] = globaltimer();
          }
        }
      }
      s_task = t;
    }
    __syncthreads();
    const int ti = s_task;
    if (ti < 0) break;
    const HluTask t = a.tasks[ti];
    switch (t.type) {
      case HT_GEMM: task_gemm<T2>(t, arena, sm); break;
      case HT_LMUL: task_lmul<T2>(t, arena, sm); break;
      case HT_RMUL: task_rmul<T2>(t, arena, sm); break;
      case HT_QR: task_qr<T2>(t, a, arena, sm); break;
      case HT_TRUNC: task_trunc<T2>(t, a, arena, slot, sm); break;
      case HT_COPY: task_copy<T2>(t, arena, reinterpret_cast<const T2*>(a.F)); break;
      case HT_ZERO: task_zero<T2>(t, arena); break;
      default: break;
    }
    __syncthreads();  // the task's writes are done (and ordered before the releases below)
    if (threadIdx.x == 0 && a.trace) a.trace[3 * (int64_t)ti + 2] = globaltimer();
    const int s1 = __ldg(a.succ_off + ti + 1);
    for (int k = __ldg(a.succ_off + ti) + threadIdx.x; k < s1; k += HX_THREADS) {
      const int sc = __ldg(a.succ + k);
      __threadfence();
      if (dec_acq_rel(a.pending + sc) == 1) {
        const int pos = atomicAdd(a.ctrl + 4, 1);
        st_release(a.queue + pos, sc);
      }
    }
  }
}

template <typename T2>
int smem_bytes() {
  return Cx<T2>::SMEM * (int)sizeof(T2);
}

template <typename T2>
int occupancy() {
  static int occ = -1;
  if (occ >= 0) return occ;
  cudaFuncSetAttribute(hlu_exec_kernel<T2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       smem_bytes<T2>());
  int o = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, hlu_exec_kernel<T2>, HX_THREADS,
                                                    smem_bytes<T2>()) != cudaSuccess)
    o = 0;
  occ = o;
  return occ;
}

}  // namespace

int hlu_exec_occupancy(int precision) {
  return precision == 0 ? occupancy<double2>() : occupancy<float2>();
}

int launch_hlu_exec(const HluExecArgs& a, int grid, cudaStream_t s) {
  HluExecArgs args = a;
  void* p[] = {&args};
  cudaError_t e;
  if (a.precision == 0) {
    occupancy<double2>();
    e = cudaLaunchKernel((const void*)hlu_exec_kernel<double2>, grid, HX_THREADS, p,
                         smem_bytes<double2>(), s);
  } else {
    occupancy<float2>();
    e = cudaLaunchKernel((const void*)hlu_exec_kernel<float2>, grid, HX_THREADS, p,
                         smem_bytes<float2>(), s);
  }
  if (e != cudaSuccess) return -1;
  return 1;
}

}  // namespace bemgpu

namespace bemgpu {
namespace {
template <typename T2>
__global__ void finite_check_kernel(const T2* p, int64_t n, int* flag) {
  int bad = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T2 v = p[i];
    if (!isfinite(v.x) || !isfinite(v.y)) bad = 1;
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}
}  // namespace

void launch_hlu_finite_check(const void* arena, int64_t n, int precision, int* flag, int nsm,
                             cudaStream_t s) {
  if (n <= 0) return;
  if (precision == 0)
    finite_check_kernel<double2><<<nsm * 4, 256, 0, s>>>(reinterpret_cast<const double2*>(arena), n, flag);
  else
    finite_check_kernel<float2><<<nsm * 4, 256, 0, s>>>(reinterpret_cast<const float2*>(arena), n, flag);
}

}  // namespace bemgpu
