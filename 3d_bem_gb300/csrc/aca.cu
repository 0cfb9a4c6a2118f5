// aca.cu -- K3: adaptive cross approximation of every admissible block, one
// CTA per block, all blocks of a matrix in one launch.
//
// Reference: BlockCluster::partialPivotACA (HMatrix/hmatrix.cpp:471-593) for
// the phi matrix and partialPivotACAextra (:595-745) with the normal-filtered
// pivot seeds of BoundaryElementSolver::getNormalFilteredPivotIndices
// (boundaryelementsolver.cpp:2052-2172) for the dPhi matrix. Both keep the
// reference's pivoting, tiny-pivot breaks, Frobenius norm estimate and
// stopping test; the random start column / seed member picks are replaced by
// a seeded hash so runs are reproducible.
//
// Two precisions share the code: T = double2 (complex FP64 storage and
// arithmetic, the plain method) and T = float2 (mixed: FP32 regular
// quadrature with an FP64-formed centroid difference, FP64 singular and
// near-singular rules, complex FP32 storage and residual updates).
//
// Layout: U column l of a block at U + uoff + l*m (unscaled residual columns),
// V row l at V + voff + l*n (residual rows), s_l = 1/pivot at S + soff + l.
// The working residual column/row of the next step live in slot `rank` of the
// same storage, so the kernel needs no scratch memory.
#include <mutex>
#include <set>

#include "bem_kernels.h"
#include "quadrature.cuh"
#include "selector.h"

namespace bemgpu {

static __constant__ QuadRules c_rules;

// class rules of the learned rule table (1, 3, 7, 13, 25 points)
struct AcaClassRules {
  float x1[SEL_CLASS_POINTS], x2[SEL_CLASS_POINTS], w[SEL_CLASS_POINTS];
  int off[SEL_C + 1];
};
static __constant__ AcaClassRules c_cls;

// The tables (always the same) go to each device's constant memory once,
// synchronously, so no later handle rewrites them under running kernels.
void aca_upload_rules(const QuadRules& r, cudaStream_t s) {
  (void)s;
  static std::mutex mu;
  static std::set<int> done;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  if (done.count(dev)) return;
  AcaClassRules cr;
  sel_class_rule_tables(cr.x1, cr.x2, cr.w, cr.off);
  if (cudaMemcpyToSymbol(c_rules, &r, sizeof(QuadRules)) == cudaSuccess &&
      cudaMemcpyToSymbol(c_cls, &cr, sizeof(AcaClassRules)) == cudaSuccess)
    done.insert(dev);
}

namespace {
constexpr double TINY = 10.0 * 2.220446049250313080847263336181640625e-16;  // global.h:53
constexpr int NW_MAX = 16;  // up to 512 threads per CTA

// complex arithmetic on the storage type
__device__ __forceinline__ double2 cx_mul(double2 a, double2 b) { return cmul(a, b); }
__device__ __forceinline__ float2 cx_mul(float2 a, float2 b) { return fmul(a, b); }
__device__ __forceinline__ double2 cx_sub(double2 a, double2 b) { return csub(a, b); }
__device__ __forceinline__ float2 cx_sub(float2 a, float2 b) { return fsub(a, b); }
__device__ __forceinline__ double2 to_d(double2 a) { return a; }
__device__ __forceinline__ double2 to_d(float2 a) { return make_double2(a.x, a.y); }
template <typename T> __device__ __forceinline__ T from_d(double2 a);
template <> __device__ __forceinline__ double2 from_d<double2>(double2 a) { return a; }
template <> __device__ __forceinline__ float2 from_d<float2>(double2 a) {
  return make_float2((float)a.x, (float)a.y);
}

// real type and complex helpers of the storage precision
template <typename T> struct Cx;
template <> struct Cx<double2> {
  using R = double;
  static __device__ __forceinline__ double2 make(double x, double y) { return make_double2(x, y); }
};
template <> struct Cx<float2> {
  using R = float;
  static __device__ __forceinline__ float2 make(float x, float y) { return make_float2(x, y); }
};

// complex reciprocal (Smith) in the storage precision
template <typename T>
__device__ __forceinline__ T cx_recip(T b) {
  using R = typename Cx<T>::R;
  if (fabs(b.x) >= fabs(b.y)) {
    const R r = b.y / b.x, d = b.x + b.y * r;
    return Cx<T>::make((R)1 / d, -r / d);
  }
  const R r = b.x / b.y, d = b.y + b.x * r;
  return Cx<T>::make(r / d, (R)-1 / d);
}

template <typename R>
struct Red {
  R v[NW_MAX];
  int i[NW_MAX];
  R cx[NW_MAX], cy[NW_MAX];
};

template <typename R>
__device__ __forceinline__ R warp_sum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block-wide sum, result returned to every thread (deterministic order)
template <int NT, typename R>
__device__ __forceinline__ R block_sum(R v, Red<R>& red) {
  constexpr int NW = NT / 32;
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red.v[w] = v;
  __syncthreads();
  R s = 0;
#pragma unroll
  for (int q = 0; q < NW; q++) s += red.v[q];
  return s;
}

// block-wide argmax, first index among equal maxima (Eigen maxCoeff)
template <int NT, typename R>
__device__ __forceinline__ void block_argmax(R v, int idx, Red<R>& red, R& best, int& bidx) {
  constexpr int NW = NT / 32;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const R v2 = __shfl_xor_sync(0xffffffffu, v, o);
    const int i2 = __shfl_xor_sync(0xffffffffu, idx, o);
    if (v2 > v || (v2 == v && i2 < idx)) {
      v = v2;
      idx = i2;
    }
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) {
    red.v[w] = v;
    red.i[w] = idx;
  }
  __syncthreads();
  best = red.v[0];
  bidx = red.i[0];
#pragma unroll
  for (int q = 1; q < NW; q++)
    if (red.v[q] > best || (red.v[q] == best && red.i[q] < bidx)) {
      best = red.v[q];
      bidx = red.i[q];
    }
}

// FP32 near-singular test on the two-float centroid difference; used only to
// pick the rule inside ACA rows/columns (the near-field blocks use the host's
// exact classification).
__device__ __forceinline__ bool near_pair32(const ElemF* __restrict__ EF, int64_t row,
                                            int64_t col, float near_r2) {
  float dx, dy, dz;
  centroid_diff(EF[row], EF[col], dx, dy, dz);
  return dx * dx + dy * dy + dz * dz < near_r2;
}

// the complex-FP64 entry (singular / near-singular pairs of the mixed path,
// every pair of the plain path); kept out of line so the FP32 fast path does
// not carry its registers
__device__ __noinline__ double2 entry64(const AcaArgs& a, int64_t row, int64_t col) {
  Ops o = ops_eval(a.E, row, col, a.k, a.near_r, c_rules);
  // impedance plane: the reflected element with the regular rule
  // (implicitPhiMatrixPlusReflected, boundaryelementsolver.cpp:2042-2050)
  if (a.Er) ops_add(o, ops_regular(a.E[row], a.Er[col], a.k, c_rules));
  double2 p, d;
  substitute(o, row == col, a.bc[col], a.alpha, p, d);
  return a.which ? d : p;
}

__device__ __noinline__ float2 entry64f(const AcaArgs& a, int64_t row, int64_t col) {
  const double2 v = entry64(a, row, col);
  return make_float2((float)v.x, (float)v.y);
}

// MODE 0: BEM entries; 2: BEM entries with an impedance plane (the
// reflected element's operators added); 1: point-cloud test kernel.
template <int MODE, typename T>
__device__ __forceinline__ T aca_entry(const AcaArgs& a, int64_t row, int64_t col) {
  if constexpr (MODE == 0 || MODE == 2) {
    if constexpr (sizeof(T) == sizeof(float2)) {
      // mixed precision: FP32 regular rule, FP64 singular / near-singular
      if (row != col && !near_pair32(a.EF, row, col, a.near_r2f)) {
        OpsF o;
        if (a.rule_tab) {  // learned order: table bin of (d / e_max, k e_max)
          float dx, dy, dz;
          centroid_diff(a.EF[row], a.EF[col], dx, dy, dz);
          const float em = a.EF[col].emax;
          const float x = __logf(sqrtf(dx * dx + dy * dy + dz * dz) / em);
          const float y = __logf(a.kf * em);
          const int ix = min(max((int)floorf((x - a.tab_x0) / a.tab_dx), 0), ACA_TAB_N - 1);
          const int iy = min(max((int)floorf((y - a.tab_y0) / a.tab_dy), 0), ACA_TAB_N - 1);
          const int c = min((int)a.rule_tab[ix * ACA_TAB_N + iy], SEL_C - 1);
          o = ops_rule32_pts(a.EF, row, col, a.kf, c_cls.off[c], c_cls.off[c + 1], c_cls.x1,
                             c_cls.x2, c_cls.w);
        } else {
          o = ops_regular32(a.EF, row, col, a.kf, c_rules);
        }
        if constexpr (MODE == 2) ops_add(o, ops_regular32_pq(a.EF[row], a.EFr[col], a.kf, c_rules));
        float2 p, d;
        substitute32(o, a.bc[col], a.alphaf, p, d);
        return a.which ? d : p;
      }
      return entry64f(a, row, col);
    } else {
      return entry64(a, row, col);
    }
  } else {
    // point-cloud Helmholtz kernel of the reference's tests
    // (Tests/tests.h:30-42): exp(ikr)/(4 pi r), 1 at r = 0
    const double* x = a.rowpts + 3 * row;
    const double* y = a.colpts + 3 * col;
    double dx = x[0] - y[0], dy = x[1] - y[1], dz = x[2] - y[2];
    double r = sqrt(dx * dx + dy * dy + dz * dz);
    if (r == 0.0) return from_d<T>(make_double2(1.0, 0.0));
    double s, c;
    sincos(a.k * r, &s, &c);
    double g = 1.0 / (4.0 * 3.14159265358979323846 * r);
    return from_d<T>(make_double2(c * g, s * g));
  }
}

// Lane q's share of the entry when Q lanes split it (Q a power of two): the
// FP32 regular rule over the points q, q + Q, ..; entries on the FP64 path
// (singular / near-singular pairs, the complex-FP64 method, the point-cloud
// kernel) come whole from lane 0. The Q shares sum to the entry (the BC
// substitution of regular entries is linear in the operators).
template <int MODE, typename T>
__device__ __forceinline__ T aca_entry_part(const AcaArgs& a, int64_t row, int64_t col, int q,
                                            int Q) {
  if constexpr ((MODE == 0 || MODE == 2) && sizeof(T) == sizeof(float2)) {
    if (row != col && !near_pair32(a.EF, row, col, a.near_r2f)) {
      const ElemF& P = a.EF[row];
      const ElemF& Qe = a.EF[col];
      OpsF o;
      if (a.rule_tab) {
        float dx, dy, dz;
        centroid_diff(P, Qe, dx, dy, dz);
        const float em = Qe.emax;
        const float x = __logf(sqrtf(dx * dx + dy * dy + dz * dz) / em);
        const float y = __logf(a.kf * em);
        const int ix = min(max((int)floorf((x - a.tab_x0) / a.tab_dx), 0), ACA_TAB_N - 1);
        const int iy = min(max((int)floorf((y - a.tab_y0) / a.tab_dy), 0), ACA_TAB_N - 1);
        const int c = min((int)a.rule_tab[ix * ACA_TAB_N + iy], SEL_C - 1);
        o = ops_pts32(P, Qe, a.kf, c_cls.x1, c_cls.x2, c_cls.w, c_cls.off[c] + q, c_cls.off[c + 1], Q);
      } else {
        o = ops_pts32(P, Qe, a.kf, c_rules.freg_x1, c_rules.freg_x2, c_rules.freg_w, q, 16, Q);
      }
      if constexpr (MODE == 2)
        ops_add(o, ops_pts32(P, a.EFr[col], a.kf, c_rules.freg_x1, c_rules.freg_x2,
                             c_rules.freg_w, q, 16, Q));
      float2 p, d;
      substitute32(o, a.bc[col], a.alphaf, p, d);
      return a.which ? d : p;
    }
    return q == 0 ? entry64f(a, row, col) : T{0, 0};
  } else {
    return q == 0 ? aca_entry<MODE, T>(a, row, col) : T{0, 0};
  }
}

// Lanes per entry of a residual row or column of cnt entries: the FP32 path
// splits each entry's rule over 4-16 lanes when at most a quarter of the CTA
// would be busy otherwise (a 32-entry column on 128 threads: 4 lanes each).
// Two lanes per entry measured slower than one (sphere, 20,480 elements).
template <int MODE, typename T, int NT>
__device__ __forceinline__ int lanes_per_entry(int cnt) {
  if constexpr (!((MODE == 0 || MODE == 2) && sizeof(T) == sizeof(float2))) return 1;
  if (4 * cnt > NT) return 1;
  int Q = 4;
  while (Q < 16 && 2 * Q * cnt <= NT) Q *= 2;
  return Q;
}

// sum over l = q, q + Q, .. < k of p[l * stride] * c[l]
template <typename T>
__device__ __forceinline__ T dot_strided_part(const T* p, int64_t stride, const T* c, int k, int q,
                                              int Q) {
  T acc{0, 0};
  for (int l = q; l < k; l += Q) {
    const T v = p[(int64_t)l * stride], cq = c[l];
    acc.x += v.x * cq.x - v.y * cq.y;
    acc.y += v.x * cq.y + v.y * cq.x;
  }
  return acc;
}

// sum_l p[l * stride] * c[l] with 4 independent loads in flight (the chain
// of dependent loads was the ACA's latency bottleneck)
template <typename T>
__device__ __forceinline__ T dot_strided(const T* p, int64_t stride, const T* c, int k) {
  T acc[4];
#pragma unroll
  for (int q = 0; q < 4; q++) acc[q] = T{0, 0};
  int l = 0;
  for (; l + 4 <= k; l += 4) {
    T v[4];
#pragma unroll
    for (int q = 0; q < 4; q++) v[q] = p[(int64_t)(l + q) * stride];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const T cq = c[l + q];
      acc[q].x += v[q].x * cq.x - v[q].y * cq.y;
      acc[q].y += v[q].x * cq.y + v[q].y * cq.x;
    }
  }
  for (; l < k; l++) {
    const T v = p[(int64_t)l * stride], cq = c[l];
    acc[0].x += v.x * cq.x - v.y * cq.y;
    acc[0].y += v.x * cq.y + v.y * cq.x;
  }
#pragma unroll
  for (int q = 1; q < 4; q++) {
    acc[0].x += acc[q].x;
    acc[0].y += acc[q].y;
  }
  return acc[0];
}

// dst[i] = A(r0+i, c0+ci) - sum_l U[:,l] (s_l V[l,ci])
template <int MODE, typename T, int NT>
__device__ void residual_col(const AcaArgs& a, const FarBlock& fb, const T* U, const T* V,
                             const T* S, int k, int ci, T* dst, T* coef) {
  for (int l = threadIdx.x; l < k; l += NT) coef[l] = cx_mul(S[l], V[(int64_t)l * fb.n + ci]);
  __syncthreads();
  // Q lanes per entry (consecutive lanes; every lane of a warp loops alike)
  const int Q = lanes_per_entry<MODE, T, NT>(fb.m);
  const int q = threadIdx.x & (Q - 1);
  for (int base = 0; base < fb.m; base += NT / Q) {
    const int i = base + threadIdx.x / Q;
    T v{0, 0};
    if (i < fb.m)
      v = cx_sub(aca_entry_part<MODE, T>(a, fb.r0 + i, fb.c0 + ci, q, Q),
                 Q == 1 ? dot_strided(U + i, (int64_t)fb.m, coef, k)
                        : dot_strided_part(U + i, (int64_t)fb.m, coef, k, q, Q));
    for (int o = Q / 2; o > 0; o >>= 1) {
      v.x += __shfl_xor_sync(0xffffffffu, v.x, o, Q);
      v.y += __shfl_xor_sync(0xffffffffu, v.y, o, Q);
    }
    if (q == 0 && i < fb.m) dst[i] = v;
  }
  __syncthreads();
}

// dst[j] = A(r0+ri, c0+j) - sum_l (U[ri,l] s_l) V[l,:]
template <int MODE, typename T, int NT>
__device__ void residual_row(const AcaArgs& a, const FarBlock& fb, const T* U, const T* V,
                             const T* S, int k, int ri, T* dst, T* coef) {
  for (int l = threadIdx.x; l < k; l += NT) coef[l] = cx_mul(U[(int64_t)l * fb.m + ri], S[l]);
  __syncthreads();
  const int Q = lanes_per_entry<MODE, T, NT>(fb.n);
  const int q = threadIdx.x & (Q - 1);
  for (int base = 0; base < fb.n; base += NT / Q) {
    const int j = base + threadIdx.x / Q;
    T v{0, 0};
    if (j < fb.n)
      v = cx_sub(aca_entry_part<MODE, T>(a, fb.r0 + ri, fb.c0 + j, q, Q),
                 Q == 1 ? dot_strided(V + j, (int64_t)fb.n, coef, k)
                        : dot_strided_part(V + j, (int64_t)fb.n, coef, k, q, Q));
    for (int o = Q / 2; o > 0; o >>= 1) {
      v.x += __shfl_xor_sync(0xffffffffu, v.x, o, Q);
      v.y += __shfl_xor_sync(0xffffffffu, v.y, o, Q);
    }
    if (q == 0 && j < fb.n) dst[j] = v;
  }
  __syncthreads();
}

// squared modulus in the storage precision (the argmax compares |v|^2, which
// orders like |v|; the FP32 path stays off the FP64 pipe)
__device__ __forceinline__ double mag2(double2 v) { return v.x * v.x + v.y * v.y; }
__device__ __forceinline__ float mag2(float2 v) { return v.x * v.x + v.y * v.y; }

// argmax_i |v[i]| over i != exclude; best = |v[bidx]| (compares |v|^2,
// which orders like |v|)
template <typename T, int NT>
__device__ void argmax_abs(const T* v, int len, int exclude, Red<typename Cx<T>::R>& red,
                           typename Cx<T>::R& best, int& bidx) {
  using R = typename Cx<T>::R;
  R bv = (R)-1;
  int bi = 0x7fffffff;
  for (int i = threadIdx.x; i < len; i += NT) {
    const R x = (i == exclude) ? (R)0 : mag2(v[i]);
    if (x > bv) {
      bv = x;
      bi = i;
    }
  }
  block_argmax<NT, R>(bv, bi, red, best, bidx);
  if (bidx < 0 || bidx >= len) {  // all entries NaN: report a zero pivot at 0
    bidx = 0;
    best = 0;
  }
  best = sqrt(best);
}

// normEstimate increment (hmatrix.cpp:570-574):
// |alpha|^2 |row|^2 |col|^2 + sum_{l<k} 2 conj(alpha) s_l (col^H U_l)(V_l row^H),
// all in the storage precision (the estimate only steers the stopping test)
template <typename T, int NT>
__device__ void norm_increment(const FarBlock& fb, const T* U, const T* V, const T* S, int k,
                               const T* col, const T* row, T alpha, Red<typename Cx<T>::R>& red,
                               typename Cx<T>::R& gain, T& incr) {
  using R = typename Cx<T>::R;
  R c0 = 0, r0 = 0;
  for (int i = threadIdx.x; i < fb.m; i += NT) c0 += mag2(col[i]);
  for (int j = threadIdx.x; j < fb.n; j += NT) r0 += mag2(row[j]);
  const R cn = block_sum<NT, R>(c0, red);
  const R rn = block_sum<NT, R>(r0, red);
  gain = mag2(alpha) * rn * cn;
  constexpr int NW = NT / 32;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  R accx = 0, accy = 0;
  const T ca = Cx<T>::make(alpha.x, -alpha.y);
  for (int l = w; l < k; l += NW) {
    const T* Ul = U + (int64_t)l * fb.m;
    const T* Vl = V + (int64_t)l * fb.n;
    R ax = 0, ay = 0, bx = 0, by = 0;
    for (int i = lane; i < fb.m; i += 32) {
      const T c = col[i], u = Ul[i];  // conj(c) * u
      ax += c.x * u.x + c.y * u.y;
      ay += c.x * u.y - c.y * u.x;
    }
    for (int j = lane; j < fb.n; j += 32) {
      const T vv = Vl[j], r = row[j];  // v * conj(r)
      bx += vv.x * r.x + vv.y * r.y;
      by += vv.y * r.x - vv.x * r.y;
    }
    ax = warp_sum(ax);
    ay = warp_sum(ay);
    bx = warp_sum(bx);
    by = warp_sum(by);
    const T t = cx_mul(cx_mul(ca, S[l]), cx_mul(Cx<T>::make(ax, ay), Cx<T>::make(bx, by)));
    accx += 2 * t.x;
    accy += 2 * t.y;
  }
  __syncthreads();
  if (lane == 0) {
    red.cx[w] = accx;
    red.cy[w] = accy;
  }
  __syncthreads();
  incr = Cx<T>::make(gain, 0);
#pragma unroll
  for (int q = 0; q < NW; q++) {
    incr.x += red.cx[q];
    incr.y += red.cy[q];
  }
  __syncthreads();
}

// Occupancy over registers: the 128-thread kernel is capped at 64 registers
// (8 CTAs per SM), the 512-thread one at 64 (2 CTAs per SM). Despite the
// spills this causes, the ACA phase at 20,480 elements drops from 24.4 ms
// (uncapped, 168 registers, 3 CTAs per SM) to 19.7 ms.
template <int MODE, typename T, int NT>
__global__ void __launch_bounds__(NT, NT == 128 ? 8 : 2) aca_kernel(AcaArgs a) {
  __shared__ T coef[ACA_MAX_KCAP];
  using R = typename Cx<T>::R;
  __shared__ Red<R> red;
  const int bi = a.order[blockIdx.x];
  const FarBlock fb = a.far[bi];
  const int m = fb.m, n = fb.n;
  int natural = min(m, n);
  if (a.max_rank > 0) natural = min(natural, a.max_rank);
  const int kmax = min(natural, fb.kcap);
  T* U = (T*)a.U + fb.uoff;
  T* V = (T*)a.V + fb.voff;
  T* S = (T*)a.S + fb.soff;
  const R tol = (R)a.tol;
  const R tiny = (R)TINY;
  int k = 0;
  T est = Cx<T>::make(0, 0);
  bool converged = false;

  if (!a.extra) {
    // --- partialPivotACA ---
    int ci = (int)(pivot_hash(a.seed, (uint64_t)fb.id, 0) % (uint64_t)n);
    residual_col<MODE, T, NT>(a, fb, U, V, S, 0, ci, U, coef);  // start column into slot 0
    int ri = -1;
    while (k < kmax) {
      const T* colv = U + (int64_t)(k > 0 ? k - 1 : 0) * m;
      R cmax;
      argmax_abs<T, NT>(colv, m, k >= 1 ? ri : -1, red, cmax, ri);
      if (cmax <= tiny && k >= 1) break;
      T* rowv = V + (int64_t)k * n;
      residual_row<MODE, T, NT>(a, fb, U, V, S, k, ri, rowv, coef);
      R rmax;
      argmax_abs<T, NT>(rowv, n, -1, red, rmax, ci);
      if (rmax <= tiny && k >= 1) break;
      T* newcol = U + (int64_t)k * m;
      residual_col<MODE, T, NT>(a, fb, U, V, S, k, ci, newcol, coef);
      const T alpha = cx_recip(rowv[ci]);
      if (threadIdx.x == 0) S[k] = alpha;
      __syncthreads();
      R gain;
      T incr;
      norm_increment<T, NT>(fb, U, V, S, k, newcol, rowv, alpha, red, gain, incr);
      k++;
      est.x += incr.x;
      est.y += incr.y;
      const R target = tol * tol * est.x;
      if (tol > 0 && gain < target) {
        converged = true;
        break;
      }
    }
  } else {
    // --- partialPivotACAextra with host-computed normal-filtered seeds ---
    const int32_t* piv = a.piv_rc + 2 * a.piv_off[bi];
    const int npiv = a.piv_cnt[bi];
    for (int p = 0; p < npiv && k < kmax; p++) {
      int ri = piv[2 * p], ci = piv[2 * p + 1];
      const T pivv = aca_entry_part<MODE, T>(a, fb.r0 + ri, fb.c0 + ci, 0, 1);
      const R pabs2 = mag2(pivv);
      if (sqrt(pabs2) < tiny) continue;
      // approximation already good at the seed?
      T approx = Cx<T>::make(0, 0);
      for (int l = 0; l < k; l++) {
        const T t = cx_mul(cx_mul(U[(int64_t)l * m + ri], S[l]), V[(int64_t)l * n + ci]);
        approx.x += t.x;
        approx.y += t.y;
      }
      if (sqrt(mag2(cx_sub(pivv, approx)) / pabs2) < tol) continue;
      residual_col<MODE, T, NT>(a, fb, U, V, S, k, ci, U + (int64_t)k * m, coef);
      bool first = true;
      while (k < kmax) {
        const T* colv = first ? U + (int64_t)k * m : U + (int64_t)(k - 1) * m;
        R cmax;
        argmax_abs<T, NT>(colv, m, first ? -1 : ri, red, cmax, ri);
        first = false;
        if (cmax <= tiny && k >= 1) break;
        T* rowv = V + (int64_t)k * n;
        residual_row<MODE, T, NT>(a, fb, U, V, S, k, ri, rowv, coef);
        R rmax;
        argmax_abs<T, NT>(rowv, n, -1, red, rmax, ci);
        if (rmax <= tiny && k >= 1) break;
        T* newcol = U + (int64_t)k * m;
        residual_col<MODE, T, NT>(a, fb, U, V, S, k, ci, newcol, coef);
        const T alpha = cx_recip(rowv[ci]);
        if (threadIdx.x == 0) S[k] = alpha;
        __syncthreads();
        R gain;
        T incr;
        norm_increment<T, NT>(fb, U, V, S, k, newcol, rowv, alpha, red, gain, incr);
        const T old = est;
        k++;
        est.x += incr.x;
        est.y += incr.y;
        const R target = tol * tol * est.x;
        if (tol > 0 && gain < target) {
          if (gain < 0.1 * target) {  // roll back the last rank (hmatrix.cpp:724-728)
            k--;
            est = old;
          }
          break;
        }
      }
    }
    converged = true;  // the seed list, not the rank cap, ends ACAextra
    if (k == kmax && kmax < natural) converged = false;
  }
  if (threadIdx.x == 0) {
    a.rank[bi] = k;
    a.flags[bi] = (!converged && k == kmax && kmax < natural) ? 1 : 0;
  }
}
}  // namespace

template <int NT>
void launch_nt(const AcaArgs& a, cudaStream_t s) {
  const unsigned g = (unsigned)a.nfar;
  const bool plane = a.mode == 0 && a.Er != nullptr;
  if (a.precision == 0) {
    if (plane) aca_kernel<2, double2, NT><<<g, NT, 0, s>>>(a);
    else if (a.mode == 0) aca_kernel<0, double2, NT><<<g, NT, 0, s>>>(a);
    else aca_kernel<1, double2, NT><<<g, NT, 0, s>>>(a);
  } else {
    if (plane) aca_kernel<2, float2, NT><<<g, NT, 0, s>>>(a);
    else if (a.mode == 0) aca_kernel<0, float2, NT><<<g, NT, 0, s>>>(a);
    else aca_kernel<1, float2, NT><<<g, NT, 0, s>>>(a);
  }
}

// a.order / a.nfar select the blocks of this launch; threads is 128 or 512
// (large blocks get 16 warps so their O(k (m+n)) residual and norm updates
// stream with enough loads in flight).
int launch_aca(const AcaArgs& a, int threads, cudaStream_t s) {
  if (a.nfar <= 0) return 0;
  if (threads >= 512) launch_nt<512>(a, s);
  else launch_nt<128>(a, s);
  return 1;
}

}  // namespace bemgpu
