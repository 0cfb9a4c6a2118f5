// recompress.cu -- K4: truncating SVD recompression of the admissible blocks.
//
// Reference: BlockCluster::compressAdmissibleBlock (HMatrix/hmatrix.cpp:101-140)
// and HArithm::RkMatRankReduction (HMatrix/harithm.cpp:158-227): QR of U and
// of V^T, SVD of the small core R_A diag(s) R_B^T, keep the smallest rank whose
// relative Frobenius tail is below the tolerance
// (GoloubReinschSvd::minRankforError, golubReinschSVD.cpp:551-585), rewrite
// U, s, V. The reference's Golub-Reinsch SVD is replaced by a one-sided
// Jacobi SVD of the core, which yields the same singular triplets.
//
// One CTA per block. The Householder QRs run in a scratch copy of the
// factors (L2-resident for all but the largest blocks): per column one block
// reduction for the norm, then one warp per remaining column applies the
// reflector. The k x k Jacobi uses the round-robin ordering, k/2 disjoint
// column pairs per round, one warp per pair. The new factors are formed by
// applying the stored reflectors to the singular vectors, straight into the
// block's own pool slots. Arithmetic in the storage precision: FP64 for
// complex-FP64 pools, FP32 for complex-FP32 pools (whose entries carry FP32
// accuracy, well inside any truncation tolerance above 1e-6).
#include "bem_kernels.h"
#include "recompress.h"

namespace bemgpu {
namespace {

constexpr int RT = 256;
constexpr int RW = RT / 32;
constexpr int MAX_SWEEPS = 30;

template <typename T2> struct CT;
template <> struct CT<double2> {
  using R = double;
  static constexpr double TH = 1e-15;  // Jacobi: pair counts as orthogonal
  static __device__ __forceinline__ double2 mk(double x, double y) { return make_double2(x, y); }
};
template <> struct CT<float2> {
  using R = float;
  static constexpr float TH = 1e-6f;
  static __device__ __forceinline__ float2 mk(float x, float y) { return make_float2(x, y); }
};

template <typename T2>
__device__ __forceinline__ T2 mul(T2 a, T2 b) {
  return CT<T2>::mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T2>
__device__ __forceinline__ T2 cjmul(T2 a, T2 b) {  // conj(a) * b
  return CT<T2>::mk(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
template <typename T2, typename R>
__device__ __forceinline__ T2 scl(T2 a, R s) {
  return CT<T2>::mk(a.x * s, a.y * s);
}
template <typename T2>
__device__ __forceinline__ T2 add(T2 a, T2 b) {
  return CT<T2>::mk(a.x + b.x, a.y + b.y);
}
template <typename T2>
__device__ __forceinline__ T2 sub(T2 a, T2 b) {
  return CT<T2>::mk(a.x - b.x, a.y - b.y);
}
template <typename R>
__device__ __forceinline__ R wsum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// sum over the CTA, returned to every thread
template <typename R>
__device__ R block_sum(R v, R* red) {
  v = wsum(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  R t = 0;
#pragma unroll
  for (int w = 0; w < RW; w++) t += red[w];
  __syncthreads();
  return t;
}

// Householder QR of A (m x k, column-major, k <= m) in place: reflector j
// (unit 2-norm, H = I - 2 v v^H) in rows j..m-1 of column j, R above the
// diagonal, diag(R) in rd.
template <typename T2>
__device__ void householder(T2* A, int m, int k, T2* rd, typename CT<T2>::R* red) {
  using R = typename CT<T2>::R;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int j = 0; j < k; j++) {
    T2* col = A + (int64_t)j * m;
    R s = 0;
    for (int i = j + 1 + tid; i < m; i += RT) s += col[i].x * col[i].x + col[i].y * col[i].y;
    s = block_sum(s, red);
    const T2 alpha = col[j];
    const R an = sqrt(alpha.x * alpha.x + alpha.y * alpha.y);
    const R xn = sqrt(an * an + s);
    const T2 ph = an > 0 ? CT<T2>::mk(alpha.x / an, alpha.y / an) : CT<T2>::mk(1, 0);
    const R vn = sqrt(s + (an + xn) * (an + xn));
    const R inv = vn > 0 ? (R)1 / vn : (R)0;
    if (tid == 0) rd[j] = scl(ph, -xn);
    __syncthreads();  // every thread has read alpha
    for (int i = j + tid; i < m; i += RT)
      col[i] = scl(i == j ? add(alpha, scl(ph, xn)) : col[i], inv);
    __syncthreads();
    for (int c = j + 1 + warp; c < k; c += RW) {
      T2* cc = A + (int64_t)c * m;
      R dx = 0, dy = 0;
      for (int i = j + lane; i < m; i += 32) {
        const T2 p = cjmul(col[i], cc[i]);
        dx += p.x;
        dy += p.y;
      }
      const T2 d = CT<T2>::mk(2 * wsum(dx), 2 * wsum(dy));
      for (int i = j + lane; i < m; i += 32) cc[i] = sub(cc[i], mul(col[i], d));
    }
    __syncthreads();
  }
}

// X (m x r, column-major) := H_0 H_1 ... H_{k-1} X with the reflectors of A
template <typename T2>
__device__ void apply_q(const T2* A, int m, int k, T2* X, int r) {
  using R = typename CT<T2>::R;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int j = k - 1; j >= 0; j--) {
    const T2* v = A + (int64_t)j * m;
    for (int c = warp; c < r; c += RW) {
      T2* x = X + (int64_t)c * m;
      R dx = 0, dy = 0;
      for (int i = j + lane; i < m; i += 32) {
        const T2 p = cjmul(v[i], x[i]);
        dx += p.x;
        dy += p.y;
      }
      const T2 d = CT<T2>::mk(2 * wsum(dx), 2 * wsum(dy));
      for (int i = j + lane; i < m; i += 32) x[i] = sub(x[i], mul(v[i], d));
    }
    __syncthreads();
  }
}

// partner pairs of the circle method: round rd, pair p of q (even) players
__device__ __forceinline__ void rr_pair(int p, int rd, int q, int& a, int& b) {
  if (p == 0) {
    a = q - 1;
    b = rd;
  } else {
    a = (rd + p) % (q - 1);
    b = (rd - p + (q - 1)) % (q - 1);
  }
}

template <typename T2>
__global__ void __launch_bounds__(RT) recompress_kernel(RecompressArgs a) {
  using R = typename CT<T2>::R;
  __shared__ T2 rdA[ACA_MAX_KCAP], rdB[ACA_MAX_KCAP];
  __shared__ double sig[ACA_MAX_KCAP];
  __shared__ int ord[ACA_MAX_KCAP];
  __shared__ R red[RW];
  __shared__ int flag, newr;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int64_t o = blockIdx.x; o < a.nfar; o += gridDim.x) {
    const int64_t b = a.order ? a.order[o] : o;
    const FarBlock fb = a.far[b];
    const int m = fb.m, n = fb.n, k = a.rank[b];
    if (k <= 0 || k > min(m, n) || k > ACA_MAX_KCAP) continue;
    if (a.tol <= 0 && (k <= a.max_rank || a.max_rank <= 0)) continue;  // hmatrix.cpp:108
    T2* U = (T2*)a.U + fb.uoff;
    T2* V = (T2*)a.V + fb.voff;
    T2* S = (T2*)a.S + fb.soff;
    T2* QA = (T2*)a.wa + fb.uoff;
    T2* QB = (T2*)a.wb + fb.voff;
    T2* C = (T2*)a.wc + a.coff[b];
    T2* Z = C + (int64_t)k * k;
    // QA = U diag(s) (m x k); QB = V^T (n x k): V is k x n row-major
    for (int64_t i = tid; i < (int64_t)m * k; i += RT) QA[i] = mul(U[i], S[i / m]);
    for (int64_t i = tid; i < (int64_t)n * k; i += RT) QB[i] = V[i];
    __syncthreads();
    householder(QA, m, k, rdA, red);
    householder(QB, n, k, rdB, red);
    // core C = R_A R_B^T (k x k); Z = I
    for (int idx = tid; idx < k * k; idx += RT) {
      const int r = idx % k, c = idx / k;
      R sx = 0, sy = 0;
      for (int l = max(r, c); l < k; l++) {
        const T2 ra = l == r ? rdA[r] : QA[(int64_t)l * m + r];
        const T2 rb = l == c ? rdB[c] : QB[(int64_t)l * n + c];
        const T2 p = mul(ra, rb);
        sx += p.x;
        sy += p.y;
      }
      C[idx] = CT<T2>::mk(sx, sy);
      Z[idx] = CT<T2>::mk(r == c ? 1 : 0, 0);
    }
    __syncthreads();
    // one-sided Jacobi on the columns of C: C Z = W diag(sigma)
    const int q = k + (k & 1);
    for (int sweep = 0; sweep < MAX_SWEEPS && q > 1; sweep++) {
      if (tid == 0) flag = 0;
      __syncthreads();
      for (int rd = 0; rd < q - 1; rd++) {
        for (int p = warp; p < q / 2; p += RW) {
          int i1, i2;
          rr_pair(p, rd, q, i1, i2);
          if (i1 >= k || i2 >= k) continue;
          const int pa = min(i1, i2), pb = max(i1, i2);
          T2* ca = C + (int64_t)pa * k;
          T2* cb = C + (int64_t)pb * k;
          R na = 0, nb = 0, gx = 0, gy = 0;
          for (int i = lane; i < k; i += 32) {
            na += ca[i].x * ca[i].x + ca[i].y * ca[i].y;
            nb += cb[i].x * cb[i].x + cb[i].y * cb[i].y;
            const T2 g = cjmul(ca[i], cb[i]);
            gx += g.x;
            gy += g.y;
          }
          na = wsum(na);
          nb = wsum(nb);
          gx = wsum(gx);
          gy = wsum(gy);
          const R ga = sqrt(gx * gx + gy * gy);
          if (na == 0 || nb == 0 || ga == 0 || ga <= CT<T2>::TH * sqrt(na * nb)) continue;
          if (lane == 0) flag = 1;
          const T2 ec = CT<T2>::mk(gx / ga, -gy / ga);  // conj(e), e = g / |g|
          const R zeta = (nb - na) / (2 * ga);
          const R t = (zeta >= 0 ? (R)1 : (R)-1) / (fabs(zeta) + sqrt((R)1 + zeta * zeta));
          const R cs = (R)1 / sqrt((R)1 + t * t), sn = cs * t;
          T2* za = Z + (int64_t)pa * k;
          T2* zb = Z + (int64_t)pb * k;
          for (int i = lane; i < k; i += 32) {
            T2 x = ca[i], y = mul(cb[i], ec);
            ca[i] = sub(scl(x, cs), scl(y, sn));
            cb[i] = add(scl(x, sn), scl(y, cs));
            x = za[i];
            y = mul(zb[i], ec);
            za[i] = sub(scl(x, cs), scl(y, sn));
            zb[i] = add(scl(x, sn), scl(y, cs));
          }
        }
        __syncthreads();
      }
      const bool more = flag != 0;
      __syncthreads();
      if (!more) break;
    }
    // singular values = column norms, sorted descending (stable rank sort)
    for (int c = warp; c < k; c += RW) {
      R s = 0;
      for (int i = lane; i < k; i += 32) s += C[(int64_t)c * k + i].x * C[(int64_t)c * k + i].x +
                                              C[(int64_t)c * k + i].y * C[(int64_t)c * k + i].y;
      s = wsum(s);
      if (lane == 0) sig[c] = sqrt((double)s);
    }
    __syncthreads();
    for (int i = tid; i < k; i += RT) {
      int pos = 0;
      for (int j = 0; j < k; j++) pos += (sig[j] > sig[i] || (sig[j] == sig[i] && j < i)) ? 1 : 0;
      ord[pos] = i;
    }
    __syncthreads();
    if (tid == 0) {  // minRankforError, at least rank 1
      int mi = (a.max_rank > 0 && a.max_rank < k) ? (int)a.max_rank : k;
      int r = mi;
      if (a.tol > 0) {
        double full = 0;
        for (int l = 0; l < k; l++) full += sig[ord[l]] * sig[ord[l]];
        double res = full;
        for (int l = 1; l <= mi; l++) {
          res -= sig[ord[l - 1]] * sig[ord[l - 1]];
          if (res / full < a.tol * a.tol) {
            r = l;
            break;
          }
        }
      }
      newr = max(r, 1);
    }
    __syncthreads();
    const int r = newr;
    // U := Q_A [W_r; 0], W column l = C column ord[l] / sigma
    for (int64_t i = tid; i < (int64_t)m * r; i += RT) {
      const int l = (int)(i / m), row = (int)(i % m);
      const int c = ord[l];
      const double sv = sig[c];
      U[i] = (row < k && sv > 0) ? scl(C[(int64_t)c * k + row], (R)(1.0 / sv)) : CT<T2>::mk(0, 0);
    }
    // V^T := Q_B [conj(Z_r); 0] (n x r column-major = V r x n row-major)
    for (int64_t i = tid; i < (int64_t)n * r; i += RT) {
      const int l = (int)(i / n), row = (int)(i % n);
      const T2 z = row < k ? Z[(int64_t)ord[l] * k + row] : CT<T2>::mk(0, 0);
      V[i] = CT<T2>::mk(z.x, -z.y);
    }
    __syncthreads();
    apply_q(QA, m, k, U, r);
    apply_q(QB, n, k, V, r);
    for (int l = tid; l < r; l += RT) S[l] = CT<T2>::mk((R)sig[ord[l]], 0);
    if (tid == 0) a.rank[b] = r;
    __syncthreads();
  }
}

}  // namespace

int launch_recompress(const RecompressArgs& a, cudaStream_t s) {
  if (a.nfar <= 0) return 0;
  const unsigned grid = (unsigned)std::min<int64_t>(a.nfar, 152 * 16);
  if (a.precision == 0)
    recompress_kernel<double2><<<grid, RT, 0, s>>>(a);
  else
    recompress_kernel<float2><<<grid, RT, 0, s>>>(a);
  return 1;
}

}  // namespace bemgpu
