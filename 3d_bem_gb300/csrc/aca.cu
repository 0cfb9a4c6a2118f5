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
// Layout: U column l of a block at U + uoff + l*m (unscaled residual columns),
// V row l at V + voff + l*n (residual rows), s_l = 1/pivot at S + soff + l.
// The working residual column/row of the next step live in slot `rank` of the
// same storage, so the kernel needs no scratch memory.
#include "bem_kernels.h"
#include "quadrature.cuh"

namespace bemgpu {

static __constant__ QuadRules c_rules;

void aca_upload_rules(const QuadRules& r, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(c_rules, &r, sizeof(QuadRules), 0, cudaMemcpyHostToDevice, s);
}

namespace {
constexpr double TINY = 10.0 * 2.220446049250313080847263336181640625e-16;  // global.h:53
constexpr int NT = 128;
constexpr int NW = NT / 32;

struct Red {
  double v[NW];
  int i[NW];
  double2 c[NW];
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block-wide sum, result returned to every thread (deterministic order)
__device__ __forceinline__ double block_sum(double v, Red& red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red.v[w] = v;
  __syncthreads();
  double s = 0;
#pragma unroll
  for (int q = 0; q < NW; q++) s += red.v[q];
  return s;
}

// block-wide argmax of |.|, first index among equal maxima (Eigen maxCoeff)
__device__ __forceinline__ void block_argmax(double v, int idx, Red& red, double& best,
                                             int& bidx) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double v2 = __shfl_xor_sync(0xffffffffu, v, o);
    int i2 = __shfl_xor_sync(0xffffffffu, idx, o);
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

template <int MODE>
__device__ __forceinline__ double2 aca_entry(const AcaArgs& a, int64_t row, int64_t col) {
  if (MODE == 0) {
    Ops o = ops_eval(a.E, row, col, a.k, a.near_r, c_rules);
    double2 p, d;
    substitute(o, row == col, a.bc[col], a.alpha, p, d);
    return a.which ? d : p;
  } else {
    // point-cloud Helmholtz kernel of the reference's tests
    // (Tests/tests.h:30-42): exp(ikr)/(4 pi r), 1 at r = 0
    const double* x = a.rowpts + 3 * row;
    const double* y = a.colpts + 3 * col;
    double dx = x[0] - y[0], dy = x[1] - y[1], dz = x[2] - y[2];
    double r = sqrt(dx * dx + dy * dy + dz * dz);
    if (r == 0.0) return make_double2(1.0, 0.0);
    double s, c;
    sincos(a.k * r, &s, &c);
    double g = 1.0 / (4.0 * 3.14159265358979323846 * r);
    return make_double2(c * g, s * g);
  }
}

// dst[i] = A(r0+i, c0+ci) - sum_l U[:,l] (s_l V[l,ci])
template <int MODE>
__device__ void residual_col(const AcaArgs& a, const FarBlock& fb, const double2* U,
                             const double2* V, const double2* S, int k, int ci, double2* dst,
                             double2* coef) {
  for (int l = threadIdx.x; l < k; l += NT) coef[l] = cmul(S[l], V[(int64_t)l * fb.n + ci]);
  __syncthreads();
  for (int i = threadIdx.x; i < fb.m; i += NT) {
    double2 v = aca_entry<MODE>(a, fb.r0 + i, fb.c0 + ci);
    for (int l = 0; l < k; l++) v = csub(v, cmul(U[(int64_t)l * fb.m + i], coef[l]));
    dst[i] = v;
  }
  __syncthreads();
}

// dst[j] = A(r0+ri, c0+j) - sum_l (U[ri,l] s_l) V[l,:]
template <int MODE>
__device__ void residual_row(const AcaArgs& a, const FarBlock& fb, const double2* U,
                             const double2* V, const double2* S, int k, int ri, double2* dst,
                             double2* coef) {
  for (int l = threadIdx.x; l < k; l += NT) coef[l] = cmul(U[(int64_t)l * fb.m + ri], S[l]);
  __syncthreads();
  for (int j = threadIdx.x; j < fb.n; j += NT) {
    double2 v = aca_entry<MODE>(a, fb.r0 + ri, fb.c0 + j);
    for (int l = 0; l < k; l++) v = csub(v, cmul(coef[l], V[(int64_t)l * fb.n + j]));
    dst[j] = v;
  }
  __syncthreads();
}

// argmax_i |col[i]| over i != exclude
__device__ void argmax_abs(const double2* v, int len, int exclude, Red& red, double& best,
                           int& bidx) {
  double bv = -1.0;
  int bi = 0x7fffffff;
  for (int i = threadIdx.x; i < len; i += NT) {
    double x = (i == exclude) ? 0.0 : sqrt(cabs2(v[i]));
    if (x > bv) {
      bv = x;
      bi = i;
    }
  }
  block_argmax(bv, bi, red, best, bidx);
  if (bidx < 0 || bidx >= len) {  // all entries NaN: report a zero pivot at 0
    bidx = 0;
    best = 0.0;
  }
}

// normEstimate increment (hmatrix.cpp:570-574):
// |alpha|^2 |row|^2 |col|^2 + sum_{l<k} 2 conj(alpha) s_l (col^H U_l)(V_l row^H)
__device__ void norm_increment(const FarBlock& fb, const double2* U, const double2* V,
                               const double2* S, int k, const double2* col, const double2* row,
                               double2 alpha, Red& red, double& gain, double2& incr) {
  double cn = 0, rn = 0;
  for (int i = threadIdx.x; i < fb.m; i += NT) cn += cabs2(col[i]);
  for (int j = threadIdx.x; j < fb.n; j += NT) rn += cabs2(row[j]);
  cn = block_sum(cn, red);
  rn = block_sum(rn, red);
  gain = cabs2(alpha) * rn * cn;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double2 acc = make_double2(0, 0);
  for (int l = w; l < k; l += NW) {
    double cux = 0, cuy = 0, vrx = 0, vry = 0;
    const double2* Ul = U + (int64_t)l * fb.m;
    const double2* Vl = V + (int64_t)l * fb.n;
    for (int i = lane; i < fb.m; i += 32) {
      double2 c = col[i], u = Ul[i];  // conj(c) * u
      cux += c.x * u.x + c.y * u.y;
      cuy += c.x * u.y - c.y * u.x;
    }
    for (int j = lane; j < fb.n; j += 32) {
      double2 v = Vl[j], r = row[j];  // v * conj(r)
      vrx += v.x * r.x + v.y * r.y;
      vry += v.y * r.x - v.x * r.y;
    }
    cux = warp_sum(cux);
    cuy = warp_sum(cuy);
    vrx = warp_sum(vrx);
    vry = warp_sum(vry);
    double2 t = cmul(cmul(cconj(alpha), S[l]), cmul(make_double2(cux, cuy), make_double2(vrx, vry)));
    acc = cadd(acc, cscale(2.0, t));
  }
  __syncthreads();
  if (lane == 0) red.c[w] = acc;
  __syncthreads();
  incr = make_double2(gain, 0.0);
#pragma unroll
  for (int q = 0; q < NW; q++) incr = cadd(incr, red.c[q]);
  __syncthreads();
}

template <int MODE>
__global__ void __launch_bounds__(NT) aca_kernel(AcaArgs a) {
  __shared__ double2 coef[ACA_MAX_KCAP];
  __shared__ Red red;
  const int bi = a.order[blockIdx.x];
  const FarBlock fb = a.far[bi];
  const int m = fb.m, n = fb.n;
  int natural = min(m, n);
  if (a.max_rank > 0) natural = min(natural, a.max_rank);
  const int kmax = min(natural, fb.kcap);
  double2* U = a.U + fb.uoff;
  double2* V = a.V + fb.voff;
  double2* S = a.S + fb.soff;
  const double tol = a.tol;
  int k = 0;
  double2 est = make_double2(0, 0);
  bool converged = false;

  if (!a.extra) {
    // --- partialPivotACA ---
    int ci = (int)(pivot_hash(a.seed, (uint64_t)fb.id, 0) % (uint64_t)n);
    residual_col<MODE>(a, fb, U, V, S, 0, ci, U, coef);  // start column into slot 0
    int ri = -1;
    while (k < kmax) {
      const double2* colv = U + (int64_t)(k > 0 ? k - 1 : 0) * m;
      double cmax;
      argmax_abs(colv, m, k >= 1 ? ri : -1, red, cmax, ri);
      if (cmax <= TINY && k >= 1) break;
      double2* rowv = V + (int64_t)k * n;
      residual_row<MODE>(a, fb, U, V, S, k, ri, rowv, coef);
      double rmax;
      argmax_abs(rowv, n, -1, red, rmax, ci);
      if (rmax <= TINY && k >= 1) break;
      double2* newcol = U + (int64_t)k * m;
      residual_col<MODE>(a, fb, U, V, S, k, ci, newcol, coef);
      double2 alpha = cdiv(make_double2(1.0, 0.0), rowv[ci]);
      if (threadIdx.x == 0) S[k] = alpha;
      __syncthreads();
      double gain;
      double2 incr;
      norm_increment(fb, U, V, S, k, newcol, rowv, alpha, red, gain, incr);
      k++;
      est = cadd(est, incr);
      double target = tol * tol * est.x;
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
      double2 pivv = aca_entry<MODE>(a, fb.r0 + ri, fb.c0 + ci);
      double pabs = sqrt(cabs2(pivv));
      if (pabs < TINY) continue;
      // approximation already good at the seed?
      double2 approx = make_double2(0, 0);
      for (int l = 0; l < k; l++)
        approx = cadd(approx, cmul(cmul(U[(int64_t)l * m + ri], S[l]), V[(int64_t)l * n + ci]));
      if (sqrt(cabs2(cdiv(csub(pivv, approx), pivv))) < tol) continue;
      residual_col<MODE>(a, fb, U, V, S, k, ci, U + (int64_t)k * m, coef);
      bool first = true;
      while (k < kmax) {
        const double2* colv = first ? U + (int64_t)k * m : U + (int64_t)(k - 1) * m;
        double cmax;
        argmax_abs(colv, m, first ? -1 : ri, red, cmax, ri);
        first = false;
        if (cmax <= TINY && k >= 1) break;
        double2* rowv = V + (int64_t)k * n;
        residual_row<MODE>(a, fb, U, V, S, k, ri, rowv, coef);
        double rmax;
        argmax_abs(rowv, n, -1, red, rmax, ci);
        if (rmax <= TINY && k >= 1) break;
        double2* newcol = U + (int64_t)k * m;
        residual_col<MODE>(a, fb, U, V, S, k, ci, newcol, coef);
        double2 alpha = cdiv(make_double2(1.0, 0.0), rowv[ci]);
        if (threadIdx.x == 0) S[k] = alpha;
        __syncthreads();
        double gain;
        double2 incr;
        norm_increment(fb, U, V, S, k, newcol, rowv, alpha, red, gain, incr);
        double2 old = est;
        k++;
        est = cadd(est, incr);
        double target = tol * tol * est.x;
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

void launch_aca(const AcaArgs& a, cudaStream_t s) {
  if (a.nfar <= 0) return;
  if (a.mode == 0)
    aca_kernel<0><<<(unsigned)a.nfar, NT, 0, s>>>(a);
  else
    aca_kernel<1><<<(unsigned)a.nfar, NT, 0, s>>>(a);
}

}  // namespace bemgpu
