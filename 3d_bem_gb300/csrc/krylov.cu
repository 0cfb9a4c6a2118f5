// krylov.cu -- K6: restarted GMRES building blocks in FP64 for R independent
// right-hand sides that share each operator application.
//
// Reference: GMRES::gmresSolve / gmresLUPreconditionedSolve
// (HMatrix/gmres.h:170-207) call Eigen's GMRES (Householder Arnoldi, Givens
// rotations, restart 300, tolerance on ||b - A x|| / ||b||). This is the same
// Krylov method (Saad & Schultz 1986) with classical Gram-Schmidt applied
// twice (CGS2) for the Arnoldi step, which maps to two dense passes over the
// basis instead of a sequence of dependent Householder reflections.
//
// Basis layout: V[q][r][i] (q = basis index, r = right-hand side), so the
// R vectors of one basis index are one N x R column-major panel.
// Hessenberg column j of RHS r: H[(r * m + j) * (m + 1) + i].
#include "bem_kernels.h"
#include "krylov.h"

#include <algorithm>
#include "quadrature.cuh"

namespace bemgpu {
namespace {

constexpr int DT = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// partial[cta][r][q] = sum_{i in chunk} conj(V[q][r][i]) w[r][i]; grid
// (chunks, task groups): the (q, r) dot products of a chunk are spread over
// gridDim.y CTAs, one warp each, so long bases (many q) at small N do not
// queue on the few CTAs of the chunks
__global__ void __launch_bounds__(DT) dot_partial_kernel(const double2* __restrict__ Vb,
                                                         const double2* __restrict__ w, int64_t N,
                                                         int R, int nq, int64_t chunk,
                                                         const GmresState* __restrict__ st,
                                                         double2* __restrict__ partial) {
  const int64_t i0 = (int64_t)blockIdx.x * chunk;
  const int64_t i1 = min(N, i0 + chunk);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int task = blockIdx.y * (DT / 32) + warp; task < nq * R; task += gridDim.y * (DT / 32)) {
    const int q = task / R, r = task % R;
    double sx = 0, sy = 0;
    if (!st[r].done) {
      const double2* v = Vb + ((int64_t)q * R + r) * N;
      const double2* ww = w + (int64_t)r * N;
      for (int64_t i = i0 + lane; i < i1; i += 32) {
        double2 a = v[i], b = ww[i];
        sx += a.x * b.x + a.y * b.y;
        sy += a.x * b.y - a.y * b.x;
      }
      sx = warp_sum(sx);
      sy = warp_sum(sy);
    }
    if (lane == 0) partial[((int64_t)blockIdx.x * R + r) * nq + q] = make_double2(sx, sy);
  }
}

// partial squared norms of R vectors: partial[cta][r]
__global__ void __launch_bounds__(DT) nrm_partial_kernel(const double2* __restrict__ w, int64_t N,
                                                         int R, int64_t chunk,
                                                         double* __restrict__ partial) {
  __shared__ double red[DT / 32];
  const int64_t i0 = (int64_t)blockIdx.x * chunk;
  const int64_t i1 = min(N, i0 + chunk);
  for (int r = 0; r < R; r++) {
    double s = 0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += DT) s += cabs2(w[(int64_t)r * N + i]);
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
      for (int q = 0; q < DT / 32; q++) t += red[q];
      partial[(int64_t)blockIdx.x * R + r] = t;
    }
    __syncthreads();
  }
}

// Fused Arnoldi kernels: grid (ceil(N / DT), R), one right-hand side r per
// blockIdx.y. Every CTA reduces the dot partials itself (one warp per q, lane
// l sums partials l, l + 32, ... in order, fixed shuffle tree: the same sums
// in every CTA), so no separate reduction launch sits between the passes.
//
// w[r] -= sum_q h[r][q] V[q][r] with h reduced from the partials; CTA x = 0
// writes h into the Hessenberg column. With norm_out, the CTA also writes the
// squared norm of its updated slice of w to norm_out[blockIdx.x * R + r].
__global__ void __launch_bounds__(DT) reduce_axpy_kernel(
    const double2* __restrict__ partial, int nct, const double2* __restrict__ Vb,
    double2* __restrict__ w, int64_t N, int R, int nq, int m, int j, int first,
    const GmresState* __restrict__ st, double2* __restrict__ H, double* __restrict__ norm_out) {
  extern __shared__ double2 hs[];  // nq
  __shared__ double red[DT / 32];
  const int r = blockIdx.y;
  if (st[r].done) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // many partials: one warp per q, lanes over the partials, fixed shuffle
  // tree; few partials (small N): one thread per q, four interleaved
  // accumulators in a fixed order (coalesced over q), so long bases do not
  // queue q by q on the warps
  const int64_t cstride = (int64_t)R * nq;
  if (nct >= 64) {
    for (int q = warp; q < nq; q += DT / 32) {
      double sx = 0, sy = 0;
      for (int c = lane; c < nct; c += 32) {
        const double2 v = partial[c * cstride + (int64_t)r * nq + q];
        sx += v.x;
        sy += v.y;
      }
      sx = warp_sum(sx);
      sy = warp_sum(sy);
      if (lane == 0) {
        const double2 sv = make_double2(sx, sy);
        hs[q] = sv;
        if (blockIdx.x == 0) {
          double2* Hc = H + ((int64_t)r * m + j) * (m + 1);
          Hc[q] = first ? sv : cadd(Hc[q], sv);
        }
      }
    }
  } else {
  for (int q = threadIdx.x; q < nq; q += DT) {
    const double2* pq = partial + (int64_t)r * nq + q;
    double a0 = 0, a1 = 0, a2 = 0, a3 = 0, b0 = 0, b1 = 0, b2 = 0, b3 = 0;
    int c = 0;
    for (; c + 4 <= nct; c += 4) {
      const double2 v0 = pq[c * cstride], v1 = pq[(c + 1) * cstride];
      const double2 v2 = pq[(c + 2) * cstride], v3 = pq[(c + 3) * cstride];
      a0 += v0.x;
      b0 += v0.y;
      a1 += v1.x;
      b1 += v1.y;
      a2 += v2.x;
      b2 += v2.y;
      a3 += v3.x;
      b3 += v3.y;
    }
    for (; c < nct; c++) {
      const double2 v = pq[c * cstride];
      a0 += v.x;
      b0 += v.y;
    }
    const double2 sv = make_double2((a0 + a1) + (a2 + a3), (b0 + b1) + (b2 + b3));
    hs[q] = sv;
    if (blockIdx.x == 0) {
      double2* Hc = H + ((int64_t)r * m + j) * (m + 1);
      Hc[q] = first ? sv : cadd(Hc[q], sv);
    }
  }
  }
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * DT + threadIdx.x;
  double n2 = 0;
  if (i < N) {
    double2 acc = w[(int64_t)r * N + i];
    for (int q = 0; q < nq; q++) acc = csub(acc, cmul(hs[q], Vb[((int64_t)q * R + r) * N + i]));
    w[(int64_t)r * N + i] = acc;
    n2 = cabs2(acc);
  }
  if (norm_out) {
    n2 = warp_sum(n2);
    if (lane == 0) red[warp] = n2;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
      for (int q = 0; q < DT / 32; q++) t += red[q];
      norm_out[(int64_t)blockIdx.x * R + r] = t;
    }
  }
}

// Finish Arnoldi step j and write V[j + 1] = w / ||w||: every CTA sums the
// nct norm partials (warp 0, fixed order) for its scaling; CTA x = 0 also
// applies the Givens rotations and updates the state (as finish_step_kernel).
// A right-hand side that converges at this step may or may not get its next
// vector written; it is not used afterwards.
__global__ void __launch_bounds__(DT) finish_scale_kernel(
    const double* __restrict__ partial, int nct, int R, int m, int j, double tol,
    GmresState* __restrict__ st, double2* __restrict__ H, double2* __restrict__ g,
    double2* __restrict__ cs, double2* __restrict__ sn, double* __restrict__ hnorm,
    const double2* __restrict__ w, double2* __restrict__ vnext, int64_t N) {
  __shared__ double hn_s;
  const int r = blockIdx.y, lane = threadIdx.x & 31;
  GmresState s = st[r];
  if (s.done) return;
  if (threadIdx.x < 32) {
    double n2 = 0;
    for (int c = lane; c < nct; c += 32) n2 += partial[(int64_t)c * R + r];
    n2 = warp_sum(n2);
    if (lane == 0) {
      const double hn = sqrt(n2);
      hn_s = hn;
      if (blockIdx.x == 0) {
        hnorm[r] = hn;
        double2* Hc = H + ((int64_t)r * m + j) * (m + 1);
        double2* cr = cs + (int64_t)r * m;
        double2* sr = sn + (int64_t)r * m;
        double2* gr = g + (int64_t)r * (m + 1);
        Hc[j + 1] = make_double2(hn, 0.0);
        for (int q = 0; q < j; q++) {
          double2 a = Hc[q], b = Hc[q + 1];
          Hc[q] = cadd(cmul(cr[q], a), cmul(sr[q], b));
          Hc[q + 1] = cadd(cscale(-1.0, cmul(cconj(sr[q]), a)), cmul(cr[q], b));
        }
        double2 a = Hc[j], b = Hc[j + 1];
        double aa = sqrt(cabs2(a));
        double rho = sqrt(cabs2(a) + cabs2(b));
        double2 c, sv;
        if (aa == 0.0) {
          c = make_double2(0, 0);
          sv = make_double2(1, 0);
        } else {
          c = make_double2(aa / rho, 0.0);
          sv = cscale(1.0 / (aa * rho), cmul(a, cconj(b)));
        }
        cr[j] = c;
        sr[j] = sv;
        Hc[j] = cadd(cmul(c, a), cmul(sv, b));
        Hc[j + 1] = make_double2(0, 0);
        double2 gj = gr[j];
        gr[j + 1] = cscale(-1.0, cmul(cconj(sv), gj));
        gr[j] = cmul(c, gj);
        s.jcount = j + 1;
        s.iters += 1;
        s.resid = sqrt(cabs2(gr[j + 1])) / s.bnorm;
        if (s.resid < tol || hn == 0.0) s.done = 1;
        st[r] = s;
      }
    }
  }
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * DT + threadIdx.x;
  if (i >= N) return;
  const double hn = hn_s;
  const double2 v = w[(int64_t)r * N + i];
  vnext[(int64_t)r * N + i] = hn > 0 ? cscale(1.0 / hn, v) : make_double2(0, 0);
}

// One thread per RHS: solve the jcount x jcount triangular system H y = g.
__global__ void trisolve_kernel(int R, int m, const GmresState* __restrict__ st,
                                const double2* __restrict__ H, const double2* __restrict__ g,
                                double2* __restrict__ y) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const int kk = st[r].jcount;
  double2* yr = y + (int64_t)r * m;
  for (int q = kk - 1; q >= 0; q--) {
    double2 s = g[(int64_t)r * (m + 1) + q];
    for (int t = q + 1; t < kk; t++) s = csub(s, cmul(H[((int64_t)r * m + t) * (m + 1) + q], yr[t]));
    yr[q] = cdiv(s, H[((int64_t)r * m + q) * (m + 1) + q]);
  }
  for (int q = kk; q < m; q++) yr[q] = make_double2(0, 0);
}

// x[r] += sum_q y[r][q] V[q][r]
__global__ void __launch_bounds__(DT) update_x_kernel(const double2* __restrict__ Vb,
                                                      double2* __restrict__ x, int64_t N, int R,
                                                      int m, const double2* __restrict__ y,
                                                      const GmresState* __restrict__ st) {
  const int r = blockIdx.y;
  const int kk = st[r].jcount;
  const int64_t i = (int64_t)blockIdx.x * DT + threadIdx.x;
  if (i >= N) return;
  double2 acc = x[(int64_t)r * N + i];
  for (int q = 0; q < kk; q++) acc = cadd(acc, cmul(y[(int64_t)r * m + q], Vb[((int64_t)q * R + r) * N + i]));
  x[(int64_t)r * N + i] = acc;
}

__global__ void __launch_bounds__(DT) add_kernel(double2* __restrict__ x,
                                                 const double2* __restrict__ d, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * DT + threadIdx.x;
  if (i >= n) return;
  x[i] = cadd(x[i], d[i]);
}

// r = b - w (stored into w), per RHS
__global__ void __launch_bounds__(DT) residual_kernel(const double2* __restrict__ b,
                                                      double2* __restrict__ w, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * DT + threadIdx.x;
  if (i >= n) return;
  w[i] = csub(b[i], w[i]);
}

// restart: beta = ||r||, V[0] = r / beta, g = [beta, 0, ...], jcount = 0
__global__ void restart_kernel(const double* __restrict__ partial, int nct, int R, int m,
                               double tol, int init, GmresState* __restrict__ st,
                               double2* __restrict__ g, double* __restrict__ hnorm) {
  const int r = blockIdx.x, lane = threadIdx.x;  // one warp per right-hand side
  if (r >= R) return;
  double n2 = 0;
  for (int c = lane; c < nct; c += 32) n2 += partial[(int64_t)c * R + r];
  n2 = warp_sum(n2);
  if (lane != 0) return;
  double beta = sqrt(n2);
  GmresState s = st[r];
  if (init) {
    s.bnorm = beta;  // first call measures ||b|| (w holds b)
    s.iters = 0;
    s.done = 0;
  }
  s.beta = beta;
  s.jcount = 0;
  s.resid = s.bnorm > 0 ? beta / s.bnorm : 0.0;
  if (!init) {
    if (s.bnorm == 0.0 || s.resid < tol) s.done = 1;
    else s.done = 0;
  }
  st[r] = s;
  hnorm[r] = beta;
  for (int q = 0; q <= m; q++) g[(int64_t)r * (m + 1) + q] = make_double2(q == 0 ? beta : 0.0, 0.0);
}

__global__ void __launch_bounds__(DT) copy_scale_kernel(const double2* __restrict__ w,
                                                        double2* __restrict__ v0, int64_t N,
                                                        const double* __restrict__ hnorm) {
  const int r = blockIdx.y;
  const int64_t i = (int64_t)blockIdx.x * DT + threadIdx.x;
  if (i >= N) return;
  const double hn = hnorm[r];
  v0[(int64_t)r * N + i] = hn > 0 ? cscale(1.0 / hn, w[(int64_t)r * N + i]) : make_double2(0, 0);
}

}  // namespace

// CTAs of the partial-sum kernels: one per 128 elements, at most 4 per SM
// (with 5 CTAs at N = 20,480 the Arnoldi dots ran at ~160 GB/s)
int krylov_num_ctas(int64_t N) {
  int64_t c = (N + 127) / 128;
  return (int)std::max<int64_t>(1, std::min<int64_t>(c, 608));
}

// CGS2 step j in five launches: dot partials, reduction + update (twice; the
// second also takes the norm partials of w), then the Givens step + scaling
int krylov_orthogonalize(const KrylovArgs& a, int j, cudaStream_t s) {
  const int nq = j + 1;
  const int nct = krylov_num_ctas(a.N);
  const int64_t chunk = (a.N + nct - 1) / nct;
  const dim3 g((unsigned)((a.N + DT - 1) / DT), (unsigned)a.R);
  const size_t hsm = (size_t)nq * sizeof(double2);
  // task groups: about two (q, r) dot products per warp
  const int tg = std::max(1, std::min(128, (nq * a.R + 2 * (DT / 32) - 1) / (2 * (DT / 32))));
  for (int pass = 0; pass < 2; pass++) {
    dot_partial_kernel<<<dim3((unsigned)nct, (unsigned)tg), DT, 0, s>>>(a.Vb, a.w, a.N, a.R, nq,
                                                                        chunk, a.st, a.cpart);
    reduce_axpy_kernel<<<g, DT, hsm, s>>>(a.cpart, nct, a.Vb, a.w, a.N, a.R, nq, a.m, j,
                                          pass == 0, a.st, a.H, pass == 1 ? a.npart : nullptr);
  }
  finish_scale_kernel<<<g, DT, 0, s>>>(a.npart, (int)g.x, a.R, a.m, j, a.tol, a.st, a.H, a.g,
                                       a.cs, a.sn, a.hnorm, a.w,
                                       a.Vb + (int64_t)(j + 1) * a.R * a.N, a.N);
  return 5;
}

void krylov_restart(const KrylovArgs& a, int init, cudaStream_t s) {
  // w holds r (or b when init); writes V[0] = r / ||r||
  const int nct = krylov_num_ctas(a.N);
  const int64_t chunk = (a.N + nct - 1) / nct;
  nrm_partial_kernel<<<nct, DT, 0, s>>>(a.w, a.N, a.R, chunk, a.npart);
  restart_kernel<<<a.R, 32, 0, s>>>(a.npart, nct, a.R, a.m, a.tol, init, a.st, a.g, a.hnorm);
  if (!init) {
    dim3 g((unsigned)((a.N + DT - 1) / DT), (unsigned)a.R);
    copy_scale_kernel<<<g, DT, 0, s>>>(a.w, a.Vb, a.N, a.hnorm);
  }
}

void krylov_axpy(double2* x, const double2* d, int64_t n, cudaStream_t s) {
  add_kernel<<<(unsigned)((n + DT - 1) / DT), DT, 0, s>>>(x, d, n);
}

void krylov_norm_partials(const double2* v, int64_t N, int R, double* partial, cudaStream_t s) {
  const int nct = krylov_num_ctas(N);
  const int64_t chunk = (N + nct - 1) / nct;
  nrm_partial_kernel<<<nct, DT, 0, s>>>(v, N, R, chunk, partial);
}

void krylov_residual(const double2* b, double2* w, int64_t n, cudaStream_t s) {
  residual_kernel<<<(unsigned)((n + DT - 1) / DT), DT, 0, s>>>(b, w, n);
}

void krylov_update(const KrylovArgs& a, cudaStream_t s) {
  trisolve_kernel<<<(a.R + 31) / 32, 32, 0, s>>>(a.R, a.m, a.st, a.H, a.g, a.y);
  dim3 g((unsigned)((a.N + DT - 1) / DT), (unsigned)a.R);
  update_x_kernel<<<g, DT, 0, s>>>(a.Vb, a.x, a.N, a.R, a.m, a.y, a.st);
}

}  // namespace bemgpu
