// post.cu -- small element-wise kernels around the solve: caller-order <->
// cluster-order gathers and the BC back-substitution
// (boundaryelementsolver.cpp:729-740) with p = i rho omega phi (:2251-2261).
#include "bem_kernels.h"
#include "post.h"
#include "quadrature.cuh"

namespace bemgpu {
namespace {
constexpr int PT = 256;

// out[r][i] = in[r][perm[i]]
__global__ void gather_kernel(const double2* __restrict__ in, double2* __restrict__ out,
                              const int64_t* __restrict__ perm, int64_t N) {
  const int r = blockIdx.y;
  const int64_t i = (int64_t)blockIdx.x * PT + threadIdx.x;
  if (i >= N) return;
  out[(int64_t)r * N + i] = in[(int64_t)r * N + perm[i]];
}

__global__ void backsub_kernel(const double2* __restrict__ x, const double2* __restrict__ g,
                               const double2* __restrict__ a, const double2* __restrict__ b,
                               const BcCoef* __restrict__ bc, const int64_t* __restrict__ perm,
                               int64_t N, double2 pfac, double2* __restrict__ phi,
                               double2* __restrict__ dphi, double2* __restrict__ p) {
  const int r = blockIdx.y;
  const int64_t i = (int64_t)blockIdx.x * PT + threadIdx.x;
  if (i >= N) return;
  const double2 xi = x[(int64_t)r * N + i], gi = g[(int64_t)r * N + i];
  const double2 ai = a[i], bi = b[i];
  double2 ph, dph;
  if (bc[i].subst) {  // |a| < |b|: the unknown was phi
    ph = xi;
    dph = cdiv(csub(gi, cmul(ai, ph)), bi);
  } else {
    dph = xi;
    ph = cdiv(csub(gi, cmul(bi, dph)), ai);
  }
  const int64_t o = (int64_t)r * N + perm[i];
  if (phi) phi[o] = ph;
  if (dphi) dphi[o] = dph;
  if (p) p[o] = cmul(pfac, ph);
}

__global__ void finite_kernel(const double2* __restrict__ v, int64_t n, int* __restrict__ bad) {
  const int64_t i = (int64_t)blockIdx.x * PT + threadIdx.x;
  if (i >= n) return;
  double2 z = v[i];
  if (!isfinite(z.x) || !isfinite(z.y)) atomicExch(bad, 1);
}
}  // namespace

// sourceTermVector of the right-hand side (BoundaryElementSolver::
// calculateBoundaryConditionAndSourceTermVector, boundaryelementsolver.cpp:
// 3386-3429, with sourceTerm :3431-3441): per collocation point (cluster
// order) the sum over the point sources of G + alpha dG rup, G = w exp(ikr) /
// (4 pi r), r = |p - s|, rup = (p - s) . n_p / r and dG = (G / r) / (ikr - 1)
// -- the reference divides by (ikr - 1) where the radial derivative would
// multiply, and this keeps its formula. Added to all R columns of rhs.
__global__ void source_rhs_kernel(const Elem* __restrict__ E, int64_t N,
                                  const double* __restrict__ src, int nsrc, double k,
                                  double2 alpha, double2* __restrict__ rhs, int R) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const Elem& e = E[i];
  double sx = 0.0, sy = 0.0;
  for (int q = 0; q < nsrc; q++) {
    const double* sq = src + 5 * q;
    const double dx = e.c[0] - sq[0], dy = e.c[1] - sq[1], dz = e.c[2] - sq[2];
    const double r = sqrt(dx * dx + dy * dy + dz * dz);
    const double rup = (dx * e.nrm[0] + dy * e.nrm[1] + dz * e.nrm[2]) / r;
    double sn, cs;
    sincos(k * r, &sn, &cs);
    const double g0 = 1.0 / (4.0 * 3.14159265358979323846 * r);
    // G = w (cos + i sin) / (4 pi r)
    const double Gx = (sq[3] * cs - sq[4] * sn) * g0, Gy = (sq[3] * sn + sq[4] * cs) * g0;
    // dG = (G / r) / (-1 + i k r)
    const double kr = k * r, den = r * (1.0 + kr * kr);
    const double dGx = (-Gx + kr * Gy) / den, dGy = (-Gy - kr * Gx) / den;
    sx += Gx + (alpha.x * dGx - alpha.y * dGy) * rup;
    sy += Gy + (alpha.x * dGy + alpha.y * dGx) * rup;
  }
  for (int r = 0; r < R; r++) {
    double2& v = rhs[(int64_t)r * N + i];
    v.x += sx;
    v.y += sy;
  }
}

int launch_source_rhs(const Elem* E, int64_t N, const double* src, int nsrc, double k,
                      double2 alpha, double2* rhs, int R, cudaStream_t s) {
  if (N <= 0 || nsrc <= 0) return 0;
  source_rhs_kernel<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(E, N, src, nsrc, k, alpha, rhs,
                                                                R);
  return 1;
}

int launch_gather(const double2* in, double2* out, const int64_t* perm, int64_t N, int R,
                  cudaStream_t s) {
  dim3 g((unsigned)((N + PT - 1) / PT), (unsigned)R);
  gather_kernel<<<g, PT, 0, s>>>(in, out, perm, N);
  return 1;
}

int launch_backsub(const double2* x, const double2* g, const double2* a, const double2* b,
                   const BcCoef* bc, const int64_t* perm, int64_t N, int R, double2 pfac, double2* phi,
                   double2* dphi, double2* p, cudaStream_t s) {
  dim3 gr((unsigned)((N + PT - 1) / PT), (unsigned)R);
  backsub_kernel<<<gr, PT, 0, s>>>(x, g, a, b, bc, perm, N, pfac, phi, dphi, p);
  return 1;
}

int launch_finite_check(const double2* v, int64_t n, int* bad, cudaStream_t s) {
  if (n <= 0) return 0;
  finite_kernel<<<(unsigned)((n + PT - 1) / PT), PT, 0, s>>>(v, n, bad);
  return 1;
}

}  // namespace bemgpu
