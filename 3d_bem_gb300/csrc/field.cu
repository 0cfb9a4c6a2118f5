// field.cu -- field evaluation: velocity potential at observation points from
// a boundary solution (BoundaryElementSolver::calculateFieldSolutionRegular,
// boundaryelementsolver.cpp:2263-2316, with BemOperatorField :2318-2353).
//
// Dense sum over (observation point, element) pairs with the 7-point rule:
// one thread per observation point, elements staged through shared memory in
// tiles, element range split over a second grid dimension so that few points
// still fill the GPU; partial sums land in a buffer and a second kernel adds
// them in a fixed order (deterministic, no atomics), adds the point sources
// and scales to sound pressure.
//
// Mixed precision (precision 1): the integrand in FP32 with two-float
// centroids (p - c_j keeps ~7 digits, the rule points are offsets from c_j),
// exp(ikr) from the hardware sin / cos after an exact reduction of
// k r / (2 pi) to [-1/2, 1/2] (absolute error ~4e-7 on [-pi, pi]), per-tile
// sums in FP32
// folded into FP64 accumulators every FIELD_TILE elements. Precision 0: the
// same sum in FP64.
#include "field.h"

namespace bemgpu {
namespace {

constexpr double kInv4Pi = 0.0795774715459476678844418816862571885;

// 7-point rule of order 5 (trianglequadraturerules.cpp:50-59 of the
// reference; orderLow = 5, boundaryelementsolver.h:653-654): barycentric xi1,
// xi2 and weight (weights sum to 1; the element area multiplies afterwards).
constexpr double kR7x1[7] = {0.33333333333333, 0.47014206410511, 0.47014206410511,
                             0.05971587178977, 0.10128650732346, 0.10128650732346,
                             0.79742698535309};
constexpr double kR7x2[7] = {0.33333333333333, 0.47014206410511, 0.05971587178977,
                             0.47014206410511, 0.10128650732346, 0.79742698535309,
                             0.10128650732346};
constexpr double kR7w[7] = {0.22500000000000, 0.13239415278851, 0.13239415278851,
                            0.13239415278851, 0.12593918054483, 0.12593918054483,
                            0.12593918054483};

__constant__ double cR7x1[7] = {kR7x1[0], kR7x1[1], kR7x1[2], kR7x1[3],
                                kR7x1[4], kR7x1[5], kR7x1[6]};
__constant__ double cR7x2[7] = {kR7x2[0], kR7x2[1], kR7x2[2], kR7x2[3],
                                kR7x2[4], kR7x2[5], kR7x2[6]};
// w / (4 pi)
__constant__ double cR7g[7] = {kR7w[0] * kInv4Pi, kR7w[1] * kInv4Pi, kR7w[2] * kInv4Pi,
                               kR7w[3] * kInv4Pi, kR7w[4] * kInv4Pi, kR7w[5] * kInv4Pi,
                               kR7w[6] * kInv4Pi};
__constant__ float cR7gf[7] = {
    (float)(kR7w[0] * kInv4Pi), (float)(kR7w[1] * kInv4Pi), (float)(kR7w[2] * kInv4Pi),
    (float)(kR7w[3] * kInv4Pi), (float)(kR7w[4] * kInv4Pi), (float)(kR7w[5] * kInv4Pi),
    (float)(kR7w[6] * kInv4Pi)};

__global__ void field_prep_kernel(const Elem* __restrict__ E, const int64_t* __restrict__ perm,
                                  int64_t N, const double2* __restrict__ phi,
                                  const double2* __restrict__ dphi, int R, int precision,
                                  FieldElemF* __restrict__ fe, void* __restrict__ coef) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  const Elem& e = E[j];
  if (precision == 1) {
    FieldElemF f;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const float hi = (float)e.c[d];
      f.c_hi[d] = hi;
      f.c_lo[d] = (float)(e.c[d] - (double)hi);
      f.nrm[d] = (float)e.nrm[d];
    }
#pragma unroll
    for (int i = 0; i < 7; i++) {
      const double a1 = cR7x1[i], a2 = cR7x2[i], a3 = 1.0 - a2 - a1;
      double on = 0.0;
#pragma unroll
      for (int d = 0; d < 3; d++) {
        const double o = (a1 * e.n1[d] + a2 * e.n2[d] + a3 * e.n3[d]) - e.c[d];
        f.q[3 * i + d] = (float)o;
        on += o * e.nrm[d];
      }
      f.qn[i] = (float)on;
    }
    f.pad[0] = f.pad[1] = f.pad[2] = 0.0f;
    fe[j] = f;
  }
  if (R == 0) return;  // element records only (the reflected elements)
  const int64_t cj = perm[j];
  const double A = e.area;
  for (int r = 0; r < R; r++) {
    const double2 p = phi[(int64_t)r * N + cj], dp = dphi[(int64_t)r * N + cj];
    if (precision == 1) {
      FieldCoefF c;
      c.a = make_float2((float)(A * p.x), (float)(A * p.y));
      c.b = make_float2((float)(A * dp.x), (float)(A * dp.y));
      static_cast<FieldCoefF*>(coef)[(int64_t)r * N + j] = c;
    } else {
      FieldCoef c;
      c.a = make_double2(A * p.x, A * p.y);
      c.b = make_double2(A * dp.x, A * dp.y);
      static_cast<FieldCoef*>(coef)[(int64_t)r * N + j] = c;
    }
  }
}

// Columns r0 .. r0 + RB - 1, element chunk blockIdx.y.
template <int RB>
__global__ void __launch_bounds__(FIELD_PTS)
    field_sum32_kernel(const FieldElemF* __restrict__ fe, const FieldCoefF* __restrict__ coef,
                       int64_t N, int64_t chunk, const double* __restrict__ pts, int64_t M,
                       float k, float kc, int r0, int R, double2* __restrict__ partial) {
  __shared__ FieldElemF se[FIELD_TILE];
  __shared__ FieldCoefF sc[RB][FIELD_TILE];
  const int64_t ip = (int64_t)blockIdx.x * FIELD_PTS + threadIdx.x;
  const int64_t e0 = (int64_t)blockIdx.y * chunk;
  const int64_t e1 = min(N, e0 + chunk);
  float ph[3] = {0.0f, 0.0f, 0.0f}, pl[3] = {0.0f, 0.0f, 0.0f};
  if (ip < M) {
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const double v = pts[3 * ip + d];
      ph[d] = (float)v;
      pl[d] = (float)(v - (double)ph[d]);
    }
  }
  double ax[RB], ay[RB];
#pragma unroll
  for (int r = 0; r < RB; r++) ax[r] = ay[r] = 0.0;
  for (int64_t t0 = e0; t0 < e1; t0 += FIELD_TILE) {
    const int nt = (int)min((int64_t)FIELD_TILE, e1 - t0);
    __syncthreads();
    const float4* src = reinterpret_cast<const float4*>(fe + t0);
    float4* dst = reinterpret_cast<float4*>(se);
    constexpr int PIECES = (int)(sizeof(FieldElemF) / sizeof(float4));
    for (int i = threadIdx.x; i < nt * PIECES; i += FIELD_PTS) dst[i] = src[i];
    for (int i = threadIdx.x; i < RB * nt; i += FIELD_PTS) {
      const int r = i / nt, j = i - r * nt;
      sc[r][j] = coef[(int64_t)(r0 + r) * N + t0 + j];
    }
    __syncthreads();
    float tx[RB], ty[RB];
#pragma unroll
    for (int r = 0; r < RB; r++) tx[r] = ty[r] = 0.0f;
    for (int j = 0; j < nt; j++) {
      const FieldElemF& E = se[j];
      const float dx = (ph[0] - E.c_hi[0]) + (pl[0] - E.c_lo[0]);
      const float dy = (ph[1] - E.c_hi[1]) + (pl[1] - E.c_lo[1]);
      const float dz = (ph[2] - E.c_hi[2]) + (pl[2] - E.c_lo[2]);
      const float dn = dx * E.nrm[0] + dy * E.nrm[1] + dz * E.nrm[2];
      float Lx = 0.0f, Ly = 0.0f, Mx = 0.0f, My = 0.0f;
#pragma unroll
      for (int i = 0; i < 7; i++) {
        const float rx = dx - E.q[3 * i], ry = dy - E.q[3 * i + 1], rz = dz - E.q[3 * i + 2];
        const float rr = rx * rx + ry * ry + rz * rz;
        const float ir = rsqrtf(rr);
        const float r = rr * ir;
        // exp(ikr): x = k r / (2 pi) reduced exactly to [-1/2, 1/2] (x - rint(x)
        // has no rounding), then the hardware sin / cos on 2 pi (x - rint(x))
        const float x = kc * r;
        const float xr = x - rintf(x);
        float sn, cs;
        __sincosf(6.28318530717959f * xr, &sn, &cs);
        const float kr = k * r;
        const float g0 = ir * cR7gf[i];  // w / (4 pi r)
        Lx = fmaf(g0, cs, Lx);
        Ly = fmaf(g0, sn, Ly);
        // w dG/dr rnq = g0 (p - q_i) . n / r^2 (cos + kr sin, sin - kr cos)
        const float tg = (dn - E.qn[i]) * (ir * ir * g0);
        Mx = fmaf(tg, fmaf(kr, sn, cs), Mx);
        My = fmaf(tg, fmaf(-kr, cs, sn), My);
      }
#pragma unroll
      for (int r = 0; r < RB; r++) {
        const FieldCoefF c = sc[r][j];
        tx[r] += (Mx * c.a.x - My * c.a.y) - (Lx * c.b.x - Ly * c.b.y);
        ty[r] += (Mx * c.a.y + My * c.a.x) - (Lx * c.b.y + Ly * c.b.x);
      }
    }
#pragma unroll
    for (int r = 0; r < RB; r++) {
      ax[r] += (double)tx[r];
      ay[r] += (double)ty[r];
    }
  }
  if (ip < M) {
#pragma unroll
    for (int r = 0; r < RB; r++)
      partial[((int64_t)blockIdx.y * R + r0 + r) * M + ip] = make_double2(ax[r], ay[r]);
  }
}

template <int RB>
__global__ void __launch_bounds__(FIELD_PTS)
    field_sum64_kernel(const Elem* __restrict__ E, const FieldCoef* __restrict__ coef, int64_t N,
                       int64_t chunk, const double* __restrict__ pts, int64_t M, double k,
                       int r0, int R, double2* __restrict__ partial) {
  __shared__ Elem se[FIELD_TILE];
  __shared__ FieldCoef sc[RB][FIELD_TILE];
  const int64_t ip = (int64_t)blockIdx.x * FIELD_PTS + threadIdx.x;
  const int64_t e0 = (int64_t)blockIdx.y * chunk;
  const int64_t e1 = min(N, e0 + chunk);
  double p[3] = {0.0, 0.0, 0.0};
  if (ip < M) {
#pragma unroll
    for (int d = 0; d < 3; d++) p[d] = pts[3 * ip + d];
  }
  double ax[RB], ay[RB];
#pragma unroll
  for (int r = 0; r < RB; r++) ax[r] = ay[r] = 0.0;
  for (int64_t t0 = e0; t0 < e1; t0 += FIELD_TILE) {
    const int nt = (int)min((int64_t)FIELD_TILE, e1 - t0);
    __syncthreads();
    const double2* src = reinterpret_cast<const double2*>(E + t0);
    double2* dst = reinterpret_cast<double2*>(se);
    for (int i = threadIdx.x; i < nt * 8; i += FIELD_PTS) dst[i] = src[i];
    for (int i = threadIdx.x; i < RB * nt; i += FIELD_PTS) {
      const int r = i / nt, j = i - r * nt;
      sc[r][j] = coef[(int64_t)(r0 + r) * N + t0 + j];
    }
    __syncthreads();
    for (int j = 0; j < nt; j++) {
      const Elem& e = se[j];
      double Lx = 0.0, Ly = 0.0, Mx = 0.0, My = 0.0;
      for (int i = 0; i < 7; i++) {
        const double a1 = cR7x1[i], a2 = cR7x2[i], a3 = 1.0 - a2 - a1;
        const double rx = p[0] - ((a1 * e.n1[0] + a2 * e.n2[0]) + a3 * e.n3[0]);
        const double ry = p[1] - ((a1 * e.n1[1] + a2 * e.n2[1]) + a3 * e.n3[1]);
        const double rz = p[2] - ((a1 * e.n1[2] + a2 * e.n2[2]) + a3 * e.n3[2]);
        const double r = sqrt(rx * rx + ry * ry + rz * rz);
        const double ir = 1.0 / r;
        const double kr = k * r;
        double sn, cs;
        sincos(kr, &sn, &cs);
        const double g0 = ir * cR7g[i];
        const double Gx = cs * g0, Gy = sn * g0;
        const double t = -(rx * e.nrm[0] + ry * e.nrm[1] + rz * e.nrm[2]) * (ir * ir);
        Lx += Gx;
        Ly += Gy;
        Mx += t * (-Gx - kr * Gy);
        My += t * (kr * Gx - Gy);
      }
#pragma unroll
      for (int r = 0; r < RB; r++) {
        const FieldCoef c = sc[r][j];
        ax[r] += (Mx * c.a.x - My * c.a.y) - (Lx * c.b.x - Ly * c.b.y);
        ay[r] += (Mx * c.a.y + My * c.a.x) - (Lx * c.b.y + Ly * c.b.x);
      }
    }
  }
  if (ip < M) {
#pragma unroll
    for (int r = 0; r < RB; r++)
      partial[((int64_t)blockIdx.y * R + r0 + r) * M + ip] = make_double2(ax[r], ay[r]);
  }
}

__global__ void field_finish_kernel(const double2* __restrict__ partial, int S, int64_t M, int R,
                                    const double* __restrict__ pts, const double* __restrict__ src,
                                    int nsrc, double k, double2 pfac, double2* __restrict__ phi_f,
                                    double2* __restrict__ p_f) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M * R) return;
  const int64_t r = i / M, ip = i - r * M;
  double ax = 0.0, ay = 0.0;
  for (int s = 0; s < S; s++) {
    const double2 v = partial[((int64_t)s * R + r) * M + ip];
    ax += v.x;
    ay += v.y;
  }
  if (nsrc > 0) {  // sourcePhiTerm: w exp(ikr) / (4 pi r)
    const double px = pts[3 * ip], py = pts[3 * ip + 1], pz = pts[3 * ip + 2];
    for (int q = 0; q < nsrc; q++) {
      const double* sq = src + 5 * q;
      const double dx = sq[0] - px, dy = sq[1] - py, dz = sq[2] - pz;
      const double rr = sqrt(dx * dx + dy * dy + dz * dz);
      double sn, cs;
      sincos(k * rr, &sn, &cs);
      const double g = kInv4Pi / rr;
      const double Gx = cs * g, Gy = sn * g;
      ax += sq[3] * Gx - sq[4] * Gy;
      ay += sq[3] * Gy + sq[4] * Gx;
    }
  }
  if (phi_f) phi_f[i] = make_double2(ax, ay);
  if (p_f) p_f[i] = make_double2(pfac.x * ax - pfac.y * ay, pfac.x * ay + pfac.y * ax);
}

template <int RB>
void sum_pass(const Elem* E, const FieldElemF* fe, const void* coef, int64_t N, int R,
              const double* pts, int64_t M, double k, int precision, int S, int64_t chunk,
              int r0, double2* partial, cudaStream_t s) {
  const dim3 grid((unsigned)((M + FIELD_PTS - 1) / FIELD_PTS), (unsigned)S);
  if (precision == 1) {
    const double kc = k / (2.0 * 3.14159265358979323846);
    field_sum32_kernel<RB><<<grid, FIELD_PTS, 0, s>>>(fe, static_cast<const FieldCoefF*>(coef), N,
                                                      chunk, pts, M, (float)k, (float)kc, r0, R,
                                                      partial);
  } else {
    field_sum64_kernel<RB><<<grid, FIELD_PTS, 0, s>>>(E, static_cast<const FieldCoef*>(coef), N,
                                                      chunk, pts, M, k, r0, R, partial);
  }
}

}  // namespace

int launch_field_prep(const Elem* E, const int64_t* perm, int64_t N, const double2* phi,
                      const double2* dphi, int R, int precision, FieldElemF* fe, void* coef,
                      cudaStream_t s) {
  if (N <= 0) return 0;
  field_prep_kernel<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(E, perm, N, phi, dphi, R,
                                                                precision, fe, coef);
  return 1;
}

int launch_field_sum(const Elem* E, const FieldElemF* fe, const void* coef, int64_t N, int R,
                     const double* pts, int64_t M, double k, int precision, int S,
                     double2* partial, cudaStream_t s) {
  if (M <= 0 || R <= 0 || S <= 0) return 0;
  const int64_t chunk = (N + S - 1) / S;
  int n = 0;
  for (int r0 = 0; r0 < R; r0 += FIELD_RB, n++) {
    switch (R - r0 >= FIELD_RB ? FIELD_RB : R - r0) {
      case 1: sum_pass<1>(E, fe, coef, N, R, pts, M, k, precision, S, chunk, r0, partial, s); break;
      case 2: sum_pass<2>(E, fe, coef, N, R, pts, M, k, precision, S, chunk, r0, partial, s); break;
      case 3: sum_pass<3>(E, fe, coef, N, R, pts, M, k, precision, S, chunk, r0, partial, s); break;
      default: sum_pass<4>(E, fe, coef, N, R, pts, M, k, precision, S, chunk, r0, partial, s); break;
    }
  }
  return n;
}

int launch_field_finish(const double2* partial, int S, int64_t M, int R, const double* pts,
                        const double* src, int nsrc, double k, double2 pfac, double2* phi_f,
                        double2* p_f, cudaStream_t s) {
  const int64_t cnt = M * R;
  if (cnt <= 0) return 0;
  field_finish_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, s>>>(partial, S, M, R, pts, src,
                                                                    nsrc, k, pfac, phi_f, p_f);
  return 1;
}

}  // namespace bemgpu
