// selector.cu -- K9/K10: the learned quadrature-order selector.
//
//  * sel_label_kernel: per (collocation element, source element, k) pair the
//    24 features and the label -- the cheapest of the 1, 3, 7, 13, 25-point
//    rules whose L, M, Mt, N all stay within a relative tolerance of a
//    reference: the 64-point product rule on the sub-triangles of an 8-fold
//    (centroid distance below 3 source sizes) or 4-fold subdivision, converged
//    to ~1e-10 from one source size on; below a distance ratio the split-polar
//    near-singular rule of boundaryelementsolver.cpp:1387-1514. FP64: the
//    labels must resolve 1e-7.
//  * mlp_*: FP32 training of the 24-64-64-5 ReLU network (forward + softmax
//    cross-entropy + backward per sample, parameter gradients one thread per
//    parameter with the samples summed in order, so the result is bitwise
//    reproducible; Adam).
//  * sel_infer / sel_near_classes: BF16 inference on the tensor cores, one warp
//    per 32 pairs (two m16 row tiles sharing the weight fragments), mma.sync
//    m16n8k16 with FP32 accumulation; low-confidence pairs get the highest
//    order (the guard band).
//  * sel_nearfield32: the mixed-precision near-field kernel with the selected
//    rule per entry; a hashed sample of entries is re-integrated with the
//    highest order and keeps that value when the two disagree.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <set>
#include <vector>

#include "bem_kernels.h"
#include "host_tree.h"
#include "quadrature.cuh"
#include "selector.h"

namespace bemgpu {

namespace {

constexpr int SEL_NPT = 1 + 3 + 7 + 13 + 25 + 16 + 64;

struct SelRules {
  int off[SEL_RULES], cnt[SEL_RULES];
  double x1[SEL_NPT], x2[SEL_NPT], w[SEL_NPT];
  float fx1[SEL_NPT], fx2[SEL_NPT], fw[SEL_NPT];
};

static __constant__ SelRules c_sel;
static __constant__ QuadRules c_rules;

// ---------------- rule tables (host) ----------------
// Symmetric Dunavant rules of degree 1, 2, 5, 7 and 10 (1, 3, 7, 13, 25
// points), as tabulated for orders n = 1, 2, 5, 7, 10 in
// trianglequadraturerules.cpp; weights sum to 1.
const double kT1[] = {1.0 / 3, 1.0 / 3, 1.0};
const double kT3[] = {1.0 / 6, 1.0 / 6, 1.0 / 3, 1.0 / 6, 2.0 / 3, 1.0 / 3, 2.0 / 3, 1.0 / 6, 1.0 / 3};
const double kT7[] = {
    0.33333333333333, 0.33333333333333, 0.22500000000000, 0.47014206410511, 0.47014206410511,
    0.13239415278851, 0.47014206410511, 0.05971587178977, 0.13239415278851, 0.05971587178977,
    0.47014206410511, 0.13239415278851, 0.10128650732346, 0.10128650732346, 0.12593918054483,
    0.10128650732346, 0.79742698535309, 0.12593918054483, 0.79742698535309, 0.10128650732346,
    0.12593918054483};
const double kT13[] = {
    0.33333333333333, 0.33333333333333, -0.14957004446768, 0.26034596607904, 0.26034596607904,
    0.17561525743321, 0.26034596607904, 0.47930806784192, 0.17561525743321, 0.47930806784192,
    0.26034596607904, 0.17561525743321, 0.06513010290222, 0.06513010290222, 0.05334723560884,
    0.06513010290222, 0.86973979419557, 0.05334723560884, 0.86973979419557, 0.06513010290222,
    0.05334723560884, 0.31286549600487, 0.63844418856981, 0.07711376089026, 0.63844418856981,
    0.04869031542532, 0.07711376089026, 0.04869031542532, 0.31286549600487, 0.07711376089026,
    0.63844418856981, 0.31286549600487, 0.07711376089026, 0.31286549600487, 0.04869031542532,
    0.07711376089026, 0.04869031542532, 0.63844418856981, 0.07711376089026};
// degree 10: one centroid point and orbits (a, b, c) with weight; the
// six-point orbits are all permutations of (a, b, 1 - a - b)
const double kT25c = 0.090817990382754;
const double kT25o3[][2] = {{0.485577633383657, 0.036725957756467},
                            {0.109481575485037, 0.045321059435528}};
const double kT25o6[][3] = {{0.141707219414880, 0.307939838764121, 0.072757916845420},
                            {0.025003534762686, 0.246672560639903, 0.028327242531057},
                            {0.009540815400299, 0.066803251012200, 0.009421666963733}};

void push_rows(std::vector<double>& X1, std::vector<double>& X2, std::vector<double>& W,
               const double* t, int n) {
  for (int i = 0; i < n; i++) {
    X1.push_back(t[3 * i]);
    X2.push_back(t[3 * i + 1]);
    W.push_back(t[3 * i + 2]);
  }
}

SelRules build_rules() {
  std::vector<double> X1, X2, W;
  SelRules R{};
  auto mark = [&](int r) { R.off[r] = (int)X1.size(); };
  auto done = [&](int r) { R.cnt[r] = (int)X1.size() - R.off[r]; };
  mark(0);
  push_rows(X1, X2, W, kT1, 1);
  done(0);
  mark(1);
  push_rows(X1, X2, W, kT3, 3);
  done(1);
  mark(2);
  push_rows(X1, X2, W, kT7, 7);
  done(2);
  mark(3);
  push_rows(X1, X2, W, kT13, 13);
  done(3);
  mark(4);
  X1.push_back(1.0 / 3);
  X2.push_back(1.0 / 3);
  W.push_back(kT25c);
  for (const auto& o : kT25o3) {  // (a, a, 1 - 2a): three points
    const double a = o[0], c = 1.0 - 2.0 * a;
    const double pts[3][2] = {{a, a}, {a, c}, {c, a}};
    for (const auto& p : pts) {
      X1.push_back(p[0]);
      X2.push_back(p[1]);
      W.push_back(o[1]);
    }
  }
  for (const auto& o : kT25o6) {  // all permutations of (a, b, c)
    const double a = o[0], b = o[1], c = 1.0 - a - b;
    const double pts[6][2] = {{a, b}, {b, a}, {a, c}, {c, a}, {b, c}, {c, b}};
    for (const auto& p : pts) {
      X1.push_back(p[0]);
      X2.push_back(p[1]);
      W.push_back(o[2]);
    }
  }
  done(4);
  mark(SEL_PLAIN);  // the reference's regular rule
  const QuadRules q = make_rules();
  for (int i = 0; i < 16; i++) {
    X1.push_back(q.reg_x1[i]);
    X2.push_back(q.reg_x2[i]);
    W.push_back(q.reg_w[i]);
  }
  done(SEL_PLAIN);
  // reference: collapsed 8 x 8 Gauss-Legendre product rule, xi1 = u,
  // xi2 = (1 - u) v, Jacobian (1 - u), weights normalised to sum 1
  mark(SEL_REF);
  double gx[8], gw[8];
  gauss_legendre(8, gx, gw);
  for (int i = 0; i < 8; i++)
    for (int j = 0; j < 8; j++) {
      const double u = 0.5 * (gx[i] + 1.0), v = 0.5 * (gx[j] + 1.0);
      X1.push_back(u);
      X2.push_back((1.0 - u) * v);
      W.push_back(2.0 * 0.25 * gw[i] * gw[j] * (1.0 - u));
    }
  done(SEL_REF);
  for (int i = 0; i < SEL_NPT; i++) {
    R.x1[i] = X1[i];
    R.x2[i] = X2[i];
    R.w[i] = W[i];
    R.fx1[i] = (float)X1[i];
    R.fx2[i] = (float)X2[i];
    R.fw[i] = (float)W[i];
  }
  return R;
}

// ---------------- features ----------------
__device__ __forceinline__ double len3(double x, double y, double z) { return sqrt(x * x + y * y + z * z); }

// 24 geometry / wavenumber features of the pair (collocation point p with
// normal np, source triangle Q), all dimensionless.
__device__ void sel_features(const double* p, const double* np, const Elem& Q, double k,
                             float* f) {
  const double h = sqrt(Q.area);
  const double rx = p[0] - Q.c[0], ry = p[1] - Q.c[1], rz = p[2] - Q.c[2];
  const double d = fmax(len3(rx, ry, rz), 1e-12 * h);
  const double hn = rx * Q.nrm[0] + ry * Q.nrm[1] + rz * Q.nrm[2];
  double e[3] = {len3(Q.n2[0] - Q.n1[0], Q.n2[1] - Q.n1[1], Q.n2[2] - Q.n1[2]),
                 len3(Q.n3[0] - Q.n2[0], Q.n3[1] - Q.n2[1], Q.n3[2] - Q.n2[2]),
                 len3(Q.n1[0] - Q.n3[0], Q.n1[1] - Q.n3[1], Q.n1[2] - Q.n3[2])};
  // angles opposite each edge by the law of cosines
  double ang[3];
  for (int i = 0; i < 3; i++) {
    const double a = e[i], b = e[(i + 1) % 3], c = e[(i + 2) % 3];
    ang[i] = acos(fmin(1.0, fmax(-1.0, (b * b + c * c - a * a) / (2.0 * b * c))));
  }
  const double emin = fmin(e[0], fmin(e[1], e[2])), emax = fmax(e[0], fmax(e[1], e[2]));
  const double emid = e[0] + e[1] + e[2] - emin - emax;
  double dv = 1e300;
  const double* V[3] = {Q.n1, Q.n2, Q.n3};
  for (int i = 0; i < 3; i++) dv = fmin(dv, len3(p[0] - V[i][0], p[1] - V[i][1], p[2] - V[i][2]));
  // barycentric coordinates of p projected onto the source plane
  const double px = p[0] - hn * Q.nrm[0], py = p[1] - hn * Q.nrm[1], pz = p[2] - hn * Q.nrm[2];
  double lam[3];
  for (int i = 0; i < 3; i++) {
    const double* A = V[(i + 1) % 3];
    const double* B = V[(i + 2) % 3];
    // signed area of (projection, A, B) along the normal over the full area
    const double ax = A[0] - px, ay = A[1] - py, az = A[2] - pz;
    const double bx = B[0] - px, by = B[1] - py, bz = B[2] - pz;
    const double cx = ay * bz - az * by, cy = az * bx - ax * bz, cz = ax * by - ay * bx;
    lam[i] = fmin(10.0, fmax(-10.0, 0.5 * (cx * Q.nrm[0] + cy * Q.nrm[1] + cz * Q.nrm[2]) / Q.area));
  }
  const double lmin = fmin(lam[0], fmin(lam[1], lam[2]));
  const double kh = fmax(k * h, 1e-6);
  f[0] = (float)(d / h);
  f[1] = (float)(h / d);
  f[2] = (float)log(d / h);
  f[3] = (float)((h / d) * (h / d));
  f[4] = (float)(hn / d);
  f[5] = (float)(fabs(hn) / h);
  f[6] = (float)(np[0] * Q.nrm[0] + np[1] * Q.nrm[1] + np[2] * Q.nrm[2]);
  f[7] = (float)((rx * np[0] + ry * np[1] + rz * np[2]) / d);
  f[8] = (float)kh;
  f[9] = (float)(k * d);
  f[10] = (float)log(kh);
  f[11] = (float)(emin / h);
  f[12] = (float)(emid / h);
  f[13] = (float)(emax / h);
  f[14] = (float)(emax * emax / (2.0 * Q.area));
  f[15] = (float)fmin(ang[0], fmin(ang[1], ang[2]));
  f[16] = (float)fmax(ang[0], fmax(ang[1], ang[2]));
  f[17] = (float)(dv / h);
  f[18] = (float)lam[0];
  f[19] = (float)lam[1];
  f[20] = (float)lam[2];
  f[21] = (float)lmin;
  f[22] = (float)(emax / d);
  f[23] = (float)((lmin >= 0 ? fabs(hn) : dv) / h);
}

// The same features from the FP32 element copies (mixed-precision path): the
// centroid offset comes from the two-float centroids, vertices are stored
// relative to their centroid, so every quantity keeps ~7 digits -- far below
// the BF16 rounding of the network input.
__device__ void sel_features32(const ElemF& P, const ElemF& Q, float k, float* f) {
  const float h = sqrtf(Q.area);
  float rx, ry, rz;
  centroid_diff(P, Q, rx, ry, rz);
  const float d = fmaxf(sqrtf(rx * rx + ry * ry + rz * rz), 1e-12f * h);
  const float hn = rx * Q.nrm[0] + ry * Q.nrm[1] + rz * Q.nrm[2];
  const float* V[3] = {Q.v, Q.v + 3, Q.v + 6};
  float e[3];
  for (int i = 0; i < 3; i++) {
    const float* A = V[i];
    const float* B = V[(i + 1) % 3];
    e[i] = sqrtf((B[0] - A[0]) * (B[0] - A[0]) + (B[1] - A[1]) * (B[1] - A[1]) +
                 (B[2] - A[2]) * (B[2] - A[2]));
  }
  float ang[3];
  for (int i = 0; i < 3; i++) {
    const float a = e[i], b = e[(i + 1) % 3], c = e[(i + 2) % 3];
    ang[i] = acosf(fminf(1.0f, fmaxf(-1.0f, (b * b + c * c - a * a) / (2.0f * b * c))));
  }
  const float emin = fminf(e[0], fminf(e[1], e[2])), emax = fmaxf(e[0], fmaxf(e[1], e[2]));
  const float emid = e[0] + e[1] + e[2] - emin - emax;
  float dv = 3e38f;
  for (int i = 0; i < 3; i++) {
    const float x = rx - V[i][0], y = ry - V[i][1], z = rz - V[i][2];
    dv = fminf(dv, sqrtf(x * x + y * y + z * z));
  }
  const float px = rx - hn * Q.nrm[0], py = ry - hn * Q.nrm[1], pz = rz - hn * Q.nrm[2];
  float lam[3];
  for (int i = 0; i < 3; i++) {
    const float* A = V[(i + 1) % 3];
    const float* B = V[(i + 2) % 3];
    const float ax = A[0] - px, ay = A[1] - py, az = A[2] - pz;
    const float bx = B[0] - px, by = B[1] - py, bz = B[2] - pz;
    const float cx = ay * bz - az * by, cy = az * bx - ax * bz, cz = ax * by - ay * bx;
    lam[i] = fminf(10.0f, fmaxf(-10.0f, 0.5f * (cx * Q.nrm[0] + cy * Q.nrm[1] + cz * Q.nrm[2]) / Q.area));
  }
  const float lmin = fminf(lam[0], fminf(lam[1], lam[2]));
  const float kh = fmaxf(k * h, 1e-6f);
  const float* np = P.nrm;
  f[0] = d / h;
  f[1] = h / d;
  f[2] = logf(d / h);
  f[3] = (h / d) * (h / d);
  f[4] = hn / d;
  f[5] = fabsf(hn) / h;
  f[6] = np[0] * Q.nrm[0] + np[1] * Q.nrm[1] + np[2] * Q.nrm[2];
  f[7] = (rx * np[0] + ry * np[1] + rz * np[2]) / d;
  f[8] = kh;
  f[9] = k * d;
  f[10] = logf(kh);
  f[11] = emin / h;
  f[12] = emid / h;
  f[13] = emax / h;
  f[14] = emax * emax / (2.0f * Q.area);
  f[15] = fminf(ang[0], fminf(ang[1], ang[2]));
  f[16] = fmaxf(ang[0], fmaxf(ang[1], ang[2]));
  f[17] = dv / h;
  f[18] = lam[0];
  f[19] = lam[1];
  f[20] = lam[2];
  f[21] = lmin;
  f[22] = emax / d;
  f[23] = (lmin >= 0 ? fabsf(hn) : dv) / h;
}

// ---------------- FP64 operators with a table rule ----------------
// The rule on each of the n^2 congruent sub-triangles of a uniform n-fold
// edge subdivision of Q (n = 1: the rule itself, points as tabulated).
__device__ Ops ops_rule_sub(const Elem& P, const Elem& Q, double k, int rule, int n) {
  Ops o{};
  const double upNq = P.nrm[0] * Q.nrm[0] + P.nrm[1] * Q.nrm[1] + P.nrm[2] * Q.nrm[2];
  const int b = c_sel.off[rule], e = b + c_sel.cnt[rule];
  const double hn = 1.0 / n;
  for (int i = 0; i < n; i++)
    for (int j = 0; j + i < n; j++)
      for (int up = 1; up >= 0; up--) {
        if (!up && i + j > n - 2) continue;
        // corners: up (i,j), (i+1,j), (i,j+1); down (i+1,j), (i+1,j+1), (i,j+1)
        const double u0 = (up ? i : i + 1) * hn, v0 = j * hn;
        const double u1 = (i + 1) * hn, v1 = (up ? j : j + 1) * hn;
        const double u2 = i * hn, v2 = (j + 1) * hn;
        for (int t = b; t < e; t++) {
          const double s1 = c_sel.x1[t], s2 = c_sel.x2[t], s3 = 1.0 - s1 - s2;
          const double x1 = n == 1 ? s1 : s1 * u0 + s2 * u1 + s3 * u2;
          const double x2 = n == 1 ? s2 : s1 * v0 + s2 * v1 + s3 * v2;
          const double x3 = 1.0 - x1 - x2;
          const double qx = x1 * Q.n1[0] + x2 * Q.n2[0] + x3 * Q.n3[0];
          const double qy = x1 * Q.n1[1] + x2 * Q.n2[1] + x3 * Q.n3[1];
          const double qz = x1 * Q.n1[2] + x2 * Q.n2[2] + x3 * Q.n3[2];
          accumulate(o, c_sel.w[t] * hn * hn, P.c[0], P.c[1], P.c[2], qx, qy, qz, P.nrm, Q.nrm,
                     upNq, k);
        }
      }
  o.L = cscale(Q.area, o.L);
  o.M = cscale(Q.area, o.M);
  o.Mt = cscale(Q.area, o.Mt);
  o.N = cscale(Q.area, o.N);
  return o;
}

__device__ __forceinline__ double cabs1(double2 a) { return sqrt(a.x * a.x + a.y * a.y); }

// max over the four operators of |a - ref| / max(|ref|, floor_rel max |ref|)
// (floor_rel = 1: every operator measured against the pair's largest)
__device__ double ops_err(const Ops& a, const Ops& r, double floor_rel) {
  const double2 av[4] = {a.L, a.M, a.Mt, a.N}, rv[4] = {r.L, r.M, r.Mt, r.N};
  double mx = 0;
  for (int i = 0; i < 4; i++) mx = fmax(mx, cabs1(rv[i]));
  const double floor_ = fmax(floor_rel * mx, 1e-300);
  double e = 0;
  for (int i = 0; i < 4; i++) e = fmax(e, cabs1(csub(av[i], rv[i])) / fmax(cabs1(rv[i]), floor_));
  return e;
}

__global__ void __launch_bounds__(128) sel_label_kernel(const Elem* __restrict__ P,
                                                        const Elem* __restrict__ Q,
                                                        const double* __restrict__ kk, int64_t n,
                                                        double tol, double near_ratio,
                                                        double floor_rel,
                                                        float* __restrict__ feat,
                                                        uint8_t* __restrict__ label,
                                                        float* __restrict__ err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Elem p = P[i], q = Q[i];
  const double k = kk[i];
  float f[SEL_NF];
  sel_features(p.c, p.nrm, q, k, f);
  for (int j = 0; j < SEL_NF; j++) feat[i * SEL_NF + j] = f[j];
  const double dc = len3(p.c[0] - q.c[0], p.c[1] - q.c[1], p.c[2] - q.c[2]);
  const double hq = sqrt(q.area);
  const Ops ref = dc < near_ratio * hq ? ops_nearsing(p, q, k, c_rules)
                                       : ops_rule_sub(p, q, k, SEL_REF, dc < 3.0 * hq ? 8 : 4);
  int lab = SEL_C;
  for (int c = 0; c < SEL_C; c++) {
    const double e = ops_err(ops_rule_sub(p, q, k, c, 1), ref, floor_rel);
    if (err) err[i * 6 + c] = (float)e;
    if (lab == SEL_C && e <= tol) {
      lab = c;
      if (!err) break;
    }
  }
  if (err) err[i * 6 + 5] = (float)ops_err(ops_rule_sub(p, q, k, SEL_PLAIN, 1), ref, floor_rel);
  label[i] = (uint8_t)lab;
}

// ---------------- FP32 training ----------------
constexpr int TB = 128;

// forward, softmax cross-entropy and the per-sample deltas
__global__ void __launch_bounds__(TB) mlp_fwd_bwd_kernel(const float* __restrict__ prm,
                                                         const float* __restrict__ X,
                                                         const uint8_t* __restrict__ y, int64_t B,
                                                         float* __restrict__ work) {
  __shared__ float W[SEL_NPARAM];
  for (int i = threadIdx.x; i < SEL_NPARAM; i += TB) W[i] = prm[i];
  __syncthreads();
  const int64_t s = (int64_t)blockIdx.x * TB + threadIdx.x;
  if (s >= B) return;
  float* H1 = work;
  float* H2 = H1 + B * SEL_H;
  float* D1 = H2 + B * SEL_H;
  float* D2 = D1 + B * SEL_H;
  float* D3 = D2 + B * SEL_H;
  float* LS = D3 + B * 8;
  float x[SEL_NF], h1[SEL_H], h2[SEL_H], z[SEL_C];
  for (int i = 0; i < SEL_NF; i++) x[i] = X[s * SEL_NF + i];
  for (int j = 0; j < SEL_H; j++) {
    float a = W[SEL_OB1 + j];
    for (int i = 0; i < SEL_NF; i++) a += x[i] * W[SEL_OW1 + i * SEL_H + j];
    h1[j] = fmaxf(a, 0.0f);
  }
  for (int j = 0; j < SEL_H; j++) {
    float a = W[SEL_OB2 + j];
    for (int i = 0; i < SEL_H; i++) a += h1[i] * W[SEL_OW2 + i * SEL_H + j];
    h2[j] = fmaxf(a, 0.0f);
  }
  float zm = -1e30f;
  for (int j = 0; j < SEL_C; j++) {
    float a = W[SEL_OB3 + j];
    for (int i = 0; i < SEL_H; i++) a += h2[i] * W[SEL_OW3 + i * SEL_C + j];
    z[j] = a;
    zm = fmaxf(zm, a);
  }
  float se = 0;
  for (int j = 0; j < SEL_C; j++) se += expf(z[j] - zm);
  const int lab = y[s];
  LS[s] = -(z[lab] - zm - logf(se));
  float d3[SEL_C];
  const float inv_b = 1.0f / (float)B;
  for (int j = 0; j < SEL_C; j++) {
    d3[j] = (expf(z[j] - zm) / se - (j == lab ? 1.0f : 0.0f)) * inv_b;
    D3[s * 8 + j] = d3[j];
  }
  float d2[SEL_H];
  for (int i = 0; i < SEL_H; i++) {
    float a = 0;
    for (int j = 0; j < SEL_C; j++) a += W[SEL_OW3 + i * SEL_C + j] * d3[j];
    d2[i] = h2[i] > 0.0f ? a : 0.0f;
    D2[s * SEL_H + i] = d2[i];
    H2[s * SEL_H + i] = h2[i];
  }
  for (int i = 0; i < SEL_H; i++) {
    float a = 0;
    for (int j = 0; j < SEL_H; j++) a += W[SEL_OW2 + i * SEL_H + j] * d2[j];
    D1[s * SEL_H + i] = h1[i] > 0.0f ? a : 0.0f;
    H1[s * SEL_H + i] = h1[i];
  }
}

// one thread per parameter (+1 for the mean loss); samples summed in order
__global__ void mlp_param_grad_kernel(const float* __restrict__ X, int64_t B,
                                      const float* __restrict__ work, float* __restrict__ grad,
                                      float* __restrict__ loss) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > SEL_NPARAM) return;
  const float* H1 = work;
  const float* H2 = H1 + B * SEL_H;
  const float* D1 = H2 + B * SEL_H;
  const float* D2 = D1 + B * SEL_H;
  const float* D3 = D2 + B * SEL_H;
  const float* LS = D3 + B * 8;
  float a = 0;
  if (p == SEL_NPARAM) {
    for (int64_t s = 0; s < B; s++) a += LS[s];
    *loss = a / (float)B;
    return;
  }
  if (p < SEL_OB1) {
    const int i = p / SEL_H, j = p % SEL_H;
    for (int64_t s = 0; s < B; s++) a += X[s * SEL_NF + i] * D1[s * SEL_H + j];
  } else if (p < SEL_OW2) {
    const int j = p - SEL_OB1;
    for (int64_t s = 0; s < B; s++) a += D1[s * SEL_H + j];
  } else if (p < SEL_OB2) {
    const int i = (p - SEL_OW2) / SEL_H, j = (p - SEL_OW2) % SEL_H;
    for (int64_t s = 0; s < B; s++) a += H1[s * SEL_H + i] * D2[s * SEL_H + j];
  } else if (p < SEL_OW3) {
    const int j = p - SEL_OB2;
    for (int64_t s = 0; s < B; s++) a += D2[s * SEL_H + j];
  } else if (p < SEL_OB3) {
    const int i = (p - SEL_OW3) / SEL_C, j = (p - SEL_OW3) % SEL_C;
    for (int64_t s = 0; s < B; s++) a += H2[s * SEL_H + i] * D3[s * 8 + j];
  } else {
    const int j = p - SEL_OB3;
    for (int64_t s = 0; s < B; s++) a += D3[s * 8 + j];
  }
  grad[p] = a;
}

__global__ void mlp_adam_kernel(float* __restrict__ prm, const float* __restrict__ g,
                                float* __restrict__ m, float* __restrict__ v, float lr, float b1,
                                float b2, float eps, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= SEL_NPARAM) return;
  const float gi = g[p];
  const float mi = b1 * m[p] + (1.0f - b1) * gi;
  const float vi = b2 * v[p] + (1.0f - b2) * gi * gi;
  m[p] = mi;
  v[p] = vi;
  prm[p] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void __launch_bounds__(TB) mlp_forward_kernel(const float* __restrict__ prm,
                                                         const float* __restrict__ X, int64_t B,
                                                         float* __restrict__ logits) {
  __shared__ float W[SEL_NPARAM];
  for (int i = threadIdx.x; i < SEL_NPARAM; i += TB) W[i] = prm[i];
  __syncthreads();
  const int64_t s = (int64_t)blockIdx.x * TB + threadIdx.x;
  if (s >= B) return;
  float x[SEL_NF], h1[SEL_H];
  for (int i = 0; i < SEL_NF; i++) x[i] = X[s * SEL_NF + i];
  for (int j = 0; j < SEL_H; j++) {
    float a = W[SEL_OB1 + j];
    for (int i = 0; i < SEL_NF; i++) a += x[i] * W[SEL_OW1 + i * SEL_H + j];
    h1[j] = fmaxf(a, 0.0f);
  }
  float z[SEL_C];
  for (int j = 0; j < SEL_C; j++) z[j] = W[SEL_OB3 + j];
  for (int i = 0; i < SEL_H; i++) {
    float a = W[SEL_OB2 + i];
    for (int t = 0; t < SEL_H; t++) a += h1[t] * W[SEL_OW2 + t * SEL_H + i];
    a = fmaxf(a, 0.0f);
    for (int j = 0; j < SEL_C; j++) z[j] += a * W[SEL_OW3 + i * SEL_C + j];
  }
  for (int j = 0; j < SEL_C; j++) logits[s * SEL_C + j] = z[j];
}

// ---------------- BF16 tensor-core inference ----------------
__device__ __forceinline__ uint16_t f2bf(float x) {
  __nv_bfloat16 b = __float2bfloat16_rn(x);
  return *reinterpret_cast<uint16_t*>(&b);
}

__device__ __forceinline__ uint32_t ld32(const uint16_t* p) {
  return *reinterpret_cast<const uint32_t*>(p);
}

// D (16 x 8, FP32) += A (16 x 16, BF16, row-major) * B (16 x 8, BF16, column-major)
__device__ __forceinline__ void mma16816(float* d, uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// One dense layer for the warp's 32 rows (two m16 row tiles sharing every B
// fragment): A (32 x K, ld lda) times W^T stored output-major (N x K, ld
// ldw). Fragments follow the m16n8k16 layout: lane = 4 g + t holds
// A(g, 2t..2t+1), A(g+8, ..), A(g, 2t+8..), A(g+8, 2t+8..); B(2t..2t+1, g),
// B(2t+8.., g); D(g, 2t..2t+1), D(g+8, ..).
template <int K, int NT>
__device__ __forceinline__ void warp_layer(const uint16_t* A, int lda, const uint16_t* Wt, int ldw,
                                           float (*acc)[NT][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int m = 0; m < 2; m++)
#pragma unroll
    for (int nt = 0; nt < NT; nt++) acc[m][nt][0] = acc[m][nt][1] = acc[m][nt][2] = acc[m][nt][3] = 0.0f;
#pragma unroll
  for (int k0 = 0; k0 < K; k0 += 16) {
    uint32_t a[2][4];
#pragma unroll
    for (int m = 0; m < 2; m++) {
      const uint16_t* r0 = A + (16 * m + g) * lda + k0 + 2 * t;
      const uint16_t* r1 = r0 + 8 * lda;
      a[m][0] = ld32(r0);
      a[m][1] = ld32(r1);
      a[m][2] = ld32(r0 + 8);
      a[m][3] = ld32(r1 + 8);
    }
#pragma unroll
    for (int nt = 0; nt < NT; nt++) {
      const uint16_t* w = Wt + (nt * 8 + g) * ldw + k0 + 2 * t;
      const uint32_t b0 = ld32(w), b1 = ld32(w + 8);
      mma16816(acc[0][nt], a[0][0], a[0][1], a[0][2], a[0][3], b0, b1);
      mma16816(acc[1][nt], a[1][0], a[1][1], a[1][2], a[1][3], b0, b1);
    }
  }
}

// bias + ReLU, back to BF16 rows of H (32 x 64)
__device__ __forceinline__ void store_hidden(float (*acc)[8][4], const float* bias, uint16_t* H) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int m = 0; m < 2; m++)
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const int c = nt * 8 + 2 * t;
      uint16_t* r0 = H + (16 * m + g) * 64 + c;
      uint16_t* r1 = r0 + 8 * 64;
      r0[0] = f2bf(fmaxf(acc[m][nt][0] + bias[c], 0.0f));
      r0[1] = f2bf(fmaxf(acc[m][nt][1] + bias[c + 1], 0.0f));
      r1[0] = f2bf(fmaxf(acc[m][nt][2] + bias[c], 0.0f));
      r1[1] = f2bf(fmaxf(acc[m][nt][3] + bias[c + 1], 0.0f));
    }
}

// two 32 x 64 BF16 tiles per warp: the input (columns 0..31) and then the
// second hidden layer in `a`, the first hidden layer in `b`
struct WarpBufs {
  uint16_t a[32 * 64];
  uint16_t b[32 * 64];
};

// the network on the warp's 32 rows (inputs staged in wb.a); lg[m] holds,
// for rows 16 m + g and 16 m + g + 8, the logits of columns 2t, 2t+1
__device__ __forceinline__ void warp_mlp(const SelBlob& B, WarpBufs& wb, float (*lg)[4]) {
  float acc[2][8][4];
  warp_layer<32, 8>(wb.a, 64, B.w1t, 32, acc);
  store_hidden(acc, B.b1, wb.b);
  __syncwarp();
  warp_layer<64, 8>(wb.b, 64, B.w2t, 64, acc);
  store_hidden(acc, B.b2, wb.a);
  __syncwarp();
  float o[2][1][4];
  warp_layer<64, 1>(wb.a, 64, B.w3t, 64, o);
  const int t = (threadIdx.x & 31) & 3;
#pragma unroll
  for (int m = 0; m < 2; m++) {
    lg[m][0] = o[m][0][0] + B.b3[2 * t];
    lg[m][1] = o[m][0][1] + B.b3[2 * t + 1];
    lg[m][2] = o[m][0][2] + B.b3[2 * t];
    lg[m][3] = o[m][0][3] + B.b3[2 * t + 1];
  }
}

// argmax over the 8 logits of a row spread over the 4 lanes of a group, and
// the softmax probability of the winner
__device__ __forceinline__ void group_argmax(float l0, float l1, int t, int& cls, float& prob) {
  float m = l0 >= l1 ? l0 : l1;
  int c = l0 >= l1 ? 2 * t : 2 * t + 1;
#pragma unroll
  for (int o = 1; o <= 2; o <<= 1) {
    const float m2 = __shfl_xor_sync(0xffffffffu, m, o);
    const int c2 = __shfl_xor_sync(0xffffffffu, c, o);
    if (m2 > m || (m2 == m && c2 < c)) {
      m = m2;
      c = c2;
    }
  }
  float se = __expf(l0 - m) + __expf(l1 - m);
  se += __shfl_xor_sync(0xffffffffu, se, 1);
  se += __shfl_xor_sync(0xffffffffu, se, 2);
  cls = c;
  prob = 1.0f / se;
}

__device__ __forceinline__ void stage_blob(const SelBlob* src, SelBlob& dst) {
  const uint4* s = reinterpret_cast<const uint4*>(src);
  uint4* d = reinterpret_cast<uint4*>(&dst);
  for (int i = threadIdx.x; i < (int)(sizeof(SelBlob) / 16); i += blockDim.x) d[i] = s[i];
  __syncthreads();
}

// normalised features of one row into the warp's BF16 input tile (ld 64)
__device__ __forceinline__ void stage_row(const SelBlob& B, const float* f, uint16_t* xrow) {
#pragma unroll
  for (int j = 0; j < SEL_NF; j++) xrow[j] = f2bf((f[j] - B.mu[j]) * B.inv_sigma[j]);
#pragma unroll
  for (int j = SEL_NF; j < 32; j++) xrow[j] = 0;
}

constexpr int IW = 4;  // warps per inference CTA

__global__ void __launch_bounds__(32 * IW) sel_infer_rows_kernel(const SelBlob* __restrict__ blob,
                                                                 const float* __restrict__ feat,
                                                                 int64_t B,
                                                                 float* __restrict__ logits,
                                                                 uint8_t* __restrict__ cls) {
  __shared__ __align__(16) SelBlob sb;
  __shared__ __align__(16) WarpBufs wb[IW];
  stage_blob(blob, sb);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int64_t nchunk = (B + 31) / 32;
  for (int64_t ch = (int64_t)blockIdx.x * IW + warp; ch < nchunk; ch += (int64_t)gridDim.x * IW) {
    const int64_t r0 = ch * 32;
    {
      float f[SEL_NF];
      const int64_t r = r0 + lane;
      for (int j = 0; j < SEL_NF; j++) f[j] = r < B ? feat[r * SEL_NF + j] : 0.0f;
      stage_row(sb, f, wb[warp].a + lane * 64);
    }
    __syncwarp();
    float lg[2][4];
    warp_mlp(sb, wb[warp], lg);
#pragma unroll
    for (int m = 0; m < 2; m++) {
      int c0, c1;
      float p0, p1;
      group_argmax(lg[m][0], lg[m][1], t, c0, p0);
      group_argmax(lg[m][2], lg[m][3], t, c1, p1);
      const int64_t ra = r0 + 16 * m + g, rb = ra + 8;
      if (logits) {
        if (ra < B) {
          logits[ra * 8 + 2 * t] = lg[m][0];
          logits[ra * 8 + 2 * t + 1] = lg[m][1];
        }
        if (rb < B) {
          logits[rb * 8 + 2 * t] = lg[m][2];
          logits[rb * 8 + 2 * t + 1] = lg[m][3];
        }
      }
      if (t == 0) {
        if (ra < B) cls[ra] = (uint8_t)c0;
        if (rb < B) cls[rb] = (uint8_t)c1;
      }
    }
    __syncwarp();
  }
}

__device__ __forceinline__ bool is_special(const uint32_t* bits, int64_t g) {
  return (bits[g >> 5] >> (g & 31)) & 1u;
}

// classes of the regular near-field entries of a mesh: a persistent grid,
// each CTA stages the network once and walks tiles, each warp 32 entries
__global__ void __launch_bounds__(32 * IW) sel_near_classes_kernel(SelNearArgs a) {
  __shared__ __align__(16) SelBlob sb;
  __shared__ __align__(16) WarpBufs wb[IW];
  stage_blob(a.blob, sb);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  for (int64_t ti = blockIdx.x; ti < a.ntiles; ti += gridDim.x) {
    const NearTile tile = a.tiles[ti];
    const NearBlock b = a.blocks[tile.block];
    const int nchunk = (tile.count + 31) / 32;
    for (int ch = warp; ch < nchunk; ch += IW) {
      {
        const int e = ch * 32 + lane;
        float f[SEL_NF];
        if (e < tile.count && !is_special(a.special_bits, b.off + tile.first + e)) {
          const int idx = tile.first + e;
          const int r = idx % b.m, c = idx / b.m;
          sel_features32(a.EF[b.r0 + r], a.EF[b.c0 + c], a.k, f);
        } else {
          for (int j = 0; j < SEL_NF; j++) f[j] = sb.mu[j];
        }
        stage_row(sb, f, wb[warp].a + lane * 64);
      }
      __syncwarp();
      float lg[2][4];
      warp_mlp(sb, wb[warp], lg);
#pragma unroll
      for (int m = 0; m < 2; m++) {
        int c0, c1;
        float p0, p1;
        group_argmax(lg[m][0], lg[m][1], t, c0, p0);
        group_argmax(lg[m][2], lg[m][3], t, c1, p1);
        if (t == 0) {
          const int ea = ch * 32 + 16 * m + g, eb = ea + 8;
          if (ea < tile.count)
            a.cls[b.off + tile.first + ea] = (uint8_t)(p0 < a.guard_prob ? SEL_C - 1 : c0);
          if (eb < tile.count)
            a.cls[b.off + tile.first + eb] = (uint8_t)(p1 < a.guard_prob ? SEL_C - 1 : c1);
        }
      }
      __syncwarp();
    }
  }
}

// ---------------- near-field entries with the selected rules ----------------
constexpr int SEL_CLASS_PTS = 1 + 3 + 7 + 13 + 25;  // classes 0-4, stored first

__device__ __forceinline__ float fabs2(float2 a) { return sqrtf(a.x * a.x + a.y * a.y); }

// One CTA per near-field tile. The tile's regular entries are first grouped
// by class in shared memory, so that a warp integrates one rule (its cost is
// the rule's points, not the largest rule among its lanes).
__global__ void __launch_bounds__(256) sel_nearfield32_kernel(SelNearfieldArgs a) {
  __shared__ float rx1[SEL_CLASS_PTS], rx2[SEL_CLASS_PTS], rw[SEL_CLASS_PTS];
  __shared__ int roff[SEL_C + 1];
  __shared__ int cnt[SEL_C], base[SEL_C + 1];
  __shared__ int16_t order[256];
  for (int i = threadIdx.x; i < SEL_CLASS_PTS; i += blockDim.x) {
    rx1[i] = c_sel.fx1[i];
    rx2[i] = c_sel.fx2[i];
    rw[i] = c_sel.fw[i];
  }
  if (threadIdx.x <= SEL_C) roff[threadIdx.x] = threadIdx.x < SEL_C ? c_sel.off[threadIdx.x] : SEL_CLASS_PTS;
  if (threadIdx.x < SEL_C) cnt[threadIdx.x] = 0;
  __syncthreads();
  const NearTile t = a.tiles[blockIdx.x];
  const NearBlock b = a.blocks[t.block];
  // group this tile's regular entries by class
  int my_cls = -1, slot = 0;
  if ((int)threadIdx.x < t.count && !is_special(a.special_bits, b.off + t.first + threadIdx.x)) {
    my_cls = min((int)a.cls[b.off + t.first + threadIdx.x], SEL_C - 1);
    slot = atomicAdd(&cnt[my_cls], 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    base[0] = 0;
    for (int c = 0; c < SEL_C; c++) base[c + 1] = base[c] + cnt[c];
  }
  __syncthreads();
  if (my_cls >= 0) order[base[my_cls] + slot] = (int16_t)threadIdx.x;
  __syncthreads();
  unsigned long long pts = 0, chk = 0, fb = 0;
  if ((int)threadIdx.x < base[SEL_C]) {
    const int le = order[threadIdx.x];
    const int e = t.first + le;
    const int64_t g = b.off + e;
    const int r = e % b.m, c = e / b.m;
    const int64_t row = b.r0 + r, col = b.c0 + c;
    const int cls = min((int)a.cls[g], SEL_C - 1);
    float2 p, d;
    substitute32(ops_rule32_pts(a.EF, row, col, a.k, roff[cls], roff[cls + 1], rx1, rx2, rw),
                 a.bc[col], a.alpha, p, d);
    pts = roff[cls + 1] - roff[cls];
    const uint32_t hsh = (uint32_t)((uint64_t)g * 2654435761ull >> 7);
    if (cls < SEL_C - 1 && a.check_every > 0 && hsh % (uint32_t)a.check_every == 0) {
      float2 p4, d4;
      substitute32(ops_rule32_pts(a.EF, row, col, a.k, roff[SEL_C - 1], roff[SEL_C], rx1, rx2, rw),
                   a.bc[col], a.alpha, p4, d4);
      pts += roff[SEL_C] - roff[SEL_C - 1];
      chk = 1;
      const float scale = fmaxf(fmaxf(fabs2(p4), fabs2(d4)), 1e-30f);
      const float diff = fmaxf(fabs2(fsub(p, p4)), fabs2(fsub(d, d4)));
      if (diff > a.check_tol * scale) {
        p = p4;
        d = d4;
        fb = 1;
      }
    }
    a.phi[g] = p;
    a.dphi[g] = d;
  }
  // per-warp sums of the counters
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    pts += __shfl_xor_sync(0xffffffffu, pts, o);
    chk += __shfl_xor_sync(0xffffffffu, chk, o);
    fb += __shfl_xor_sync(0xffffffffu, fb, o);
  }
  if ((threadIdx.x & 31) == 0 && a.counters) {
    if (pts) atomicAdd(&a.counters[0], pts);
    if (chk) atomicAdd(&a.counters[1], chk);
    if (fb) atomicAdd(&a.counters[2], fb);
  }
}

uint16_t host_bf16(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);  // NaN stays NaN
  const uint32_t lsb = (u >> 16) & 1u;
  u += 0x7fffu + lsb;  // round to nearest even
  return (uint16_t)(u >> 16);
}

}  // namespace

// The rule tables go to each device's constant memory once (synchronously),
// so that concurrent sweep workers never rewrite them under running kernels.
void sel_upload_rules(cudaStream_t s) {
  (void)s;
  static std::mutex mu;
  static std::set<int> done;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  if (done.count(dev)) return;
  static const SelRules R = build_rules();
  static const QuadRules Q = make_rules();
  if (cudaMemcpyToSymbol(c_sel, &R, sizeof(SelRules)) == cudaSuccess &&
      cudaMemcpyToSymbol(c_rules, &Q, sizeof(QuadRules)) == cudaSuccess)
    done.insert(dev);
}

void launch_sel_label(const Elem* P, const Elem* Q, const double* k, int64_t n, double tol,
                      double near_ratio, double floor_rel, float* feat, uint8_t* label,
                      float* err, cudaStream_t s) {
  if (n <= 0) return;
  sel_upload_rules(s);
  sel_label_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(P, Q, k, n, tol, near_ratio,
                                                               floor_rel, feat, label, err);
}

void launch_mlp_grad(const float* params, const float* X, const uint8_t* y, int64_t B,
                     float* grad, float* loss, float* work, cudaStream_t s) {
  if (B <= 0) return;
  mlp_fwd_bwd_kernel<<<(unsigned)((B + TB - 1) / TB), TB, 0, s>>>(params, X, y, B, work);
  mlp_param_grad_kernel<<<(SEL_NPARAM + 1 + 127) / 128, 128, 0, s>>>(X, B, work, grad, loss);
}

void launch_mlp_adam(float* params, const float* grad, float* m, float* v, int64_t step,
                     float lr, float b1, float b2, float eps, cudaStream_t s) {
  const float c1 = 1.0f - std::pow(b1, (float)step), c2 = 1.0f - std::pow(b2, (float)step);
  mlp_adam_kernel<<<(SEL_NPARAM + 255) / 256, 256, 0, s>>>(params, grad, m, v, lr, b1, b2, eps,
                                                            c1, c2);
}

void launch_mlp_forward(const float* params, const float* X, int64_t B, float* logits,
                        cudaStream_t s) {
  if (B <= 0) return;
  mlp_forward_kernel<<<(unsigned)((B + TB - 1) / TB), TB, 0, s>>>(params, X, B, logits);
}

void launch_sel_infer_rows(const SelBlob* blob, const float* feat, int64_t B, float* logits,
                           uint8_t* cls, cudaStream_t s) {
  if (B <= 0) return;
  const int64_t nchunk = (B + 31) / 32;
  const unsigned grid = (unsigned)std::min<int64_t>((nchunk + IW - 1) / IW, 152 * 8);
  sel_infer_rows_kernel<<<grid, 32 * IW, 0, s>>>(blob, feat, B, logits, cls);
}

void launch_sel_near_classes(const SelNearArgs& a, cudaStream_t s) {
  if (a.ntiles <= 0) return;
  const unsigned grid = (unsigned)std::min<int64_t>(a.ntiles, 152 * 8);
  sel_near_classes_kernel<<<grid, 32 * IW, 0, s>>>(a);
}

void launch_sel_nearfield32(const SelNearfieldArgs& a, cudaStream_t s) {
  if (a.ntiles <= 0) return;
  sel_upload_rules(s);
  sel_nearfield32_kernel<<<(unsigned)a.ntiles, 256, 0, s>>>(a);
}

void sel_class_rule_tables(float* x1, float* x2, float* w, int* off) {
  static const SelRules R = build_rules();
  for (int i = 0; i < SEL_CLASS_PTS; i++) {
    x1[i] = R.fx1[i];
    x2[i] = R.fx2[i];
    w[i] = R.fw[i];
  }
  for (int c = 0; c < SEL_C; c++) off[c] = R.off[c];
  off[SEL_C] = SEL_CLASS_PTS;
}

void sel_make_blob(const float* prm, const float* mu, const float* sigma, SelBlob& B) {
  std::memset(&B, 0, sizeof(B));
  for (int j = 0; j < SEL_H; j++) {
    for (int i = 0; i < SEL_NF; i++) B.w1t[j * 32 + i] = host_bf16(prm[SEL_OW1 + i * SEL_H + j]);
    for (int i = 0; i < SEL_H; i++) B.w2t[j * SEL_H + i] = host_bf16(prm[SEL_OW2 + i * SEL_H + j]);
    B.b1[j] = prm[SEL_OB1 + j];
    B.b2[j] = prm[SEL_OB2 + j];
  }
  for (int j = 0; j < 8; j++) {
    for (int i = 0; i < SEL_H; i++)
      B.w3t[j * SEL_H + i] = j < SEL_C ? host_bf16(prm[SEL_OW3 + i * SEL_C + j]) : (uint16_t)0;
    B.b3[j] = j < SEL_C ? prm[SEL_OB3 + j] : -1e30f;
  }
  for (int i = 0; i < SEL_NF; i++) {
    B.mu[i] = mu[i];
    B.inv_sigma[i] = sigma[i] > 0 ? 1.0f / sigma[i] : 1.0f;
  }
}

}  // namespace bemgpu
