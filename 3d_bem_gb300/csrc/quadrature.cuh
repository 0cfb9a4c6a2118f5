// quadrature.cuh -- device evaluation of the collocation operators L, M, Mt, N
// of one (collocation point, triangle) pair and of the BC-substituted matrix
// entries. Included by every kernel file that generates matrix entries; each
// translation unit gets its own constant-memory copy of the rule tables.
//
// Reference (KG93/3d_BEM): boundaryelementsolver.cpp:844-894 (dispatch and the
// regular 16-point rule), :896-1029 (singular polar integration),
// :1387-1514 (near-singular split-polar rule), global.cpp:955-1228 (point
// projection), :2004-2040 (BC substitution).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bem_types.h"

namespace bemgpu {

// ----- complex helpers (double2 / float2 as complex) -----
__host__ __device__ __forceinline__ double2 cmk(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return cmk(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) { return cmk(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return cmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ double2 cscale(double s, double2 a) { return cmk(s * a.x, s * a.y); }
__host__ __device__ __forceinline__ double2 cconj(double2 a) { return cmk(a.x, -a.y); }
__host__ __device__ __forceinline__ double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }
__host__ __device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  // Smith's algorithm for complex division
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, d = b.x + b.y * r;
    return cmk((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  }
  double r = b.x / b.y, d = b.y + b.x * r;
  return cmk((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}

struct Ops {
  double2 L, M, Mt, N;
};

// ----- the element integrand, shared by the regular and near-singular rules -----
// G = exp(ikr) / (4 pi r); dG/dr = G/r (ikr - 1); d2G/dr2 = G/r^2 (2 - 2ikr - k^2 r^2)
// (boundaryelementsolver.cpp:872-887, :1486-1500)
__device__ __forceinline__ void accumulate(Ops& o, double w, double px, double py, double pz,
                                           double qx, double qy, double qz, const double* np,
                                           const double* nq, double upNq, double k) {
  double rx = px - qx, ry = py - qy, rz = pz - qz;
  double rr = rx * rx + ry * ry + rz * rz;
  double r = sqrt(rr);
  double ir = 1.0 / r;
  double rnq = -(rx * nq[0] + ry * nq[1] + rz * nq[2]) * ir;
  double rnp = (rx * np[0] + ry * np[1] + rz * np[2]) * ir;
  double s, c;
  sincos(k * r, &s, &c);
  double g0 = ir * (1.0 / (4.0 * 3.14159265358979323846));
  double2 G = cmk(c * g0, s * g0);
  double kr = k * r;
  // dG = G/r * (ikr - 1)
  double2 Gr = cscale(ir, G);
  double2 dG = cmk(-Gr.x - kr * Gr.y, -Gr.y + kr * Gr.x);
  // d2G = G/rr * (2 - k^2 rr - 2ikr)
  double2 Grr = cscale(ir * ir, G);
  double a2 = 2.0 - kr * kr, b2 = -2.0 * kr;
  double2 d2G = cmk(Grr.x * a2 - Grr.y * b2, Grr.x * b2 + Grr.y * a2);
  o.L.x += w * G.x;
  o.L.y += w * G.y;
  double wm = w * rnq, wt = w * rnp;
  o.M.x += wm * dG.x;
  o.M.y += wm * dG.y;
  o.Mt.x += wt * dG.x;
  o.Mt.y += wt * dG.y;
  double f1 = -(upNq + rnp * rnq) * ir, f2 = rnp * rnq;
  o.N.x += w * (f1 * dG.x + f2 * d2G.x);
  o.N.y += w * (f1 * dG.y + f2 * d2G.y);
}

// Regular rule: 16-point triangle rule scaled by the area (:857-893).
__device__ __forceinline__ Ops ops_regular(const Elem& P, const Elem& Q, double k,
                                           const QuadRules& R) {
  Ops o{};
  double upNq = P.nrm[0] * Q.nrm[0] + P.nrm[1] * Q.nrm[1] + P.nrm[2] * Q.nrm[2];
#pragma unroll
  for (int i = 0; i < 16; i++) {
    double a1 = R.reg_x1[i], a2 = R.reg_x2[i], a3 = 1.0 - a2 - a1;
    double qx = a1 * Q.n1[0] + a2 * Q.n2[0] + a3 * Q.n3[0];
    double qy = a1 * Q.n1[1] + a2 * Q.n2[1] + a3 * Q.n3[1];
    double qz = a1 * Q.n1[2] + a2 * Q.n2[2] + a3 * Q.n3[2];
    accumulate(o, R.reg_w[i], P.c[0], P.c[1], P.c[2], qx, qy, qz, P.nrm, Q.nrm, upNq, k);
  }
  double A = Q.area;
  o.L = cscale(A, o.L);
  o.M = cscale(A, o.M);
  o.Mt = cscale(A, o.Mt);
  o.N = cscale(A, o.N);
  return o;
}

// Singular rule for the panel's own collocation point (:896-1029): three
// sub-triangles at the centroid, angular Gauss-Legendre (16 symmetric pairs),
// closed-form radial integral; M = Mt = 0 on a flat panel.
__device__ __forceinline__ Ops ops_singular(const Elem& T, double k, const QuadRules& R) {
  const double* nodes[3] = {T.n1, T.n2, T.n3};
  double Ls_x = 0, Ls_y = 0, Ns_x = 0, Ns_y = 0;
  for (int s = 0; s < 3; s++) {
    const double* P1 = nodes[s];
    const double* P2 = nodes[(s + 1) % 3];
    double cx = T.c[0] - P1[0], cy = T.c[1] - P1[1], cz = T.c[2] - P1[2];
    double bx = T.c[0] - P2[0], by = T.c[1] - P2[1], bz = T.c[2] - P2[2];
    double ax = P2[0] - P1[0], ay = P2[1] - P1[1], az = P2[2] - P1[2];
    double b2 = bx * bx + by * by + bz * bz, c2 = cx * cx + cy * cy + cz * cz,
           a2 = ax * ax + ay * ay + az * az;
    double b = sqrt(b2), c = sqrt(c2);
    if (c < b) {
      double t = c;
      c = b;
      b = t;
    }
    double A = acos((b2 + c2 - a2) / (2.0 * b * c));
    double sA, cA;
    sincos(A, &sA, &cA);
    double B = atan((b * sA) / (c - b * cA));
    double sB = sin(B);
    double half = 0.5 * A;
    double lx = 0, ly = 0, nx = 0, ny = 0;
#pragma unroll 4
    for (int i = 0; i < 16; i++) {
      double th1 = R.gl_x[i] * half + half;
      double th2 = -R.gl_x[i] * half + half;
      double r1 = c * sB / sin(th1 + B);
      double r2 = c * sB / sin(th2 + B);
      double s1, c1, s2, c2v;
      sincos(k * r1, &s1, &c1);
      sincos(k * r2, &s2, &c2v);
      double w = R.gl_w[i];
      lx += w * (c1 + c2v);
      ly += w * (s1 + s2);
      nx += w * (c1 / r1 + c2v / r2);
      ny += w * (s1 / r1 + s2 / r2);
    }
    Ls_x += lx * half;
    Ls_y += ly * half;
    Ns_x += nx * half;
    Ns_y += ny * half;
  }
  const double PI = 3.14159265358979323846;
  double LTx = Ls_x / (2.0 * PI), LTy = Ls_y / (2.0 * PI);
  double NTx = Ns_x / (4.0 * PI), NTy = Ns_y / (4.0 * PI);
  Ops o{};
  // L = (i / 2k) (1 - LT)
  double ik2 = 1.0 / (2.0 * k);
  o.L = cmk(ik2 * LTy, ik2 * (1.0 - LTx));
  // N = ik/2 - NT
  o.N = cmk(-NTx, 0.5 * k - NTy);
  o.M = cmk(0, 0);
  o.Mt = cmk(0, 0);
  return o;
}

// Closest point of triangle Q to p (global.cpp:955-1228), with the 0.05
// barycentric classification; returns the region code
// 0 interior, 1..3 node 1..3, 4 side 21, 5 side 32, 6 side 13.
// The minimisation over the triangle's (s, t) parameter domain is D. Eberly's
// published point-to-triangle distance algorithm ("Distance Between Point and
// Triangle in 3D", Geometric Tools), which the reference also follows region
// by region; the same branches and quadratic-form names are kept because the
// near-singular classification has to agree with the reference bit for bit.
__device__ __forceinline__ int project_point(const Elem& Q, const double* p, double* out) {
  double d[3], e0[3], e1[3];
  for (int i = 0; i < 3; i++) {
    d[i] = Q.n1[i] - p[i];
    e0[i] = Q.n2[i] - Q.n1[i];
    e1[i] = Q.n3[i] - Q.n1[i];
  }
  double a00 = e0[0] * e0[0] + e0[1] * e0[1] + e0[2] * e0[2];
  double a01 = e0[0] * e1[0] + e0[1] * e1[1] + e0[2] * e1[2];
  double a11 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
  double b0 = d[0] * e0[0] + d[1] * e0[1] + d[2] * e0[2];
  double b1 = d[0] * e1[0] + d[1] * e1[1] + d[2] * e1[2];
  double det = fmax(a00 * a11 - a01 * a01, 0.0);
  double s = a01 * b1 - a11 * b0;
  double t = a01 * b0 - a00 * b1;
  if (s + t <= det) {
    if (s < 0.0) {
      if (t < 0.0) {
        if (b0 < 0.0) {
          t = 0.0;
          s = (-b0 >= a00) ? 1.0 : -b0 / a00;
        } else {
          s = 0.0;
          t = (b1 >= 0.0) ? 0.0 : ((-b1 >= a11) ? 1.0 : -b1 / a11);
        }
      } else {
        s = 0.0;
        t = (b1 >= 0.0) ? 0.0 : ((-b1 >= a11) ? 1.0 : -b1 / a11);
      }
    } else if (t < 0.0) {
      t = 0.0;
      s = (b0 >= 0.0) ? 0.0 : ((-b0 >= a00) ? 1.0 : -b0 / a00);
    } else {
      s /= det;
      t /= det;
    }
  } else {
    if (s < 0.0) {
      double tmp0 = a01 + b0, tmp1 = a11 + b1;
      if (tmp1 > tmp0) {
        double numer = tmp1 - tmp0, denom = a00 - 2.0 * a01 + a11;
        if (numer >= denom) { s = 1.0; t = 0.0; }
        else { s = numer / denom; t = 1.0 - s; }
      } else {
        s = 0.0;
        t = (tmp1 <= 0.0) ? 1.0 : ((b1 >= 0.0) ? 0.0 : -b1 / a11);
      }
    } else if (t < 0.0) {
      double tmp0 = a01 + b1, tmp1 = a00 + b0;
      if (tmp1 > tmp0) {
        double numer = tmp1 - tmp0, denom = a00 - 2.0 * a01 + a11;
        if (numer >= denom) { t = 1.0; s = 0.0; }
        else { t = numer / denom; s = 1.0 - t; }
      } else {
        t = 0.0;
        s = (tmp1 <= 0.0) ? 1.0 : ((b0 >= 0.0) ? 0.0 : -b0 / a00);
      }
    } else {
      double numer = a11 + b1 - a01 - b0;
      if (numer <= 0.0) { s = 0.0; t = 1.0; }
      else {
        double denom = a00 - 2.0 * a01 + a11;
        if (numer >= denom) { s = 1.0; t = 0.0; }
        else { s = numer / denom; t = 1.0 - s; }
      }
    }
  }
  const double EPS = 0.05;
  double c1 = 1.0 - s - t, c2 = s, c3 = t;
  int sig = (c1 > EPS) + (c2 > EPS) + (c3 > EPS);
  int reg;
  if (sig == 3) {
    reg = 0;
  } else if (sig == 2) {
    if (c1 > EPS && c2 > EPS) { reg = 4; c1 += c3 / 2.0; c2 += c3 / 2.0; c3 = 0.0; }
    else if (c1 > EPS && c3 > EPS) { reg = 6; c1 += c2 / 2.0; c3 += c2 / 2.0; c2 = 0.0; }
    else { reg = 5; c2 += c1 / 2.0; c3 += c1 / 2.0; c1 = 0.0; }
  } else {
    if (c1 > EPS) { reg = 1; c1 = 1; c2 = 0; c3 = 0; }
    else if (c2 > EPS) { reg = 2; c1 = 0; c2 = 1; c3 = 0; }
    else { reg = 3; c1 = 0; c2 = 0; c3 = 1; }
  }
  for (int i = 0; i < 3; i++) out[i] = c1 * Q.n1[i] + c2 * Q.n2[i] + c3 * Q.n3[i];
  return reg;
}

// Near-singular split-polar rule (:1387-1514): project p onto the source
// triangle, split there into 1-3 sub-triangles, 5 x 5 polar Gauss-Legendre.
static __device__ __noinline__ Ops ops_nearsing(const Elem& P, const Elem& Q, double k,
                                         const QuadRules& R) {
  Ops o{};
  double upNq = P.nrm[0] * Q.nrm[0] + P.nrm[1] * Q.nrm[1] + P.nrm[2] * Q.nrm[2];
  double Pp[3];
  int reg = project_point(Q, P.c, Pp);
  // sub-triangles as (first, second, third) vertex pointers
  const double* V[3][3];
  int ns = 0;
  switch (reg) {
    case 0:
      V[0][0] = Pp; V[0][1] = Q.n1; V[0][2] = Q.n2;
      V[1][0] = Pp; V[1][1] = Q.n2; V[1][2] = Q.n3;
      V[2][0] = Pp; V[2][1] = Q.n3; V[2][2] = Q.n1;
      ns = 3;
      break;
    case 1: V[0][0] = Q.n1; V[0][1] = Q.n2; V[0][2] = Q.n3; ns = 1; break;
    case 2: V[0][0] = Q.n2; V[0][1] = Q.n3; V[0][2] = Q.n1; ns = 1; break;
    case 3: V[0][0] = Q.n3; V[0][1] = Q.n1; V[0][2] = Q.n2; ns = 1; break;
    case 4:
      V[0][0] = Pp; V[0][1] = Q.n3; V[0][2] = Q.n1;
      V[1][0] = Pp; V[1][1] = Q.n2; V[1][2] = Q.n3;
      ns = 2;
      break;
    case 5:
      V[0][0] = Pp; V[0][1] = Q.n3; V[0][2] = Q.n1;
      V[1][0] = Pp; V[1][1] = Q.n1; V[1][2] = Q.n2;
      ns = 2;
      break;
    default:
      V[0][0] = Pp; V[0][1] = Q.n1; V[0][2] = Q.n2;
      V[1][0] = Pp; V[1][1] = Q.n2; V[1][2] = Q.n3;
      ns = 2;
      break;
  }
  for (int s = 0; s < ns; s++) {
    const double *A1 = V[s][0], *A2 = V[s][1], *A3 = V[s][2];
    double s13[3], s23[3], s12[3];
    for (int i = 0; i < 3; i++) {
      s13[i] = A3[i] - A1[i];
      s23[i] = A3[i] - A2[i];
      s12[i] = A2[i] - A1[i];
    }
    double q13 = s13[0] * s13[0] + s13[1] * s13[1] + s13[2] * s13[2];
    double q23 = s23[0] * s23[0] + s23[1] * s23[1] + s23[2] * s23[2];
    double q12 = s12[0] * s12[0] + s12[1] * s12[1] + s12[2] * s12[2];
    double l13 = sqrt(q13), l23 = sqrt(q23), l12 = sqrt(q12);
    double angP = acos((q13 + q12 - q23) / (2.0 * l13 * l12));
    double ang2 = acos((q23 + q12 - q13) / (2.0 * l23 * l12));
    double e0[3], e1[3];
    for (int i = 0; i < 3; i++) e0[i] = s12[i] / l12;
    double dd = e0[0] * s13[0] + e0[1] * s13[1] + e0[2] * s13[2];
    for (int i = 0; i < 3; i++) e1[i] = s13[i] - dd * e0[i];
    double n1 = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    for (int i = 0; i < 3; i++) e1[i] /= n1;
    double sa2 = sin(ang2);
    Ops acc{};
    for (int i = 0; i < 5; i++) {
      double th = (angP + R.line_x[i] * angP) / 2.0;
      double sth, cth;
      sincos(th, &sth, &cth);
      double rmax = l12 * sa2 / sin(th + ang2);
      for (int j = 0; j < 5; j++) {
        double rs = (rmax + R.line_x[j] * rmax) / 2.0;
        double x = rs * cth, y = rs * sth;
        double qx = A1[0] + x * e0[0] + y * e1[0];
        double qy = A1[1] + x * e0[1] + y * e1[1];
        double qz = A1[2] + x * e0[2] + y * e1[2];
        double w = rmax / 2.0 * rs * R.line_w[i] * R.line_w[j];
        accumulate(acc, w, P.c[0], P.c[1], P.c[2], qx, qy, qz, P.nrm, Q.nrm, upNq, k);
      }
    }
    double f = angP / 2.0;
    o.L = cadd(o.L, cscale(f, acc.L));
    o.M = cadd(o.M, cscale(f, acc.M));
    o.Mt = cadd(o.Mt, cscale(f, acc.Mt));
    o.N = cadd(o.N, cscale(f, acc.N));
  }
  return o;
}

// Near-singular test |p_i - p_j| < 4 * averageTriangleDim (:851), evaluated
// without contraction so it classifies exactly like the host code.
__device__ __forceinline__ bool near_pair(const Elem& P, const Elem& Q, double near_r) {
  double dx = __dsub_rn(P.c[0], Q.c[0]), dy = __dsub_rn(P.c[1], Q.c[1]),
         dz = __dsub_rn(P.c[2], Q.c[2]);
  double s = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  return __dsqrt_rn(s) < near_r;
}

// Dispatch of BemOperatorsConst (:844-856).
__device__ __forceinline__ Ops ops_eval(const Elem* __restrict__ E, int64_t row, int64_t col,
                                        double k, double near_r, const QuadRules& R) {
  const Elem& P = E[row];
  const Elem& Q = E[col];
  if (row == col) return ops_singular(P, k, R);
  if (near_pair(P, Q, near_r)) return ops_nearsing(P, Q, k, R);
  return ops_regular(P, Q, k, R);
}

// ----- FP32 regular rule (mixed precision) -----
__host__ __device__ __forceinline__ float2 fmk(float r, float i) { return make_float2(r, i); }
__host__ __device__ __forceinline__ float2 fadd(float2 a, float2 b) { return fmk(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 fsub(float2 a, float2 b) { return fmk(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 fmul(float2 a, float2 b) {
  return fmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

struct OpsF {
  float2 L, M, Mt, N;
};

// c_p - c_q from the two-float centroids (see ElemF), all FP32
__device__ __forceinline__ void centroid_diff(const ElemF& P, const ElemF& Q, float& dx,
                                              float& dy, float& dz) {
  dx = (P.c_hi[0] - Q.c_hi[0]) + (P.c_lo[0] - Q.c_lo[0]);
  dy = (P.c_hi[1] - Q.c_hi[1]) + (P.c_lo[1] - Q.c_lo[1]);
  dz = (P.c_hi[2] - Q.c_hi[2]) + (P.c_lo[2] - Q.c_lo[2]);
}

// Same integrand and 16-point rule as ops_regular, evaluated in FP32. The
// centroid difference c_p - c_q keeps ~7 significant digits (two-float
// centroids); source points are offsets from c_q, so r = |p - q| keeps ~7
// significant digits even for neighbouring panels.
__device__ __forceinline__ OpsF ops_regular32_pq(const ElemF& P, const ElemF& Q, float k,
                                                 const QuadRules& R) {
  float dx, dy, dz;
  centroid_diff(P, Q, dx, dy, dz);
  const float npx = P.nrm[0], npy = P.nrm[1], npz = P.nrm[2];
  const float nqx = Q.nrm[0], nqy = Q.nrm[1], nqz = Q.nrm[2];
  const float upNq = npx * nqx + npy * nqy + npz * nqz;
  const float inv4pi = 0.0795774715459476679f;
  float Lx = 0, Ly = 0, Mx = 0, My = 0, Tx = 0, Ty = 0, Nx = 0, Ny = 0;
#pragma unroll 2
  for (int i = 0; i < 16; i++) {
    const float a1 = R.freg_x1[i], a2 = R.freg_x2[i], a3 = 1.0f - a2 - a1, w = R.freg_w[i];
    const float rx = dx - (a1 * Q.v[0] + a2 * Q.v[3] + a3 * Q.v[6]);
    const float ry = dy - (a1 * Q.v[1] + a2 * Q.v[4] + a3 * Q.v[7]);
    const float rz = dz - (a1 * Q.v[2] + a2 * Q.v[5] + a3 * Q.v[8]);
    const float rr = rx * rx + ry * ry + rz * rz;
    const float ir = rsqrtf(rr);
    const float r = rr * ir;
    const float rnq = -(rx * nqx + ry * nqy + rz * nqz) * ir;
    const float rnp = (rx * npx + ry * npy + rz * npz) * ir;
    const float kr = k * r;
    float s, c;
    sincosf(kr, &s, &c);
    const float g0 = ir * inv4pi;
    const float Gx = c * g0, Gy = s * g0;
    const float Grx = Gx * ir, Gry = Gy * ir;
    const float dGx = -Grx - kr * Gry, dGy = -Gry + kr * Grx;
    const float Grrx = Grx * ir, Grry = Gry * ir;
    const float a2c = 2.0f - kr * kr, b2c = -2.0f * kr;
    const float d2Gx = Grrx * a2c - Grry * b2c, d2Gy = Grrx * b2c + Grry * a2c;
    Lx += w * Gx;
    Ly += w * Gy;
    const float wm = w * rnq, wt = w * rnp;
    Mx += wm * dGx;
    My += wm * dGy;
    Tx += wt * dGx;
    Ty += wt * dGy;
    const float f1 = -(upNq + rnp * rnq) * ir, f2 = rnp * rnq;
    Nx += w * (f1 * dGx + f2 * d2Gx);
    Ny += w * (f1 * dGy + f2 * d2Gy);
  }
  const float A = Q.area;
  OpsF o;
  o.L = fmk(A * Lx, A * Ly);
  o.M = fmk(A * Mx, A * My);
  o.Mt = fmk(A * Tx, A * Ty);
  o.N = fmk(A * Nx, A * Ny);
  return o;
}

__device__ __forceinline__ OpsF ops_regular32(const ElemF* __restrict__ EF, int64_t row,
                                              int64_t col, float k, const QuadRules& R) {
  return ops_regular32_pq(EF[row], EF[col], k, R);
}

// Sums of operator sets: an entry with an impedance plane adds the operators
// of the column element reflected in the plane to its own (the substitution
// is affine in L, M, Mt, N and the reflected part has no jump terms).
__device__ __forceinline__ void ops_add(OpsF& a, const OpsF& b) {
  a.L = fadd(a.L, b.L);
  a.M = fadd(a.M, b.M);
  a.Mt = fadd(a.Mt, b.Mt);
  a.N = fadd(a.N, b.N);
}
__device__ __forceinline__ void ops_add(Ops& a, const Ops& b) {
  a.L = cadd(a.L, b.L);
  a.M = cadd(a.M, b.M);
  a.Mt = cadd(a.Mt, b.Mt);
  a.N = cadd(a.N, b.N);
}

// FP32 BC substitution for off-diagonal regular entries (no jump terms).
// The same FP32 integrand with any rule: points [b, e) of the tables x1, x2, w.
__device__ __forceinline__ OpsF ops_rule32_pts(const ElemF* __restrict__ EF, int64_t row,
                                               int64_t col, float k, int b, int e,
                                               const float* x1, const float* x2, const float* wt) {
  float dx, dy, dz;
  centroid_diff(EF[row], EF[col], dx, dy, dz);
  const ElemF& Q = EF[col];
  const float npx = EF[row].nrm[0], npy = EF[row].nrm[1], npz = EF[row].nrm[2];
  const float nqx = Q.nrm[0], nqy = Q.nrm[1], nqz = Q.nrm[2];
  const float upNq = npx * nqx + npy * nqy + npz * nqz;
  const float inv4pi = 0.0795774715459476679f;
  float Lx = 0, Ly = 0, Mx = 0, My = 0, Tx = 0, Ty = 0, Nx = 0, Ny = 0;
  for (int i = b; i < e; i++) {
    const float a1 = x1[i], a2 = x2[i], a3 = 1.0f - a2 - a1, w = wt[i];
    const float rx = dx - (a1 * Q.v[0] + a2 * Q.v[3] + a3 * Q.v[6]);
    const float ry = dy - (a1 * Q.v[1] + a2 * Q.v[4] + a3 * Q.v[7]);
    const float rz = dz - (a1 * Q.v[2] + a2 * Q.v[5] + a3 * Q.v[8]);
    const float rr = rx * rx + ry * ry + rz * rz;
    const float ir = rsqrtf(rr);
    const float r = rr * ir;
    const float rnq = -(rx * nqx + ry * nqy + rz * nqz) * ir;
    const float rnp = (rx * npx + ry * npy + rz * npz) * ir;
    const float kr = k * r;
    float s, c;
    sincosf(kr, &s, &c);
    const float g0 = ir * inv4pi;
    const float Gx = c * g0, Gy = s * g0;
    const float Grx = Gx * ir, Gry = Gy * ir;
    const float dGx = -Grx - kr * Gry, dGy = -Gry + kr * Grx;
    const float Grrx = Grx * ir, Grry = Gry * ir;
    const float a2c = 2.0f - kr * kr, b2c = -2.0f * kr;
    const float d2Gx = Grrx * a2c - Grry * b2c, d2Gy = Grrx * b2c + Grry * a2c;
    Lx += w * Gx;
    Ly += w * Gy;
    const float wm = w * rnq, wtt = w * rnp;
    Mx += wm * dGx;
    My += wm * dGy;
    Tx += wtt * dGx;
    Ty += wtt * dGy;
    const float f1 = -(upNq + rnp * rnq) * ir, f2 = rnp * rnq;
    Nx += w * (f1 * dGx + f2 * d2Gx);
    Ny += w * (f1 * dGy + f2 * d2Gy);
  }
  const float A = Q.area;
  OpsF o;
  o.L = fmk(A * Lx, A * Ly);
  o.M = fmk(A * Mx, A * My);
  o.Mt = fmk(A * Tx, A * Ty);
  o.N = fmk(A * Nx, A * Ny);
  return o;
}

// sin and cos of 2 pi x for x >= 0 (x in turns): the quarter turn q =
// rint(4 x) is split off exactly (x - q / 4 has no rounding, by Sterbenz'
// lemma), the rest t = 2 pi (x - q / 4) lies in [-pi/4, pi/4], where the
// Taylor series of sin to t^9 and of cos to t^8 are within 2.5e-8 of the
// functions, and the quadrant rotates (sin t, cos t) by q quarter turns.
// Maximum error 7.6e-8 (FP32 rounding of the result), relative accuracy near
// zero, no slow path for large arguments. The ACA entries need this: the
// hardware sin / cos (absolute error ~4e-7) moved the mixed solution of an
// ill-conditioned body by ~4e-6 at ACA 1e-6.
__device__ __forceinline__ void sincos_turns(float x, float& sn, float& cs) {
  const int iq = __float2int_rn(4.0f * x);
  const float t = 6.28318530717959f * fmaf(-0.25f, (float)iq, x);
  const float t2 = t * t;
  float ps = fmaf(t2, 2.75573192e-6f, -1.98412698e-4f);  // 1/9!, -1/7!
  ps = fmaf(t2, ps, 8.33333333e-3f);                    // 1/5!
  ps = fmaf(t2, ps, -0.166666667f);                     // -1/3!
  const float st = fmaf(t * t2, ps, t);
  float pc = fmaf(t2, 2.48015873e-5f, -1.38888889e-3f);  // 1/8!, -1/6!
  pc = fmaf(t2, pc, 4.16666667e-2f);                    // 1/4!
  pc = fmaf(t2, pc, -0.5f);                             // -1/2!
  const float ct = fmaf(t2, pc, 1.0f);
  const float a = (iq & 1) ? ct : st, b = (iq & 1) ? st : ct;
  sn = (iq & 2) ? -a : a;
  cs = ((iq ^ (iq >> 1)) & 1) ? -b : b;
}

// The same FP32 integrand over the points b, b + s, b + 2 s, .. < e of the
// tables x1, x2, wt: one lane's share when s lanes split an entry's rule (the
// operators are sums over the points, so the shares add up to the entry).
__device__ __forceinline__ OpsF ops_pts32(const ElemF& P, const ElemF& Q, float k,
                                          const float* x1, const float* x2, const float* wt,
                                          int b, int e, int s) {
  float dx, dy, dz;
  centroid_diff(P, Q, dx, dy, dz);
  const float npx = P.nrm[0], npy = P.nrm[1], npz = P.nrm[2];
  const float nqx = Q.nrm[0], nqy = Q.nrm[1], nqz = Q.nrm[2];
  const float upNq = npx * nqx + npy * nqy + npz * nqz;
  const float inv4pi = 0.0795774715459476679f;
  const float kc = k * 0.159154943091895336f;  // k / (2 pi)
  float Lx = 0, Ly = 0, Mx = 0, My = 0, Tx = 0, Ty = 0, Nx = 0, Ny = 0;
  for (int i = b; i < e; i += s) {
    const float a1 = x1[i], a2 = x2[i], a3 = 1.0f - a2 - a1, w = wt[i];
    const float rx = dx - (a1 * Q.v[0] + a2 * Q.v[3] + a3 * Q.v[6]);
    const float ry = dy - (a1 * Q.v[1] + a2 * Q.v[4] + a3 * Q.v[7]);
    const float rz = dz - (a1 * Q.v[2] + a2 * Q.v[5] + a3 * Q.v[8]);
    const float rr = rx * rx + ry * ry + rz * rz;
    const float ir = rsqrtf(rr);
    const float r = rr * ir;
    const float rnq = -(rx * nqx + ry * nqy + rz * nqz) * ir;
    const float rnp = (rx * npx + ry * npy + rz * npz) * ir;
    const float kr = k * r;
    float sn, cs;
    sincos_turns(kc * r, sn, cs);
    const float g0 = ir * inv4pi;
    const float Gx = cs * g0, Gy = sn * g0;
    const float Grx = Gx * ir, Gry = Gy * ir;
    const float dGx = -Grx - kr * Gry, dGy = -Gry + kr * Grx;
    const float Grrx = Grx * ir, Grry = Gry * ir;
    const float a2c = 2.0f - kr * kr, b2c = -2.0f * kr;
    const float d2Gx = Grrx * a2c - Grry * b2c, d2Gy = Grrx * b2c + Grry * a2c;
    Lx += w * Gx;
    Ly += w * Gy;
    const float wm = w * rnq, wtt = w * rnp;
    Mx += wm * dGx;
    My += wm * dGy;
    Tx += wtt * dGx;
    Ty += wtt * dGy;
    const float f1 = -(upNq + rnp * rnq) * ir, f2 = rnp * rnq;
    Nx += w * (f1 * dGx + f2 * d2Gx);
    Ny += w * (f1 * dGy + f2 * d2Gy);
  }
  const float A = Q.area;
  OpsF o;
  o.L = fmk(A * Lx, A * Ly);
  o.M = fmk(A * Mx, A * My);
  o.Mt = fmk(A * Tx, A * Ty);
  o.N = fmk(A * Nx, A * Ny);
  return o;
}

__device__ __forceinline__ void substitute32(const OpsF& o, const BcCoef& bc, float2 alpha,
                                             float2& phi, float2& dphi) {
  const float2 X = fadd(o.L, fmul(alpha, o.Mt));
  const float2 Y = fadd(o.M, fmul(alpha, o.N));
  if (bc.subst) {
    const float2 t = fmul(X, bc.finv_main);
    phi = fmk(-t.x, -t.y);
    const float2 u = fmul(bc.fratio, X);
    dphi = fmk(-u.x - Y.x, -u.y - Y.y);
  } else {
    phi = fmul(Y, bc.finv_main);
    dphi = fadd(X, fmul(bc.fratio, Y));
  }
}

// BC substitution of implicitPhiMatrix2 / implicitDPhiMatrix2 (:2004-2040).
// bc[col] holds a, b, b/a or a/b and the substitution flag.
__device__ __forceinline__ void substitute(const Ops& o, bool diag, const BcCoef& bc,
                                           double2 alpha, double2& phi, double2& dphi) {
  // X = L + alpha Mt + [diag] alpha/2 ; Y = M + alpha N - [diag] / 2
  double2 X = cadd(o.L, cmul(alpha, o.Mt));
  double2 Y = cadd(o.M, cmul(alpha, o.N));
  if (diag) {
    X = cadd(X, cscale(0.5, alpha));
    Y.x -= 0.5;
  }
  if (bc.subst) {  // |a| < |b|: unknown is phi
    phi = cscale(-1.0, cmul(X, bc.inv_main));            // -X / b
    dphi = csub(cscale(-1.0, cmul(bc.ratio, X)), Y);     // -(a/b) X - Y
  } else {           // unknown is dphi
    phi = cmul(Y, bc.inv_main);                          // Y / a
    dphi = cadd(X, cmul(bc.ratio, Y));                   // X + (b/a) Y
  }
}

}  // namespace bemgpu
