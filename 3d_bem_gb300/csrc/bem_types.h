// bem_types.h -- plain data shared by the host runtime and the kernels.
#pragma once
#include <stdint.h>
#ifdef __CUDACC__
#include <cuda_runtime.h>
#else
#include <vector_types.h>
#endif

namespace bemgpu {

// One boundary element in cluster order: nodes, unit normal, collocation
// point (centroid) and area -- 16 doubles, one 128-byte line.
struct __align__(16) Elem {
  double n1[3], n2[3], n3[3];
  double nrm[3];
  double c[3];
  double area;
};

// FP32 companion of Elem for the mixed-precision rules: vertices relative to
// the element's own centroid (small numbers, so FP32 keeps ~7 digits of the
// local geometry), unit normal, area, and the centroid as an unevaluated sum
// c = c_hi + c_lo of two floats. The pair difference
// (c_hi,i - c_hi,j) + (c_lo,i - c_lo,j) is then accurate to ~1e-7 relative
// without any FP64 instruction (GB300's FP64 rate is 1/64 of FP32).
struct __align__(16) ElemF {
  float v[9];    // node1 - c, node2 - c, node3 - c
  float nrm[3];
  float area;
  float c_hi[3];
  float c_lo[3];
  float emax;    // longest edge (rule-table lookup of ACA entries)
};

// Rule tables: 16-point triangle rule (order 8), 5-point Gauss-Legendre
// (near-singular rule), positive half of the 32-point Gauss-Legendre rule
// (singular rule). Values: trianglequadraturerules.cpp:91-110,
// linequadraturerules.cpp:61-76 and :77-120 of the reference.
struct QuadRules {
  double reg_x1[16], reg_x2[16], reg_w[16];
  double line_x[5], line_w[5];
  double gl_x[16], gl_w[16];
  float freg_x1[16], freg_x2[16], freg_w[16];
};

// Per-column Robin data after the substitution rule |a| < |b|
// (boundaryelementsolver.cpp:3423): when subst, inv_main = 1/b and
// ratio = a/b; otherwise inv_main = 1/a and ratio = b/a.
struct BcCoef {
  double2 inv_main;
  double2 ratio;
  int subst;
  int pad;
  float2 finv_main;  // FP32 copies for the mixed-precision kernels
  float2 fratio;
};

// Dense near-field block (column-major m x n at data offset `off`, complex).
struct NearBlock {
  int64_t r0, c0, off;
  int32_t m, n;
};

// Admissible block stored as U (m x kcap, column-major), s (kcap) and
// V (kcap x n, row-major): block = U diag(s) V. `rank` is written by the ACA
// kernel.
struct FarBlock {
  int64_t r0, c0;
  int64_t uoff, voff, soff;  // complex-element offsets into the U / V / s pools
  int32_t m, n;
  int32_t kcap;        // reserved rank
  int32_t id;          // index in the reference partition order
};

// Tile of consecutive entries of one near-field block (column-major order).
struct NearTile {
  int32_t block;
  int32_t first;
  int32_t count;
  int32_t pad;
};

}  // namespace bemgpu
