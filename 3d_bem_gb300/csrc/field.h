// field.h -- launch interface of the field-evaluation kernels (field.cu):
// velocity potential at observation points from a boundary solution,
// phi(p) = sum_sources + sum_j (Mk_j phi_j - Lk_j dphi_j), Mk and Lk by the
// 7-point triangle rule of order 5 (BoundaryElementSolver::BemOperatorField,
// boundaryelementsolver.cpp:2318-2353).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bem_types.h"

namespace bemgpu {

// FP32 element record of the mixed-precision field kernel (160 bytes):
// centroid as two floats (c_hi + c_lo), the 7 rule points as offsets o_i from
// the centroid, unit normal n, and n . o_i (so (p - q_i) . n costs one
// subtraction per rule point).
struct __align__(16) FieldElemF {
  float c_hi[3], c_lo[3];
  float q[21];
  float nrm[3];
  float qn[7];
  float pad[3];
};
static_assert(sizeof(FieldElemF) == 160, "FieldElemF is ten 16-byte pieces");

// Coefficients of one element and right-hand side: a = A phi, b = A dphi
// (A the element area), complex.
struct FieldCoefF {
  float2 a, b;
};
struct FieldCoef {
  double2 a, b;
};

constexpr int FIELD_PTS = 256;  // observation points (threads) per CTA
constexpr int FIELD_TILE = 128; // elements per shared-memory tile
constexpr int FIELD_RB = 4;     // right-hand sides per pass

// Element records (precision 1 only) and the coefficients of R columns:
// phi, dphi are N x R complex FP64 in the caller's order, perm[j] the caller
// index of cluster-order element j. coef: R x N FieldCoefF (precision 1) or
// FieldCoef (precision 0). R = 0: the records only (perm, phi, dphi, coef
// unused).
int launch_field_prep(const Elem* E, const int64_t* perm, int64_t N, const double2* phi,
                      const double2* dphi, int R, int precision, FieldElemF* fe, void* coef,
                      cudaStream_t s);

// Partial sums over S element chunks: partial[(s R + r) M + i] for the M
// points pts (M x 3, FP64) and all R columns. k is the wavenumber.
int launch_field_sum(const Elem* E, const FieldElemF* fe, const void* coef, int64_t N, int R,
                     const double* pts, int64_t M, double k, int precision, int S,
                     double2* partial, cudaStream_t s);

// phi_f = sum over the S partials + point sources (src: nsrc x 5 doubles x, y,
// z, Re w, Im w; sourcePhiTerm, boundaryelementsolver.cpp:3443-3450), added to
// every column; p_f = pfac phi_f. phi_f, p_f (M x R complex) may be null.
int launch_field_finish(const double2* partial, int S, int64_t M, int R, const double* pts,
                        const double* src, int nsrc, double k, double2 pfac, double2* phi_f,
                        double2* p_f, cudaStream_t s);

}  // namespace bemgpu
