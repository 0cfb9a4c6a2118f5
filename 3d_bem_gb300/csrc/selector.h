// selector.h -- learned quadrature-order selector: pair features, labels at
// escalating orders, the MLP's training kernels, BF16 tensor-core inference
// and the near-field kernel that integrates each pair with its selected rule.
//
// The reference integrates every regular pair with one fixed 16-point rule
// (boundaryelementsolver.cpp:857-893); the selector picks per pair the
// cheapest of the 1, 3, 7, 13, 25-point rules of the same family
// (trianglequadraturerules.cpp orders 1, 2, 5, 7, 10).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bem_types.h"

namespace bemgpu {

constexpr int SEL_NF = 24;       // features per pair
constexpr int SEL_H = 64;        // hidden width (two layers)
constexpr int SEL_C = 5;         // classes: 1, 3, 7, 13, 25 points
constexpr int SEL_NPARAM = SEL_NF * SEL_H + SEL_H + SEL_H * SEL_H + SEL_H + SEL_H * SEL_C + SEL_C;
constexpr int SEL_RULES = 7;     // the 5 classes, the plain 16-point rule, the 64-point reference
constexpr int SEL_PLAIN = 5;
constexpr int SEL_REF = 6;

// Offsets of the flat FP32 parameter vector: W1 (24 x 64, row-major: input i
// to hidden j at i * 64 + j), b1, W2 (64 x 64), b2, W3 (64 x 5), b3.
constexpr int SEL_OW1 = 0;
constexpr int SEL_OB1 = SEL_OW1 + SEL_NF * SEL_H;
constexpr int SEL_OW2 = SEL_OB1 + SEL_H;
constexpr int SEL_OB2 = SEL_OW2 + SEL_H * SEL_H;
constexpr int SEL_OW3 = SEL_OB2 + SEL_H;
constexpr int SEL_OB3 = SEL_OW3 + SEL_H * SEL_C;

// Device image of a trained selector in the layout the inference kernel
// stages into shared memory: transposed BF16 weights (output-major, inputs
// padded: 32 for layer 1, 64 for layers 2-3, 8 outputs for layer 3), FP32
// biases (padded logits get -1e30) and the feature normalisation.
struct SelBlob {
  uint16_t w1t[SEL_H * 32];
  uint16_t w2t[SEL_H * SEL_H];
  uint16_t w3t[8 * SEL_H];
  float b1[SEL_H], b2[SEL_H], b3[8];
  float mu[SEL_NF], inv_sigma[SEL_NF];
};

// FP32 training work area per sample: H1, H2, D1, D2 (64 each), P/D3 (8), loss (1)
constexpr int SEL_WORK_PER_SAMPLE = 4 * SEL_H + 8 + 1;

// Host-built rule tables (classes 0-4, plain 16-point, 64-point reference).
void sel_upload_rules(cudaStream_t s);

// Labels: per pair (P, Q elements, wavenumber k) the features, the cheapest
// class whose rule reaches relative error tol against the reference (the
// 64-point rule on a subdivision of Q, or the split-polar near-singular rule
// when the centroid distance is below near_ratio * sqrt(area_Q)); 5 when
// none does. The error of an operator is relative to max(|ref|, floor_rel
// times the pair's largest operator). err (may be null): npairs x 6 relative
// errors of the 5 classes and the plain 16-point rule.
void launch_sel_label(const Elem* P, const Elem* Q, const double* k, int64_t n, double tol,
                      double near_ratio, double floor_rel, float* feat, uint8_t* label,
                      float* err, cudaStream_t s);

// FP32 training: forward + softmax cross-entropy, backward, parameter
// gradients (deterministic: one thread per parameter, samples in order) and
// the mean loss. work: B * SEL_WORK_PER_SAMPLE floats.
void launch_mlp_grad(const float* params, const float* X, const uint8_t* y, int64_t B,
                     float* grad, float* loss, float* work, cudaStream_t s);
void launch_mlp_adam(float* params, const float* grad, float* m, float* v, int64_t step,
                     float lr, float b1, float b2, float eps, cudaStream_t s);
void launch_mlp_forward(const float* params, const float* X, int64_t B, float* logits,
                        cudaStream_t s);

// BF16 tensor-core inference over arbitrary feature rows (raw features):
// logits (B x 8, padded) and classes.
void launch_sel_infer_rows(const SelBlob* blob, const float* feat, int64_t B, float* logits,
                           uint8_t* cls, cudaStream_t s);

// Near-field classes for a mesh: per regular near-field entry the selected
// class (low-confidence pairs, top softmax probability below guard_prob, get
// the highest order). Special entries are left untouched.
struct SelNearArgs {
  const SelBlob* blob;
  const ElemF* EF;  // features in FP32 from the mixed-precision element copies
  const NearBlock* blocks;
  const NearTile* tiles;
  int64_t ntiles;
  const uint32_t* special_bits;
  double k;
  float guard_prob;
  uint8_t* cls;  // per near-field entry
};
void launch_sel_near_classes(const SelNearArgs& a, cudaStream_t s);

// Mixed-precision regular near-field entries with the selected rules. Every
// check_every-th entry (by hash) whose class is below the highest is also
// integrated with the highest order; if the two differ by more than
// check_tol (relative), the entry keeps the highest-order value.
// counters: [0] points used, [1] checked, [2] fell back.
struct SelNearfieldArgs {
  const ElemF* EF;
  const BcCoef* bc;
  const NearBlock* blocks;
  const NearTile* tiles;
  int64_t ntiles;
  const uint32_t* special_bits;
  const uint8_t* cls;
  float k;
  float2 alpha;
  float2 *phi, *dphi;
  int check_every;
  float check_tol;
  unsigned long long* counters;
};
void launch_sel_nearfield32(const SelNearfieldArgs& a, cudaStream_t s);

// FP32 copies of the class rules (1, 3, 7, 13, 25 points, in this order,
// 49 points) and their offsets (off[5] = 49), for other kernels' tables.
constexpr int SEL_CLASS_POINTS = 49;
void sel_class_rule_tables(float* x1, float* x2, float* w, int* off);

// Convert flat FP32 parameters + normalisation into the device blob layout.
void sel_make_blob(const float* params, const float* mu, const float* sigma, SelBlob& out);

}  // namespace bemgpu
