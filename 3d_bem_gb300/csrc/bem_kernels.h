// bem_kernels.h -- launch interfaces of the CUDA kernels (host <-> device).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bem_types.h"

namespace bemgpu {

constexpr int ACA_MAX_KCAP = 512;  // largest per-block rank reservation

// Seeded stand-in for the reference's QRandomGenerator picks
// (hmatrix.cpp:508, boundaryelementsolver.cpp:2156-2158): splitmix64 finaliser.
__host__ __device__ inline uint64_t pivot_hash(uint64_t seed, uint64_t a, uint64_t b) {
  uint64_t z = seed ^ (a * 0x9E3779B97F4A7C15ull) ^ (b * 0xC2B2AE3D27D4EB4Full);
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

#ifdef __CUDACC__
__device__ __forceinline__ double2 load_c(const double2* p) { return __ldg(p); }
__device__ __forceinline__ double2 load_c(const float2* p) {
  float2 v = __ldg(p);
  return make_double2((double)v.x, (double)v.y);
}
#endif

struct LeafRows {
  int64_t start;
  int32_t size;
  int32_t pad;
};

struct NearfieldArgs {
  int precision;  // 0: complex FP64 output, 1: complex FP32 output (FP32 regular rule)
  const Elem* E;
  const ElemF* EF;
  const BcCoef* bc;
  const NearBlock* blocks;
  const NearTile* tiles;
  int64_t ntiles;
  const uint32_t* special_bits;
  const int64_t* sp_entry;
  const int32_t* sp_row;
  const int32_t* sp_col;
  int64_t nspecial;
  double k;
  double2 alpha;
  void* phi;   // double2 or float2 per precision
  void* dphi;
  // impedance plane: the elements reflected in it (cluster order), null
  // without a plane; every entry adds the reflected element's operators
  const Elem* Er = nullptr;
  const ElemF* EFr = nullptr;
};

struct AcaArgs {
  int mode;       // 0 = BEM entries, 1 = point-cloud Helmholtz kernel (tests)
  int precision;  // 0: complex FP64, 1: complex FP32 storage + FP32 regular rule
  const Elem* E;
  const ElemF* EF;
  const BcCoef* bc;
  double k;
  double near_r;
  double2 alpha;
  float kf;        // FP32 copies for the mixed path
  float near_r2f;
  float2 alphaf;
  int which;  // 0 phi, 1 dphi
  const double* rowpts;
  const double* colpts;
  const FarBlock* far;
  const int32_t* order;
  int64_t nfar;
  void* U;
  void* V;
  void* S;
  int32_t* rank;
  int32_t* flags;
  double tol;
  int max_rank;
  uint64_t seed;
  int extra;
  const int64_t* piv_off;
  const int32_t* piv_cnt;
  const int32_t* piv_rc;
  // learned rule table of the FP32 regular entries (null: the 16-point rule):
  // class (1/3/7/13/25 points) by x = log(d / e_max), y = log(k e_max) bins
  const uint8_t* rule_tab;
  float tab_x0, tab_dx, tab_y0, tab_dy;
  // impedance plane (mode 0 only): reflected elements, null without a plane
  const Elem* Er;
  const ElemF* EFr;
};

constexpr int ACA_TAB_N = 12;  // rule-table bins per axis

// Optional skip of a launch's work: when every flag f[i * stride] (i < n) is
// nonzero the kernels take an empty work range (an early return instead made
// the FP32 H-matvec ~19 % slower even when open, through its register
// allocation). GMRES gates the operator products of its
// Arnoldi steps with the right-hand sides' converged flags, so the steps it
// runs past convergence (it checks on the host every few steps) cost no work.
struct HmvGate {
  const int* f;
  int stride, n;
};
#ifdef __CUDACC__
__device__ __forceinline__ bool gate_closed(const HmvGate& g) {
  if (!g.f) return false;
  for (int i = 0; i < g.n; i++)
    if (!g.f[(int64_t)i * g.stride]) return false;
  return true;
}
#endif

struct HmvArgs {
  int precision;  // 0: double2 storage, 1: float2 storage
  int fp32_math;  // float2 storage only: 0 FP64 arithmetic, 1 FP32 products with
                  // compensated FP32 sums, 2 two-float (FP64-accurate) on FP32 units
  int nrhs;
  const FarBlock* far;
  const int32_t* rank;
  int64_t nfar;
  const NearBlock* nearb;
  const LeafRows* leaves;
  int64_t nleaves;
  const int32_t* list_off;
  const int32_t* list;
  const void* U;
  const void* V;
  const void* S;
  const void* F;
  const double2* x;
  int64_t ldx;
  double2* t;
  int64_t ldt;
  double2* y;
  int64_t ldy;
  int accumulate;
  float2* xf;  // FP32 scratch copies of x (ldx x nrhs) and t (ldt x nrhs)
  float2* tf;  // for the FP32-arithmetic variant
  // optional pass-V work list: items (far block, first row), 16 rows each,
  // built from the block ranks; null = one CTA per far block
  const int2* vwork;
  int64_t nvwork;
  HmvGate gate;  // null f: always run
  // two-float products only: remainders of the near-field entries (F + Flo
  // = the FP64 entries), null when the pool holds FP32-computed entries
  const void* Flo = nullptr;
};

void nearfield_upload_rules(const QuadRules& r, cudaStream_t s);
// hi = (float) v, lo = (float) (v - hi) for n complex values
void launch_split_twofloat(const double2* v, float2* hi, float2* lo, int64_t n, cudaStream_t s);
void aca_upload_rules(const QuadRules& r, cudaStream_t s);
void launch_nearfield(const NearfieldArgs& a, cudaStream_t s);
void launch_operators(const Elem* E, const int64_t* rows, const int64_t* cols, int64_t count,
                      double k, double near_r, double2* out, cudaStream_t s);
void launch_points_nearfield(const NearBlock* blocks, int64_t nblocks, const NearTile* tiles,
                             int64_t ntiles, const double* rp, const double* cp, double k,
                             double2* F, cudaStream_t s);
int launch_aca(const AcaArgs& a, int threads, cudaStream_t s);
constexpr int ACA_BIG_MN = 512;  // blocks with m + n >= this get 512-thread CTAs
int launch_hmatvec(const HmvArgs& a, cudaStream_t s);  // returns kernels launched

// Fixed device scratch of the allocation-free H-matvec (complex FP64 entries,
// 32 MiB): holds ldt x nrhs projections of one pass.
constexpr int64_t HMV_NOALLOC_SCRATCH = int64_t(1) << 21;
int64_t hmatvec_noalloc_capacity();
cudaError_t hmatvec_noalloc_scratch(double2** out);

}  // namespace bemgpu
