// nearfield.cu -- K1/K2: dense near-field blocks of both BC-substituted
// matrices (phi = right-hand-side operator, dPhi = system operator) from one
// operator evaluation per entry.
//
// The reference fills every inadmissible leaf entry by entry and evaluates the
// operators twice, once per matrix (BlockCluster::fullRankAssembly,
// HMatrix/hmatrix.cpp:350-374, called from assembleBlocks / assembleBlocksExtra
// :793-846 with implicitPhiMatrix2 / implicitDPhiMatrix2,
// boundaryelementsolver.cpp:2004-2040). Here one thread owns one entry and
// writes both matrices. Regular pairs (16-point rule) and special pairs
// (i == j singular rule, near-singular split-polar rule) run in separate
// kernels so every warp follows one rule.
#include <mutex>
#include <set>

#include "bem_kernels.h"
#include "quadrature.cuh"

namespace bemgpu {

static __constant__ QuadRules c_rules;

// The tables (always the same) go to each device's constant memory once,
// synchronously, so no later handle rewrites them under running kernels.
void nearfield_upload_rules(const QuadRules& r, cudaStream_t s) {
  (void)s;
  static std::mutex mu;
  static std::set<int> done;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  if (done.count(dev)) return;
  if (cudaMemcpyToSymbol(c_rules, &r, sizeof(QuadRules)) == cudaSuccess) done.insert(dev);
}

__device__ __forceinline__ void store(double2* p, int64_t g, double2 v) { p[g] = v; }
__device__ __forceinline__ void store(float2* p, int64_t g, double2 v) {
  p[g] = make_float2((float)v.x, (float)v.y);
}

// Regular entries of all near-field blocks; entries the host classified as
// special (flag bit set) are left to nearfield_special.
__global__ void __launch_bounds__(256) nearfield_regular_kernel(
    const Elem* __restrict__ E, const BcCoef* __restrict__ bc,
    const NearBlock* __restrict__ blocks, const NearTile* __restrict__ tiles,
    const uint32_t* __restrict__ special_bits, double k, double2 alpha,
    double2* __restrict__ phi, double2* __restrict__ dphi, const Elem* __restrict__ Er) {
  const NearTile t = tiles[blockIdx.x];
  if ((int)threadIdx.x >= t.count) return;
  const NearBlock b = blocks[t.block];
  const int e = t.first + threadIdx.x;
  const int64_t g = b.off + e;
  if (special_bits[g >> 5] & (1u << (g & 31))) return;
  const int r = e % b.m, c = e / b.m;
  const int64_t row = b.r0 + r, col = b.c0 + c;
  Ops o = ops_regular(E[row], E[col], k, c_rules);
  if (Er) ops_add(o, ops_regular(E[row], Er[col], k, c_rules));
  double2 p, d;
  substitute(o, false, bc[col], alpha, p, d);
  phi[g] = p;
  dphi[g] = d;
}

// Mixed precision: the same entries with the FP32 regular rule, stored as
// complex FP32.
__global__ void __launch_bounds__(256) nearfield_regular32_kernel(
    const Elem* __restrict__ E, const ElemF* __restrict__ EF, const BcCoef* __restrict__ bc,
    const NearBlock* __restrict__ blocks, const NearTile* __restrict__ tiles,
    const uint32_t* __restrict__ special_bits, float k, float2 alpha, float2* __restrict__ phi,
    float2* __restrict__ dphi, const ElemF* __restrict__ EFr) {
  const NearTile t = tiles[blockIdx.x];
  if ((int)threadIdx.x >= t.count) return;
  const NearBlock b = blocks[t.block];
  const int e = t.first + threadIdx.x;
  const int64_t g = b.off + e;
  if (special_bits[g >> 5] & (1u << (g & 31))) return;
  const int r = e % b.m, c = e / b.m;
  const int64_t row = b.r0 + r, col = b.c0 + c;
  OpsF o = ops_regular32(EF, row, col, k, c_rules);
  if (EFr) ops_add(o, ops_regular32_pq(EF[row], EFr[col], k, c_rules));
  float2 p, d;
  substitute32(o, bc[col], alpha, p, d);
  phi[g] = p;
  dphi[g] = d;
}

// Special entries: (global entry index, row, col) triples sorted so that the
// singular (row == col) ones come first. Always FP64 arithmetic.
template <typename T>
__global__ void __launch_bounds__(128) nearfield_special_kernel(
    const Elem* __restrict__ E, const BcCoef* __restrict__ bc,
    const int64_t* __restrict__ sp_entry, const int32_t* __restrict__ sp_row,
    const int32_t* __restrict__ sp_col, int64_t count, double k, double2 alpha,
    T* __restrict__ phi, T* __restrict__ dphi, const Elem* __restrict__ Er) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int64_t row = sp_row[i], col = sp_col[i];
  Ops o = (row == col) ? ops_singular(E[row], k, c_rules)
                       : ops_nearsing(E[row], E[col], k, c_rules);
  // the reflected element always takes the regular rule (BemOperatorsReflected,
  // boundaryelementsolver.cpp:1516-1554)
  if (Er) ops_add(o, ops_regular(E[row], Er[col], k, c_rules));
  double2 p, d;
  substitute(o, row == col, bc[col], alpha, p, d);
  const int64_t g = sp_entry[i];
  store(phi, g, p);
  store(dphi, g, d);
}

// Raw operators L, M, Mt, N for arbitrary pairs (reference BemOperatorsConst,
// boundaryelementsolver.cpp:844-894), used by bem_operators().
__global__ void operators_kernel(const Elem* __restrict__ E, const int64_t* __restrict__ rows,
                                 const int64_t* __restrict__ cols, int64_t count, double k,
                                 double near_r, double2* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int64_t row = rows[i], col = cols[i];
  Ops o;
  if (row == col) o = ops_singular(E[row], k, c_rules);
  else if (near_pair(E[row], E[col], near_r)) o = ops_nearsing(E[row], E[col], k, c_rules);
  else o = ops_regular(E[row], E[col], k, c_rules);
  out[4 * i + 0] = o.L;
  out[4 * i + 1] = o.M;
  out[4 * i + 2] = o.Mt;
  out[4 * i + 3] = o.N;
}

// Dense blocks of the point-cloud test kernel exp(ikr)/(4 pi r), 1 at r = 0
// (Tests/tests.h:30-42).
__global__ void __launch_bounds__(256) points_nearfield_kernel(
    const NearBlock* __restrict__ blocks, const NearTile* __restrict__ tiles,
    const double* __restrict__ rp, const double* __restrict__ cp, double k,
    double2* __restrict__ F) {
  const NearTile t = tiles[blockIdx.x];
  if ((int)threadIdx.x >= t.count) return;
  const NearBlock b = blocks[t.block];
  const int e = t.first + threadIdx.x;
  const int r = e % b.m, c = e / b.m;
  const double* x = rp + 3 * (b.r0 + r);
  const double* y = cp + 3 * (b.c0 + c);
  double dx = x[0] - y[0], dy = x[1] - y[1], dz = x[2] - y[2];
  double d = sqrt(dx * dx + dy * dy + dz * dz);
  double2 v = make_double2(1.0, 0.0);
  if (d != 0.0) {
    double sn, cs;
    sincos(k * d, &sn, &cs);
    double g = 1.0 / (4.0 * 3.14159265358979323846 * d);
    v = make_double2(cs * g, sn * g);
  }
  F[b.off + e] = v;
}

void launch_points_nearfield(const NearBlock* blocks, int64_t nblocks, const NearTile* tiles,
                             int64_t ntiles, const double* rp, const double* cp, double k,
                             double2* F, cudaStream_t s) {
  (void)nblocks;
  if (ntiles > 0) points_nearfield_kernel<<<(unsigned)ntiles, 256, 0, s>>>(blocks, tiles, rp, cp, k, F);
}

namespace {
__global__ void split_twofloat_kernel(const double2* __restrict__ v, float2* __restrict__ hi,
                                      float2* __restrict__ lo, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 x = v[i];
  const float rh = (float)x.x, ih = (float)x.y;
  hi[i] = make_float2(rh, ih);
  lo[i] = make_float2((float)(x.x - (double)rh), (float)(x.y - (double)ih));
}
}  // namespace

void launch_split_twofloat(const double2* v, float2* hi, float2* lo, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  split_twofloat_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(v, hi, lo, n);
}

void launch_nearfield(const NearfieldArgs& a, cudaStream_t s) {
  const unsigned g = (unsigned)((a.nspecial + 127) / 128);
  if (a.precision == 0) {
    if (a.ntiles > 0)
      nearfield_regular_kernel<<<(unsigned)a.ntiles, 256, 0, s>>>(
          a.E, a.bc, a.blocks, a.tiles, a.special_bits, a.k, a.alpha, (double2*)a.phi,
          (double2*)a.dphi, a.Er);
    if (a.nspecial > 0)
      nearfield_special_kernel<double2><<<g, 128, 0, s>>>(a.E, a.bc, a.sp_entry, a.sp_row,
                                                          a.sp_col, a.nspecial, a.k, a.alpha,
                                                          (double2*)a.phi, (double2*)a.dphi,
                                                          a.Er);
  } else {
    if (a.ntiles > 0)
      nearfield_regular32_kernel<<<(unsigned)a.ntiles, 256, 0, s>>>(
          a.E, a.EF, a.bc, a.blocks, a.tiles, a.special_bits, (float)a.k,
          make_float2((float)a.alpha.x, (float)a.alpha.y), (float2*)a.phi, (float2*)a.dphi,
          a.EFr);
    if (a.nspecial > 0)
      nearfield_special_kernel<float2><<<g, 128, 0, s>>>(a.E, a.bc, a.sp_entry, a.sp_row,
                                                         a.sp_col, a.nspecial, a.k, a.alpha,
                                                         (float2*)a.phi, (float2*)a.dphi, a.Er);
  }
}

void launch_operators(const Elem* E, const int64_t* rows, const int64_t* cols, int64_t count,
                      double k, double near_r, double2* out, cudaStream_t s) {
  if (count <= 0) return;
  operators_kernel<<<(unsigned)((count + 127) / 128), 128, 0, s>>>(E, rows, cols, count, k,
                                                                   near_r, out);
}

}  // namespace bemgpu
