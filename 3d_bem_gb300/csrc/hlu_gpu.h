// hlu_gpu.h -- H-LU factorization on the GPU: a task program built once per
// mesh on the host (symbolic factorization) and executed per frequency by one
// persistent dataflow kernel.
//
// The recursion is the reference's HArithm::LUDecomposition
// (HMatrix/harithm.cpp:1192-1296) with QR diagonal leaves, forwSubsMatVal /
// forwSubsMatValTransposed for the off-diagonal blocks (:1450-1595) and
// truncated H-matrix products for the Schur complement (hmultiply.cpp:138-197,
// recursiveHMatSubstraction harithm.cpp:1915-2005). With every low-rank block
// held at exactly the preconditioner rank kc (columns beyond the truncation's
// rank are zero) the shape of every intermediate is independent of the
// matrix entries, so the whole factorization unrolls into a fixed list of
// small dense tasks over one device arena:
//
//   GEMM   C (+)= alpha op(A) op(B)            (products with leaves, panels)
//   LMUL   X := op(M) X, M <= 64 x 64          (Q^H and R^{-T} of a diagonal leaf)
//   RMUL   X := X op(M)                        (R^{-1} from the right)
//   QR     diagonal leaf -> Q, R, Q^H, R^{-1}  (the sweep kernels' apply matrices)
//   TRUNC  [A_1 .. A_p] [B_1 .. B_p]^T -> rank kc (Householder QR of both
//          sides, one-sided Jacobi SVD of the core, the rule of
//          GoloubReinschSvd::minRankforError, golubReinschSVD.cpp:551-585)
//   COPY   C (+)= alpha op(A) (loads of the near-field blocks)
//   ZERO   C := 0
//
// Each task lists the tasks whose results it reads or whose inputs it
// overwrites (read-after-write, write-after-write and write-after-read on the
// row segments of every buffer, one segment per leaf cluster). Tasks are
// numbered in a topological order; the kernel's CTAs claim them in that order
// and wait (bounded) on the done flags of their dependencies.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "hlu.h"
#include "hlu_solve.h"
#include "host_tree.h"

namespace bemgpu {

enum HluTaskType : int32_t {
  HT_GEMM = 0,
  HT_LMUL = 1,
  HT_RMUL = 2,
  HT_QR = 3,
  HT_TRUNC = 4,
  HT_COPY = 5,
  HT_ZERO = 6,
};

// operand transforms (2 bits each)
constexpr int HOP_N = 0, HOP_T = 1, HOP_C = 2;
// flags: bits 0-1 op(A) (LMUL / RMUL: op(M)), bits 2-3 op(B), bit 4 accumulate
// into C, bit 5 negate the product, bits 8-10 source pool of A (COPY):
// 0 arena, 1 near-field pool F
constexpr int HF_ACC = 16, HF_NEG = 32;
constexpr int HF_SRC_SHIFT = 8;

// A truncation's scratch: A and B gathered (m x kt, n x kt), then either the
// QR path's reflector heads, singular values, core and Jacobi rotations, or
// the range finder's panels (m x L and n x L twice, kt x L, L x L; L <= 14).
inline int64_t trunc_scratch(int64_t m, int64_t n, int64_t kt) {
  const int64_t k2 = kt > 32 ? kt : 32, L = 14;
  const int64_t qr = 3 * k2 + 2 * kt * kt;
  const int64_t rng = 2 * (m + n) * L + kt * L + L * L + 2 * L;
  return (m + n) * kt + (qr > rng ? qr : rng) + 64;
}
// truncations up to this many complex elements of scratch use their CTA's slot
constexpr int64_t HLU_CTA_SCRATCH = int64_t(1) << 16;
// complex elements of the executor's dynamic shared memory per CTA
constexpr int64_t HLU_SMEM_ELEMS = 6144;
// subspace truncation (rank <= 2, no tolerance): basis width and the shared
// memory of its buffers (Q m x 8, Z n x 8, T kt x 8, V and R 8 x 8, 8 values)
constexpr int HLU_SUB_L = 8;
#ifdef __CUDACC__
__host__ __device__
#endif
inline int64_t hlu_sub_buffers(int64_t m, int64_t n, int64_t kt) {
  return (m + n + kt) * HLU_SUB_L + 2 * HLU_SUB_L * HLU_SUB_L + HLU_SUB_L;
}

struct HluTask {
  int32_t type, flags;
  int32_t m, n, q;     // GEMM: C m x n, inner q; LMUL: X m x n (M m x m);
                       // RMUL: X m x n (M n x n); QR: m; TRUNC: target m x n,
                       // q = static column bound; COPY / ZERO: m x n
  int32_t x0, x1;      // TRUNC: first input pair, pair count; QR: output slot
  int32_t lda, ldb, ldc;
  int64_t a, b, c;     // arena offsets (elements); TRUNC: c = A' (m x kc), b = B',
                       // a = offset of its own scratch region, -1: the CTA's slot
};

// One column block of a truncation: the A-side piece (rows ra .. ra + ma of
// A', others zero) and the B-side piece (rows rb .. rb + mb of B') with the
// same columns. Element (r, l) of a piece = src[off + r * rs + l * cs]
// (kind 0, arena), the identity (kind 1), or, for the loads of the assembled
// ACA blocks, U (kind 2: U pool, column-major, column l scaled by
// S[soff + l]) / V^T (kind 3: V pool, row-major) with the block's current ACA
// rank as the column count.
struct HluTruncPair {
  int64_t aoff, boff;       // kind 2: uoff / soff packed as aoff = uoff, boff = voff
  int64_t soff;             // kind 2 / 3: S pool offset
  int32_t ars, acs, brs, bcs;  // strides of the A / B pieces (kind 0)
  int32_t ra, ma, rb, mb;   // placements
  int32_t cols;             // columns (static); kinds 2 / 3: the reservation
  int32_t akind, bkind;     // 0 strided (arena), 1 identity, 2 U pool * S, 3 V pool^T
  int32_t neg;              // bit 0: negate the A piece, bit 1: the B piece
  int32_t rank_idx;         // kinds 2 / 3: far-block index of the runtime rank
  int32_t pad;
};

// Where the QR task of a diagonal leaf puts its results.
struct HluQrOut {
  int64_t q, r;          // arena: Q (L leaf data), R (U leaf data), m x m column-major
  int64_t qh, rinv;      // arena: Q^H and R^{-1}, row-major (the sweep apply matrices)
};

struct HluProgram {
  std::vector<HluTask> tasks;
  std::vector<int32_t> dep_off, deps;  // CSR, topological: deps[i] < i
  std::vector<int32_t> succ_off, succ;  // the reverse CSR (successors), ascending
  std::vector<int32_t> queue_init;     // ready queue at launch: tasks without
                                       // dependencies, then -1
  int32_t nready0 = 0;                 // their count
  std::vector<HluTruncPair> pairs;
  std::vector<HluQrOut> qr;
  int64_t arena = 0;                   // complex elements
  int64_t scratch = 0;                 // per-CTA TRUNC scratch (complex elements)
  int64_t big_scratch = 0;             // regions of the large truncations (task.a)
  int32_t kc = 0;                      // rank of every low-rank block
  int32_t max_kt = 0;                  // largest truncation width
  FlatFactor L, U;                     // leaf lists with arena offsets (data empty)
  int64_t qh_base = 0, rinv_base = 0;  // apply matrices of the sweeps (arena offsets)
  bool df_ok = false;                  // the dataflow sweeps apply (else sequential)
  std::string df_why;
  // statistics of the program
  int64_t levels = 0;                  // longest dependency chain (tasks)
  double cost_path = 0, cost_total = 0;  // model cost of the critical path / all tasks
  int64_t counts[8] = {};              // tasks per type
  int64_t path_counts[8] = {};         // tasks per type on the critical path
};

// Builds the program for the partition of `tree` (blocks in minPartition
// order, near / far index tables as laid out for the pools). kc in [1, 64].
// Returns false with the reason when the partition does not have the
// structure the program needs (e.g. a low-rank diagonal block).
bool hlu_gpu_plan(const HTree& tree, const Layout& L, int64_t kc, HluProgram& P,
                  std::string* why);

// The dataflow sweeps' plan without the apply matrices (those are written by
// the QR tasks at the offsets `moff` of the plan); false as hlu_df_plan.
bool hlu_df_plan_structure(const FlatFactor& f, int64_t N, int elem_bytes, HluDfPlan& p,
                           std::string* why);

struct HluExecArgs {
  int precision;                 // 0 complex FP64, 1 complex FP32 (FP32 arithmetic)
  void* arena;
  const void *F, *U, *V, *S;     // the system matrix's pools (storage precision)
  const int32_t* rank;           // its ACA ranks
  const HluTask* tasks;
  int32_t ntasks;
  const int32_t* succ_off;       // CSR of the successors (the dependency graph reversed)
  const int32_t* succ;
  const HluTruncPair* pairs;
  const HluQrOut* qr;
  int* pending;                  // per task: dependencies not yet done (indegree at launch)
  int* queue;                    // ntasks slots of ready tasks: the tasks without
                                 // dependencies first, -1 in the others at launch
  int* ctrl;                     // [0] pop counter, [1] error word, [2] bad pivots,
                                 // [3] non-finite flag, [4] push counter (initial ready count)
  void* scratch;                 // grid x scratch_per_cta complex elements
  int64_t scratch_per_cta;
  void* big_scratch;             // regions of the large truncations (HluTask.a)
  int32_t kc;
  double tol;                    // truncation tolerance (0: rank kc)
  int32_t range_power;           // power iterations of the randomized range finder (0 or 1)
  int64_t wait_cycles;           // bound of one dependency wait (clock64 cycles)
  unsigned long long* trace;     // optional: per task claim, start, end (ns)
};

// One launch of `grid` CTAs (the per-CTA scratch must hold grid slots; any
// number of them may be resident at a time); returns the kernels launched
// (1), or -1 when the launch was refused.
int launch_hlu_exec(const HluExecArgs& a, int grid, cudaStream_t s);
// Most CTAs of the executor an SM holds at once, for a precision (sizes the grid).
int hlu_exec_occupancy(int precision);
// flag |= 1 when the n arena values (complex, the precision's type) hold a NaN
// or an Inf.
void launch_hlu_finite_check(const void* arena, int64_t n, int precision, int* flag, int nsm,
                             cudaStream_t s);
// Largest diagonal leaf the QR task holds in shared memory.
constexpr int HLU_GPU_MAX_LEAF = 48;

}  // namespace bemgpu
