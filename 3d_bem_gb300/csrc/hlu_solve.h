// hlu_solve.h -- launch interface of the H-LU block-triangular solve kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bem_kernels.h"

namespace bemgpu {

constexpr int HLU_MAX_RANK = 512;  // largest low-rank leaf of a factor
constexpr int HLU_MAX_LEAF = 512;  // largest diagonal leaf (leaf_size - 1)

// One sweep over a flattened factor: upper = 0 applies L^{-1} (y = Q^H w on
// diagonal leaves), upper = 1 applies U^{-1}. data holds the factor in complex
// FP64 (precision 0) or complex FP32 (precision 1, FP32 arithmetic). w (R x N,
// complex FP64) is consumed, x gets the result. Returns the kernels launched.
int launch_hlu_sweep(const int32_t* sched, int nops, const int64_t* leaves, const void* data,
                     int precision, double2* w, double2* x, int64_t N, int R, int upper,
                     cudaStream_t s);

// ---- dataflow form of the same sweep ----
//
// The factor re-indexed by its diagonal leaves ("chunks", numbered in solve
// order: increasing rows for L, decreasing for U). Every off-diagonal leaf
// covers whole chunks, and in solve order its columns come before its rows.
// For chunk i the one leaf that holds rows(i) x cols(i - 1) is its "corner":
// the driver applies it right after solving chunk i - 1. The other leaves
// that touch rows(i) were complete HLU_DF_LAG or more chunks earlier
// ("early", summed by item E(i) with several steps of slack) or later
// ("late": at most HLU_DF_LAG - 2 leaves, one per column chunk, summed by
// item R(i) right after chunk i - 2 is solved). A low-rank leaf's t = V x is
// accumulated chunk by chunk as the columns are solved (prefix "pre",
// complete "fin") by items C(j), so no consumer reduces over a long column
// range on the critical path.
constexpr int HLU_DF_MAX_M = 32;     // rows of a diagonal leaf
constexpr int HLU_DF_MAX_RANK = 32;  // rank of a low-rank leaf
constexpr int HLU_DF_MAX_R = 8;      // right-hand sides per launch (slot stride)
constexpr int HLU_DF_LAG = 8;        // early / late boundary, in chunks
constexpr int HLU_DF_NLATE = HLU_DF_LAG - 2;
constexpr int HLU_DF_STAGE_BYTES = 64 * 1024;  // R(i)'s shared-memory staging of late leaves

struct HluDfChunk {
  int32_t r0, m;        // rows of the diagonal leaf
  int32_t corner;       // leaf index holding rows(i) x cols(i - 1), -1 if none
  int32_t cro;          // row offset of this chunk inside the corner leaf
  int32_t cco;          // column offset of chunk i - 1 inside the corner leaf
  int32_t cflags;       // bit 0 low rank, bit 1 with earlier column chunks,
                        // bit 2 full leaf whose columns are exactly chunk i - 1,
                        // bit 3 low rank with columns before chunk i - 2 (their
                        // prefix pre is complete once C(i - 3) is done)
  int32_t rbeg, ebeg;   // starts of the late and early row lists
  int32_t cbeg;         // start of the column pair list (ends: the next
                        // chunk's, a sentinel chunk closes them)
  int32_t cco2;         // low rank with bit 1: column offset of chunk i - 2 in the leaf
  int64_t moff;         // offset of the m x m apply matrix (row-major)
  int32_t cm, cn, ck;   // corner leaf: rows, columns, rank
  int32_t cc0;          // corner leaf: first column
  int64_t cdata;        // corner leaf: data offset
  int32_t cw2;          // low rank with bit 1: columns of chunk i - 2 (its row count;
                        // in the U sweep they follow chunk i - 1's in the leaf)
  int32_t pad1;         // 80 bytes: five 16-byte copies
};
static_assert(sizeof(HluDfChunk) == 80, "HluDfChunk is copied in 16-byte pieces");

// row list entry of chunk i: the contribution of one leaf to rows(i)
struct HluDfRow {
  int32_t leaf, ro;  // leaf and the row offset of chunk i inside it
  int32_t mode;      // 0 full; low rank: 1 t = fin, 2 t = pre2 + V x(i - 2), 3 t = V x(i - 2)
  int32_t co2;       // column offset of chunk i - 2 inside the leaf (modes 2, 3)
  int32_t soff;      // late entries: staging offset (factor elements), -1 = read from global
};

// column pair list of chunk j: row l of a low-rank leaf's V over cols(j)
struct HluDfCol {
  int32_t leaf, co;  // leaf and the column offset of chunk j inside it
  int32_t flags;     // bit 0 first chunk of the leaf (no prefix yet), bit 1 last (write
                     // fin), bit 2 second to last (write pre2), bit 3 read pre2
                     // (else pre)
  int32_t l;         // row of V (0 <= l < rank)
};

// device copy of one factor's plan
struct HluDfDev {
  const HluDfChunk* chunks = nullptr;  // D + 1
  const HluDfRow* rows = nullptr;   // late
  const HluDfRow* erows = nullptr;  // early
  const HluDfCol* cols = nullptr;
  const int64_t* slot = nullptr;  // per leaf: offset of its k x HLU_DF_MAX_R pre/fin slots
  int64_t nslot = 0;              // pre2 of a leaf: pre + nslot (its prefix through the
                                  // second-to-last column chunk)
  const void* diag = nullptr;     // apply matrices, factor precision
  int D = 0;
};

// Workspace shared by the sweeps of one handle, vectors in the factor type
// (HLU_DF_MAX_R x N each): xi (the solution as the helpers read it; unused
// for FP64 factors, where x itself is read), acc and eacc (all and early
// contributions); pre and fin (nslot values each); ctrl (4 + 4 D ints,
// cleared by every launch), err (sticky error word: nonzero after a wait ran
// out of time).
struct HluDfWork {
  void* xi = nullptr;
  void* acc = nullptr;
  void* eacc = nullptr;
  void* pre = nullptr;
  void* fin = nullptr;
  int* ctrl = nullptr;
  int* err = nullptr;
  unsigned long long* trace = nullptr;  // optional: 4 x D driver timestamps (ns)
  // bound of one wait (ns): a driver may wait for helpers that start only
  // when other streams' kernels leave an SM free
  unsigned long long wait_ns = 10000000000ull;
};

// w (R x N) -> x (R x N) with one launch of 1 driver + `helpers`
// CTAs (R <= HLU_DF_MAX_R; w is only read). Returns the kernels launched.
// gate: optional early exit (bem_kernels.h HmvGate; all its flags set -> no work)
int launch_hlu_df(const HluDfDev& p, const int64_t* leaves, const void* data, int precision,
                  const double2* w, double2* x, int64_t N, int R, const HluDfWork& ws, int helpers,
                  cudaStream_t s, HmvGate gate = HmvGate{nullptr, 0, 0});

}  // namespace bemgpu
