// hlu.h -- host-side H-LU factorization (the producer of the block-triangular
// factors whose solves run on the GPU) and the dense helpers it needs.
#pragma once
#include <stdint.h>

#include <complex>
#include <memory>
#include <string>
#include <vector>

#include "hlu_solve.h"
#include "host_tree.h"

namespace bemgpu {

using cd = std::complex<double>;

// Truncation of a low-rank product A B^T (A m x k, B n x k, column-major) to
// rank <= max_rank and relative Frobenius tail <= tol (the rule of
// GoloubReinschSvd::minRankforError, golubReinschSVD.cpp:551-585); QR of both
// factors, SVD of the k x k core. Singular values are folded into A.
void rk_truncate(int64_t m, int64_t n, int64_t& k, std::vector<cd>& A, std::vector<cd>& B,
                 int64_t max_rank, double tol);

// Flat leaf list of a block-triangular factor:
// per leaf r0, m, c0, n, kind (0 full, 1 low-rank, 2 diagonal Q, 3 diagonal R),
// rank, data offset (complex elements). Low-rank data: U (m x k col-major)
// then V (k x n row-major). Schedule: the order of leaf applications of the
// reference's recursive substitution (forward for L, backward for U); op >= 0
// is a diagonal leaf index, op < 0 is -(off-diagonal leaf index) - 1.
struct FlatFactor {
  std::vector<int64_t> leaves;  // 7 per leaf
  std::vector<cd> data;
  std::vector<int32_t> schedule;
  int64_t nleaves() const { return (int64_t)leaves.size() / 7; }
};

// Input block of the matrix to factor: full (F, m x n col-major) or low rank
// (A m x k, B n x k: block = A B^T), in the partition order of `blocks`.
struct InBlock {
  bool lowrank = false;
  int64_t k = 0;
  std::vector<cd> F, A, B;
};

// H-LU of the matrix given by the partition and its blocks (consumed), with
// the reference's structure (HArithm::LUDecomposition, harithm.cpp:1192-1296):
// QR diagonal leaves (L leaf = Q, U leaf = R), forwSubsMatVal /
// forwSubsMatValTransposed for the off-diagonal blocks, truncated H-matrix
// products for the Schur complement. Truncation: max_rank / tol.
void hlu_factor(const HTree& tree, const std::vector<HBlockDesc>& blocks,
                std::vector<InBlock>& in, int64_t max_rank, double tol, FlatFactor& L,
                FlatFactor& U);

// Plan of the dataflow sweep (hlu_solve.h) for one flattened factor: chunks
// in solve order with their corner leaves, row and column lists, pre/fin slot
// offsets, and the m x m apply matrix of every diagonal leaf, row-major:
// conj(Q) stored like Q (y = Q^H s) for L, R^{-1} for U (back substitution
// done once here, per column of the identity, instead of once per sweep).
struct HluDfPlan {
  std::vector<HluDfChunk> chunks;  // D + 1, the last one a sentinel
  std::vector<HluDfRow> rows, erows;  // late and early row lists
  std::vector<HluDfCol> cols;
  std::vector<int64_t> slot;       // per leaf, -1 for none
  int64_t nslot = 0;               // complex values in each of pre and fin
  std::vector<cd> diag;
  int D() const { return (int)chunks.size() - 1; }
};

// False (with the reason) when the factor does not have the dataflow form's
// structure: diagonal leaves that do not tile [0, N) or exceed 32 rows, a leaf
// that is not aligned with them or not below the diagonal in solve order, a
// rank above 32, a zero pivot. The sweep then runs on launch_hlu_sweep.
// elem_bytes: size of one factor element (16 complex FP64, 8 complex FP32),
// for the staging offsets of the late entries.
bool hlu_df_plan(const FlatFactor& f, int64_t N, int elem_bytes, HluDfPlan& p, std::string* why);

}  // namespace bemgpu
