// hlu.cpp -- oracle restatement of the H-LU preconditioner (test
// infrastructure only; never linked by the GPU library).
//
// HMatrix(const HMatrix&, rank, relError) (HMatrix/hmatrix.cpp:770-776): every
// admissible block recompressed to the preconditioner rank
// (compressAdmissibleBlock, :101-140), then HArithm::LUDecomposition /
// recursiveLUDecomposition (harithm.cpp:1192-1296) with QR diagonal leaves
// (qrInLUDecomp, harithm.h:13): lu(A11); U12 = L11^{-1} A12 (forwSubsMatVal,
// :1450-1511); L21 = A21 U11^{-1} (forwSubsMatValTransposed, :1522-1595);
// A22 -= L21 U12 (HMultiply::multiplyHMat, hmultiply.cpp:138-197, and
// recursiveHMatSubstraction, harithm.cpp:1915-2005, truncating to the rank);
// lu(A22). The factors come out as flat leaf lists (the format of
// orc_lower_solve / orc_upper_solve), and orc_solve_precond runs the
// left-preconditioned GMRES of GMRES::gmresLUPreconditionedSolve
// (gmres.h:191-207) on them.
//
// Written for clarity: dense arithmetic on the blocks in the reference's
// order; independent sub-blocks run as OpenMP tasks, as in the reference.
#include <chrono>
#include <cstring>
#include <memory>
#include <numeric>
#include <omp.h>

#include "bem_oracle.h"
#include "oracle_core.hpp"

namespace orc {
namespace {

enum class NK { Zero, Dense, LowRank, Split };

// one node of the block-cluster tree; low rank: block = U W^T (U m x k,
// W n x k, column-major)
struct HNode {
  int64_t r0 = 0, m = 0, c0 = 0, n = 0, rc = -1, cc = -1;
  NK kind = NK::Zero;
  std::vector<cd> D;
  std::vector<cd> U, W;
  int64_t k = 0;
  std::unique_ptr<HNode> ch[4];
  const HBlock* src = nullptr;  // the assembled block of a low-rank leaf, until loaded
};

// compressAdmissibleBlock of one assembled block into a low-rank leaf
void load_lowrank(HNode& nd, int64_t rank, double tol) {
  HBlock c = *nd.src;
  recompress_block(c, rank, tol);
  nd.k = c.rank;
  nd.U.assign(nd.m * nd.k, 0.0);
  nd.W.assign(nd.n * nd.k, 0.0);
  for (int64_t l = 0; l < nd.k; l++) {
    for (int64_t i = 0; i < nd.m; i++) nd.U[l * nd.m + i] = c.U[l * nd.m + i] * c.s[l];
    for (int64_t j = 0; j < nd.n; j++) nd.W[l * nd.n + j] = c.V[l * nd.n + j];
  }
  nd.src = nullptr;
}

void lowrank_leaves(HNode& nd, std::vector<HNode*>& out) {
  if (nd.kind == NK::Split) {
    for (auto& q : nd.ch) lowrank_leaves(*q, out);
  } else if (nd.kind == NK::LowRank && nd.src) {
    out.push_back(&nd);
  }
}

struct Ctx {
  const ClusterTree* t;
  int64_t rank;
  double tol;
};

// truncation of U W^T (k columns) to the rank rule of minRankforError: QR of
// both factors, SVD of the k x k core
void lr_truncate(int64_t m, int64_t n, int64_t& k, std::vector<cd>& U, std::vector<cd>& W,
                 const Ctx& cx) {
  if (k == 0) return;
  std::vector<cd> A = U, QA, RA, B = W, QB, RB;
  householder_qr(m, k, A, QA, RA);
  householder_qr(n, k, B, QB, RB);
  const int64_t pa = std::min(m, k), pb = std::min(n, k), q = std::max(pa, pb);
  std::vector<cd> C(q * q, 0.0);  // RA RB^T, padded square
  for (int64_t c = 0; c < pb; c++)
    for (int64_t r = 0; r < pa; r++) {
      cd acc = 0;
      for (int64_t l = 0; l < k; l++) acc += RA[l * pa + r] * RB[l * pb + c];
      C[c * q + r] = acc;
    }
  std::vector<double> sig;
  std::vector<cd> Uc, Vc;
  jacobi_svd(q, C, sig, Uc, Vc);  // C = Uc diag(sig) Vc^H
  int64_t r = min_rank_for_error(sig, cx.rank, cx.tol);
  while (r > 0 && sig[r - 1] == 0.0) r--;
  std::vector<cd> U2(m * r, 0.0), W2(n * r, 0.0);
  for (int64_t l = 0; l < r; l++) {
    for (int64_t i = 0; i < m; i++) {
      cd acc = 0;
      for (int64_t t = 0; t < pa; t++) acc += QA[t * m + i] * Uc[l * q + t];
      U2[l * m + i] = acc * sig[l];
    }
    for (int64_t j = 0; j < n; j++) {  // U W^T = QA Uc S Vc^H QB^T
      cd acc = 0;
      for (int64_t t = 0; t < pb; t++) acc += QB[t * n + j] * std::conj(Vc[l * q + t]);
      W2[l * n + j] = acc;
    }
  }
  U = std::move(U2);
  W = std::move(W2);
  k = r;
}

std::unique_ptr<HNode> node(const Ctx& cx, int64_t rc, int64_t cc) {
  auto nd = std::make_unique<HNode>();
  const Cluster &R = cx.t->c[rc], &C = cx.t->c[cc];
  nd->rc = rc;
  nd->cc = cc;
  nd->r0 = R.start;
  nd->m = R.size;
  nd->c0 = C.start;
  nd->n = C.size;
  return nd;
}

// the truncated copy of the matrix as a node tree (partition order)
std::unique_ptr<HNode> build(const Ctx& cx, const std::vector<HBlock>& blk, size_t& next,
                             int64_t rc, int64_t cc) {
  auto nd = node(cx, rc, cc);
  const HBlock& b = blk[next];
  if (b.info.rc == rc && b.info.cc == cc) {
    // a partition leaf at this node (the partition lists the blocks in the
    // same depth-first order)
    next++;
    if (b.info.adm) {  // truncated to the rank afterwards (load_lowrank)
      nd->kind = NK::LowRank;
      nd->src = &b;
    } else {
      nd->kind = NK::Dense;
      nd->D = b.full;
    }
    return nd;
  }
  const Cluster &R = cx.t->c[rc], &C = cx.t->c[cc];
  nd->kind = NK::Split;
  nd->ch[0] = build(cx, blk, next, R.son1, C.son1);
  nd->ch[1] = build(cx, blk, next, R.son1, C.son2);
  nd->ch[2] = build(cx, blk, next, R.son2, C.son1);
  nd->ch[3] = build(cx, blk, next, R.son2, C.son2);
  return nd;
}

// Y (H.m x p, ld) += s H X (H.n x p, ld)
void hmv(const HNode& H, const cd* X, int64_t ldx, int64_t p, cd* Y, int64_t ldy, cd s) {
  if (H.kind == NK::Zero) return;
  if (H.kind == NK::Dense) {
    for (int64_t c = 0; c < p; c++)
      for (int64_t j = 0; j < H.n; j++) {
        const cd x = s * X[c * ldx + j];
        for (int64_t i = 0; i < H.m; i++) Y[c * ldy + i] += H.D[j * H.m + i] * x;
      }
    return;
  }
  if (H.kind == NK::LowRank) {
    for (int64_t c = 0; c < p; c++)
      for (int64_t l = 0; l < H.k; l++) {
        cd t = 0;
        for (int64_t j = 0; j < H.n; j++) t += H.W[l * H.n + j] * X[c * ldx + j];
        t *= s;
        for (int64_t i = 0; i < H.m; i++) Y[c * ldy + i] += H.U[l * H.m + i] * t;
      }
    return;
  }
  for (const auto& q : H.ch) hmv(*q, X + (q->c0 - H.c0), ldx, p, Y + (q->r0 - H.r0), ldy, s);
}

// Y (H.n x p) += s H^T X (H.m x p)
void hmvT(const HNode& H, const cd* X, int64_t ldx, int64_t p, cd* Y, int64_t ldy, cd s) {
  if (H.kind == NK::Zero) return;
  if (H.kind == NK::Dense) {
    for (int64_t c = 0; c < p; c++)
      for (int64_t j = 0; j < H.n; j++) {
        cd acc = 0;
        for (int64_t i = 0; i < H.m; i++) acc += H.D[j * H.m + i] * X[c * ldx + i];
        Y[c * ldy + j] += s * acc;
      }
    return;
  }
  if (H.kind == NK::LowRank) {
    for (int64_t c = 0; c < p; c++)
      for (int64_t l = 0; l < H.k; l++) {
        cd t = 0;
        for (int64_t i = 0; i < H.m; i++) t += H.U[l * H.m + i] * X[c * ldx + i];
        t *= s;
        for (int64_t j = 0; j < H.n; j++) Y[c * ldy + j] += H.W[l * H.n + j] * t;
      }
    return;
  }
  for (const auto& q : H.ch) hmvT(*q, X + (q->r0 - H.r0), ldx, p, Y + (q->c0 - H.c0), ldy, s);
}

std::vector<cd> to_dense(const HNode& H) {
  std::vector<cd> D(H.m * H.n, 0.0), I(H.n * H.n, 0.0);
  for (int64_t i = 0; i < H.n; i++) I[i * H.n + i] = 1.0;
  hmv(H, I.data(), H.n, H.n, D.data(), H.m, 1.0);
  return D;
}

// X := L^{-1} X (X: L.m x p); diagonal leaves of L hold Q (X := Q^H X)
void lsolve(const HNode& L, cd* X, int64_t ldx, int64_t p) {
  if (L.kind == NK::Dense) {
    std::vector<cd> T(L.m);
    for (int64_t c = 0; c < p; c++) {
      for (int64_t i = 0; i < L.m; i++) {
        cd acc = 0;
        for (int64_t t = 0; t < L.m; t++) acc += std::conj(L.D[i * L.m + t]) * X[c * ldx + t];
        T[i] = acc;
      }
      for (int64_t i = 0; i < L.m; i++) X[c * ldx + i] = T[i];
    }
    return;
  }
  const HNode &L11 = *L.ch[0], &L21 = *L.ch[2], &L22 = *L.ch[3];
  lsolve(L11, X, ldx, p);
  hmv(L21, X, ldx, p, X + L11.m, ldx, -1.0);
  lsolve(L22, X + L11.m, ldx, p);
}

// X := U^{-T} X (X: U.n x p); diagonal leaves of U hold R
void utsolve(const HNode& U, cd* X, int64_t ldx, int64_t p) {
  if (U.kind == NK::Dense) {
    for (int64_t c = 0; c < p; c++)
      for (int64_t i = 0; i < U.m; i++) {  // R^T y = x: forward substitution
        cd s = X[c * ldx + i];
        for (int64_t t = 0; t < i; t++) s -= U.D[i * U.m + t] * X[c * ldx + t];
        X[c * ldx + i] = s / U.D[i * U.m + i];
      }
    return;
  }
  const HNode &U11 = *U.ch[0], &U12 = *U.ch[1], &U22 = *U.ch[3];
  utsolve(U11, X, ldx, p);
  hmvT(U12, X, ldx, p, X + U11.n, ldx, -1.0);
  utsolve(U22, X + U11.n, ldx, p);
}

// a product in the target's index ranges: low rank (U W^T) or dense
struct Prod {
  bool dense = false;
  int64_t m = 0, n = 0, k = 0;
  std::vector<cd> D, U, W;
};

// acc += p (both low rank after converting a dense p), truncated
void lr_add(Prod& acc, Prod p, const Ctx& cx) {
  if (p.dense) {  // identity on the shorter side
    Prod r;
    r.m = p.m;
    r.n = p.n;
    if (p.m <= p.n) {
      r.k = p.m;
      r.U.assign(p.m * p.m, 0.0);
      for (int64_t i = 0; i < p.m; i++) r.U[i * p.m + i] = 1.0;
      r.W.resize(p.n * p.m);
      for (int64_t i = 0; i < p.m; i++)
        for (int64_t j = 0; j < p.n; j++) r.W[i * p.n + j] = p.D[j * p.m + i];
    } else {
      r.k = p.n;
      r.U = p.D;
      r.W.assign(p.n * p.n, 0.0);
      for (int64_t i = 0; i < p.n; i++) r.W[i * p.n + i] = 1.0;
    }
    p = std::move(r);
  }
  if (p.k == 0) return;
  if (acc.k == 0) {
    acc.U = std::move(p.U);
    acc.W = std::move(p.W);
    acc.k = p.k;
    return;
  }
  acc.U.insert(acc.U.end(), p.U.begin(), p.U.end());
  acc.W.insert(acc.W.end(), p.W.begin(), p.W.end());
  acc.k += p.k;
  lr_truncate(acc.m, acc.n, acc.k, acc.U, acc.W, cx);
}

// P = A B
Prod product(const HNode& A, const HNode& B, const Ctx& cx) {
  Prod P;
  P.m = A.m;
  P.n = B.n;
  if (A.kind == NK::Zero || B.kind == NK::Zero) return P;
  if (A.kind == NK::LowRank) {  // A.U (B^T A.W)^T
    P.k = A.k;
    P.U = A.U;
    P.W.assign(B.n * A.k, 0.0);
    hmvT(B, A.W.data(), A.n, A.k, P.W.data(), B.n, 1.0);
    return P;
  }
  if (B.kind == NK::LowRank) {  // (A B.U) B.W^T
    P.k = B.k;
    P.U.assign(A.m * B.k, 0.0);
    hmv(A, B.U.data(), B.m, B.k, P.U.data(), A.m, 1.0);
    P.W = B.W;
    return P;
  }
  if (A.kind == NK::Split && B.kind == NK::Split) {
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++) {
        Prod q;
        q.m = A.ch[2 * i]->m;
        q.n = B.ch[j]->n;
        for (int l = 0; l < 2; l++) lr_add(q, product(*A.ch[2 * i + l], *B.ch[2 * l + j], cx), cx);
        if (q.k == 0) continue;
        const int64_t ro = A.ch[2 * i]->r0 - A.r0, co = B.ch[j]->c0 - B.c0;
        Prod e;  // q embedded in P's ranges
        e.m = P.m;
        e.n = P.n;
        e.k = q.k;
        e.U.assign(P.m * q.k, 0.0);
        e.W.assign(P.n * q.k, 0.0);
        for (int64_t l = 0; l < q.k; l++) {
          for (int64_t r = 0; r < q.m; r++) e.U[l * P.m + ro + r] = q.U[l * q.m + r];
          for (int64_t c = 0; c < q.n; c++) e.W[l * P.n + co + c] = q.W[l * q.n + c];
        }
        lr_add(P, std::move(e), cx);
      }
    return P;
  }
  P.dense = true;  // a dense leaf operand: one side is small
  P.D.assign(P.m * P.n, 0.0);
  if (A.kind == NK::Dense && B.kind == NK::Dense) {
    hmv(A, B.D.data(), B.m, B.n, P.D.data(), P.m, 1.0);
  } else if (A.kind == NK::Dense) {  // P^T = B^T A^T
    std::vector<cd> At(A.n * A.m), Pt(B.n * A.m, 0.0);
    for (int64_t i = 0; i < A.m; i++)
      for (int64_t j = 0; j < A.n; j++) At[i * A.n + j] = A.D[j * A.m + i];
    hmvT(B, At.data(), A.n, A.m, Pt.data(), B.n, 1.0);
    for (int64_t i = 0; i < A.m; i++)
      for (int64_t j = 0; j < B.n; j++) P.D[j * P.m + i] = Pt[i * B.n + j];
  } else {
    hmv(A, B.D.data(), B.m, B.n, P.D.data(), P.m, 1.0);
  }
  return P;
}

// C -= P restricted to C ((ro, co): C's offset in P)
void subtract(HNode& C, const Prod& P, int64_t ro, int64_t co, const Ctx& cx) {
  if (!P.dense && P.k == 0) return;
  if (C.kind == NK::Dense) {
    for (int64_t j = 0; j < C.n; j++)
      for (int64_t i = 0; i < C.m; i++) {
        cd v;
        if (P.dense) {
          v = P.D[(co + j) * P.m + ro + i];
        } else {
          v = 0;
          for (int64_t l = 0; l < P.k; l++) v += P.U[l * P.m + ro + i] * P.W[l * P.n + co + j];
        }
        C.D[j * C.m + i] -= v;
      }
    return;
  }
  if (C.kind == NK::Split) {
    for (auto& q : C.ch) subtract(*q, P, ro + (q->r0 - C.r0), co + (q->c0 - C.c0), cx);
    return;
  }
  Prod acc;  // low rank (or zero): C + (-P restricted), truncated
  acc.m = C.m;
  acc.n = C.n;
  acc.k = C.k;
  acc.U = std::move(C.U);
  acc.W = std::move(C.W);
  Prod s;
  s.m = C.m;
  s.n = C.n;
  if (P.dense) {
    s.dense = true;
    s.D.resize(C.m * C.n);
    for (int64_t j = 0; j < C.n; j++)
      for (int64_t i = 0; i < C.m; i++) s.D[j * C.m + i] = -P.D[(co + j) * P.m + ro + i];
  } else {
    s.k = P.k;
    s.U.resize(C.m * P.k);
    s.W.resize(C.n * P.k);
    for (int64_t l = 0; l < P.k; l++) {
      for (int64_t i = 0; i < C.m; i++) s.U[l * C.m + i] = -P.U[l * P.m + ro + i];
      for (int64_t j = 0; j < C.n; j++) s.W[l * C.n + j] = P.W[l * P.n + co + j];
    }
  }
  lr_add(acc, std::move(s), cx);
  C.kind = NK::LowRank;
  C.k = acc.k;
  C.U = std::move(acc.U);
  C.W = std::move(acc.W);
}

// sub-problems of at least this many entries run as OpenMP tasks (they write
// disjoint blocks and read finished ones)
constexpr int64_t TASK_ENTRIES = 128 * 128;

// C -= A B
void mul_subtract(HNode& C, const HNode& A, const HNode& B, const Ctx& cx) {
  if (A.kind == NK::Zero || B.kind == NK::Zero) return;
  if (C.kind == NK::Split && A.kind == NK::Split && B.kind == NK::Split) {
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++) {
        HNode& Cq = *C.ch[2 * i + j];
#pragma omp task default(shared) firstprivate(i, j) if (Cq.m * Cq.n >= TASK_ENTRIES)
        for (int l = 0; l < 2; l++) mul_subtract(Cq, *A.ch[2 * i + l], *B.ch[2 * l + j], cx);
      }
#pragma omp taskwait
    return;
  }
  subtract(C, product(A, B, cx), 0, 0, cx);
}

// X := L^{-1} X
void left_solve(const HNode& L, HNode& X, const Ctx& cx) {
  switch (X.kind) {
    case NK::Zero: return;
    case NK::Dense: lsolve(L, X.D.data(), X.m, X.n); return;
    case NK::LowRank: lsolve(L, X.U.data(), X.m, X.k); return;
    case NK::Split:
      for (int j = 0; j < 2; j++) {  // the block columns are independent
#pragma omp task default(shared) firstprivate(j) if (X.m * X.n >= 2 * TASK_ENTRIES)
        {
          left_solve(*L.ch[0], *X.ch[j], cx);
          mul_subtract(*X.ch[2 + j], *L.ch[2], *X.ch[j], cx);
          left_solve(*L.ch[3], *X.ch[2 + j], cx);
        }
      }
#pragma omp taskwait
  }
}

// X := X U^{-1}
void right_solve(HNode& X, const HNode& U, const Ctx& cx) {
  switch (X.kind) {
    case NK::Zero: return;
    case NK::Dense: {
      std::vector<cd> T(X.n * X.m);
      for (int64_t i = 0; i < X.m; i++)
        for (int64_t j = 0; j < X.n; j++) T[i * X.n + j] = X.D[j * X.m + i];
      utsolve(U, T.data(), X.n, X.m);
      for (int64_t i = 0; i < X.m; i++)
        for (int64_t j = 0; j < X.n; j++) X.D[j * X.m + i] = T[i * X.n + j];
      return;
    }
    case NK::LowRank: utsolve(U, X.W.data(), X.n, X.k); return;
    case NK::Split:
      for (int i = 0; i < 2; i++) {  // the block rows are independent
#pragma omp task default(shared) firstprivate(i) if (X.m * X.n >= 2 * TASK_ENTRIES)
        {
          right_solve(*X.ch[2 * i], *U.ch[0], cx);
          mul_subtract(*X.ch[2 * i + 1], *X.ch[2 * i], *U.ch[1], cx);
          right_solve(*X.ch[2 * i + 1], *U.ch[3], cx);
        }
      }
#pragma omp taskwait
  }
}

void factor(HNode& A, HNode& L, HNode& U, const Ctx& cx) {
  if (A.kind != NK::Split) {
    std::vector<cd> D = A.kind == NK::Dense ? A.D : to_dense(A), Q, R;
    householder_qr(A.m, A.n, D, Q, R);
    L.kind = NK::Dense;
    L.D = std::move(Q);
    U.kind = NK::Dense;
    U.D = std::move(R);
    return;
  }
  const Cluster &R = cx.t->c[A.rc], &C = cx.t->c[A.cc];
  L.kind = U.kind = NK::Split;
  L.ch[0] = node(cx, R.son1, C.son1);
  L.ch[1] = node(cx, R.son1, C.son2);
  L.ch[3] = node(cx, R.son2, C.son2);
  U.ch[0] = node(cx, R.son1, C.son1);
  U.ch[2] = node(cx, R.son2, C.son1);
  U.ch[3] = node(cx, R.son2, C.son2);
  factor(*A.ch[0], *L.ch[0], *U.ch[0], cx);
#pragma omp task default(shared) if (A.m * A.n >= 4 * TASK_ENTRIES)
  left_solve(*L.ch[0], *A.ch[1], cx);
  right_solve(*A.ch[2], *U.ch[0], cx);
#pragma omp taskwait
  U.ch[1] = std::move(A.ch[1]);
  L.ch[2] = std::move(A.ch[2]);
  mul_subtract(*A.ch[3], *L.ch[2], *U.ch[1], cx);
  factor(*A.ch[3], *L.ch[3], *U.ch[3], cx);
}

// flat leaf list: r0, m, c0, n, kind (0 dense, 1 low rank, 2 Q, 3 R), rank,
// data offset; low rank data = U (m x k) then W^T (k x n row-major)
void flatten(const HNode& H, bool diag, int64_t dkind, std::vector<int64_t>& lv,
             std::vector<cd>& data) {
  if (H.kind == NK::Zero) return;
  if (H.kind == NK::Split) {
    for (const auto& q : H.ch)
      if (q) flatten(*q, diag && q->r0 == q->c0 && q->m == q->n && q->rc == q->cc, dkind, lv, data);
    return;
  }
  const int64_t off = (int64_t)data.size();
  int64_t kind = H.kind == NK::Dense ? (diag ? dkind : 0) : 1;
  if (H.kind == NK::LowRank) {
    if (H.k == 0) return;
    data.insert(data.end(), H.U.begin(), H.U.end());
    data.insert(data.end(), H.W.begin(), H.W.end());
  } else {
    data.insert(data.end(), H.D.begin(), H.D.end());
  }
  const int64_t v[7] = {H.r0, H.m, H.c0, H.n, kind, H.kind == NK::LowRank ? H.k : 0, off};
  lv.insert(lv.end(), v, v + 7);
}

}  // namespace

// H-LU of the block list (partition order) of an assembled H-matrix
void hlu_factor_blocks(const ClusterTree& t, const std::vector<HBlock>& blk, int64_t rank,
                       double tol, std::vector<int64_t>& Ll, std::vector<cd>& Ld,
                       std::vector<int64_t>& Ul, std::vector<cd>& Ud) {
  Ctx cx{&t, rank, tol};
  size_t next = 0;
  auto A = build(cx, blk, next, 0, 0);
  // the truncated copy HMatrix(const HMatrix&, rank, relError): blocks
  // recompressed independently
  std::vector<HNode*> lr;
  lowrank_leaves(*A, lr);
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t i = 0; i < (int64_t)lr.size(); i++) load_lowrank(*lr[i], rank, tol);
  HNode L, U;
  L.r0 = U.r0 = A->r0;
  L.m = U.m = A->m;
  L.c0 = U.c0 = A->c0;
  L.n = U.n = A->n;
  L.rc = U.rc = A->rc;
  L.cc = U.cc = A->cc;
#pragma omp parallel
#pragma omp single
  factor(*A, L, U, cx);
  Ll.clear();
  Ld.clear();
  Ul.clear();
  Ud.clear();
  flatten(L, true, 2, Ll, Ld);
  flatten(U, true, 3, Ul, Ud);
}

}  // namespace orc
