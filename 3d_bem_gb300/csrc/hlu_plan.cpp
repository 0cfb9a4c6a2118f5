// hlu_plan.cpp -- symbolic H-LU factorization: the task program of the GPU
// executor (hlu_exec.cu), built once per mesh and rank.
//
// The recursion follows HArithm::LUDecomposition / recursiveLUDecomposition
// (HMatrix/harithm.cpp:1192-1296): lu(A11); U12 = L11^{-1} A12
// (forwSubsMatVal :1450-1511); L21 = A21 U11^{-1} (forwSubsMatValTransposed
// :1522-1595); A22 -= L21 U12 (HMultiply::multiplyHMat hmultiply.cpp:138-197
// with recursiveHMatSubstraction harithm.cpp:1915-2005); lu(A22); diagonal
// leaves by QR (qrInLUDecomp, harithm.h:13). Instead of computing, every step
// appends tasks (hlu_gpu.h) on arena buffers and records which earlier tasks
// each one depends on. Low-rank blocks keep exactly kc columns; a product of
// two subdivided blocks into a low-rank target is formed from its eight
// sub-products in one truncation (the reference truncates after each
// quadrant sum; one truncation of the whole sum keeps at least as much).
#include <algorithm>
#include <cmath>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <unordered_map>

#include "hlu_gpu.h"

namespace bemgpu {

namespace {

enum Kind { ZERO, FULL, RK, SUB };

// A column-major window of the arena. gr / gc: global index of its first row /
// column (the hazard segments of row- or column-segmented buffers).
struct View {
  int64_t off = -1;
  int32_t ld = 0;
  int32_t buf = -1;
  int64_t gr = 0, gc = 0, rows = 0, cols = 0;
  View sub(int64_t r, int64_t c, int64_t nr, int64_t nc) const {
    View v = *this;
    v.off = off + r + c * (int64_t)ld;
    v.gr = gr + r;
    v.gc = gc + c;
    v.rows = nr;
    v.cols = nc;
    return v;
  }
};

struct SNode {
  int64_t r0 = 0, m = 0, c0 = 0, n = 0, rc = -1, cc = -1;
  Kind kind = ZERO;
  View F;     // FULL: m x n
  View A, B;  // RK: A m x kc, B n x kc, stored contiguously (A then B)
  std::unique_ptr<SNode> s[4];
};

// A product in the index ranges of its target: dense, or low rank as pieces,
// each a pair of views (a: m x w, b: n x w) with product a b^T.
struct Piece {
  View a, b;
  int64_t width = 0;
};

struct Prod {
  int64_t m = 0, n = 0, r0 = 0, c0 = 0;
  bool dense = false;
  View D;                    // dense m x n
  std::vector<Piece> pieces; // low rank (empty: zero)
};

struct Cell {
  int32_t last = -1;
  std::vector<int32_t> rd;
};

struct Buf {
  int axis = 0;  // 0 one cell, 1 segmented by rows (gr), 2 by columns (gc)
  int64_t leaf_base = 0;
  int64_t cell0 = 0;
  int32_t ncell = 1;
};

struct Access {
  int32_t buf;
  int32_t c0, c1;  // cell range within the buffer
  int mode;        // 1 read, 2 write, 3 both
};

class Planner {
 public:
  Planner(const HTree& t, const Layout& L, int64_t kc, HluProgram& P)
      : t_(t), L_(L), kc_(kc), P_(P) {
    // leaf cluster ordinal of every index (the hazard segments)
    leaf_of_.assign(L.N, -1);
    int64_t ord = 0;
    walk_leaves(0, ord);
    nleaf_ = ord;
  }

  bool run(std::string* why) {
    try {
      size_t next = 0;
      std::unique_ptr<SNode> A = build(next, 0, 0);
      if (next != L_.blocks.size()) throw std::runtime_error("partition walk mismatch");
      SNode Ln, Un;
      copy_shape(*A, Ln);
      copy_shape(*A, Un);
      lu(*A, Ln, Un);
      flatten_lower(Ln, P_.L);
      flatten_upper(Un, P_.U);
      place_apply_matrices();
      order_and_finish();
    } catch (const std::exception& e) {
      if (why) *why = e.what();
      return false;
    }
    return true;
  }

 private:
  const HTree& t_;
  const Layout& L_;
  int64_t kc_;
  HluProgram& P_;
  std::vector<int64_t> leaf_of_;
  int64_t nleaf_ = 0;
  std::vector<Buf> bufs_;
  std::vector<Cell> cells_;
  std::vector<std::vector<int32_t>> tdeps_;
  std::vector<double> cost_;

  void walk_leaves(int64_t c, int64_t& ord) {
    const HCluster& C = t_.c[c];
    if (C.son1 < 0) {
      for (int64_t r = C.start; r < C.start + C.size; r++) leaf_of_[r] = ord;
      ord++;
      return;
    }
    walk_leaves(C.son1, ord);
    walk_leaves(C.son2, ord);
  }

  // ---- arena and buffers ----
  int64_t alloc(int64_t elems) {
    const int64_t a = (P_.arena + 15) / 16 * 16;
    P_.arena = a + std::max<int64_t>(elems, 1);
    return a;
  }
  int32_t new_buf(int axis, int64_t g0, int64_t len) {
    Buf b;
    b.axis = axis;
    if (axis != 0 && len > 0) {
      b.leaf_base = leaf_of_[g0];
      b.ncell = (int32_t)(leaf_of_[g0 + len - 1] - b.leaf_base + 1);
    }
    b.cell0 = (int64_t)cells_.size();
    cells_.resize(cells_.size() + b.ncell);
    bufs_.push_back(b);
    return (int32_t)bufs_.size() - 1;
  }
  // column-major m x n window at a fresh arena offset
  View new_view(int axis, int64_t gr, int64_t gc, int64_t m, int64_t n) {
    View v;
    v.off = alloc(m * n);
    v.ld = (int32_t)std::max<int64_t>(m, 1);
    v.gr = gr;
    v.gc = gc;
    v.rows = m;
    v.cols = n;
    const int64_t g0 = axis == 2 ? gc : gr, len = axis == 2 ? n : m;
    v.buf = new_buf(axis, g0, len);
    return v;
  }
  Access acc(const View& v, int mode) const {
    const Buf& b = bufs_[v.buf];
    Access a{v.buf, 0, b.ncell - 1, mode};
    if (b.axis != 0) {
      const int64_t g0 = b.axis == 1 ? v.gr : v.gc, len = b.axis == 1 ? v.rows : v.cols;
      if (len <= 0) return Access{v.buf, 0, -1, mode};
      a.c0 = (int32_t)(leaf_of_[g0] - b.leaf_base);
      a.c1 = (int32_t)(leaf_of_[g0 + len - 1] - b.leaf_base);
      if (a.c0 < 0 || a.c1 >= b.ncell) throw std::runtime_error("hazard range outside its buffer");
    }
    return a;
  }

  int32_t emit(const HluTask& t, std::initializer_list<Access> acs, double cost) {
    return emit_v(t, std::vector<Access>(acs), cost);
  }
  int32_t emit_v(const HluTask& t, const std::vector<Access>& acs, double cost) {
    const int32_t idx = (int32_t)P_.tasks.size();
    std::vector<int32_t> d;
    for (const Access& a : acs)
      for (int32_t c = a.c0; c <= a.c1; c++) {
        Cell& cl = cells_[bufs_[a.buf].cell0 + c];
        if (cl.last >= 0) d.push_back(cl.last);
        if (a.mode & 2) d.insert(d.end(), cl.rd.begin(), cl.rd.end());
      }
    for (const Access& a : acs)
      if (a.mode == 1)
        for (int32_t c = a.c0; c <= a.c1; c++) cells_[bufs_[a.buf].cell0 + c].rd.push_back(idx);
    for (const Access& a : acs)
      if (a.mode & 2)
        for (int32_t c = a.c0; c <= a.c1; c++) {
          Cell& cl = cells_[bufs_[a.buf].cell0 + c];
          cl.last = idx;
          cl.rd.clear();
        }
    std::sort(d.begin(), d.end());
    d.erase(std::unique(d.begin(), d.end()), d.end());
    d.erase(std::remove(d.begin(), d.end(), idx), d.end());
    P_.tasks.push_back(t);
    tdeps_.push_back(std::move(d));
    cost_.push_back(cost);
    P_.counts[t.type]++;
    return idx;
  }

  // ---- task helpers ----
  // C (m x n) (+)= (-) op(A) op(B)
  void gemm(const View& C, const View& A, int opa, const View& B, int opb, int64_t m, int64_t n,
            int64_t q, bool accumulate, bool neg) {
    if (m == 0 || n == 0) return;
    if (q == 0) {
      if (!accumulate) zero(C);
      return;
    }
    HluTask t{};
    t.type = HT_GEMM;
    t.flags = opa | (opb << 2) | (accumulate ? HF_ACC : 0) | (neg ? HF_NEG : 0);
    t.m = (int32_t)m;
    t.n = (int32_t)n;
    t.q = (int32_t)q;
    t.a = A.off;
    t.lda = A.ld;
    t.b = B.off;
    t.ldb = B.ld;
    t.c = C.off;
    t.ldc = C.ld;
    emit(t, {acc(A, 1), acc(B, 1), acc(C, accumulate ? 3 : 2)},
         2.0 + (double)m * n * q / 4096.0);
  }
  void zero(const View& C) {
    if (C.rows == 0 || C.cols == 0) return;
    HluTask t{};
    t.type = HT_ZERO;
    t.m = (int32_t)C.rows;
    t.n = (int32_t)C.cols;
    t.c = C.off;
    t.ldc = C.ld;
    emit(t, {acc(C, 2)}, 1.0 + (double)C.rows * C.cols / 65536.0);
  }
  // X (rows x p) := op(M) X, M = rows x rows (in place)
  void lmul(const View& X, const View& M, int op) {
    if (X.rows == 0 || X.cols == 0) return;
    if (X.rows > 64) throw std::runtime_error("diagonal leaf above 64 rows");
    HluTask t{};
    t.type = HT_LMUL;
    t.flags = op;
    t.m = (int32_t)X.rows;
    t.n = (int32_t)X.cols;
    t.a = M.off;
    t.lda = M.ld;
    t.c = X.off;
    t.ldc = X.ld;
    emit(t, {acc(M, 1), acc(X, 3)}, 2.5 + (double)X.rows * X.rows * X.cols / 4096.0);
  }
  // X (p x cols) := X op(M), M = cols x cols (in place)
  void rmul(const View& X, const View& M, int op) {
    if (X.rows == 0 || X.cols == 0) return;
    if (X.cols > 64) throw std::runtime_error("diagonal leaf above 64 rows");
    HluTask t{};
    t.type = HT_RMUL;
    t.flags = op;
    t.m = (int32_t)X.rows;
    t.n = (int32_t)X.cols;
    t.a = M.off;
    t.lda = M.ld;
    t.c = X.off;
    t.ldc = X.ld;
    emit(t, {acc(M, 1), acc(X, 3)}, 2.5 + (double)X.rows * X.cols * X.cols / 4096.0);
  }

  // ---- structure ----
  static void copy_shape(const SNode& a, SNode& b) {
    b.r0 = a.r0;
    b.m = a.m;
    b.c0 = a.c0;
    b.n = a.n;
    b.rc = a.rc;
    b.cc = a.cc;
  }
  std::unique_ptr<SNode> make_node(int64_t rc, int64_t cc) {
    auto nd = std::make_unique<SNode>();
    nd->rc = rc;
    nd->cc = cc;
    nd->r0 = t_.c[rc].start;
    nd->m = t_.c[rc].size;
    nd->c0 = t_.c[cc].start;
    nd->n = t_.c[cc].size;
    return nd;
  }
  void make_rk(SNode& nd) {
    nd.kind = RK;
    const int64_t off = alloc((nd.m + nd.n) * kc_);
    nd.A.off = off;
    nd.A.ld = (int32_t)std::max<int64_t>(nd.m, 1);
    nd.A.gr = nd.r0;
    nd.A.rows = nd.m;
    nd.A.cols = kc_;
    nd.A.buf = new_buf(1, nd.r0, nd.m);
    nd.B.off = off + nd.m * kc_;
    nd.B.ld = (int32_t)std::max<int64_t>(nd.n, 1);
    nd.B.gr = nd.c0;
    nd.B.rows = nd.n;
    nd.B.cols = kc_;
    nd.B.buf = new_buf(1, nd.c0, nd.n);
  }
  void make_full(SNode& nd) {
    nd.kind = FULL;
    nd.F = new_view(0, nd.r0, nd.c0, nd.m, nd.n);
  }

  // the partition leaves become the matrix to factor; their loads are the
  // first tasks (near-field copies, truncations of the assembled ACA blocks)
  std::unique_ptr<SNode> build(size_t& next, int64_t rc, int64_t cc) {
    auto nd = make_node(rc, cc);
    if (next >= L_.blocks.size()) throw std::runtime_error("partition walk past the end");
    const HBlockDesc& b = L_.blocks[next];
    if (b.rc == rc && b.cc == cc) {
      const size_t bi = next++;
      if (b.adm) {
        make_rk(*nd);
        load_far(bi, *nd);
      } else {
        make_full(*nd);
        load_near(bi, *nd);
      }
      return nd;
    }
    const HCluster &R = t_.c[rc], &C = t_.c[cc];
    if (R.son1 < 0 || C.son1 < 0) throw std::runtime_error("partition block below a leaf");
    nd->kind = SUB;
    nd->s[0] = build(next, R.son1, C.son1);
    nd->s[1] = build(next, R.son1, C.son2);
    nd->s[2] = build(next, R.son2, C.son1);
    nd->s[3] = build(next, R.son2, C.son2);
    return nd;
  }
  int64_t near_index(size_t bi) {
    if (near_of_.empty()) {
      near_of_.assign(L_.blocks.size(), -1);
      far_of_.assign(L_.blocks.size(), -1);
      int64_t ni = 0, fi = 0;
      for (size_t i = 0; i < L_.blocks.size(); i++)
        (L_.blocks[i].adm ? far_of_[i] = fi++ : near_of_[i] = ni++);
    }
    return near_of_[bi];
  }
  std::vector<int64_t> near_of_, far_of_;
  void load_near(size_t bi, SNode& nd) {
    const NearBlock& nb = L_.near[near_index(bi)];
    if (nb.m != nd.m || nb.n != nd.n) throw std::runtime_error("near block shape");
    HluTask t{};
    t.type = HT_COPY;
    t.flags = 1 << HF_SRC_SHIFT;
    t.m = (int32_t)nd.m;
    t.n = (int32_t)nd.n;
    t.a = nb.off;
    t.lda = (int32_t)nd.m;
    t.c = nd.F.off;
    t.ldc = nd.F.ld;
    emit(t, {acc(nd.F, 2)}, 2.5 + (double)nd.m * nd.n / 65536.0);
  }
  void load_far(size_t bi, SNode& nd) {
    near_index(bi);
    const int64_t fi = far_of_[bi];
    const FarBlock& fb = L_.far[fi];
    if (fb.m != nd.m || fb.n != nd.n) throw std::runtime_error("far block shape");
    HluTruncPair p{};
    p.akind = 2;
    p.bkind = 3;
    p.aoff = fb.uoff;
    p.boff = fb.voff;
    p.soff = fb.soff;
    p.ars = 1;
    p.acs = fb.m;
    p.brs = 1;
    p.bcs = fb.n;
    p.ra = 0;
    p.ma = fb.m;
    p.rb = 0;
    p.mb = fb.n;
    p.cols = fb.kcap;
    p.rank_idx = (int32_t)fi;
    trunc_out(nd.A, nd.B, nd.m, nd.n, {p}, {}, fb.kcap);
  }

  // model cost (microseconds) of a truncation, by the executor's path: the
  // shared-memory subspace path for ranks <= 2, the dense sum of a small
  // target, the range finder for a small rank of a wide sum, Householder QR
  // otherwise (fitted to traced factorizations; it only orders the claims)
  double trunc_cost(int64_t m, int64_t n, int64_t kt) const {
    if (kc_ <= 2 && hlu_sub_buffers(m, n, kt) <= HLU_SMEM_ELEMS)
      return 30.0 + (double)(m + n) * kt / 80.0;
    if (m <= 32 && n <= 32) return 60.0 + 0.2 * (double)kt * (m < n ? m : n);
    if (kc_ <= 8 && kt > kc_ + 6 && m > kc_ + 6 && n > kc_ + 6)
      return 150.0 + (double)(m + n) * kt / 50.0;
    return 100.0 + (double)(m + n) * kt * kt / 4096.0;
  }

  // TRUNC task writing A' (m x kc at Ao), B' (n x kc at Bo)
  void trunc_out(const View& Ao, const View& Bo, int64_t m, int64_t n,
                 const std::vector<HluTruncPair>& pairs, const std::vector<Access>& reads,
                 int64_t kt) {
    HluTask t{};
    t.type = HT_TRUNC;
    t.m = (int32_t)m;
    t.n = (int32_t)n;
    t.q = (int32_t)kt;
    t.x0 = (int32_t)P_.pairs.size();
    t.x1 = (int32_t)pairs.size();
    t.c = Ao.off;
    t.b = Bo.off;
    P_.pairs.insert(P_.pairs.end(), pairs.begin(), pairs.end());
    std::vector<Access> a = reads;
    a.push_back(acc(Ao, 2));
    a.push_back(acc(Bo, 2));
    P_.max_kt = std::max<int32_t>(P_.max_kt, (int32_t)kt);
    // scratch: a per-CTA slot for the common small truncations, a region of
    // its own for each large one (the loads of big ACA blocks, products into
    // big low-rank blocks)
    const int64_t sc = trunc_scratch(m, n, kt);
    if (sc <= HLU_CTA_SCRATCH) {
      t.a = -1;
      P_.scratch = std::max(P_.scratch, sc);
    } else {
      t.a = P_.big_scratch;
      P_.big_scratch += (sc + 31) / 32 * 32;
    }
    emit_v(t, a, trunc_cost(m, n, kt));
  }

  // ---- H-matrix times panel ----
  // Y (H.m x p) (+)= alpha H X (H.n x p); X and Y are views with p columns
  void hmul(const SNode& H, const View& X, const View& Y, bool neg) {
    switch (H.kind) {
      case ZERO: return;
      case FULL: gemm(Y, H.F, HOP_N, X, HOP_N, H.m, X.cols, H.n, true, neg); return;
      case RK: {
        View T = new_view(0, 0, 0, kc_, X.cols);
        gemm(T, H.B, HOP_T, X, HOP_N, kc_, X.cols, H.n, false, false);
        gemm(Y, H.A, HOP_N, T, HOP_N, H.m, X.cols, kc_, true, neg);
        return;
      }
      case SUB:
        for (int q = 0; q < 4; q++) {
          const SNode& S = *H.s[q];
          hmul(S, X.sub(S.c0 - H.c0, 0, S.n, X.cols), Y.sub(S.r0 - H.r0, 0, S.m, Y.cols), neg);
        }
    }
  }
  // Y (H.n x p) (+)= alpha H^T X (H.m x p)
  void hmulT(const SNode& H, const View& X, const View& Y, bool neg) {
    switch (H.kind) {
      case ZERO: return;
      case FULL: gemm(Y, H.F, HOP_T, X, HOP_N, H.n, X.cols, H.m, true, neg); return;
      case RK: {
        View T = new_view(0, 0, 0, kc_, X.cols);
        gemm(T, H.A, HOP_T, X, HOP_N, kc_, X.cols, H.m, false, false);
        gemm(Y, H.B, HOP_N, T, HOP_N, H.n, X.cols, kc_, true, neg);
        return;
      }
      case SUB:
        for (int q = 0; q < 4; q++) {
          const SNode& S = *H.s[q];
          hmulT(S, X.sub(S.r0 - H.r0, 0, S.m, X.cols), Y.sub(S.c0 - H.c0, 0, S.n, Y.cols), neg);
        }
    }
  }
  // Y (p x H.n) (+)= alpha X (p x H.m) H  (row panels)
  void rpmul(const View& X, const SNode& H, const View& Y, bool neg) {
    switch (H.kind) {
      case ZERO: return;
      case FULL: gemm(Y, X, HOP_N, H.F, HOP_N, X.rows, H.n, H.m, true, neg); return;
      case RK: {
        View T = new_view(0, 0, 0, X.rows, kc_);
        gemm(T, X, HOP_N, H.A, HOP_N, X.rows, kc_, H.m, false, false);
        gemm(Y, T, HOP_N, H.B, HOP_T, X.rows, H.n, kc_, true, neg);
        return;
      }
      case SUB:
        for (int q = 0; q < 4; q++) {
          const SNode& S = *H.s[q];
          rpmul(X.sub(0, S.r0 - H.r0, X.rows, S.m), S, Y.sub(0, S.c0 - H.c0, Y.rows, S.n), neg);
        }
    }
  }

  // X := L^{-1} X (X: L.m x p)
  void lower_solve(const SNode& L, const View& X) {
    if (L.kind == FULL) {
      lmul(X, L.F, HOP_C);  // Q^H X
      return;
    }
    if (L.kind != SUB) throw std::runtime_error("lower factor block kind");
    const SNode &L11 = *L.s[0], &L21 = *L.s[2], &L22 = *L.s[3];
    lower_solve(L11, X.sub(0, 0, L11.m, X.cols));
    hmul(L21, X.sub(0, 0, L11.m, X.cols), X.sub(L11.m, 0, L22.m, X.cols), true);
    lower_solve(L22, X.sub(L11.m, 0, L22.m, X.cols));
  }
  // X := U^{-T} X (X: U.n x p)
  void upperT_solve(const SNode& U, const View& X) {
    if (U.kind == FULL) {
      lmul(X, rinv_cm(U), HOP_N);  // (R^{-1})^T X
      return;
    }
    if (U.kind != SUB) throw std::runtime_error("upper factor block kind");
    const SNode &U11 = *U.s[0], &U12 = *U.s[1], &U22 = *U.s[3];
    upperT_solve(U11, X.sub(0, 0, U11.n, X.cols));
    hmulT(U12, X.sub(0, 0, U11.n, X.cols), X.sub(U11.n, 0, U22.n, X.cols), true);
    upperT_solve(U22, X.sub(U11.n, 0, U22.n, X.cols));
  }
  // X := X U^{-1} (X: p x U.m)
  void rsolve(const View& X, const SNode& U) {
    if (U.kind == FULL) {
      rmul(X, rinv_cm(U), HOP_T);  // X R^{-1}
      return;
    }
    if (U.kind != SUB) throw std::runtime_error("upper factor block kind");
    const SNode &U11 = *U.s[0], &U12 = *U.s[1], &U22 = *U.s[3];
    rsolve(X.sub(0, 0, X.rows, U11.m), U11);
    rpmul(X.sub(0, 0, X.rows, U11.m), U12, X.sub(0, U11.m, X.rows, U22.m), true);
    rsolve(X.sub(0, U11.m, X.rows, U22.m), U22);
  }

  // ---- truncation inputs ----
  // a low-rank pair: A piece a (rows at ra of A'), B piece b (rows at rb of B')
  HluTruncPair lr_pair(const View& a, const View& b, int64_t ra, int64_t rb, bool neg,
                       std::vector<Access>& rd) {
    HluTruncPair p{};
    p.akind = p.bkind = 0;
    p.aoff = a.off;
    p.ars = 1;
    p.acs = a.ld;
    p.boff = b.off;
    p.brs = 1;
    p.bcs = b.ld;
    p.ra = (int32_t)ra;
    p.ma = (int32_t)a.rows;
    p.rb = (int32_t)rb;
    p.mb = (int32_t)b.rows;
    p.cols = (int32_t)a.cols;
    p.neg = neg ? 1 : 0;
    p.rank_idx = -1;
    rd.push_back(acc(a, 1));
    rd.push_back(acc(b, 1));
    return p;
  }
  // a dense h x w block d as a low-rank pair (the reference's dense_to_rk
  // step: identity on the shorter side), placed at ra / rb
  HluTruncPair dense_pair(const View& d, int64_t ra, int64_t rb, bool neg,
                          std::vector<Access>& rd) {
    HluTruncPair p{};
    p.rank_idx = -1;
    p.ra = (int32_t)ra;
    p.rb = (int32_t)rb;
    rd.push_back(acc(d, 1));
    if (d.rows <= d.cols) {  // A = I (h), B = d^T (w x h)
      p.akind = 1;
      p.ma = (int32_t)d.rows;
      p.bkind = 0;
      p.boff = d.off;
      p.brs = d.ld;  // B(r, l) = d(l, r) = d[l + r ld]
      p.bcs = 1;
      p.mb = (int32_t)d.cols;
      p.cols = (int32_t)d.rows;
      p.neg = neg ? 2 : 0;
    } else {  // A = d (h x w), B = I (w)
      p.akind = 0;
      p.aoff = d.off;
      p.ars = 1;
      p.acs = d.ld;
      p.ma = (int32_t)d.rows;
      p.bkind = 1;
      p.mb = (int32_t)d.cols;
      p.cols = (int32_t)d.cols;
      p.neg = neg ? 1 : 0;
    }
    return p;
  }
  void trunc_pairs(const View& Ao, const View& Bo, int64_t m, int64_t n,
                   const std::vector<HluTruncPair>& pr, const std::vector<Access>& rd) {
    int64_t kt = 0;
    for (const HluTruncPair& p : pr) kt += p.cols;
    if (kt == 0) {
      zero(Ao);
      zero(Bo);
      return;
    }
    trunc_out(Ao, Bo, m, n, pr, rd, kt);
  }

  // ---- products ----
  Prod mul(const SNode& A, const SNode& B) {
    Prod P;
    P.m = A.m;
    P.n = B.n;
    P.r0 = A.r0;
    P.c0 = B.c0;
    if (A.kind == ZERO || B.kind == ZERO) return P;
    if (A.kind == RK) {  // A.A (B^T A.B)^T
      View PB = new_view(1, B.c0, 0, B.n, kc_);
      zero(PB);
      hmulT(B, A.B, PB, false);
      Piece pc;
      pc.a = A.A;
      pc.b = PB;
      pc.width = kc_;
      P.pieces.push_back(pc);
      return P;
    }
    if (B.kind == RK) {  // (A B.A) B.B^T
      View PA = new_view(1, A.r0, 0, A.m, kc_);
      zero(PA);
      hmul(A, B.A, PA, false);
      Piece pc;
      pc.a = PA;
      pc.b = B.B;
      pc.width = kc_;
      P.pieces.push_back(pc);
      return P;
    }
    if (A.kind == SUB && B.kind == SUB) {  // eight sub-products, one truncation
      std::vector<HluTruncPair> pr;
      std::vector<Access> rd;
      for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++)
          for (int l = 0; l < 2; l++) {
            const SNode &Ai = *A.s[2 * i + l], &Bj = *B.s[2 * l + j];
            Prod q = mul(Ai, Bj);
            const int64_t ro = Ai.r0 - A.r0, co = Bj.c0 - B.c0;
            if (q.dense) {
              pr.push_back(dense_pair(q.D, ro, co, false, rd));
            } else {
              for (const Piece& pc : q.pieces) pr.push_back(lr_pair(pc.a, pc.b, ro, co, false, rd));
            }
          }
      View PA = new_view(1, A.r0, 0, A.m, kc_), PB = new_view(1, B.c0, 0, B.n, kc_);
      trunc_pairs(PA, PB, A.m, B.n, pr, rd);
      Piece pc;
      pc.a = PA;
      pc.b = PB;
      pc.width = kc_;
      P.pieces.push_back(pc);
      return P;
    }
    // a full leaf operand: one side is small, the product is dense
    P.dense = true;
    P.D = new_view(P.m >= P.n ? 1 : 2, A.r0, B.c0, P.m, P.n);
    if (A.kind == FULL && B.kind == FULL) {
      gemm(P.D, A.F, HOP_N, B.F, HOP_N, A.m, B.n, A.n, false, false);
    } else if (A.kind == FULL) {
      zero(P.D);
      rpmul(A.F, B, P.D, false);
    } else {
      zero(P.D);
      hmul(A, B.F, P.D, false);
    }
    return P;
  }

  // C -= P restricted to C's ranges ((ro, co): C's offset inside P)
  void sub_into(SNode& C, const Prod& P, int64_t ro, int64_t co) {
    if (!P.dense && P.pieces.empty()) return;
    switch (C.kind) {
      case FULL:
        if (P.dense) {
          HluTask t{};
          t.type = HT_COPY;
          t.flags = HF_ACC | HF_NEG;
          t.m = (int32_t)C.m;
          t.n = (int32_t)C.n;
          const View d = P.D.sub(ro, co, C.m, C.n);
          t.a = d.off;
          t.lda = d.ld;
          t.c = C.F.off;
          t.ldc = C.F.ld;
          emit(t, {acc(d, 1), acc(C.F, 3)}, 2.5 + (double)C.m * C.n / 65536.0);
        } else {
          for (const Piece& pc : P.pieces)
            gemm(C.F, pc.a.sub(ro, 0, C.m, pc.width), HOP_N, pc.b.sub(co, 0, C.n, pc.width),
                 HOP_T, C.m, C.n, pc.width, true, true);
        }
        return;
      case RK: {
        std::vector<HluTruncPair> pr;
        std::vector<Access> rd;
        pr.push_back(lr_pair(C.A, C.B, 0, 0, false, rd));
        if (P.dense) {
          pr.push_back(dense_pair(P.D.sub(ro, co, C.m, C.n), 0, 0, true, rd));
        } else {
          for (const Piece& pc : P.pieces)
            pr.push_back(lr_pair(pc.a.sub(ro, 0, C.m, pc.width), pc.b.sub(co, 0, C.n, pc.width),
                                 0, 0, true, rd));
        }
        trunc_pairs(C.A, C.B, C.m, C.n, pr, rd);
        return;
      }
      case ZERO: throw std::runtime_error("update of a zero block");
      case SUB:
        for (int q = 0; q < 4; q++) {
          SNode& S = *C.s[q];
          sub_into(S, P, ro + (S.r0 - C.r0), co + (S.c0 - C.c0));
        }
        return;
    }
  }

  // C -= A B (truncated), recursing while all three are subdivided
  void mul_sub(SNode& C, const SNode& A, const SNode& B) {
    if (A.kind == ZERO || B.kind == ZERO) return;
    if (C.kind == SUB && A.kind == SUB && B.kind == SUB) {
      for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++)
          for (int l = 0; l < 2; l++) mul_sub(*C.s[2 * i + j], *A.s[2 * i + l], *B.s[2 * l + j]);
      return;
    }
    const Prod P = mul(A, B);
    sub_into(C, P, 0, 0);
  }

  // X := L^{-1} X (forwSubsMatVal)
  void solve_lower_left(const SNode& L, SNode& X) {
    switch (X.kind) {
      case ZERO: return;
      case FULL: lower_solve(L, X.F); return;
      case RK: lower_solve(L, X.A); return;
      case SUB: {
        if (L.kind != SUB) throw std::runtime_error("subdivided block beside a leaf factor");
        const SNode &L11 = *L.s[0], &L21 = *L.s[2], &L22 = *L.s[3];
        for (int j = 0; j < 2; j++) {
          solve_lower_left(L11, *X.s[j]);
          mul_sub(*X.s[2 + j], L21, *X.s[j]);
          solve_lower_left(L22, *X.s[2 + j]);
        }
        return;
      }
    }
  }
  // X := X U^{-1} (forwSubsMatValTransposed)
  void solve_upper_right(SNode& X, const SNode& U) {
    switch (X.kind) {
      case ZERO: return;
      case FULL: rsolve(X.F, U); return;
      case RK: upperT_solve(U, X.B); return;
      case SUB: {
        if (U.kind != SUB) throw std::runtime_error("subdivided block beside a leaf factor");
        const SNode &U11 = *U.s[0], &U12 = *U.s[1], &U22 = *U.s[3];
        for (int i = 0; i < 2; i++) {
          solve_upper_right(*X.s[2 * i], U11);
          mul_sub(*X.s[2 * i + 1], *X.s[2 * i], U12);
          solve_upper_right(*X.s[2 * i + 1], U22);
        }
        return;
      }
    }
  }

  // ---- the factorization ----
  std::unordered_map<int64_t, View> rinv_map_;  // U leaf data offset -> R^{-1} view
  std::vector<int64_t> leaf_r0_, leaf_m_;       // leaf clusters in row order
  std::vector<int64_t> qh_off_, rinv_off_;      // apply matrices per leaf ordinal
  int64_t qh_base_ = 0, rinv_base_ = 0;

  void lu(SNode& A, SNode& L, SNode& U) {
    if (A.kind != SUB) {
      if (A.kind != FULL || A.m != A.n || A.r0 != A.c0)
        throw std::runtime_error("diagonal block is not a square full leaf");
      if (A.m > HLU_GPU_MAX_LEAF) throw std::runtime_error("diagonal leaf above 48 rows");
      const int64_t o = leaf_of_[A.r0];
      if (leaf_r0_[o] != A.r0 || leaf_m_[o] != A.m)
        throw std::runtime_error("diagonal leaf is not a leaf cluster");
      L.kind = FULL;
      L.F = new_view(0, A.r0, A.c0, A.m, A.m);
      U.kind = FULL;
      U.F = new_view(0, A.r0, A.c0, A.m, A.m);
      View ri;
      ri.off = rinv_off_[o];
      ri.ld = (int32_t)A.m;
      ri.rows = ri.cols = A.m;
      ri.buf = new_buf(0, 0, 0);
      rinv_map_[U.F.off] = ri;
      HluQrOut q{L.F.off, U.F.off, qh_off_[o], rinv_off_[o]};
      HluTask t{};
      t.type = HT_QR;
      t.m = (int32_t)A.m;
      t.x0 = (int32_t)P_.qr.size();
      t.a = A.F.off;
      t.lda = A.F.ld;
      P_.qr.push_back(q);
      emit(t, {acc(A.F, 1), acc(L.F, 2), acc(U.F, 2), acc(ri, 2)}, 25.0);
      return;
    }
    const HCluster &R = t_.c[A.rc], &C = t_.c[A.cc];
    L.kind = SUB;
    U.kind = SUB;
    L.s[0] = make_node(R.son1, C.son1);
    L.s[1] = make_node(R.son1, C.son2);  // stays ZERO
    L.s[3] = make_node(R.son2, C.son2);
    U.s[0] = make_node(R.son1, C.son1);
    U.s[2] = make_node(R.son2, C.son1);  // stays ZERO
    U.s[3] = make_node(R.son2, C.son2);
    lu(*A.s[0], *L.s[0], *U.s[0]);
    solve_lower_left(*L.s[0], *A.s[1]);   // U12 = L11^{-1} A12
    solve_upper_right(*A.s[2], *U.s[0]);  // L21 = A21 U11^{-1}
    U.s[1] = std::move(A.s[1]);
    L.s[2] = std::move(A.s[2]);
    mul_sub(*A.s[3], *L.s[2], *U.s[1]);   // A22 -= L21 U12
    lu(*A.s[3], *L.s[3], *U.s[3]);
  }
  View rinv_cm(const SNode& U) {
    auto it = rinv_map_.find(U.F.off);
    if (it == rinv_map_.end()) throw std::runtime_error("R^{-1} of an unfactored leaf");
    return it->second;
  }

  // ---- flattening (the sweeps' leaf lists, hlu.cpp's order) ----
  void emit_leaf(const SNode& nd, int64_t kind, FlatFactor& F) {
    const int64_t off = kind == 1 ? nd.A.off : nd.F.off;
    const int64_t v[7] = {nd.r0, nd.m, nd.c0, nd.n, kind, kind == 1 ? kc_ : 0, off};
    F.leaves.insert(F.leaves.end(), v, v + 7);
  }
  void emit_offdiag(const SNode& nd, FlatFactor& F) {
    if (nd.kind == ZERO) return;
    if (nd.kind == SUB) {
      for (int q = 0; q < 4; q++) emit_offdiag(*nd.s[q], F);
      return;
    }
    const int32_t idx = (int32_t)F.nleaves();
    emit_leaf(nd, nd.kind == FULL ? 0 : 1, F);
    F.schedule.push_back(-idx - 1);
  }
  void flatten_lower(const SNode& L, FlatFactor& F) {
    if (L.kind != SUB) {
      const int32_t idx = (int32_t)F.nleaves();
      emit_leaf(L, 2, F);
      F.schedule.push_back(idx);
      return;
    }
    flatten_lower(*L.s[0], F);
    emit_offdiag(*L.s[2], F);
    flatten_lower(*L.s[3], F);
  }
  void flatten_upper(const SNode& U, FlatFactor& F) {
    if (U.kind != SUB) {
      const int32_t idx = (int32_t)F.nleaves();
      emit_leaf(U, 3, F);
      F.schedule.push_back(idx);
      return;
    }
    flatten_upper(*U.s[3], F);
    emit_offdiag(*U.s[1], F);
    flatten_upper(*U.s[0], F);
  }

 public:
  // apply matrices of the sweeps: Q^H of the leaves in increasing row order
  // (the lower sweep's chunk order), R^{-1} in decreasing order (the upper
  // sweep's); both laid out once, before the recursion
  void plan_apply_layout() {
    leaf_r0_.assign(nleaf_, 0);
    leaf_m_.assign(nleaf_, 0);
    for (int64_t r = 0; r < L_.N; r++) {
      const int64_t o = leaf_of_[r];
      if (leaf_m_[o] == 0) leaf_r0_[o] = r;
      leaf_m_[o]++;
    }
    int64_t tot = 0;
    for (int64_t o = 0; o < nleaf_; o++) tot += leaf_m_[o] * leaf_m_[o];
    qh_base_ = alloc(tot);
    rinv_base_ = alloc(tot);
    qh_off_.assign(nleaf_, 0);
    rinv_off_.assign(nleaf_, 0);
    int64_t a = 0;
    for (int64_t o = 0; o < nleaf_; o++) {
      qh_off_[o] = qh_base_ + a;
      a += leaf_m_[o] * leaf_m_[o];
    }
    a = 0;
    for (int64_t o = nleaf_ - 1; o >= 0; o--) {
      rinv_off_[o] = rinv_base_ + a;
      a += leaf_m_[o] * leaf_m_[o];
    }
    P_.qh_base = qh_base_;
    P_.rinv_base = rinv_base_;
  }

 private:
  void place_apply_matrices() {
    // the sweep plans' chunk offsets must equal this layout
    HluDfPlan pl, pu;
    std::string w;
    const bool okl = hlu_df_plan_structure(P_.L, L_.N, 8, pl, &w);
    const bool oku = okl && hlu_df_plan_structure(P_.U, L_.N, 8, pu, &w);
    P_.df_ok = okl && oku;
    P_.df_why = w;
    if (!P_.df_ok) return;
    for (int i = 0; i < pl.D(); i++) {
      const int64_t o = leaf_of_[pl.chunks[i].r0];
      if (qh_base_ + pl.chunks[i].moff != qh_off_[o])
        throw std::runtime_error("lower sweep apply matrices out of place");
    }
    for (int i = 0; i < pu.D(); i++) {
      const int64_t o = leaf_of_[pu.chunks[i].r0];
      if (rinv_base_ + pu.chunks[i].moff != rinv_off_[o])
        throw std::runtime_error("upper sweep apply matrices out of place");
    }
  }

  // ---- order, dependencies, statistics, bounds ----
  void order_and_finish() {
    const int64_t nt = (int64_t)P_.tasks.size();
    std::vector<double> est(nt, 0.0);
    std::vector<int64_t> lev(nt, 1);
    double path = 0, total = 0;
    for (int64_t i = 0; i < nt; i++) {
      double s = 0;
      int64_t lv = 1;
      for (int32_t d : tdeps_[i]) {
        if (d >= i) throw std::runtime_error("dependency on a later task");
        s = std::max(s, est[d] + cost_[d]);
        lv = std::max(lv, lev[d] + 1);
      }
      est[i] = s;
      lev[i] = lv;
      path = std::max(path, s + cost_[i]);
      total += cost_[i];
      P_.levels = std::max(P_.levels, lv);
    }
    P_.cost_path = path;
    P_.cost_total = total;
    {  // task types along the critical path of the cost model
      int64_t at = -1;
      for (int64_t i = 0; i < nt; i++)
        if (at < 0 || est[i] + cost_[i] > est[at] + cost_[at]) at = i;
      while (at >= 0) {
        P_.path_counts[P_.tasks[at].type]++;
        int64_t nx = -1;
        for (int32_t d : tdeps_[at])
          if (nx < 0 || est[d] + cost_[d] > est[nx] + cost_[nx]) nx = d;
        at = nx;
      }
    }
    // claim order: earliest start in the cost model (a list schedule); every
    // dependency starts strictly earlier, so the order is topological
    std::vector<int32_t> ord(nt);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int32_t a, int32_t b) { return est[a] < est[b]; });
    std::vector<int32_t> pos(nt);
    for (int64_t i = 0; i < nt; i++) pos[ord[i]] = (int32_t)i;
    std::vector<HluTask> tasks(nt);
    P_.dep_off.assign(nt + 1, 0);
    P_.deps.clear();
    for (int64_t i = 0; i < nt; i++) {
      const int32_t o = ord[i];
      tasks[i] = P_.tasks[o];
      std::vector<int32_t> d;
      for (int32_t x : tdeps_[o]) d.push_back(pos[x]);
      std::sort(d.begin(), d.end());
      d.erase(std::unique(d.begin(), d.end()), d.end());
      for (int32_t x : d)
        if (x >= i) throw std::runtime_error("claim order is not topological");
      P_.deps.insert(P_.deps.end(), d.begin(), d.end());
      P_.dep_off[i + 1] = (int32_t)P_.deps.size();
    }
    P_.tasks = std::move(tasks);
    // successors (the reverse CSR) and the ready queue at launch: the
    // executor pops ready tasks, and the task that completes a successor's
    // last dependency pushes it
    std::vector<int32_t> cnt(nt + 1, 0);
    for (int32_t x : P_.deps) cnt[x + 1]++;
    P_.succ_off.assign(nt + 1, 0);
    for (int64_t i = 0; i < nt; i++) P_.succ_off[i + 1] = P_.succ_off[i] + cnt[i + 1];
    P_.succ.assign(P_.deps.size(), 0);
    std::vector<int32_t> fill(P_.succ_off.begin(), P_.succ_off.end() - 1);
    for (int64_t i = 0; i < nt; i++)
      for (int32_t k = P_.dep_off[i]; k < P_.dep_off[i + 1]; k++)
        P_.succ[fill[P_.deps[k]]++] = (int32_t)i;
    P_.queue_init.assign(nt, -1);
    P_.nready0 = 0;
    for (int64_t i = 0; i < nt; i++)
      if (P_.dep_off[i + 1] == P_.dep_off[i]) P_.queue_init[P_.nready0++] = (int32_t)i;
    validate();
  }

  // every access of every task inside the arena and the pools
  void validate() const {
    const int64_t A = P_.arena;
    auto span = [&](int64_t off, int64_t r, int64_t c, int64_t rs, int64_t cs, int64_t lim,
                    const char* what) {
      if (r <= 0 || c <= 0) return;
      const int64_t hi = off + (r - 1) * rs + (c - 1) * cs;
      if (off < 0 || hi >= lim || rs < 0 || cs < 0) throw std::runtime_error(what);
    };
    auto op_span = [&](int64_t off, int op, int64_t r, int64_t c, int64_t ld, const char* w) {
      if (op == HOP_N) span(off, r, c, 1, ld, A, w);
      else span(off, r, c, ld, 1, A, w);
    };
    for (const HluTask& t : P_.tasks) {
      switch (t.type) {
        case HT_GEMM:
          op_span(t.a, t.flags & 3, t.m, t.q, t.lda, "GEMM A out of range");
          op_span(t.b, (t.flags >> 2) & 3, t.q, t.n, t.ldb, "GEMM B out of range");
          span(t.c, t.m, t.n, 1, t.ldc, A, "GEMM C out of range");
          if (t.lda < 1 || t.ldb < 1 || t.ldc < t.m) throw std::runtime_error("GEMM leading dim");
          break;
        case HT_LMUL:
          span(t.a, t.m, t.m, 1, t.lda, A, "LMUL M out of range");
          span(t.c, t.m, t.n, 1, t.ldc, A, "LMUL X out of range");
          if (t.m > 64 || t.ldc < t.m) throw std::runtime_error("LMUL shape");
          break;
        case HT_RMUL:
          span(t.a, t.n, t.n, 1, t.lda, A, "RMUL M out of range");
          span(t.c, t.m, t.n, 1, t.ldc, A, "RMUL X out of range");
          if (t.n > 64 || t.ldc < t.m) throw std::runtime_error("RMUL shape");
          break;
        case HT_QR: {
          if (t.x0 < 0 || t.x0 >= (int32_t)P_.qr.size() || t.m > HLU_GPU_MAX_LEAF)
            throw std::runtime_error("QR slot");
          const HluQrOut& q = P_.qr[t.x0];
          span(t.a, t.m, t.m, 1, t.lda, A, "QR input out of range");
          for (int64_t o : {q.q, q.r, q.qh, q.rinv}) span(o, t.m, t.m, 1, t.m, A, "QR output");
          break;
        }
        case HT_TRUNC: {
          span(t.c, t.m, P_.kc, 1, t.m, A, "TRUNC A' out of range");
          span(t.b, t.n, P_.kc, 1, t.n, A, "TRUNC B' out of range");
          int64_t kt = 0;
          if (t.x0 < 0 || t.x1 < 1 || t.x1 > 64 || t.x0 + t.x1 > (int32_t)P_.pairs.size())
            throw std::runtime_error("TRUNC pairs");
          if (t.a >= 0 ? t.a + trunc_scratch(t.m, t.n, t.q) > P_.big_scratch
                       : trunc_scratch(t.m, t.n, t.q) > P_.scratch)
            throw std::runtime_error("TRUNC scratch");
          for (int32_t i = t.x0; i < t.x0 + t.x1; i++) {
            const HluTruncPair& p = P_.pairs[i];
            kt += p.cols;
            if (p.ra < 0 || p.ra + p.ma > t.m || p.rb < 0 || p.rb + p.mb > t.n)
              throw std::runtime_error("TRUNC placement");
            if (p.akind == 0) span(p.aoff, p.ma, p.cols, p.ars, p.acs, A, "TRUNC A piece");
            if (p.bkind == 0) span(p.boff, p.mb, p.cols, p.brs, p.bcs, A, "TRUNC B piece");
            if (p.akind == 1 && p.ma != p.cols) throw std::runtime_error("TRUNC identity");
            if (p.bkind == 1 && p.mb != p.cols) throw std::runtime_error("TRUNC identity");
            if (p.akind == 2) {
              span(p.aoff, p.ma, p.cols, 1, p.acs, L_.u_size, "TRUNC U pool");
              span(p.soff, p.cols, 1, 1, 1, L_.s_size, "TRUNC S pool");
              if (p.rank_idx < 0 || p.rank_idx >= (int32_t)L_.far.size())
                throw std::runtime_error("TRUNC rank index");
            }
            if (p.bkind == 3) span(p.boff, p.mb, p.cols, 1, p.bcs, L_.v_size, "TRUNC V pool");
          }
          if (kt != t.q || kt > P_.max_kt) throw std::runtime_error("TRUNC width");
          break;
        }
        case HT_COPY: {
          const int src = (t.flags >> HF_SRC_SHIFT) & 7;
          span(t.a, t.m, t.n, 1, t.lda, src == 1 ? L_.near_entries : A, "COPY source");
          span(t.c, t.m, t.n, 1, t.ldc, A, "COPY target");
          break;
        }
        case HT_ZERO: span(t.c, t.m, t.n, 1, t.ldc, A, "ZERO target"); break;
        default: throw std::runtime_error("task type");
      }
    }
  }
};

}  // namespace

bool hlu_gpu_plan(const HTree& tree, const Layout& L, int64_t kc, HluProgram& P,
                  std::string* why) {
  P = HluProgram();
  if (kc < 1 || kc > 64) {
    if (why) *why = "preconditioner rank outside 1..64";
    return false;
  }
  if (L.N <= 0 || L.blocks.empty() || tree.c.empty()) {
    if (why) *why = "no partition";
    return false;
  }
  P.kc = (int32_t)kc;
  Planner pl(tree, L, kc, P);
  pl.plan_apply_layout();
  if (!pl.run(why)) {
    P = HluProgram();
    return false;
  }
  return true;
}

}  // namespace bemgpu
