// hlu.cpp -- host H-LU factorization producing the block-triangular factors
// whose forward / backward solves run on the GPU (hlu_solve.cu).
//
// Reference: HArithm::LUDecomposition / recursiveLUDecomposition
// (HMatrix/harithm.cpp:1192-1296) with QR diagonal leaves (qrInLUDecomp,
// harithm.h:13), forwSubsMatVal / forwSubsMatValTransposed (:1450-1595),
// HMultiply::multiplyHMat (hmultiply.cpp:138-197) and
// recursiveHMatSubstraction (harithm.cpp:1915-2005), all truncating to the
// preconditioner rank (bemparameters.h:27). The same recursion is written here
// with this library's own node type and dense helpers.
#include "hlu.h"
#include "hlu_gpu.h"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <stdexcept>

namespace bemgpu {

namespace {

// ---------------- dense helpers (column-major) ----------------
// C (m x n) += alpha * op(A) * op(B); op = 'N' or 'T' (plain transpose) or 'C'
void gemm(char ta, char tb, int64_t m, int64_t n, int64_t k, cd alpha, const cd* A, int64_t lda,
          const cd* B, int64_t ldb, cd* C, int64_t ldc) {
  for (int64_t j = 0; j < n; j++)
    for (int64_t l = 0; l < k; l++) {
      cd b = (tb == 'N') ? B[l + j * ldb] : (tb == 'T' ? B[j + l * ldb] : std::conj(B[j + l * ldb]));
      if (b == cd(0)) continue;
      b *= alpha;
      if (ta == 'N') {
        const cd* a = A + l * lda;
        cd* c = C + j * ldc;
        for (int64_t i = 0; i < m; i++) c[i] += a[i] * b;
      } else {
        for (int64_t i = 0; i < m; i++) {
          cd a = A[l + i * lda];
          if (ta == 'C') a = std::conj(a);
          C[i + j * ldc] += a * b;
        }
      }
    }
}

// Householder QR: A (m x k) -> Q (m x p), R (p x k), p = min(m, k)
void qr_thin(int64_t m, int64_t k, std::vector<cd> A, std::vector<cd>& Q, std::vector<cd>& R) {
  const int64_t p = std::min(m, k);
  std::vector<std::vector<cd>> vs(p);
  for (int64_t j = 0; j < p; j++) {
    double xn = 0;
    for (int64_t i = j; i < m; i++) xn += std::norm(A[j * m + i]);
    xn = std::sqrt(xn);
    std::vector<cd> v(A.begin() + j * m + j, A.begin() + j * m + m);
    const cd x0 = v[0];
    const cd ph = std::abs(x0) > 0 ? x0 / std::abs(x0) : cd(1.0);
    v[0] += ph * xn;
    double vn = 0;
    for (auto& z : v) vn += std::norm(z);
    vn = std::sqrt(vn);
    if (vn > 0)
      for (auto& z : v) z /= vn;
    for (int64_t c = j; c < k; c++) {
      cd d = 0;
      for (int64_t i = j; i < m; i++) d += std::conj(v[i - j]) * A[c * m + i];
      for (int64_t i = j; i < m; i++) A[c * m + i] -= 2.0 * v[i - j] * d;
    }
    vs[j] = std::move(v);
  }
  R.assign(p * k, 0.0);
  for (int64_t c = 0; c < k; c++)
    for (int64_t r = 0; r <= std::min(c, p - 1); r++) R[c * p + r] = A[c * m + r];
  Q.assign(m * p, 0.0);
  for (int64_t j = 0; j < p; j++) Q[j * m + j] = 1.0;
  for (int64_t j = p - 1; j >= 0; j--) {
    const auto& v = vs[j];
    for (int64_t c = 0; c < p; c++) {
      cd d = 0;
      for (int64_t i = j; i < m; i++) d += std::conj(v[i - j]) * Q[c * m + i];
      for (int64_t i = j; i < m; i++) Q[c * m + i] -= 2.0 * v[i - j] * d;
    }
  }
}

// One-sided (Hestenes) Jacobi SVD of a p x q complex matrix C (column-major):
// the q columns are rotated until pairwise orthogonal, C V = U diag(s), so
// C = U diag(s) V^H with U p x q, V q x q, s sorted descending. Real and
// imaginary parts are kept in separate arrays so that the pair loops
// vectorize; the caller passes the orientation with the fewer columns.
void jacobi_svd(int64_t p, int64_t q, const cd* C, std::vector<double>& s, std::vector<cd>& U,
                std::vector<cd>& V) {
  std::vector<double> ar(p * q), ai(p * q), vr(q * q, 0.0), vi(q * q, 0.0), nrm(q);
  for (int64_t i = 0; i < p * q; i++) {
    ar[i] = C[i].real();
    ai[i] = C[i].imag();
  }
  for (int64_t i = 0; i < q; i++) vr[i * q + i] = 1.0;
  auto colnorm = [&](int64_t j) {
    const double *xr = &ar[j * p], *xi = &ai[j * p];
    double t = 0;
    for (int64_t i = 0; i < p; i++) t += xr[i] * xr[i] + xi[i] * xi[i];
    return t;
  };
  for (int64_t j = 0; j < q; j++) nrm[j] = colnorm(j);
  // columns below 1e-30 of the squared Frobenius norm (rotations keep it) are
  // rounding noise: their relative test never settles, so they take no
  // rotations
  double fro = 0;
  for (int64_t j = 0; j < q; j++) fro += nrm[j];
  const double floor2 = 1e-30 * fro;
  // rotate columns x, y (length len) of a split array by (c, s, e)
  auto rot = [](double* xr, double* xi, double* yr, double* yi, int64_t len, double c, double sn,
                double er, double ei) {
    for (int64_t i = 0; i < len; i++) {
      // y' = y conj(e)
      const double tr = yr[i] * er + yi[i] * ei, ti = yi[i] * er - yr[i] * ei;
      const double pr = xr[i], pi = xi[i];
      xr[i] = c * pr - sn * tr;
      xi[i] = c * pi - sn * ti;
      yr[i] = sn * pr + c * tr;
      yi[i] = sn * pi + c * ti;
    }
  };
  for (int sweep = 0; sweep < 60; sweep++) {
    double off = 0;
    for (int64_t a = 0; a < q - 1; a++)
      for (int64_t b = a + 1; b < q; b++) {
        const double na = nrm[a], nb = nrm[b];
        if (!(na > floor2) || !(nb > floor2)) continue;
        const double *xr = &ar[a * p], *xi = &ai[a * p], *yr = &ar[b * p], *yi = &ai[b * p];
        double gr = 0, gi = 0;  // g = <x, y> = sum conj(x) y
        for (int64_t i = 0; i < p; i++) {
          gr += xr[i] * yr[i] + xi[i] * yi[i];
          gi += xr[i] * yi[i] - xi[i] * yr[i];
        }
        const double ga = std::hypot(gr, gi);
        const double rel = ga / std::sqrt(na * nb);
        if (ga == 0.0 || rel <= 1e-15) continue;
        off = std::max(off, rel);
        const double er = gr / ga, ei = gi / ga;
        const double zeta = (nb - na) / (2.0 * ga);
        const double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / std::sqrt(1.0 + t * t), sn = c * t;
        rot(&ar[a * p], &ai[a * p], &ar[b * p], &ai[b * p], p, c, sn, er, ei);
        rot(&vr[a * q], &vi[a * q], &vr[b * q], &vi[b * q], q, c, sn, er, ei);
        nrm[a] = colnorm(a);
        nrm[b] = colnorm(b);
      }
    if (off < 1e-15) break;
  }
  std::vector<double> sv(q);
  for (int64_t j = 0; j < q; j++) sv[j] = std::sqrt(nrm[j]);
  std::vector<int64_t> ord(q);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int64_t x, int64_t y) { return sv[x] > sv[y]; });
  s.resize(q);
  U.assign(p * q, 0.0);
  V.resize(q * q);
  for (int64_t jj = 0; jj < q; jj++) {
    const int64_t j = ord[jj];
    s[jj] = sv[j];
    for (int64_t i = 0; i < p; i++)
      U[jj * p + i] = sv[j] > 0 ? cd(ar[j * p + i], ai[j * p + i]) / sv[j] : cd(0.0);
    for (int64_t i = 0; i < q; i++) V[jj * q + i] = cd(vr[j * q + i], vi[j * q + i]);
  }
}

int64_t min_rank(const std::vector<double>& sv, int64_t max_rank, double rel) {
  const int64_t nz = (int64_t)sv.size();
  if (rel <= 0) return max_rank <= 0 ? nz : std::min(nz, max_rank);
  int64_t mi = max_rank > 0 ? std::min(max_rank, nz) : nz;
  double full = 0;
  for (double v : sv) full += v * v;
  double res = full;
  for (int64_t r = 1; r <= mi; r++) {
    res -= sv[r - 1] * sv[r - 1];
    if (res / full < rel * rel) return r;
  }
  return mi;
}

}  // namespace

namespace {

// Householder QR of X (rows x cols, column-major, in place): R in the upper
// triangle, reflector j (unit 2-norm) in v[j * rows + j .. rows), so that
// X = H_0 ... H_{p-1} [R; 0] with H_j = I - 2 v_j v_j^H.
void householder_inplace(int64_t rows, int64_t cols, cd* X, cd* v) {
  const int64_t p = std::min(rows, cols);
  for (int64_t j = 0; j < p; j++) {
    cd* x = X + j * rows;
    double xn = 0;
    for (int64_t i = j; i < rows; i++) xn += std::norm(x[i]);
    xn = std::sqrt(xn);
    cd* vj = v + j * rows;
    for (int64_t i = j; i < rows; i++) vj[i] = x[i];
    const cd x0 = x[j];
    const cd ph = std::abs(x0) > 0 ? x0 / std::abs(x0) : cd(1.0);
    vj[j] += ph * xn;
    double vn = 0;
    for (int64_t i = j; i < rows; i++) vn += std::norm(vj[i]);
    vn = std::sqrt(vn);
    if (vn > 0)
      for (int64_t i = j; i < rows; i++) vj[i] /= vn;
    for (int64_t c = j; c < cols; c++) {
      cd* y = X + c * rows;
      cd d = 0;
      for (int64_t i = j; i < rows; i++) d += std::conj(vj[i]) * y[i];
      d *= 2.0;
      for (int64_t i = j; i < rows; i++) y[i] -= vj[i] * d;
    }
  }
}

// Y (rows x r, column-major) := H_0 ... H_{p-1} Y
void apply_q(int64_t rows, int64_t p, const cd* v, int64_t r, cd* Y) {
  for (int64_t j = p - 1; j >= 0; j--) {
    const cd* vj = v + j * rows;
    for (int64_t c = 0; c < r; c++) {
      cd* y = Y + c * rows;
      cd d = 0;
      for (int64_t i = j; i < rows; i++) d += std::conj(vj[i]) * y[i];
      d *= 2.0;
      for (int64_t i = j; i < rows; i++) y[i] -= vj[i] * d;
    }
  }
}

// grow-only scratch of one thread (no allocation per truncation)
struct TruncScratch {
  std::vector<cd> xa, va, xb, vb, core, ct;
  cd* get(std::vector<cd>& b, size_t n) {
    if (b.size() < n) b.resize(n);
    return b.data();
  }
};

}  // namespace

void rk_truncate(int64_t m, int64_t n, int64_t& k, std::vector<cd>& A, std::vector<cd>& B,
                 int64_t max_rank, double tol) {
  if (k == 0) return;
  thread_local TruncScratch ws;
  // A = Qa Ra, B = Qb Rb (Householder, Q kept as reflectors)
  cd* xa = ws.get(ws.xa, (size_t)(m * k));
  cd* va = ws.get(ws.va, (size_t)(m * k));
  cd* xb = ws.get(ws.xb, (size_t)(n * k));
  cd* vb = ws.get(ws.vb, (size_t)(n * k));
  std::copy(A.begin(), A.begin() + m * k, xa);
  std::copy(B.begin(), B.begin() + n * k, xb);
  householder_inplace(m, k, xa, va);
  householder_inplace(n, k, xb, vb);
  const int64_t pa = std::min(m, k), pb = std::min(n, k);
  // core = Ra Rb^T (pa x pb); R entries (r, l) with r <= l
  cd* C = ws.get(ws.core, (size_t)(pa * pb));
  for (int64_t c = 0; c < pb; c++)
    for (int64_t r = 0; r < pa; r++) {
      cd acc = 0;
      for (int64_t l = std::max(r, c); l < k; l++) acc += xa[l * m + r] * xb[l * n + c];
      C[c * pa + r] = acc;
    }
  // core = W diag(sig) Z^H with W pa x q, Z pb x q, q = min(pa, pb)
  std::vector<double> sig;
  std::vector<cd> W, Z;
  const int64_t q = std::min(pa, pb);
  if (pa >= pb) {
    jacobi_svd(pa, pb, C, sig, W, Z);
  } else {  // C^T = U' S V'^H  ->  C = conj(V') S U'^T
    cd* Ct = ws.get(ws.ct, (size_t)(pb * pa));
    for (int64_t c = 0; c < pb; c++)
      for (int64_t r = 0; r < pa; r++) Ct[r * pb + c] = C[c * pa + r];
    std::vector<cd> Up, Vp;
    jacobi_svd(pb, pa, Ct, sig, Up, Vp);
    W.resize(pa * q);
    Z.resize(pb * q);
    for (size_t i = 0; i < W.size(); i++) W[i] = std::conj(Vp[i]);
    for (size_t i = 0; i < Z.size(); i++) Z[i] = std::conj(Up[i]);
  }
  int64_t r = min_rank(sig, max_rank, tol);
  while (r > 0 && sig[r - 1] == 0.0) r--;  // exact zeros carry nothing
  // A' = Qa [W S; 0], B' = Qb [conj(Z); 0] (A B^T = Qa W S Z^H Qb^T)
  std::vector<cd> An(m * r, 0.0), Bn(n * r, 0.0);
  for (int64_t l = 0; l < r; l++) {
    for (int64_t t = 0; t < pa; t++) An[l * m + t] = W[l * pa + t] * sig[l];
    for (int64_t t = 0; t < pb; t++) Bn[l * n + t] = std::conj(Z[l * pb + t]);
  }
  apply_q(m, pa, va, r, An.data());
  apply_q(n, pb, vb, r, Bn.data());
  A = std::move(An);
  B = std::move(Bn);
  k = r;
}

namespace {

enum Kind { ZERO, FULL, RK, SUB };

struct Node {
  int64_t r0 = 0, m = 0, c0 = 0, n = 0, rc = -1, cc = -1;
  Kind kind = ZERO;
  std::vector<cd> F;     // m x n
  int64_t k = 0;
  std::vector<cd> A, B;  // A m x k, B n x k: block = A B^T
  std::unique_ptr<Node> s[4];
};

struct Ctx {
  const HTree* t;
  int64_t rank;
  double tol;
};

std::unique_ptr<Node> make_node(const HTree& t, int64_t rc, int64_t cc) {
  auto nd = std::make_unique<Node>();
  nd->rc = rc;
  nd->cc = cc;
  nd->r0 = t.c[rc].start;
  nd->m = t.c[rc].size;
  nd->c0 = t.c[cc].start;
  nd->n = t.c[cc].size;
  return nd;
}

// rebuild the block-cluster tree of the partition (same DFS as build_blocks)
std::unique_ptr<Node> build(const HTree& t, const std::vector<HBlockDesc>& blocks,
                            std::vector<InBlock>& in, size_t& next, int64_t rc, int64_t cc) {
  auto nd = make_node(t, rc, cc);
  const HBlockDesc& b = blocks[next];
  if (b.rc == rc && b.cc == cc) {  // a partition leaf
    InBlock& ib = in[next++];
    if (ib.lowrank) {
      nd->kind = RK;
      nd->k = ib.k;
      nd->A = std::move(ib.A);
      nd->B = std::move(ib.B);
    } else {
      nd->kind = FULL;
      nd->F = std::move(ib.F);
    }
    return nd;
  }
  nd->kind = SUB;
  const HCluster &R = t.c[rc], &C = t.c[cc];
  nd->s[0] = build(t, blocks, in, next, R.son1, C.son1);
  nd->s[1] = build(t, blocks, in, next, R.son1, C.son2);
  nd->s[2] = build(t, blocks, in, next, R.son2, C.son1);
  nd->s[3] = build(t, blocks, in, next, R.son2, C.son2);
  return nd;
}

// Y (H.m x p, ld) += alpha H X (H.n x p, ld)
void hmul(const Node& H, const cd* X, int64_t ldx, int64_t p, cd* Y, int64_t ldy, cd alpha) {
  switch (H.kind) {
    case ZERO: return;
    case FULL: gemm('N', 'N', H.m, p, H.n, alpha, H.F.data(), H.m, X, ldx, Y, ldy); return;
    case RK: {
      std::vector<cd> T(H.k * p, 0.0);
      gemm('T', 'N', H.k, p, H.n, 1.0, H.B.data(), H.n, X, ldx, T.data(), H.k);
      gemm('N', 'N', H.m, p, H.k, alpha, H.A.data(), H.m, T.data(), H.k, Y, ldy);
      return;
    }
    case SUB:
      for (int q = 0; q < 4; q++) {
        const Node& S = *H.s[q];
        hmul(S, X + (S.c0 - H.c0), ldx, p, Y + (S.r0 - H.r0), ldy, alpha);
      }
  }
}

// Y (H.n x p) += alpha H^T X (H.m x p)
void hmulT(const Node& H, const cd* X, int64_t ldx, int64_t p, cd* Y, int64_t ldy, cd alpha) {
  switch (H.kind) {
    case ZERO: return;
    case FULL: gemm('T', 'N', H.n, p, H.m, alpha, H.F.data(), H.m, X, ldx, Y, ldy); return;
    case RK: {
      std::vector<cd> T(H.k * p, 0.0);
      gemm('T', 'N', H.k, p, H.m, 1.0, H.A.data(), H.m, X, ldx, T.data(), H.k);
      gemm('N', 'N', H.n, p, H.k, alpha, H.B.data(), H.n, T.data(), H.k, Y, ldy);
      return;
    }
    case SUB:
      for (int q = 0; q < 4; q++) {
        const Node& S = *H.s[q];
        hmulT(S, X + (S.r0 - H.r0), ldx, p, Y + (S.c0 - H.c0), ldy, alpha);
      }
  }
}

std::vector<cd> dense_of(const Node& H) {
  std::vector<cd> D(H.m * H.n, 0.0), I(H.n * H.n, 0.0);
  for (int64_t i = 0; i < H.n; i++) I[i * H.n + i] = 1.0;
  hmul(H, I.data(), H.n, H.n, D.data(), H.m, 1.0);
  return D;
}

// X = L^{-1} X, L block lower triangular with diagonal Q leaves (L leaf = Q)
void lower_solve(const Node& L, cd* X, int64_t ldx, int64_t p) {
  if (L.kind == FULL) {  // X = Q^H X
    std::vector<cd> T(L.m * p, 0.0);
    gemm('C', 'N', L.m, p, L.m, 1.0, L.F.data(), L.m, X, ldx, T.data(), L.m);
    for (int64_t j = 0; j < p; j++)
      for (int64_t i = 0; i < L.m; i++) X[i + j * ldx] = T[i + j * L.m];
    return;
  }
  const Node &L11 = *L.s[0], &L21 = *L.s[2], &L22 = *L.s[3];
  lower_solve(L11, X, ldx, p);
  hmul(L21, X, ldx, p, X + L11.m, ldx, -1.0);
  lower_solve(L22, X + L11.m, ldx, p);
}

// X = U^{-T} X (solve U^T Y = X), U block upper triangular with R leaves
void upperT_solve(const Node& U, cd* X, int64_t ldx, int64_t p) {
  if (U.kind == FULL) {  // R^T y = x, R upper -> forward substitution
    for (int64_t j = 0; j < p; j++) {
      cd* x = X + j * ldx;
      for (int64_t i = 0; i < U.m; i++) {
        cd s = x[i];
        for (int64_t t = 0; t < i; t++) s -= U.F[i * U.m + t] * x[t];
        x[i] = s / U.F[i * U.m + i];
      }
    }
    return;
  }
  const Node &U11 = *U.s[0], &U12 = *U.s[1], &U22 = *U.s[3];
  upperT_solve(U11, X, ldx, p);
  hmulT(U12, X, ldx, p, X + U11.n, ldx, -1.0);
  upperT_solve(U22, X + U11.n, ldx, p);
}

// a product P = A B in C's index ranges: dense (m x n) or low rank (A m x k, B n x k)
struct Prod {
  bool lowrank = false;
  int64_t m = 0, n = 0, k = 0;
  std::vector<cd> D, A, B;
};

Prod dense_to_rk(Prod P) {
  // a dense product only occurs with a small side: factor it trivially
  Prod r;
  r.lowrank = true;
  r.m = P.m;
  r.n = P.n;
  if (P.m <= P.n) {
    r.k = P.m;
    r.A.assign(P.m * P.m, 0.0);
    for (int64_t i = 0; i < P.m; i++) r.A[i * P.m + i] = 1.0;
    r.B.resize(P.n * P.m);
    for (int64_t i = 0; i < P.m; i++)
      for (int64_t j = 0; j < P.n; j++) r.B[i * P.n + j] = P.D[j * P.m + i];
  } else {
    r.k = P.n;
    r.A = std::move(P.D);
    r.B.assign(P.n * P.n, 0.0);
    for (int64_t i = 0; i < P.n; i++) r.B[i * P.n + i] = 1.0;
  }
  return r;
}

Prod mul(const Node& A, const Node& B, const Ctx& cx);

// sum of products as a truncated low-rank product over [m x n]
void rk_add(Prod& acc, Prod p, const Ctx& cx) {
  if (!p.lowrank) p = dense_to_rk(std::move(p));
  if (p.k == 0) return;
  if (acc.k == 0) {
    acc = std::move(p);
    return;
  }
  acc.A.insert(acc.A.end(), p.A.begin(), p.A.end());
  acc.B.insert(acc.B.end(), p.B.begin(), p.B.end());
  acc.k += p.k;
  rk_truncate(acc.m, acc.n, acc.k, acc.A, acc.B, cx.rank, cx.tol);
}

// P = A B for nodes with A.n == B.m
Prod mul(const Node& A, const Node& B, const Ctx& cx) {
  Prod P;
  P.m = A.m;
  P.n = B.n;
  if (A.kind == ZERO || B.kind == ZERO) {
    P.lowrank = true;
    return P;
  }
  if (A.kind == RK) {  // A.A (A.B^T B)
    P.lowrank = true;
    P.k = A.k;
    P.A = A.A;
    P.B.assign(B.n * A.k, 0.0);
    hmulT(B, A.B.data(), A.n, A.k, P.B.data(), B.n, 1.0);
    return P;
  }
  if (B.kind == RK) {  // (A B.A) B.B^T
    P.lowrank = true;
    P.k = B.k;
    P.A.assign(A.m * B.k, 0.0);
    hmul(A, B.A.data(), B.m, B.k, P.A.data(), A.m, 1.0);
    P.B = B.B;
    return P;
  }
  if (A.kind == SUB && B.kind == SUB) {
    // quadrant products, each a truncated sum, stacked into one low-rank block
    P.lowrank = true;
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++) {
        Prod q;
        q.lowrank = true;
        q.m = A.s[2 * i]->m;
        q.n = B.s[j]->n;
        for (int l = 0; l < 2; l++) rk_add(q, mul(*A.s[2 * i + l], *B.s[2 * l + j], cx), cx);
        if (q.k == 0) continue;
        const int64_t ro = A.s[2 * i]->r0 - A.r0, co = B.s[j]->c0 - B.c0;
        Prod e;
        e.lowrank = true;
        e.m = P.m;
        e.n = P.n;
        e.k = q.k;
        e.A.assign(P.m * q.k, 0.0);
        e.B.assign(P.n * q.k, 0.0);
        for (int64_t l = 0; l < q.k; l++) {
          for (int64_t r = 0; r < q.m; r++) e.A[l * P.m + ro + r] = q.A[l * q.m + r];
          for (int64_t c = 0; c < q.n; c++) e.B[l * P.n + co + c] = q.B[l * q.n + c];
        }
        rk_add(P, std::move(e), cx);
      }
    return P;
  }
  // one operand is a full leaf: one side of the product is small -> dense
  P.lowrank = false;
  P.D.assign(P.m * P.n, 0.0);
  if (A.kind == FULL && B.kind == FULL) {
    gemm('N', 'N', A.m, B.n, A.n, 1.0, A.F.data(), A.m, B.F.data(), B.m, P.D.data(), P.m);
  } else if (A.kind == FULL) {  // A FULL (few rows), B SUB: P^T = B^T A^T
    std::vector<cd> At(A.n * A.m), Pt(B.n * A.m, 0.0);
    for (int64_t i = 0; i < A.m; i++)
      for (int64_t j = 0; j < A.n; j++) At[i * A.n + j] = A.F[j * A.m + i];
    hmulT(B, At.data(), A.n, A.m, Pt.data(), B.n, 1.0);
    for (int64_t i = 0; i < A.m; i++)
      for (int64_t j = 0; j < B.n; j++) P.D[j * P.m + i] = Pt[i * B.n + j];
  } else {  // A SUB, B FULL (few columns)
    hmul(A, B.F.data(), B.m, B.n, P.D.data(), P.m, 1.0);
  }
  return P;
}

// C -= P restricted to C's ranges; (ro, co) = offset of C inside P
void sub_into(Node& C, const Prod& P, int64_t ro, int64_t co, const Ctx& cx) {
  if (P.lowrank && P.k == 0) return;
  switch (C.kind) {
    case FULL:
      if (P.lowrank) {
        for (int64_t j = 0; j < C.n; j++)
          for (int64_t l = 0; l < P.k; l++) {
            const cd b = P.B[l * P.n + co + j];
            for (int64_t i = 0; i < C.m; i++) C.F[j * C.m + i] -= P.A[l * P.m + ro + i] * b;
          }
      } else {
        for (int64_t j = 0; j < C.n; j++)
          for (int64_t i = 0; i < C.m; i++) C.F[j * C.m + i] -= P.D[(co + j) * P.m + ro + i];
      }
      return;
    case RK:
    case ZERO: {
      Prod s;  // the restriction of P as a low-rank block
      s.lowrank = true;
      s.m = C.m;
      s.n = C.n;
      if (P.lowrank) {
        s.k = P.k;
        s.A.resize(C.m * P.k);
        s.B.resize(C.n * P.k);
        for (int64_t l = 0; l < P.k; l++) {
          for (int64_t i = 0; i < C.m; i++) s.A[l * C.m + i] = -P.A[l * P.m + ro + i];
          for (int64_t j = 0; j < C.n; j++) s.B[l * C.n + j] = P.B[l * P.n + co + j];
        }
      } else {
        Prod d;
        d.m = C.m;
        d.n = C.n;
        d.D.resize(C.m * C.n);
        for (int64_t j = 0; j < C.n; j++)
          for (int64_t i = 0; i < C.m; i++) d.D[j * C.m + i] = -P.D[(co + j) * P.m + ro + i];
        s = dense_to_rk(std::move(d));
      }
      Prod acc;
      acc.lowrank = true;
      acc.m = C.m;
      acc.n = C.n;
      if (C.kind == RK && C.k > 0) {
        acc.k = C.k;
        acc.A = std::move(C.A);
        acc.B = std::move(C.B);
      }
      rk_add(acc, std::move(s), cx);
      C.kind = RK;
      C.k = acc.k;
      C.A = std::move(acc.A);
      C.B = std::move(acc.B);
      return;
    }
    case SUB:
      for (int q = 0; q < 4; q++) {
        Node& S = *C.s[q];
        sub_into(S, P, ro + (S.r0 - C.r0), co + (S.c0 - C.c0), cx);
      }
      return;
  }
}

// Independent sub-problems of at least this many matrix entries run as
// OpenMP tasks (they write disjoint blocks and only read finished ones).
constexpr int64_t TASK_MIN = 128 * 128;

// C -= A B (truncated), recursing while all three are subdivided
void mul_sub(Node& C, const Node& A, const Node& B, const Ctx& cx) {
  if (A.kind == ZERO || B.kind == ZERO) return;
  if (C.kind == SUB && A.kind == SUB && B.kind == SUB) {
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++) {
        Node& Cq = *C.s[2 * i + j];
#pragma omp task default(shared) firstprivate(i, j) if (Cq.m * Cq.n >= TASK_MIN)
        for (int l = 0; l < 2; l++) mul_sub(Cq, *A.s[2 * i + l], *B.s[2 * l + j], cx);
      }
#pragma omp taskwait
    return;
  }
  const Prod P = mul(A, B, cx);
  sub_into(C, P, 0, 0, cx);
}

// X := L^{-1} X (forwSubsMatVal, harithm.cpp:1450-1511)
void solve_lower_left(const Node& L, Node& X, const Ctx& cx) {
  switch (X.kind) {
    case ZERO: return;
    case FULL: lower_solve(L, X.F.data(), X.m, X.n); return;
    case RK: lower_solve(L, X.A.data(), X.m, X.k); return;
    case SUB: {
      if (L.kind != SUB) {  // cannot happen for partition-shaped operands
        X.F = dense_of(X);
        X.kind = FULL;
        for (auto& s : X.s) s.reset();
        lower_solve(L, X.F.data(), X.m, X.n);
        return;
      }
      const Node &L11 = *L.s[0], &L21 = *L.s[2], &L22 = *L.s[3];
      for (int j = 0; j < 2; j++) {  // the two block columns are independent
#pragma omp task default(shared) firstprivate(j) if (X.m * X.n >= 2 * TASK_MIN)
        {
          solve_lower_left(L11, *X.s[j], cx);
          mul_sub(*X.s[2 + j], L21, *X.s[j], cx);
          solve_lower_left(L22, *X.s[2 + j], cx);
        }
      }
#pragma omp taskwait
      return;
    }
  }
}

// X := X U^{-1} (forwSubsMatValTransposed, harithm.cpp:1522-1595)
void solve_upper_right(Node& X, const Node& U, const Ctx& cx) {
  switch (X.kind) {
    case ZERO: return;
    case FULL: {  // X^T := U^{-T} X^T
      std::vector<cd> T(X.n * X.m);
      for (int64_t i = 0; i < X.m; i++)
        for (int64_t j = 0; j < X.n; j++) T[i * X.n + j] = X.F[j * X.m + i];
      upperT_solve(U, T.data(), X.n, X.m);
      for (int64_t i = 0; i < X.m; i++)
        for (int64_t j = 0; j < X.n; j++) X.F[j * X.m + i] = T[i * X.n + j];
      return;
    }
    case RK: upperT_solve(U, X.B.data(), X.n, X.k); return;
    case SUB: {
      if (U.kind != SUB) {
        X.F = dense_of(X);
        X.kind = FULL;
        for (auto& s : X.s) s.reset();
        solve_upper_right(X, U, cx);
        return;
      }
      const Node &U11 = *U.s[0], &U12 = *U.s[1], &U22 = *U.s[3];
      for (int i = 0; i < 2; i++) {  // the two block rows are independent
#pragma omp task default(shared) firstprivate(i) if (X.m * X.n >= 2 * TASK_MIN)
        {
          solve_upper_right(*X.s[2 * i], U11, cx);
          mul_sub(*X.s[2 * i + 1], *X.s[2 * i], U12, cx);
          solve_upper_right(*X.s[2 * i + 1], U22, cx);
        }
      }
#pragma omp taskwait
      return;
    }
  }
}

// recursiveLUDecomposition (harithm.cpp:1202-1296); A is consumed
void lu(Node& A, Node& L, Node& U, const Ctx& cx) {
  if (A.kind != SUB) {
    if (A.kind != FULL) A.F = dense_of(A);
    std::vector<cd> Q, R;
    qr_thin(A.m, A.n, A.F, Q, R);  // diagonal leaves are square
    L.kind = FULL;
    L.F = std::move(Q);
    U.kind = FULL;
    U.F = std::move(R);
    A.F.clear();
    return;
  }
  const HTree& t = *cx.t;
  const HCluster &R = t.c[A.rc], &C = t.c[A.cc];
  L.kind = SUB;
  U.kind = SUB;
  L.s[0] = make_node(t, R.son1, C.son1);
  L.s[1] = make_node(t, R.son1, C.son2);  // stays ZERO
  L.s[3] = make_node(t, R.son2, C.son2);
  U.s[0] = make_node(t, R.son1, C.son1);
  U.s[2] = make_node(t, R.son2, C.son1);  // stays ZERO
  U.s[3] = make_node(t, R.son2, C.son2);
  lu(*A.s[0], *L.s[0], *U.s[0], cx);
#pragma omp task default(shared) if (A.m * A.n >= 4 * TASK_MIN)
  solve_lower_left(*L.s[0], *A.s[1], cx);  // U12 = L11^{-1} A12
  solve_upper_right(*A.s[2], *U.s[0], cx);  // L21 = A21 U11^{-1}
#pragma omp taskwait
  U.s[1] = std::move(A.s[1]);
  L.s[2] = std::move(A.s[2]);
  mul_sub(*A.s[3], *L.s[2], *U.s[1], cx);  // A22 -= L21 U12
  lu(*A.s[3], *L.s[3], *U.s[3], cx);
}

// ---------------- flattening ----------------
void emit_leaf(const Node& nd, int64_t kind, FlatFactor& F) {
  const int64_t off = (int64_t)F.data.size();
  int64_t rank = 0;
  if (kind == 1) {
    rank = nd.k;
    F.data.insert(F.data.end(), nd.A.begin(), nd.A.end());
    // V = B^T as k x n row-major: row l is column l of B
    F.data.insert(F.data.end(), nd.B.begin(), nd.B.end());
  } else {
    F.data.insert(F.data.end(), nd.F.begin(), nd.F.end());
  }
  const int64_t v[7] = {nd.r0, nd.m, nd.c0, nd.n, kind, rank, off};
  F.leaves.insert(F.leaves.end(), v, v + 7);
}

// every leaf of an off-diagonal subtree, appended to the schedule
void emit_offdiag(const Node& nd, FlatFactor& F) {
  if (nd.kind == ZERO || (nd.kind == RK && nd.k == 0)) return;
  if (nd.kind == SUB) {
    for (int q = 0; q < 4; q++) emit_offdiag(*nd.s[q], F);
    return;
  }
  const int32_t idx = (int32_t)F.nleaves();
  emit_leaf(nd, nd.kind == FULL ? 0 : 1, F);
  F.schedule.push_back(-idx - 1);
}

// forwardSubstitution order (harithm.cpp:1314-1340): L11, L21 x1, L22
void flatten_lower(const Node& L, FlatFactor& F) {
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

// backwardSubstitution order (harithm.cpp:1386-1412): U22, U12 x2, U11
void flatten_upper(const Node& U, FlatFactor& F) {
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

}  // namespace

void hlu_factor(const HTree& tree, const std::vector<HBlockDesc>& blocks, std::vector<InBlock>& in,
                int64_t max_rank, double tol, FlatFactor& L, FlatFactor& U) {
  if (blocks.empty()) throw std::runtime_error("hlu_factor: empty partition");
  size_t next = 0;
  std::unique_ptr<Node> A = build(tree, blocks, in, next, 0, 0);
  Ctx cx{&tree, max_rank, tol};
  Node Ln, Un;
  Ln.r0 = Un.r0 = A->r0;
  Ln.m = Un.m = A->m;
  Ln.c0 = Un.c0 = A->c0;
  Ln.n = Un.n = A->n;
  Ln.rc = Un.rc = A->rc;
  Ln.cc = Un.cc = A->cc;
#pragma omp parallel
#pragma omp single
  lu(*A, Ln, Un, cx);
  L = FlatFactor();
  U = FlatFactor();
  flatten_lower(Ln, L);
  flatten_upper(Un, U);
}

namespace {
bool df_plan_impl(const FlatFactor& f, int64_t N, int elem_bytes, HluDfPlan& p,
                  std::string* why, bool with_diag) {
  p = HluDfPlan();
  auto fail = [&](const char* s) {
    if (why) *why = s;
    p = HluDfPlan();
    return false;
  };
  const int64_t nl = f.nleaves();
  const int64_t* lv = f.leaves.data();
  std::vector<int32_t> diag;
  for (int32_t op : f.schedule)
    if (op >= 0) diag.push_back(op);
  const int D = (int)diag.size();
  if (D == 0 || N <= 0) return fail("no diagonal leaves");
  std::vector<int32_t> chunk_of(N, -1);
  std::vector<int64_t> cr0(D), cm(D);
  for (int i = 0; i < D; i++) {
    const int64_t* L = lv + 7 * (int64_t)diag[i];
    if (L[0] != L[2] || L[1] != L[3] || L[1] < 1 || L[1] > HLU_DF_MAX_M || L[0] < 0 ||
        L[0] + L[1] > N)
      return fail("diagonal leaf shape");
    for (int64_t r = L[0]; r < L[0] + L[1]; r++) {
      if (chunk_of[r] >= 0) return fail("diagonal leaves overlap");
      chunk_of[r] = i;
    }
    cr0[i] = L[0];
    cm[i] = L[1];
  }
  for (int64_t r = 0; r < N; r++)
    if (chunk_of[r] < 0) return fail("diagonal leaves do not cover the rows");
  // chunks [lo, hi] (solve order) that tile [a, a + len) exactly
  auto span = [&](int64_t a, int64_t len, int& lo, int& hi) {
    if (len < 1 || a < 0 || a + len > N) return false;
    const int c1 = chunk_of[a], c2 = chunk_of[a + len - 1];
    lo = std::min(c1, c2);
    hi = std::max(c1, c2);
    int64_t tot = 0;
    for (int c = lo; c <= hi; c++) {
      if (cr0[c] < a || cr0[c] + cm[c] > a + len) return false;
      tot += cm[c];
    }
    return tot == len;
  };
  std::vector<std::vector<HluDfRow>> rl(D), el(D);  // late, early
  std::vector<std::vector<HluDfCol>> cl(D);
  std::vector<HluDfChunk> ch(D + 1);
  for (int i = 0; i <= D; i++) {
    ch[i] = HluDfChunk{};
    ch[i].corner = -1;
  }
  p.slot.assign(nl, -1);
  for (int32_t op : f.schedule) {
    if (op >= 0) continue;
    const int32_t o = -op - 1;
    const int64_t* L = lv + 7 * (int64_t)o;
    const int64_t kind = L[4], k = L[5];
    if (kind != 0 && kind != 1) return fail("off-diagonal leaf kind");
    const bool lr = kind == 1;
    if (lr && (k < 1 || k > HLU_DF_MAX_RANK)) return fail("low-rank leaf rank");
    int ra, rb, ca, cb;
    if (!span(L[0], L[1], ra, rb) || !span(L[2], L[3], ca, cb))
      return fail("leaf not aligned with the diagonal leaves");
    if (cb >= ra) return fail("leaf not below the diagonal in solve order");
    bool uses_fin = false;
    for (int i = ra; i <= rb; i++) {
      const int32_t ro = (int32_t)(cr0[i] - L[0]);
      if (cb == i - 1) {
        if (ch[i].corner >= 0) return fail("two corner leaves");
        ch[i].corner = o;
        ch[i].cro = ro;
        ch[i].cco = (int32_t)(cr0[i - 1] - L[2]);
        ch[i].cflags = (lr ? 1 : 0) | (lr && ca < cb ? 2 : 0) | (!lr && ca == cb ? 4 : 0) |
                       (lr && ca + 1 < cb ? 8 : 0);
        ch[i].cco2 = lr && ca < cb ? (int32_t)(cr0[i - 2] - L[2]) : 0;
        ch[i].cw2 = lr && ca < cb ? (int32_t)cm[i - 2] : 0;
        ch[i].cm = (int32_t)L[1];
        ch[i].cn = (int32_t)L[3];
        ch[i].ck = (int32_t)k;
        ch[i].cc0 = (int32_t)L[2];
        ch[i].cdata = L[6];
      } else {
        auto& list = cb <= i - HLU_DF_LAG ? el[i] : rl[i];
        if (!lr) {
          list.push_back(HluDfRow{o, ro, 0, 0, -1});
        } else if (cb == i - 2) {
          list.push_back(HluDfRow{o, ro, ca < cb ? 2 : 3, (int32_t)(cr0[i - 2] - L[2]), -1});
        } else {
          list.push_back(HluDfRow{o, ro, 1, 0, -1});
          uses_fin = true;
        }
      }
    }
    if (!lr) continue;
    // prefixes of t = V x: pre over cols ca..cb-2, read by the corner (rows
    // cb + 1, which adds chunks cb - 1 and cb itself, so it waits on nothing
    // solved after chunk cb - 2); pre2 over ca..cb-1, read by mode 2 (rows
    // cb + 2) and by the last step into fin (mode 1)
    const bool uses_pre = ca < cb && ra <= cb + 2;
    if (!uses_pre && !uses_fin) continue;
    p.slot[o] = p.nslot;
    p.nslot += k * HLU_DF_MAX_R;
    for (int j = ca; j <= cb; j++) {
      const bool last = j == cb;
      if (last && !uses_fin) continue;
      const int32_t fl = (j == ca ? 1 : 0) | (last ? 2 : 0) | (j == cb - 1 ? 4 : 0) |
                         (last && ca < cb ? 8 : 0);
      for (int32_t l = 0; l < (int32_t)k; l++)
        cl[j].push_back(HluDfCol{o, (int32_t)(cr0[j] - L[2]), fl, l});
    }
  }
  // CSR lists, apply matrices
  int64_t moff = 0;
  for (int i = 0; i < D; i++) {
    ch[i].r0 = (int32_t)cr0[i];
    ch[i].m = (int32_t)cm[i];
    ch[i].moff = moff;
    // late entries: at most one per column chunk i - LAG + 1 .. i - 2; their
    // constants (full: F rows, low rank: U rows and V over cols(i - 2)) get
    // staging offsets, 32 rows per column / rank, within the staging budget
    if ((int)rl[i].size() > HLU_DF_NLATE) return fail("too many late leaves");
    int64_t so = 0;
    const int64_t budget = HLU_DF_STAGE_BYTES / elem_bytes;
    for (HluDfRow& r : rl[i]) {
      const int64_t* L = lv + 7 * (int64_t)r.leaf;
      const int64_t need = L[4] == 0 ? (L[3] <= 2 * HLU_DF_MAX_M ? 32 * L[3] : budget + 1)
                                     : 32 * L[5] * (r.mode >= 2 ? 2 : 1);
      if (so + need <= budget) {
        r.soff = (int32_t)so;
        so += need;
      }
    }
    ch[i].rbeg = (int32_t)p.rows.size();
    p.rows.insert(p.rows.end(), rl[i].begin(), rl[i].end());
    ch[i].ebeg = (int32_t)p.erows.size();
    p.erows.insert(p.erows.end(), el[i].begin(), el[i].end());
    ch[i].cbeg = (int32_t)p.cols.size();
    p.cols.insert(p.cols.end(), cl[i].begin(), cl[i].end());
    const int64_t* L = lv + 7 * (int64_t)diag[i];
    const int64_t m = L[1];
    if (!with_diag) {
      if (L[4] != 2 && L[4] != 3) return fail("diagonal leaf kind");
      moff += m * m;
      continue;
    }
    const cd* Dd = f.data.data() + L[6];
    if (L[6] < 0 || L[6] + m * m > (int64_t)f.data.size()) return fail("diagonal leaf data");
    p.diag.resize(moff + m * m);
    cd* M = p.diag.data() + moff;
    if (L[4] == 2) {  // Q (column-major): M[row][t] = conj(Q[t, row]) = conj(Q[row * m + t])
      for (int64_t e = 0; e < m * m; e++) M[e] = std::conj(Dd[e]);
    } else if (L[4] == 3) {  // R upper (column-major): M = R^{-1} row-major
      for (int64_t t = 0; t < m; t++) {
        if (Dd[t + t * m] == cd(0.0)) return fail("zero pivot");
        for (int64_t row = 0; row < m; row++) M[row * m + t] = 0.0;
        // column t of R^{-1}: R y = e_t
        M[t * m + t] = 1.0 / Dd[t + t * m];
        for (int64_t row = t - 1; row >= 0; row--) {
          cd acc = 0.0;
          for (int64_t q = row + 1; q <= t; q++) acc += Dd[row + q * m] * M[q * m + t];
          M[row * m + t] = -acc / Dd[row + row * m];
        }
      }
    } else {
      return fail("diagonal leaf kind");
    }
    moff += m * m;
  }
  ch[D].r0 = (int32_t)N;
  ch[D].rbeg = (int32_t)p.rows.size();
  ch[D].ebeg = (int32_t)p.erows.size();
  ch[D].cbeg = (int32_t)p.cols.size();
  ch[D].moff = moff;
  p.chunks = std::move(ch);
  return true;
}
}  // namespace

bool hlu_df_plan(const FlatFactor& f, int64_t N, int elem_bytes, HluDfPlan& p,
                 std::string* why) {
  return df_plan_impl(f, N, elem_bytes, p, why, true);
}

bool hlu_df_plan_structure(const FlatFactor& f, int64_t N, int elem_bytes, HluDfPlan& p,
                           std::string* why) {
  return df_plan_impl(f, N, elem_bytes, p, why, false);
}

}  // namespace bemgpu

