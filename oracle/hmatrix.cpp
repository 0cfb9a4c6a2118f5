// hmatrix.cpp -- oracle restatement of the cluster tree, block partition, ACA
// and truncating recompression (test infrastructure only).
#include <algorithm>
#include <cstdio>
#include <numeric>

#include "oracle_core.hpp"

namespace orc {

// ---------------------------------------------------------------------------
// Cluster tree: bisection of the triangle midpoints' bounding box along its
// longest side at the half (clustertree.h:262-310), leaf when size < leaf,
// then depth-first renumbering so every cluster is contiguous
// (clustertree.cpp:265-283).
// ---------------------------------------------------------------------------
namespace {
struct BuildNode {
  std::vector<int64_t> idx;
  Box box;
  int64_t son1 = -1, son2 = -1, level = 0;
  bool leaf = false;
};

Box box_of(const std::vector<V3>& pts, const std::vector<int64_t>& idx) {
  Box b;
  for (int64_t i : idx) b.add(pts[i]);
  return b;
}

void split(std::vector<BuildNode>& nodes, int64_t id, const std::vector<V3>& pts,
           int64_t leaf) {
  BuildNode& nd = nodes[id];
  if ((int64_t)nd.idx.size() < leaf || nd.idx.size() <= 1) {
    nd.leaf = true;
    return;
  }
  V3 side = nd.box.hi - nd.box.lo;
  int ax = 0;
  double best = std::fabs(side[0]);
  for (int i = 1; i < 3; i++)
    if (std::fabs(side[i]) > best) { best = std::fabs(side[i]); ax = i; }
  if (!(best > 0.0)) {  // all midpoints coincide: cannot split (guard)
    nd.leaf = true;
    return;
  }
  Box b1 = nd.box, b2 = nd.box;
  b1.lo[ax] = nd.box.lo[ax] + 0.5 * side[ax];
  b2.hi[ax] = nd.box.lo[ax] + 0.5 * side[ax];
  std::vector<int64_t> i1, i2;
  for (int64_t t : nd.idx) {
    V3 m = pts[t];
    bool in1 = (b1.hi.x - m.x >= 0 && b1.hi.y - m.y >= 0 && b1.hi.z - m.z >= 0) &&
               (b1.lo.x - m.x <= 0 && b1.lo.y - m.y <= 0 && b1.lo.z - m.z <= 0);
    (in1 ? i1 : i2).push_back(t);
  }
  int64_t lvl = nd.level;
  BuildNode s1, s2;
  s1.box = box_of(pts, i1);
  s1.idx = std::move(i1);
  s1.level = lvl + 1;
  s2.box = box_of(pts, i2);
  s2.idx = std::move(i2);
  s2.level = lvl + 1;
  int64_t id1 = (int64_t)nodes.size();
  nodes.push_back(std::move(s1));
  nodes[id].son1 = id1;
  split(nodes, id1, pts, leaf);
  int64_t id2 = (int64_t)nodes.size();
  nodes.push_back(std::move(s2));
  nodes[id].son2 = id2;
  split(nodes, id2, pts, leaf);
}

void reorder(std::vector<BuildNode>& nodes, int64_t id, int64_t& next,
             std::vector<int64_t>& perm, std::vector<int64_t>& start) {
  BuildNode& nd = nodes[id];
  if (nd.leaf) {
    start[id] = next;
    for (int64_t t : nd.idx) perm[next++] = t;
  } else {
    reorder(nodes, nd.son1, next, perm, start);
    reorder(nodes, nd.son2, next, perm, start);
    start[id] = start[nd.son1];
  }
}
}  // namespace

ClusterTree build_cluster_tree(const std::vector<V3>& pts, int64_t leaf) {
  ClusterTree ct;
  int64_t n = (int64_t)pts.size();
  std::vector<BuildNode> nodes;
  nodes.reserve(4 * (n / std::max<int64_t>(leaf, 1) + 2));
  BuildNode root;
  root.idx.resize(n);
  std::iota(root.idx.begin(), root.idx.end(), 0);
  root.box = box_of(pts, root.idx);
  nodes.push_back(std::move(root));
  split(nodes, 0, pts, leaf);
  ct.perm.assign(n, 0);
  std::vector<int64_t> start(nodes.size(), 0);
  int64_t next = 0;
  reorder(nodes, 0, next, ct.perm, start);
  ct.c.resize(nodes.size());
  for (size_t i = 0; i < nodes.size(); i++) {
    Cluster& c = ct.c[i];
    c.start = start[i];
    c.size = (int64_t)nodes[i].idx.size();
    c.son1 = nodes[i].son1;
    c.son2 = nodes[i].son2;
    c.level = nodes[i].level;
    c.leaf = nodes[i].leaf;
    c.box = nodes[i].box;  // boxes are of midpoints, invariant under renumbering
  }
  return ct;
}

// clusterDistance (hmatrix.cpp:1070-1129): axis-aligned box distance, with
// strict overlap tests per axis.
double cluster_distance(const Box& a, const Box& b) {
  const V3 &p1 = a.lo, &q1 = a.hi, &p2 = b.lo, &q2 = b.hi;
  bool ov[3];
  for (int i = 0; i < 3; i++)
    ov[i] = (p1[i] < q2[i] && q1[i] > p2[i]) || (p2[i] < q1[i] && q2[i] > p1[i]);
  int nov = ov[0] + ov[1] + ov[2];
  auto gap = [&](int i) { return std::min(std::fabs(p1[i] - q2[i]), std::fabs(p2[i] - q1[i])); };
  if (nov == 3) return 0.0;
  if (nov == 2) {
    if (!ov[0]) return gap(0);
    if (!ov[1]) return gap(1);
    return gap(2);
  }
  if (nov == 1) {
    int i = ov[0] ? 1 : 0, j = ov[0] ? 2 : (ov[1] ? 2 : 1);
    double d1 = gap(i), d2 = gap(j);
    return std::sqrt(d1 * d1 + d2 * d2);
  }
  double dx = gap(0), dy = gap(1), dz = gap(2);
  return std::sqrt(dx * dx + dy * dy + dz * dz);
}

// clusterSize (hmatrix.cpp:1131-1135): box diagonal.
double cluster_diameter(const Box& a) { return norm(a.hi - a.lo); }

// createBlockClusterChildren (hmatrix.cpp:958-1007) with isBlockAdmissible
// (:1052-1068): min(diam)/dist < eta.
static void partition_rec(const ClusterTree& rt, const ClusterTree& ct, int64_t r, int64_t c,
                          double eta, std::vector<BlockInfo>& out) {
  const Cluster& R = rt.c[r];
  const Cluster& C = ct.c[c];
  double dist = cluster_distance(R.box, C.box);
  bool adm = false;
  if (dist != 0.0)
    adm = std::min(cluster_diameter(R.box), cluster_diameter(C.box)) / dist < eta;
  if (adm || R.leaf || C.leaf) {
    out.push_back({R.start, R.size, C.start, C.size, adm, r, c});
    return;
  }
  partition_rec(rt, ct, R.son1, C.son1, eta, out);
  partition_rec(rt, ct, R.son1, C.son2, eta, out);
  partition_rec(rt, ct, R.son2, C.son1, eta, out);
  partition_rec(rt, ct, R.son2, C.son2, eta, out);
}

std::vector<BlockInfo> build_partition(const ClusterTree& rt, const ClusterTree& ct,
                                       double eta) {
  std::vector<BlockInfo> out;
  if (!rt.c.empty() && !ct.c.empty()) partition_rec(rt, ct, 0, 0, eta, out);
  return out;
}

// ---------------------------------------------------------------------------
// ACA with partial pivoting (hmatrix.cpp:471-593).
// ---------------------------------------------------------------------------
static int64_t argmax_abs(const std::vector<cd>& v) {
  int64_t best = 0;
  double bv = -1.0;
  for (int64_t i = 0; i < (int64_t)v.size(); i++) {
    double a = std::abs(v[i]);
    if (a > bv) { bv = a; best = i; }
  }
  return best;
}

static double sqnorm(const std::vector<cd>& v) {
  double s = 0;
  for (auto& x : v) s += std::norm(x);
  return s;
}

namespace {
struct RkBuilder {
  int64_t m, n;
  std::vector<std::vector<cd>> U, V;  // U columns (m), V rows (n)
  std::vector<cd> s;
  // (U_k s_k V_k)(row i, :) residual subtraction
  void sub_row(int64_t i, std::vector<cd>& row) const {
    for (size_t l = 0; l < s.size(); l++) {
      cd f = U[l][i] * s[l];
      for (int64_t j = 0; j < n; j++) row[j] -= f * V[l][j];
    }
  }
  void sub_col(int64_t j, std::vector<cd>& col) const {
    for (size_t l = 0; l < s.size(); l++) {
      cd f = s[l] * V[l][j];
      for (int64_t i = 0; i < m; i++) col[i] -= U[l][i] * f;
    }
  }
  cd entry(int64_t i, int64_t j) const {
    cd acc = 0;
    for (size_t l = 0; l < s.size(); l++) acc += U[l][i] * s[l] * V[l][j];
    return acc;
  }
  void finish(HBlock& blk) {
    int64_t k = (int64_t)s.size();
    if (k == 0) {  // nothing sampled: rank-1 zero block (hmatrix.cpp:587-592)
      blk.rank = 1;
      blk.U.assign(m, 0.0);
      blk.s.assign(1, 0.0);
      blk.V.assign(n, 0.0);
      return;
    }
    blk.rank = k;
    blk.U.resize(m * k);
    blk.V.resize(k * n);
    blk.s = s;
    for (int64_t l = 0; l < k; l++) {
      for (int64_t i = 0; i < m; i++) blk.U[l * m + i] = U[l][i];
      for (int64_t j = 0; j < n; j++) blk.V[l * n + j] = V[l][j];
    }
  }
};

// normEstimate update (hmatrix.cpp:570-574): |alpha|^2 |row|^2 |col|^2 plus
// 2 conj(alpha) s_i (col^H U_i)(V_i row^H) over earlier terms.
cd norm_update(const RkBuilder& rk, const std::vector<cd>& row, const std::vector<cd>& col,
               cd alpha) {
  cd add = std::abs(alpha * alpha) * sqnorm(row) * sqnorm(col);
  int64_t k = (int64_t)rk.s.size();
  for (int64_t l = 0; l < k - 1; l++) {
    cd cu = 0, vr = 0;
    for (int64_t i = 0; i < rk.m; i++) cu += std::conj(col[i]) * rk.U[l][i];
    for (int64_t j = 0; j < rk.n; j++) vr += rk.V[l][j] * std::conj(row[j]);
    add += 2.0 * std::conj(alpha) * rk.s[l] * cu * vr;
  }
  return add;
}
}  // namespace

void aca_partial_pivot(HBlock& blk, int64_t max_rank, double tol, const EntryFn& f,
                       uint64_t seed, uint64_t block_id) {
  const BlockInfo& b = blk.info;
  int64_t m = b.m, n = b.n;
  int64_t kmax = std::min(m, n);
  if (max_rank > 0) kmax = std::min(kmax, max_rank);
  RkBuilder rk{m, n, {}, {}, {}};
  std::vector<cd> row(n), col(m);
  cd est = 0;
  int64_t ri = 0, ci = (int64_t)(pivot_hash(seed, block_id, 0) % (uint64_t)n);
  for (int64_t i = 0; i < m; i++) col[i] = f(b.r0 + i, b.c0 + ci);
  while ((int64_t)rk.s.size() < kmax) {
    int64_t k = (int64_t)rk.s.size();
    if (k >= 1) col[ri] = 0.0;
    ri = argmax_abs(col);
    if (std::abs(col[ri]) <= TINY && k >= 1) break;
    for (int64_t j = 0; j < n; j++) row[j] = f(b.r0 + ri, b.c0 + j);
    rk.sub_row(ri, row);
    ci = argmax_abs(row);
    double maxrow = std::abs(row[ci]);
    if (maxrow <= TINY && k >= 1) break;
    for (int64_t i = 0; i < m; i++) col[i] = f(b.r0 + i, b.c0 + ci);
    cd alpha = 1.0 / row[ci];
    rk.sub_col(ci, col);
    rk.U.push_back(col);
    rk.V.push_back(row);
    rk.s.push_back(alpha);
    est += norm_update(rk, row, col, alpha);
    double target = std::real(tol * tol * est);
    double gain = std::norm(alpha) * sqnorm(row) * sqnorm(col);
    if (tol > 0 && gain < target) break;
  }
  rk.finish(blk);
}

// ACA with seeded pivots for dPhi blocks (hmatrix.cpp:595-745).
void aca_partial_pivot_extra(HBlock& blk, int64_t max_rank, double tol, const EntryFn& f,
                             const std::vector<std::pair<int64_t, int64_t>>& pivots) {
  const BlockInfo& b = blk.info;
  int64_t m = b.m, n = b.n;
  int64_t kmax = std::min(m, n);
  if (max_rank > 0) kmax = std::min(kmax, max_rank);
  RkBuilder rk{m, n, {}, {}, {}};
  std::vector<cd> row(n), col(m);
  cd est = 0;
  for (size_t pi = 0; pi < pivots.size() && (int64_t)rk.s.size() < kmax; pi++) {
    int64_t ri = pivots[pi].first, ci = pivots[pi].second;
    cd piv = f(b.r0 + ri, b.c0 + ci);
    if (std::abs(piv) < TINY) continue;
    if (std::abs((piv - rk.entry(ri, ci)) / piv) < tol) continue;
    for (int64_t i = 0; i < m; i++) col[i] = f(b.r0 + i, b.c0 + ci);
    rk.sub_col(ci, col);
    bool first = true;
    while ((int64_t)rk.s.size() < kmax) {
      int64_t k = (int64_t)rk.s.size();
      std::vector<double> ca(m);
      for (int64_t i = 0; i < m; i++) ca[i] = std::abs(col[i]);
      if (!first) ca[ri] = 0.0;
      {
        int64_t best = 0;
        double bv = -1;
        for (int64_t i = 0; i < m; i++)
          if (ca[i] > bv) { bv = ca[i]; best = i; }
        ri = best;
      }
      first = false;
      if (std::abs(col[ri]) <= TINY && k >= 1) break;
      for (int64_t j = 0; j < n; j++) row[j] = f(b.r0 + ri, b.c0 + j);
      rk.sub_row(ri, row);
      ci = argmax_abs(row);
      if (std::abs(row[ci]) <= TINY && k >= 1) break;
      for (int64_t i = 0; i < m; i++) col[i] = f(b.r0 + i, b.c0 + ci);
      cd alpha = 1.0 / row[ci];
      rk.sub_col(ci, col);
      rk.U.push_back(col);
      rk.V.push_back(row);
      rk.s.push_back(alpha);
      cd old = est;
      est += norm_update(rk, row, col, alpha);
      double target = std::real(tol * tol * est);
      double gain = std::norm(alpha) * sqnorm(row) * sqnorm(col);
      if (tol > 0 && gain < target) {
        if (gain < 0.1 * target) {  // roll back the last rank (:724-728)
          rk.U.pop_back();
          rk.V.pop_back();
          rk.s.pop_back();
          est = old;
        }
        break;
      }
    }
  }
  rk.finish(blk);
}

// getNormalFilteredPivotIndices (boundaryelementsolver.cpp:2052-2172):
// greedy grouping of the block's rows (and columns) by normal direction
// (|n_ref . n| >= cos(angle) stays in the group), at most 20 groups per side,
// one seeded member per group, all row-group x column-group pairs.
static std::vector<std::vector<int64_t>> normal_groups(const Mesh& mesh, int64_t start,
                                                       int64_t count, double fv) {
  const int64_t maxc = 20;
  std::vector<std::vector<int64_t>> g(maxc);
  for (int64_t i = 0; i < count; i++) g[0].push_back(start + i);
  int64_t nun = count, ci = 0;
  while (nun > 1 && ci < maxc - 1) {
    g[ci + 1].clear();
    std::vector<int64_t> keep;
    keep.push_back(g[ci][0]);
    V3 ref = mesh.normal[g[ci][0]];
    for (size_t i = 1; i < g[ci].size(); i++) {
      int64_t t = g[ci][i];
      if (std::fabs(dot(ref, mesh.normal[t])) < fv) g[ci + 1].push_back(t);
      else keep.push_back(t);
    }
    g[ci] = keep;
    nun = (int64_t)g[ci + 1].size();
    if (nun >= 1) ci++;
  }
  g.resize(ci + 1);
  return g;
}

std::vector<std::pair<int64_t, int64_t>> normal_filtered_pivots(const Mesh& mesh,
                                                                const BlockInfo& b,
                                                                double angle, uint64_t seed,
                                                                uint64_t block_id) {
  double fv = std::cos(angle);
  auto rg = normal_groups(mesh, b.r0, b.m, fv);
  auto cg = normal_groups(mesh, b.c0, b.n, fv);
  std::vector<std::pair<int64_t, int64_t>> piv;
  int64_t nr = (int64_t)rg.size(), nc = (int64_t)cg.size();
  for (int64_t i = 0; i < nr; i++)
    for (int64_t j = 0; j < nc; j++) {
      uint64_t q = (uint64_t)(i * nc + j);
      int64_t a = (int64_t)(pivot_hash(seed, block_id, 2 * q + 1) % rg[i].size());
      int64_t c = (int64_t)(pivot_hash(seed, block_id, 2 * q + 2) % cg[j].size());
      piv.push_back({rg[i][a] - b.r0, cg[j][c] - b.c0});
    }
  return piv;
}

// ---------------------------------------------------------------------------
// Dense helpers: Householder QR and one-sided Jacobi SVD (textbook forms).
// ---------------------------------------------------------------------------
void householder_qr(int64_t m, int64_t k, std::vector<cd>& A, std::vector<cd>& Q,
                    std::vector<cd>& R) {
  // A: m x k col-major, overwritten. Q: m x p (p = min(m,k)), R: p x k.
  int64_t p = std::min(m, k);
  std::vector<std::vector<cd>> vs;
  for (int64_t j = 0; j < p; j++) {
    double xn = 0;
    for (int64_t i = j; i < m; i++) xn += std::norm(A[j * m + i]);
    xn = std::sqrt(xn);
    std::vector<cd> v(m - j);
    for (int64_t i = j; i < m; i++) v[i - j] = A[j * m + i];
    cd x0 = v[0];
    cd ph = (std::abs(x0) > 0) ? x0 / std::abs(x0) : cd(1.0, 0.0);
    cd alpha = -ph * xn;
    v[0] -= alpha;
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
    vs.push_back(std::move(v));
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

void jacobi_svd(int64_t n, std::vector<cd>& A, std::vector<double>& sigma,
                std::vector<cd>& U, std::vector<cd>& V) {
  // A: n x n col-major -> A = U diag(sigma) V^H, sigma descending.
  V.assign(n * n, 0.0);
  for (int64_t i = 0; i < n; i++) V[i * n + i] = 1.0;
  // columns below 1e-30 of the squared Frobenius norm (kept by the rotations)
  // are rounding noise and take no rotations: the relative test between two
  // of them never settles
  double fro = 0;
  for (int64_t i = 0; i < n * n; i++) fro += std::norm(A[i]);
  const double floor2 = 1e-30 * fro;
  for (int sweep = 0; sweep < 60; sweep++) {
    double off = 0;
    for (int64_t p = 0; p < n - 1; p++)
      for (int64_t q = p + 1; q < n; q++) {
        double al = 0, be = 0;
        cd ga = 0;
        for (int64_t i = 0; i < n; i++) {
          al += std::norm(A[p * n + i]);
          be += std::norm(A[q * n + i]);
          ga += std::conj(A[p * n + i]) * A[q * n + i];
        }
        double g = std::abs(ga);
        if (!(al > floor2) || !(be > floor2)) continue;
        if (g == 0.0 || g <= 1e-15 * std::sqrt(al * be)) continue;
        off = std::max(off, g / std::sqrt(al * be));
        cd e = ga / g;  // e^{i phi}
        double zeta = (be - al) / (2.0 * g);
        double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
        double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
        for (int64_t i = 0; i < n; i++) {
          cd ap = A[p * n + i], aq = A[q * n + i] * std::conj(e);
          A[p * n + i] = c * ap - s * aq;
          A[q * n + i] = s * ap + c * aq;
          cd vp = V[p * n + i], vq = V[q * n + i] * std::conj(e);
          V[p * n + i] = c * vp - s * vq;
          V[q * n + i] = s * vp + c * vq;
        }
      }
    if (off < 1e-15) break;
  }
  std::vector<double> sv(n);
  for (int64_t j = 0; j < n; j++) {
    double s = 0;
    for (int64_t i = 0; i < n; i++) s += std::norm(A[j * n + i]);
    sv[j] = std::sqrt(s);
  }
  std::vector<int64_t> ord(n);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return sv[a] > sv[b]; });
  sigma.resize(n);
  U.assign(n * n, 0.0);
  std::vector<cd> V2(n * n);
  for (int64_t jj = 0; jj < n; jj++) {
    int64_t j = ord[jj];
    sigma[jj] = sv[j];
    for (int64_t i = 0; i < n; i++) {
      U[jj * n + i] = sv[j] > 0 ? A[j * n + i] / sv[j] : (i == jj ? 1.0 : 0.0);
      V2[jj * n + i] = V[j * n + i];
    }
  }
  V = V2;
}

// minRankforError (golubReinschSVD.cpp:551-585).
int64_t min_rank_for_error(const std::vector<double>& sv, int64_t max_rank, double rel) {
  int64_t nz = (int64_t)sv.size();
  if (rel <= 0) return max_rank <= 0 ? nz : std::min(nz, max_rank);
  int64_t mi = nz;
  if (max_rank > 0) mi = std::min(max_rank, nz);
  double full = 0;
  for (double s : sv) full += s * s;
  double res = full, e2 = rel * rel;
  for (int64_t r = 1; r <= mi; r++) {
    res -= sv[r - 1] * sv[r - 1];
    if (res / full < e2) return r;
  }
  return mi;
}

// compressAdmissibleBlock (hmatrix.cpp:101-140): QR of U and of V^T, SVD of the
// small core R_A diag(s) R_B^T, truncate by minRankforError.
void recompress_block(HBlock& blk, int64_t rank, double tol) {
  if (!blk.info.adm) return;
  int64_t m = blk.info.m, n = blk.info.n, k = blk.rank;
  if (tol <= 0 && (k <= rank || rank <= 0)) return;
  std::vector<cd> A = blk.U, QA, RA;
  householder_qr(m, k, A, QA, RA);
  std::vector<cd> Bt(n * k);  // V^T: n x k col-major
  for (int64_t l = 0; l < k; l++)
    for (int64_t j = 0; j < n; j++) Bt[l * n + j] = blk.V[l * n + j];
  std::vector<cd> QB, RB;
  householder_qr(n, k, Bt, QB, RB);
  int64_t pa = std::min(m, k), pb = std::min(n, k);
  // core = RA (pa x k) * diag(s) * RB^T (k x pb), padded to square q x q
  int64_t q = std::max(pa, pb);
  std::vector<cd> C(q * q, 0.0);
  for (int64_t c = 0; c < pb; c++)
    for (int64_t r = 0; r < pa; r++) {
      cd acc = 0;
      for (int64_t l = 0; l < k; l++) acc += RA[l * pa + r] * blk.s[l] * RB[l * pb + c];
      C[c * q + r] = acc;
    }
  std::vector<double> sig;
  std::vector<cd> Uc, Vc;
  jacobi_svd(q, C, sig, Uc, Vc);
  int64_t r = min_rank_for_error(sig, rank, tol);
  if (r < 1) r = 1;
  std::vector<cd> U(m * r, 0.0), V(r * n, 0.0), s(r);
  for (int64_t l = 0; l < r; l++) {
    s[l] = sig[l];
    for (int64_t i = 0; i < m; i++) {
      cd acc = 0;
      for (int64_t t = 0; t < pa; t++) acc += QA[t * m + i] * Uc[l * q + t];
      U[l * m + i] = acc;
    }
    // VAdj row l = conj(Vc[:, l])^T * QB^T
    for (int64_t j = 0; j < n; j++) {
      cd acc = 0;
      for (int64_t t = 0; t < pb; t++) acc += std::conj(Vc[l * q + t]) * QB[t * n + j];
      V[l * n + j] = acc;
    }
  }
  blk.rank = r;
  blk.U = std::move(U);
  blk.V = std::move(V);
  blk.s = std::move(s);
}

}  // namespace orc
