// host_tree.cpp -- cluster tree, partition, element geometry and the flat index
// tables of the kernels. Compiled with -ffp-contract=off so the geometry and
// the near-singular classification are bit-identical to the device's.
#include "host_tree.h"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <stdexcept>

namespace bemgpu {

namespace {
struct BuildNode {
  std::vector<int64_t> idx;
  HBox box;
  int64_t son1 = -1, son2 = -1, level = 0;
  bool leaf = false;
};

HBox box_of(const std::vector<double>& p, const std::vector<int64_t>& idx) {
  HBox b;
  for (int d = 0; d < 3; d++) {
    b.lo[d] = INFINITY;
    b.hi[d] = -INFINITY;
  }
  for (int64_t i : idx)
    for (int d = 0; d < 3; d++) {
      b.lo[d] = std::min(b.lo[d], p[3 * i + d]);
      b.hi[d] = std::max(b.hi[d], p[3 * i + d]);
    }
  return b;
}

void split(std::vector<BuildNode>& nodes, int64_t id, const std::vector<double>& p, int64_t leaf) {
  if ((int64_t)nodes[id].idx.size() < leaf || nodes[id].idx.size() <= 1) {
    nodes[id].leaf = true;
    return;
  }
  const HBox box = nodes[id].box;
  double side[3];
  for (int d = 0; d < 3; d++) side[d] = box.hi[d] - box.lo[d];
  int ax = 0;
  for (int d = 1; d < 3; d++)
    if (std::fabs(side[d]) > std::fabs(side[ax])) ax = d;
  if (!(std::fabs(side[ax]) > 0.0)) {  // coincident midpoints cannot be split
    nodes[id].leaf = true;
    return;
  }
  HBox b1 = box;
  b1.lo[ax] = box.lo[ax] + 0.5 * side[ax];
  std::vector<int64_t> i1, i2;
  for (int64_t t : nodes[id].idx) {
    const double* m = &p[3 * t];
    bool in1 = (b1.hi[0] - m[0] >= 0 && b1.hi[1] - m[1] >= 0 && b1.hi[2] - m[2] >= 0) &&
               (b1.lo[0] - m[0] <= 0 && b1.lo[1] - m[1] <= 0 && b1.lo[2] - m[2] <= 0);
    (in1 ? i1 : i2).push_back(t);
  }
  const int64_t lvl = nodes[id].level;
  BuildNode s1, s2;
  s1.box = box_of(p, i1);
  s1.idx = std::move(i1);
  s1.level = lvl + 1;
  s2.box = box_of(p, i2);
  s2.idx = std::move(i2);
  s2.level = lvl + 1;
  int64_t id1 = (int64_t)nodes.size();
  nodes.push_back(std::move(s1));
  nodes[id].son1 = id1;
  split(nodes, id1, p, leaf);
  int64_t id2 = (int64_t)nodes.size();
  nodes.push_back(std::move(s2));
  nodes[id].son2 = id2;
  split(nodes, id2, p, leaf);
}

void renumber(std::vector<BuildNode>& nodes, int64_t id, int64_t& next, std::vector<int64_t>& perm,
              std::vector<int64_t>& start) {
  if (nodes[id].leaf) {
    start[id] = next;
    for (int64_t t : nodes[id].idx) perm[next++] = t;
  } else {
    renumber(nodes, nodes[id].son1, next, perm, start);
    renumber(nodes, nodes[id].son2, next, perm, start);
    start[id] = start[nodes[id].son1];
  }
}
}  // namespace

HTree build_tree(const std::vector<double>& pts, int64_t leaf) {
  HTree t;
  const int64_t n = (int64_t)pts.size() / 3;
  std::vector<BuildNode> nodes;
  BuildNode root;
  root.idx.resize(n);
  std::iota(root.idx.begin(), root.idx.end(), 0);
  root.box = box_of(pts, root.idx);
  nodes.push_back(std::move(root));
  split(nodes, 0, pts, leaf);
  t.perm.assign(n, 0);
  std::vector<int64_t> start(nodes.size(), 0);
  int64_t next = 0;
  renumber(nodes, 0, next, t.perm, start);
  t.c.resize(nodes.size());
  for (size_t i = 0; i < nodes.size(); i++) {
    HCluster& c = t.c[i];
    c.start = start[i];
    c.size = (int64_t)nodes[i].idx.size();
    c.son1 = nodes[i].son1;
    c.son2 = nodes[i].son2;
    c.level = nodes[i].level;
    c.leaf = nodes[i].leaf;
    c.box = nodes[i].box;
  }
  return t;
}

static double box_distance(const HBox& a, const HBox& b) {
  bool ov[3];
  for (int i = 0; i < 3; i++)
    ov[i] = (a.lo[i] < b.hi[i] && a.hi[i] > b.lo[i]) || (b.lo[i] < a.hi[i] && b.hi[i] > a.lo[i]);
  const int nov = ov[0] + ov[1] + ov[2];
  auto gap = [&](int i) { return std::min(std::fabs(a.lo[i] - b.hi[i]), std::fabs(b.lo[i] - a.hi[i])); };
  if (nov == 3) return 0.0;
  if (nov == 2) return !ov[0] ? gap(0) : (!ov[1] ? gap(1) : gap(2));
  if (nov == 1) {
    int i = ov[0] ? 1 : 0, j = ov[0] ? 2 : (ov[1] ? 2 : 1);
    double d1 = gap(i), d2 = gap(j);
    return std::sqrt(d1 * d1 + d2 * d2);
  }
  double dx = gap(0), dy = gap(1), dz = gap(2);
  return std::sqrt(dx * dx + dy * dy + dz * dz);
}

static double box_diameter(const HBox& a) {
  double dx = a.hi[0] - a.lo[0], dy = a.hi[1] - a.lo[1], dz = a.hi[2] - a.lo[2];
  return std::sqrt(dx * dx + dy * dy + dz * dz);
}

static void blocks_rec(const HTree& rt, const HTree& ct, int64_t r, int64_t c, double eta,
                       std::vector<HBlockDesc>& out) {
  const HCluster& R = rt.c[r];
  const HCluster& C = ct.c[c];
  double dist = box_distance(R.box, C.box);
  bool adm = false;
  if (dist != 0.0) adm = std::min(box_diameter(R.box), box_diameter(C.box)) / dist < eta;
  if (adm || R.leaf || C.leaf) {
    out.push_back({R.start, R.size, C.start, C.size, adm, r, c});
    return;
  }
  blocks_rec(rt, ct, R.son1, C.son1, eta, out);
  blocks_rec(rt, ct, R.son1, C.son2, eta, out);
  blocks_rec(rt, ct, R.son2, C.son1, eta, out);
  blocks_rec(rt, ct, R.son2, C.son2, eta, out);
}

std::vector<HBlockDesc> build_blocks(const HTree& rows, const HTree& cols, double eta) {
  std::vector<HBlockDesc> out;
  if (!rows.c.empty() && !cols.c.empty()) blocks_rec(rows, cols, 0, 0, eta, out);
  return out;
}

void prepare_elements(const double* tri, const std::vector<int64_t>& perm, std::vector<Elem>& E,
                      double& avgdim) {
  const int64_t n = (int64_t)perm.size();
  E.resize(n);
  double acc = 0;
  for (int64_t i = 0; i < n; i++) {
    const double* t = tri + 9 * perm[i];
    Elem& e = E[i];
    for (int d = 0; d < 3; d++) {
      e.n1[d] = t[d];
      e.n2[d] = t[3 + d];
      e.n3[d] = t[6 + d];
    }
    // normal: (n2 - n1) x (n3 - n1), normalised
    double a[3], b[3];
    for (int d = 0; d < 3; d++) {
      a[d] = e.n2[d] - e.n1[d];
      b[d] = e.n3[d] - e.n1[d];
    }
    double cx = a[1] * b[2] - a[2] * b[1], cy = a[2] * b[0] - a[0] * b[2],
           cz = a[0] * b[1] - a[1] * b[0];
    double cn = std::sqrt(cx * cx + cy * cy + cz * cz);
    e.nrm[0] = cx / cn;
    e.nrm[1] = cy / cn;
    e.nrm[2] = cz / cn;
    // centroid: (n1 + n2 + n3) / 3
    for (int d = 0; d < 3; d++) e.c[d] = ((e.n1[d] + e.n2[d]) + e.n3[d]) / 3.0;
    // area: |(n1 - n2) x (n1 - n3)| / 2
    double u[3], v[3];
    for (int d = 0; d < 3; d++) {
      u[d] = e.n1[d] - e.n2[d];
      v[d] = e.n1[d] - e.n3[d];
    }
    double x = u[1] * v[2] - u[2] * v[1], y = u[2] * v[0] - u[0] * v[2], z = u[0] * v[1] - u[1] * v[0];
    e.area = std::sqrt(x * x + y * y + z * z) / 2.0;
    acc += std::sqrt(e.area);
  }
  avgdim = n > 0 ? acc / n / 2.0 : 0.0;
}

bool host_near_pair(const Elem& P, const Elem& Q, double near_r) {
  double dx = P.c[0] - Q.c[0], dy = P.c[1] - Q.c[1], dz = P.c[2] - Q.c[2];
  double s = (dx * dx + dy * dy) + dz * dz;
  return std::sqrt(s) < near_r;
}

static void normal_groups(const std::vector<Elem>& E, int64_t start, int64_t count, double fv,
                          std::vector<std::vector<int64_t>>& g) {
  const int64_t maxc = 20;
  g.assign(maxc, {});
  for (int64_t i = 0; i < count; i++) g[0].push_back(start + i);
  int64_t nun = count, ci = 0;
  while (nun > 1 && ci < maxc - 1) {
    g[ci + 1].clear();
    std::vector<int64_t> keep{g[ci][0]};
    const double* ref = E[g[ci][0]].nrm;
    for (size_t i = 1; i < g[ci].size(); i++) {
      const double* nn = E[g[ci][i]].nrm;
      double d = ref[0] * nn[0] + ref[1] * nn[1] + ref[2] * nn[2];
      if (std::fabs(d) < fv) g[ci + 1].push_back(g[ci][i]);
      else keep.push_back(g[ci][i]);
    }
    g[ci] = keep;
    nun = (int64_t)g[ci + 1].size();
    if (nun >= 1) ci++;
  }
  g.resize(ci + 1);
}

void pivot_seeds(const std::vector<Elem>& E, const HBlockDesc& b, double angle, uint64_t seed,
                 uint64_t block_id, std::vector<int32_t>& out) {
  const double fv = std::cos(angle);
  std::vector<std::vector<int64_t>> rg, cg;
  normal_groups(E, b.r0, b.m, fv, rg);
  normal_groups(E, b.c0, b.n, fv, cg);
  const int64_t nr = (int64_t)rg.size(), nc = (int64_t)cg.size();
  for (int64_t i = 0; i < nr; i++)
    for (int64_t j = 0; j < nc; j++) {
      uint64_t q = (uint64_t)(i * nc + j);
      int64_t a = (int64_t)(pivot_hash(seed, block_id, 2 * q + 1) % rg[i].size());
      int64_t c = (int64_t)(pivot_hash(seed, block_id, 2 * q + 2) % cg[j].size());
      out.push_back((int32_t)(rg[i][a] - b.r0));
      out.push_back((int32_t)(cg[j][c] - b.c0));
    }
}

void build_layout(const HTree& rows, const HTree& cols, const std::vector<Elem>* E, double near_r,
                  double eta, int64_t kcap_default, int64_t max_rank, bool pivots, uint64_t seed,
                  Layout& L) {
  L = Layout();
  L.N = rows.perm.size();
  L.blocks = build_blocks(rows, cols, eta);
  const int64_t nb = (int64_t)L.blocks.size();
  // near / far split, in partition order
  std::vector<int64_t> near_idx(nb, -1), far_idx(nb, -1);
  for (int64_t i = 0; i < nb; i++) {
    const HBlockDesc& b = L.blocks[i];
    if (b.adm) {
      FarBlock f{};
      f.r0 = b.r0;
      f.c0 = b.c0;
      f.m = (int32_t)b.m;
      f.n = (int32_t)b.n;
      int64_t kc = std::min<int64_t>(std::min(b.m, b.n), kcap_default);
      if (max_rank > 0) kc = std::min(kc, max_rank);
      kc = std::min<int64_t>(kc, ACA_MAX_KCAP);
      f.kcap = (int32_t)std::max<int64_t>(kc, 1);
      f.uoff = L.u_size;
      f.voff = L.v_size;
      f.soff = L.s_size;
      f.id = (int32_t)i;
      L.u_size += (int64_t)f.kcap * b.m;
      L.v_size += (int64_t)f.kcap * b.n;
      L.s_size += f.kcap;
      far_idx[i] = (int64_t)L.far.size();
      L.far.push_back(f);
    } else {
      NearBlock nbk{};
      nbk.r0 = b.r0;
      nbk.c0 = b.c0;
      nbk.m = (int32_t)b.m;
      nbk.n = (int32_t)b.n;
      nbk.off = L.near_entries;
      L.near_entries += b.m * b.n;
      near_idx[i] = (int64_t)L.near.size();
      L.near.push_back(nbk);
    }
  }
  // ACA launch order: largest blocks first
  L.far_order.resize(L.far.size());
  std::iota(L.far_order.begin(), L.far_order.end(), 0);
  std::stable_sort(L.far_order.begin(), L.far_order.end(), [&](int32_t a, int32_t b) {
    return (int64_t)L.far[a].m + L.far[a].n > (int64_t)L.far[b].m + L.far[b].n;
  });
  L.nbig = 0;
  while (L.nbig < (int64_t)L.far_order.size() &&
         (int64_t)L.far[L.far_order[L.nbig]].m + L.far[L.far_order[L.nbig]].n >= ACA_BIG_MN)
    L.nbig++;
  // near-field tiles of <= 256 entries
  for (size_t bi = 0; bi < L.near.size(); bi++) {
    const int64_t cnt = (int64_t)L.near[bi].m * L.near[bi].n;
    for (int64_t f = 0; f < cnt; f += 256)
      L.tiles.push_back({(int32_t)bi, (int32_t)f, (int32_t)std::min<int64_t>(256, cnt - f), 0});
  }
  // special entries (singular and near-singular) of the near field
  L.special_bits.assign((L.near_entries + 31) / 32, 0u);
  if (E) {
    std::vector<std::pair<int64_t, std::pair<int32_t, int32_t>>> sing, nsing;
    for (const NearBlock& b : L.near)
      for (int c = 0; c < b.n; c++)
        for (int r = 0; r < b.m; r++) {
          const int64_t row = b.r0 + r, col = b.c0 + c;
          const int64_t g = b.off + (int64_t)c * b.m + r;
          if (row == col) sing.push_back({g, {(int32_t)row, (int32_t)col}});
          else if (host_near_pair((*E)[row], (*E)[col], near_r))
            nsing.push_back({g, {(int32_t)row, (int32_t)col}});
          else continue;
          L.special_bits[g >> 5] |= 1u << (g & 31);
        }
    for (auto* v : {&sing, &nsing})
      for (auto& e : *v) {
        L.sp_entry.push_back(e.first);
        L.sp_row.push_back(e.second.first);
        L.sp_col.push_back(e.second.second);
      }
  }
  // leaf row lists for the matvec U pass
  std::vector<int64_t> leaf_of_row(L.N, -1);
  for (const HCluster& c : rows.c)
    if (c.leaf && c.size > 0) {
      for (int64_t i = c.start; i < c.start + c.size; i++) leaf_of_row[i] = (int64_t)L.leaves.size();
      L.leaves.push_back({c.start, (int32_t)c.size, 0});
    }
  std::sort(L.leaves.begin(), L.leaves.end(),
            [](const LeafRows& a, const LeafRows& b) { return a.start < b.start; });
  for (int64_t i = 0; i < (int64_t)L.leaves.size(); i++)
    for (int64_t r = L.leaves[i].start; r < L.leaves[i].start + L.leaves[i].size; r++) leaf_of_row[r] = i;
  std::vector<std::vector<int32_t>> per_leaf(L.leaves.size());
  for (int64_t i = 0; i < nb; i++) {
    const HBlockDesc& b = L.blocks[i];
    if (b.m == 0) continue;
    int64_t l0 = leaf_of_row[b.r0], l1 = leaf_of_row[b.r0 + b.m - 1];
    int32_t code = b.adm ? (int32_t)far_idx[i] : (int32_t)(-near_idx[i] - 1);
    for (int64_t l = l0; l <= l1; l++) per_leaf[l].push_back(code);
  }
  L.list_off.assign(L.leaves.size() + 1, 0);
  for (size_t l = 0; l < per_leaf.size(); l++) {
    L.list_off[l + 1] = L.list_off[l] + (int32_t)per_leaf[l].size();
    L.list.insert(L.list.end(), per_leaf[l].begin(), per_leaf[l].end());
  }
  // ACAextra pivot seeds
  L.piv_off.assign(L.far.size(), 0);
  L.piv_cnt.assign(L.far.size(), 0);
  if (pivots && E) {
    std::vector<int32_t> buf;
    for (size_t fi = 0; fi < L.far.size(); fi++) {
      buf.clear();
      pivot_seeds(*E, L.blocks[L.far[fi].id], 0.44, seed, (uint64_t)L.far[fi].id, buf);
      L.piv_off[fi] = (int64_t)L.piv_rc.size() / 2;
      L.piv_cnt[fi] = (int32_t)(buf.size() / 2);
      L.piv_rc.insert(L.piv_rc.end(), buf.begin(), buf.end());
    }
  }
}

// Gauss-Legendre nodes (ascending) and weights on [-1, 1] by Newton iteration
// on the Legendre recurrence.
void gauss_legendre(int n, double* x, double* w) {
  const double PI = 3.14159265358979323846;
  for (int i = 0; i < n; i++) {
    double z = std::cos(PI * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; k++) {
        double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = pk;
      }
      double dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= n; k++) {
      double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = pk;
    }
    double dp = n * (z * p1 - p0) / (z * z - 1.0);
    x[n - 1 - i] = z;
    w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

// 16-point Dunavant rule (order 8) in the point order of
// trianglequadraturerules.cpp:91-110.
QuadRules make_rules() {
  QuadRules R{};
  static const double t8[16][3] = {
      {0.33333333333333, 0.33333333333333, 0.14431560767779},
      {0.45929258829272, 0.45929258829272, 0.09509163426728},
      {0.45929258829272, 0.08141482341455, 0.09509163426728},
      {0.08141482341455, 0.45929258829272, 0.09509163426728},
      {0.17056930775176, 0.17056930775176, 0.10321737053472},
      {0.17056930775176, 0.65886138449648, 0.10321737053472},
      {0.65886138449648, 0.17056930775176, 0.10321737053472},
      {0.05054722831703, 0.05054722831703, 0.03245849762320},
      {0.05054722831703, 0.89890554336594, 0.03245849762320},
      {0.89890554336594, 0.05054722831703, 0.03245849762320},
      {0.26311282963464, 0.72849239295540, 0.02723031417443},
      {0.72849239295540, 0.00839477740996, 0.02723031417443},
      {0.00839477740996, 0.26311282963464, 0.02723031417443},
      {0.72849239295540, 0.26311282963464, 0.02723031417443},
      {0.26311282963464, 0.00839477740996, 0.02723031417443},
      {0.00839477740996, 0.72849239295540, 0.02723031417443}};
  for (int i = 0; i < 16; i++) {
    R.reg_x1[i] = t8[i][0];
    R.reg_x2[i] = t8[i][1];
    R.reg_w[i] = t8[i][2];
    R.freg_x1[i] = (float)t8[i][0];
    R.freg_x2[i] = (float)t8[i][1];
    R.freg_w[i] = (float)t8[i][2];
  }
  gauss_legendre(5, R.line_x, R.line_w);
  double x32[32], w32[32];
  gauss_legendre(32, x32, w32);
  for (int i = 0; i < 16; i++) {
    R.gl_x[i] = x32[16 + i];
    R.gl_w[i] = w32[16 + i];
  }
  return R;
}

}  // namespace bemgpu
