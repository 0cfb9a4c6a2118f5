// bem_oracle.cpp -- C API of the CPU FP64 oracle (test infrastructure only).
#include "bem_oracle.h"

#include <omp.h>

#include <chrono>
#include <cstring>
#include <memory>

#include "oracle_core.hpp"

using namespace orc;

struct orc_problem {
  Mesh mesh;
  ClusterTree tree;
  std::vector<BlockInfo> blocks;
  Mesh refl;              // impedance plane: reflected elements (cluster order)
  bool has_refl = false;
  std::vector<double> src;  // point sources, rows x, y, z, Re w, Im w
  const Mesh* reflected() const { return has_refl ? &refl : nullptr; }
};

struct orc_hmatrix {
  int64_t nrows = 0, ncols = 0;
  std::vector<HBlock> blk;
};

static inline const cd* C(const double* p) { return reinterpret_cast<const cd*>(p); }
static inline cd* C(double* p) { return reinterpret_cast<cd*>(p); }

extern "C" {

orc_problem* orc_create(const double* tri, int64_t n, int64_t leaf, double eta) {
  auto* p = new orc_problem();
  // midpoints in caller order -> cluster tree (ClusterTree(BoundaryElements*),
  // clustertree.h:77-86 computes triangleMidpoint first)
  std::vector<V3> mids(n);
  for (int64_t i = 0; i < n; i++) {
    const double* t = tri + 9 * i;
    V3 s = (V3(t[0], t[1], t[2]) + V3(t[3], t[4], t[5])) + V3(t[6], t[7], t[8]);
    mids[i] = V3(s.x / 3.0, s.y / 3.0, s.z / 3.0);
  }
  p->tree = build_cluster_tree(mids, leaf);
  p->mesh.tri.resize(n);
  for (int64_t i = 0; i < n; i++) {
    const double* t = tri + 9 * p->tree.perm[i];
    p->mesh.tri[i] = {V3(t[0], t[1], t[2]), V3(t[3], t[4], t[5]), V3(t[6], t[7], t[8])};
  }
  mesh_prepare(p->mesh);
  p->blocks = build_partition(p->tree, p->tree, eta);
  return p;
}

void orc_set_sources(orc_problem* p, const double* src, int64_t nsrc) {
  p->src.assign(src, src + (nsrc > 0 ? 5 * nsrc : 0));
}

void orc_set_plane(orc_problem* p, const double* point, const double* normal) {
  if (!normal || (normal[0] == 0 && normal[1] == 0 && normal[2] == 0)) {
    p->has_refl = false;
    return;
  }
  p->refl = reflect_mesh(p->mesh, V3(point[0], point[1], point[2]),
                         V3(normal[0], normal[1], normal[2]));
  p->has_refl = true;
}

void orc_destroy(orc_problem* p) { delete p; }
int64_t orc_n(const orc_problem* p) { return p->mesh.n; }
void orc_perm(const orc_problem* p, int64_t* perm) {
  std::memcpy(perm, p->tree.perm.data(), sizeof(int64_t) * p->tree.perm.size());
}
int64_t orc_num_clusters(const orc_problem* p) { return (int64_t)p->tree.c.size(); }
void orc_clusters(const orc_problem* p, int64_t* info, double* boxes) {
  for (size_t i = 0; i < p->tree.c.size(); i++) {
    const Cluster& c = p->tree.c[i];
    int64_t* o = info + 6 * i;
    o[0] = c.start; o[1] = c.size; o[2] = c.son1; o[3] = c.son2; o[4] = c.level; o[5] = c.leaf;
    double* b = boxes + 6 * i;
    for (int d = 0; d < 3; d++) { b[d] = c.box.lo[d]; b[3 + d] = c.box.hi[d]; }
  }
}
int64_t orc_num_blocks(const orc_problem* p) { return (int64_t)p->blocks.size(); }
void orc_blocks(const orc_problem* p, int64_t* info) {
  for (size_t i = 0; i < p->blocks.size(); i++) {
    const BlockInfo& b = p->blocks[i];
    int64_t* o = info + 5 * i;
    o[0] = b.r0; o[1] = b.m; o[2] = b.c0; o[3] = b.n; o[4] = b.adm;
  }
}
void orc_geometry(const orc_problem* p, double* normals, double* areas, double* colloc,
                  double* avgdim) {
  const Mesh& m = p->mesh;
  for (int64_t i = 0; i < m.n; i++) {
    for (int d = 0; d < 3; d++) {
      if (normals) normals[3 * i + d] = m.normal[i][d];
      if (colloc) colloc[3 * i + d] = m.colloc[i][d];
    }
    if (areas) areas[i] = m.area[i];
  }
  if (avgdim) *avgdim = m.avgdim;
}

void orc_operators(const orc_problem* p, double k, const int64_t* rows, const int64_t* cols,
                   int64_t cnt, double* out) {
  OperatorCtx ctx(&p->mesh, k, p->reflected());
  cd* o = C(out);
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t e = 0; e < cnt; e++) {
    Ops r = ctx.eval(rows[e], cols[e]);
    o[4 * e + 0] = r.L;
    o[4 * e + 1] = r.M;
    o[4 * e + 2] = r.Mt;
    o[4 * e + 3] = r.N;
  }
}

void orc_entries(const orc_problem* p, double k, int coupling, const double* a,
                 const double* b, const int64_t* rows, const int64_t* cols, int64_t cnt,
                 double* phi, double* dphi) {
  OperatorCtx ctx(&p->mesh, k, p->reflected());
  Coupling cp = coupling_parameter(coupling, k);
  EntryGen g{&ctx, cp.alpha, cp.alpha_half, C(a), C(b), 0};
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t e = 0; e < cnt; e++) {
    cd x, y;
    g.both(rows[e], cols[e], x, y);
    if (phi) C(phi)[e] = x;
    if (dphi) C(dphi)[e] = y;
  }
}

static orc_hmatrix* assemble(const std::vector<BlockInfo>& blocks, int64_t nr, int64_t nc,
                             const EntryFn& f, const Mesh* mesh_for_pivots, double tol,
                             int64_t max_rank, uint64_t seed, int nthreads) {
  auto* h = new orc_hmatrix();
  h->nrows = nr;
  h->ncols = nc;
  h->blk.resize(blocks.size());
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
  // blocks as independent tasks (hmatrix.cpp:793-846 uses omp tasks)
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (int64_t i = 0; i < (int64_t)blocks.size(); i++) {
    HBlock& b = h->blk[i];
    b.info = blocks[i];
    if (b.info.adm) {
      if (mesh_for_pivots) {
        auto piv = normal_filtered_pivots(*mesh_for_pivots, b.info, 0.44, seed, (uint64_t)i);
        aca_partial_pivot_extra(b, max_rank, tol, f, piv);
      } else {
        aca_partial_pivot(b, max_rank, tol, f, seed, (uint64_t)i);
      }
    } else {  // fullRankAssembly (hmatrix.cpp:350-374)
      b.full.resize(b.info.m * b.info.n);
      for (int64_t c = 0; c < b.info.n; c++)
        for (int64_t r = 0; r < b.info.m; r++)
          b.full[c * b.info.m + r] = f(b.info.r0 + r, b.info.c0 + c);
    }
  }
  return h;
}

orc_hmatrix* orc_hassemble(const orc_problem* p, double k, int coupling, const double* a,
                           const double* b, int which, double tol, int64_t max_rank,
                           uint64_t seed, int nthreads) {
  OperatorCtx ctx(&p->mesh, k, p->reflected());
  Coupling cp = coupling_parameter(coupling, k);
  EntryGen g{&ctx, cp.alpha, cp.alpha_half, C(a), C(b), which};
  EntryFn f = [&g](int64_t r, int64_t c) { return g(r, c); };
  return assemble(p->blocks, p->mesh.n, p->mesh.n, f, which == 1 ? &p->mesh : nullptr, tol,
                  max_rank, seed, nthreads);
}

void orc_hdestroy(orc_hmatrix* h) { delete h; }

// HArithm::MVM (harithm.cpp:3-28): y += sum over blocks; per-thread partial
// sums replace the omp critical scatter.
void orc_hmatvec(const orc_hmatrix* h, const double* xd, double* yd) {
  const cd* x = C(xd);
  cd* y = C(yd);
  int nt = omp_get_max_threads();
  std::vector<std::vector<cd>> part(nt, std::vector<cd>(h->nrows, 0.0));
#pragma omp parallel num_threads(nt)
  {
    std::vector<cd>& acc = part[omp_get_thread_num()];
    std::vector<cd> t;
#pragma omp for schedule(dynamic, 4)
    for (int64_t bi = 0; bi < (int64_t)h->blk.size(); bi++) {
      const HBlock& b = h->blk[bi];
      int64_t m = b.info.m, n = b.info.n;
      if (b.info.adm) {
        int64_t k = b.rank;
        t.assign(k, 0.0);
        for (int64_t l = 0; l < k; l++) {
          cd s = 0;
          const cd* v = &b.V[l * n];
          for (int64_t j = 0; j < n; j++) s += v[j] * x[b.info.c0 + j];
          t[l] = s * b.s[l];
        }
        for (int64_t l = 0; l < k; l++) {
          const cd* u = &b.U[l * m];
          for (int64_t i = 0; i < m; i++) acc[b.info.r0 + i] += u[i] * t[l];
        }
      } else {
        for (int64_t j = 0; j < n; j++) {
          cd xv = x[b.info.c0 + j];
          const cd* f = &b.full[j * m];
          for (int64_t i = 0; i < m; i++) acc[b.info.r0 + i] += f[i] * xv;
        }
      }
    }
  }
  for (int64_t i = 0; i < h->nrows; i++) {
    cd s = 0;
    for (int ti = 0; ti < nt; ti++) s += part[ti][i];
    y[i] += s;
  }
}

void orc_hdense(const orc_hmatrix* h, double* out) {
  cd* o = C(out);
  int64_t N = h->nrows;
  for (const HBlock& b : h->blk) {
    int64_t m = b.info.m, n = b.info.n;
    for (int64_t c = 0; c < n; c++)
      for (int64_t r = 0; r < m; r++) {
        cd v;
        if (b.info.adm) {
          v = 0;
          for (int64_t l = 0; l < b.rank; l++) v += b.U[l * m + r] * b.s[l] * b.V[l * n + c];
        } else {
          v = b.full[c * m + r];
        }
        o[(b.info.c0 + c) * N + b.info.r0 + r] = v;
      }
  }
}

void orc_hranks(const orc_hmatrix* h, int64_t* ranks) {
  for (size_t i = 0; i < h->blk.size(); i++) ranks[i] = h->blk[i].info.adm ? h->blk[i].rank : -1;
}

int64_t orc_hblock(const orc_hmatrix* h, int64_t bi, double* U, double* s, double* V,
                   double* full) {
  const HBlock& b = h->blk[bi];
  if (b.info.adm) {
    if (U) std::memcpy(U, b.U.data(), sizeof(cd) * b.U.size());
    if (s) std::memcpy(s, b.s.data(), sizeof(cd) * b.s.size());
    if (V) std::memcpy(V, b.V.data(), sizeof(cd) * b.V.size());
    return b.rank;
  }
  if (full) std::memcpy(full, b.full.data(), sizeof(cd) * b.full.size());
  return -1;
}

void orc_hrecompress(orc_hmatrix* h, int64_t rank, double tol) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i = 0; i < (int64_t)h->blk.size(); i++) recompress_block(h->blk[i], rank, tol);
}

orc_hmatrix* orc_hassemble_points(const double* rowpts, int64_t nr, const double* colpts,
                                  int64_t nc, double k, int64_t leaf, double eta, double tol,
                                  int64_t max_rank, uint64_t seed, int64_t* rowperm,
                                  int64_t* colperm) {
  std::vector<V3> rp(nr), cp(nc);
  for (int64_t i = 0; i < nr; i++) rp[i] = V3(rowpts[3 * i], rowpts[3 * i + 1], rowpts[3 * i + 2]);
  for (int64_t i = 0; i < nc; i++) cp[i] = V3(colpts[3 * i], colpts[3 * i + 1], colpts[3 * i + 2]);
  ClusterTree rt = build_cluster_tree(rp, leaf), ct = build_cluster_tree(cp, leaf);
  std::vector<V3> rps(nr), cps(nc);
  for (int64_t i = 0; i < nr; i++) rps[i] = rp[rt.perm[i]];
  for (int64_t i = 0; i < nc; i++) cps[i] = cp[ct.perm[i]];
  if (rowperm) std::memcpy(rowperm, rt.perm.data(), sizeof(int64_t) * nr);
  if (colperm) std::memcpy(colperm, ct.perm.data(), sizeof(int64_t) * nc);
  auto blocks = build_partition(rt, ct, eta);
  // Tests/tests.h:30-42: exp(ikr)/(4 pi r), 1 at r = 0
  EntryFn f = [&](int64_t r, int64_t c) -> cd {
    double d = norm(rps[r] - cps[c]);
    if (d == 0.0) return 1.0;
    return std::exp(cd(0.0, k * d)) / (PI4 * d);
  };
  return assemble(blocks, nr, nc, f, nullptr, tol, max_rank, seed, 0);
}

// GMRES(m) of Saad & Schultz (1986) with CGS2 Arnoldi and complex Givens
// rotations; the tolerance is on ||b - A x|| / ||b|| as in Eigen's GMRES used
// by gmres.h:170-207.
using MatVec = std::function<void(const std::vector<cd>&, std::vector<cd>&)>;

static int64_t gmres_core(int64_t n, const MatVec& A, const std::vector<cd>& b, std::vector<cd>& x,
                          double tol, int64_t restart, int64_t maxit, double* rel) {
  auto nrm = [](const std::vector<cd>& v) {
    double s = 0;
    for (auto& z : v) s += std::norm(z);
    return std::sqrt(s);
  };
  double bn = nrm(b);
  if (bn == 0.0) {
    std::fill(x.begin(), x.end(), cd(0.0));
    if (rel) *rel = 0;
    return 0;
  }
  std::vector<cd> r(n), w(n);
  int64_t it = 0;
  double res = 0;
  while (true) {
    A(x, w);
    for (int64_t i = 0; i < n; i++) r[i] = b[i] - w[i];
    double beta = nrm(r);
    res = beta / bn;
    if (res < tol || it >= maxit) break;
    int64_t m = restart;
    std::vector<std::vector<cd>> V;
    V.push_back(r);
    for (auto& z : V[0]) z /= beta;
    std::vector<std::vector<cd>> H(m + 1, std::vector<cd>(m, 0.0));
    std::vector<cd> cs(m), sn(m), g(m + 1, 0.0);
    g[0] = beta;
    int64_t j = 0;
    bool done = false;
    for (; j < m && it < maxit; j++) {
      A(V[j], w);
      std::vector<cd> h(j + 2, 0.0);
      for (int pass = 0; pass < 2; pass++) {
        std::vector<cd> hp(j + 1, 0.0);
        for (int64_t q = 0; q <= j; q++) {
          cd s = 0;
          for (int64_t i = 0; i < n; i++) s += std::conj(V[q][i]) * w[i];
          hp[q] = s;
        }
        for (int64_t q = 0; q <= j; q++)
          for (int64_t i = 0; i < n; i++) w[i] -= hp[q] * V[q][i];
        for (int64_t q = 0; q <= j; q++) h[q] += hp[q];
      }
      double hn = nrm(w);
      h[j + 1] = hn;
      for (int64_t q = 0; q < j; q++) {  // previous rotations
        cd a = h[q], bb = h[q + 1];
        h[q] = cs[q] * a + sn[q] * bb;
        h[q + 1] = -std::conj(sn[q]) * a + cs[q] * bb;
      }
      cd a = h[j], bb = h[j + 1];
      double rho = std::sqrt(std::norm(a) + std::norm(bb));
      if (std::abs(a) == 0.0) {
        cs[j] = 0.0;
        sn[j] = 1.0;
      } else {
        cs[j] = std::abs(a) / rho;
        sn[j] = (a / std::abs(a)) * std::conj(bb) / rho;
      }
      h[j] = cs[j] * a + sn[j] * bb;
      h[j + 1] = 0.0;
      g[j + 1] = -std::conj(sn[j]) * g[j];
      g[j] = cs[j] * g[j];
      for (int64_t q = 0; q <= j; q++) H[q][j] = h[q];
      it++;
      res = std::abs(g[j + 1]) / bn;
      if (hn > 0) {
        std::vector<cd> vn(n);
        for (int64_t i = 0; i < n; i++) vn[i] = w[i] / hn;
        V.push_back(std::move(vn));
      }
      if (res < tol || hn == 0.0) {
        j++;
        done = true;
        break;
      }
    }
    // back-substitution H y = g, x += V y
    int64_t kk = j;
    std::vector<cd> y(kk);
    for (int64_t q = kk - 1; q >= 0; q--) {
      cd s = g[q];
      for (int64_t t = q + 1; t < kk; t++) s -= H[q][t] * y[t];
      y[q] = s / H[q][q];
    }
    for (int64_t q = 0; q < kk; q++)
      for (int64_t i = 0; i < n; i++) x[i] += y[q] * V[q][i];
    if (done) {
      A(x, w);
      for (int64_t i = 0; i < n; i++) r[i] = b[i] - w[i];
      res = nrm(r) / bn;
      if (res < tol) break;
    }
    if (it >= maxit) {
      A(x, w);
      for (int64_t i = 0; i < n; i++) r[i] = b[i] - w[i];
      res = nrm(r) / bn;
      break;
    }
  }
  if (rel) *rel = res;
  return it;
}

int64_t orc_gmres(const orc_hmatrix* h, const double* b, double* x, double tol, int64_t restart,
                  int64_t maxit, double* rel_resid) {
  int64_t n = h->nrows;
  std::vector<cd> bv(C(b), C(b) + n), xv(C(x), C(x) + n);
  MatVec A = [h, n](const std::vector<cd>& in, std::vector<cd>& out) {
    std::fill(out.begin(), out.end(), cd(0.0));
    orc_hmatvec(h, reinterpret_cast<const double*>(in.data()), reinterpret_cast<double*>(out.data()));
  };
  int64_t it = gmres_core(n, A, bv, xv, tol, restart, maxit, rel_resid);
  std::memcpy(x, xv.data(), sizeof(cd) * n);
  return it;
}

// Flat block-triangular solves equivalent to the recursions
// forwardSubstitution / backwardSubstitution (harithm.cpp:1314-1412): an
// off-diagonal leaf is applied once every unknown of its column range is
// known and before any diagonal leaf of its row range is solved.
namespace {
struct Leaf {
  int64_t r0, m, c0, n, kind, rank, off;
};
std::vector<Leaf> leaves(int64_t nblk, const int64_t* b) {
  std::vector<Leaf> L(nblk);
  for (int64_t i = 0; i < nblk; i++) {
    const int64_t* o = b + 7 * i;
    L[i] = {o[0], o[1], o[2], o[3], o[4], o[5], o[6]};
  }
  return L;
}
void apply_sub(const Leaf& lf, const cd* data, const cd* x, cd* y) {  // y -= B x
  if (lf.kind == 0) {
    for (int64_t j = 0; j < lf.n; j++)
      for (int64_t i = 0; i < lf.m; i++) y[lf.r0 + i] -= data[lf.off + j * lf.m + i] * x[lf.c0 + j];
  } else {
    const cd* U = data + lf.off;
    const cd* V = U + lf.m * lf.rank;
    for (int64_t l = 0; l < lf.rank; l++) {
      cd t = 0;
      for (int64_t j = 0; j < lf.n; j++) t += V[l * lf.n + j] * x[lf.c0 + j];
      for (int64_t i = 0; i < lf.m; i++) y[lf.r0 + i] -= U[l * lf.m + i] * t;
    }
  }
}
}  // namespace

void orc_lower_solve(int64_t n, int64_t nblk, const int64_t* blocks, const double* data,
                     const double* b, double* y) {
  auto L = leaves(nblk, blocks);
  const cd* D = C(data);
  std::vector<cd> w(C(b), C(b) + n);
  cd* Y = C(y);
  std::vector<Leaf> diag, off;
  for (auto& l : L) (l.kind >= 2 ? diag : off).push_back(l);
  std::sort(diag.begin(), diag.end(), [](const Leaf& a, const Leaf& c) { return a.r0 < c.r0; });
  std::stable_sort(off.begin(), off.end(), [](const Leaf& a, const Leaf& c) { return a.r0 < c.r0; });
  size_t op = 0;
  for (const Leaf& d : diag) {
    while (op < off.size() && off[op].r0 <= d.r0) apply_sub(off[op++], D, Y, w.data());
    // leaf: y = Q^H w (QR leaves, harithm.cpp:1324-1327)
    for (int64_t i = 0; i < d.m; i++) {
      cd s = 0;
      for (int64_t t = 0; t < d.m; t++) s += std::conj(D[d.off + i * d.m + t]) * w[d.r0 + t];
      Y[d.r0 + i] = s;
    }
  }
}

void orc_upper_solve(int64_t n, int64_t nblk, const int64_t* blocks, const double* data,
                     const double* yv, double* x) {
  auto L = leaves(nblk, blocks);
  const cd* D = C(data);
  std::vector<cd> w(C(yv), C(yv) + n);
  cd* X = C(x);
  std::vector<Leaf> diag, off;
  for (auto& l : L) (l.kind >= 2 ? diag : off).push_back(l);
  std::sort(diag.begin(), diag.end(), [](const Leaf& a, const Leaf& c) { return a.r0 > c.r0; });
  std::stable_sort(off.begin(), off.end(),
                   [](const Leaf& a, const Leaf& c) { return a.r0 + a.m > c.r0 + c.m; });
  size_t op = 0;
  for (const Leaf& d : diag) {
    while (op < off.size() && off[op].r0 + off[op].m >= d.r0 + d.m) apply_sub(off[op++], D, X, w.data());
    // leaf: solve R x = w (harithm.cpp:1396-1399)
    for (int64_t i = d.m - 1; i >= 0; i--) {
      cd s = w[d.r0 + i];
      for (int64_t t = i + 1; t < d.m; t++) s -= D[d.off + t * d.m + i] * X[d.r0 + t];
      X[d.r0 + i] = s / D[d.off + i * d.m + i];
    }
  }
}

// H-LU factors of an assembled H-matrix (hlu.cpp): flat leaf lists of L and U
// in the format of orc_lower_solve / orc_upper_solve.
struct orc_hlu {
  std::vector<int64_t> Ll, Ul;
  std::vector<cd> Ld, Ud;
};

orc_hlu* orc_hlu_factor(const orc_problem* p, const orc_hmatrix* h, int64_t rank, double tol) {
  auto* f = new orc_hlu();
  hlu_factor_blocks(p->tree, h->blk, rank, tol, f->Ll, f->Ld, f->Ul, f->Ud);
  return f;
}

void orc_hlu_sizes(const orc_hlu* f, int64_t* out) {
  out[0] = (int64_t)f->Ll.size() / 7;
  out[1] = (int64_t)f->Ld.size();
  out[2] = (int64_t)f->Ul.size() / 7;
  out[3] = (int64_t)f->Ud.size();
}

void orc_hlu_get(const orc_hlu* f, int64_t* Ll, double* Ld, int64_t* Ul, double* Ud) {
  if (Ll) std::memcpy(Ll, f->Ll.data(), f->Ll.size() * sizeof(int64_t));
  if (Ld) std::memcpy(Ld, f->Ld.data(), f->Ld.size() * sizeof(cd));
  if (Ul) std::memcpy(Ul, f->Ul.data(), f->Ul.size() * sizeof(int64_t));
  if (Ud) std::memcpy(Ud, f->Ud.data(), f->Ud.size() * sizeof(cd));
}

void orc_hlu_free(orc_hlu* f) { delete f; }

// hMatrixSolve (boundaryelementsolver.cpp:526-744): phi H-matrix by ACA,
// rhs = phi * g, dPhi H-matrix by ACAextra, GMRES (with precond_rank >= 1:
// the H-LU preconditioner of the dPhi matrix truncated to that rank, initial
// guess (LU)^{-1} rhs and GMRES on (LU)^{-1} A x = (LU)^{-1} rhs,
// :657-700 and GMRES::gmresLUPreconditionedSolve, gmres.h:191-207), BC
// back-substitution (:729-740), p = i rho omega phi (:2251-2261).
int orc_solve_precond(const orc_problem* p, double freq, double c, double rho, int coupling,
                      const double* a_in, const double* b_in, const double* g_in, int64_t R,
                      double aca_tol, int64_t max_rank, double gmres_tol, int64_t restart,
                      int64_t maxit, uint64_t seed, int nthreads, int64_t precond_rank,
                      double precond_tol, double* phi_out, double* dphi_out, double* p_out,
                      double* stats);

// The unpreconditioned solve.
int orc_solve(const orc_problem* p, double freq, double c, double rho, int coupling,
              const double* a_in, const double* b_in, const double* g_in, int64_t R,
              double aca_tol, int64_t max_rank, double gmres_tol, int64_t restart,
              int64_t maxit, uint64_t seed, int nthreads, double* phi_out, double* dphi_out,
              double* p_out, double* stats) {
  return orc_solve_precond(p, freq, c, rho, coupling, a_in, b_in, g_in, R, aca_tol, max_rank,
                           gmres_tol, restart, maxit, seed, nthreads, 0, 0.0, phi_out, dphi_out,
                           p_out, stats);
}

int orc_solve_precond(const orc_problem* p, double freq, double c, double rho, int coupling,
                      const double* a_in, const double* b_in, const double* g_in, int64_t R,
                      double aca_tol, int64_t max_rank, double gmres_tol, int64_t restart,
                      int64_t maxit, uint64_t seed, int nthreads, int64_t precond_rank,
                      double precond_tol, double* phi_out, double* dphi_out, double* p_out,
                      double* stats) {
  using clk = std::chrono::steady_clock;
  auto t0 = clk::now();
  if (nthreads > 0) omp_set_num_threads(nthreads);
  int64_t N = p->mesh.n;
  const auto& perm = p->tree.perm;
  std::vector<cd> a(N), b(N), g(N * R);
  for (int64_t i = 0; i < N; i++) {
    a[i] = C(a_in)[perm[i]];
    b[i] = C(b_in)[perm[i]];
    for (int64_t r = 0; r < R; r++) g[r * N + i] = C(g_in)[r * N + perm[i]];
  }
  double k = 2.0 * PI * freq / c;
  auto secs = [](clk::time_point s, clk::time_point e) {
    return std::chrono::duration<double>(e - s).count();
  };
  auto t1 = clk::now();
  orc_hmatrix* hphi = orc_hassemble(p, k, coupling, (double*)a.data(), (double*)b.data(), 0,
                                    aca_tol, max_rank, seed, nthreads);
  auto t2 = clk::now();
  // rhs = sourceTermVector + phi g (boundaryelementsolver.cpp:578-579); the
  // source term of each collocation point restates sourceTerm (:3431-3441),
  // whose derivative factor divides by (ikr - 1) as written there
  std::vector<cd> rhs(N * R, 0.0);
  if (!p->src.empty()) {
    const Coupling cp = coupling_parameter(coupling, k);
    const cd ik(0.0, k);
    for (int64_t i = 0; i < N; i++) {
      cd sum = 0.0;
      for (size_t q = 0; q + 4 < p->src.size(); q += 5) {
        const V3 rv = p->mesh.colloc[i] - V3(p->src[q], p->src[q + 1], p->src[q + 2]);
        const double r = norm(rv);
        const double rup = dot(rv, p->mesh.normal[i]) / r;
        const cd ikr = ik * r;
        const cd G = cd(p->src[q + 3], p->src[q + 4]) * std::exp(ikr) / (PI4 * r);
        const cd dG = (G / r) / (ikr - 1.0);
        sum += G + cp.alpha * dG * rup;
      }
      for (int64_t r = 0; r < R; r++) rhs[r * N + i] = sum;
    }
  }
  for (int64_t r = 0; r < R; r++) orc_hmatvec(hphi, (double*)&g[r * N], (double*)&rhs[r * N]);
  orc_hdestroy(hphi);
  auto t3 = clk::now();
  orc_hmatrix* hd = orc_hassemble(p, k, coupling, (double*)a.data(), (double*)b.data(), 1, aca_tol,
                                  max_rank, seed, nthreads);
  auto t4 = clk::now();
  int64_t itmax = 0;
  double resmax = 0;
  std::vector<cd> x(N * R, 0.0);
  double t_factor = 0;
  if (precond_rank >= 1) {
    auto tf = clk::now();
    orc_hlu* f = orc_hlu_factor(p, hd, precond_rank, precond_tol);
    t_factor = secs(tf, clk::now());
    const int64_t nl = (int64_t)f->Ll.size() / 7, nu = (int64_t)f->Ul.size() / 7;
    auto prec = [&](const std::vector<cd>& in, std::vector<cd>& out) {  // out = (LU)^{-1} in
      std::vector<cd> y(N);
      orc_lower_solve(N, nl, f->Ll.data(), (const double*)f->Ld.data(), (const double*)in.data(),
                      (double*)y.data());
      orc_upper_solve(N, nu, f->Ul.data(), (const double*)f->Ud.data(), (const double*)y.data(),
                      (double*)out.data());
    };
    MatVec A = [&](const std::vector<cd>& in, std::vector<cd>& out) {
      std::vector<cd> w(N, 0.0);
      orc_hmatvec(hd, reinterpret_cast<const double*>(in.data()), reinterpret_cast<double*>(w.data()));
      prec(w, out);
    };
    for (int64_t r = 0; r < R; r++) {
      std::vector<cd> b(rhs.begin() + r * N, rhs.begin() + (r + 1) * N), bp(N), xr(N);
      prec(b, bp);
      xr = bp;  // initial guess (LU)^{-1} rhs
      double res = 0;
      const int64_t it = gmres_core(N, A, bp, xr, gmres_tol, restart, maxit, &res);
      std::copy(xr.begin(), xr.end(), x.begin() + r * N);
      itmax = std::max(itmax, it);
      resmax = std::max(resmax, res);
    }
    orc_hlu_free(f);
  } else {
    for (int64_t r = 0; r < R; r++) {
      double res = 0;
      int64_t it = orc_gmres(hd, (double*)&rhs[r * N], (double*)&x[r * N], gmres_tol, restart, maxit, &res);
      itmax = std::max(itmax, it);
      resmax = std::max(resmax, res);
    }
  }
  int64_t maxrank = 0;
  for (auto& bl : hd->blk)
    if (bl.info.adm) maxrank = std::max(maxrank, bl.rank);
  orc_hdestroy(hd);
  auto t5 = clk::now();
  const cd I(0.0, 1.0);
  for (int64_t r = 0; r < R; r++)
    for (int64_t i = 0; i < N; i++) {
      cd xi = x[r * N + i], ph, dph;
      cd gi = g[r * N + i];
      if (std::abs(a[i]) < std::abs(b[i])) {
        ph = xi;
        dph = (gi - a[i] * ph) / b[i];
      } else {
        dph = xi;
        ph = (gi - b[i] * dph) / a[i];
      }
      int64_t o = r * N + perm[i];
      if (phi_out) C(phi_out)[o] = ph;
      if (dphi_out) C(dphi_out)[o] = dph;
      if (p_out) C(p_out)[o] = (freq != 0 ? I * rho * PI2 * freq : I * rho * PI2) * ph;
    }
  auto t6 = clk::now();
  if (stats) {
    stats[0] = secs(t1, t2);
    stats[1] = secs(t2, t3);
    stats[2] = secs(t3, t4);
    stats[3] = secs(t4, t5);
    stats[4] = (double)itmax;
    stats[5] = resmax;
    stats[6] = secs(t0, t6);
    stats[7] = (double)maxrank;
    if (precond_rank >= 1) stats[8] = t_factor;  // the caller passes 9 values
  }
  return 0;
}

void orc_dense(const orc_problem* p, double k, int coupling, const double* a, const double* b,
               double* phi, double* dphi, int nthreads) {
  OperatorCtx ctx(&p->mesh, k, p->reflected());
  Coupling cp = coupling_parameter(coupling, k);
  EntryGen g{&ctx, cp.alpha, cp.alpha_half, C(a), C(b), 0};
  int64_t N = p->mesh.n;
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (int64_t c = 0; c < N; c++)
    for (int64_t r = 0; r < N; r++) {
      cd x, y;
      g.both(r, c, x, y);
      if (phi) C(phi)[c * N + r] = x;
      if (dphi) C(dphi)[c * N + r] = y;
    }
}

int64_t orc_triangle_rule(int64_t order, double* out) {
  Rule2D r = triangle_rule((int)order);
  for (int i = 0; i < r.size(); i++) {
    out[3 * i] = r.x1[i];
    out[3 * i + 1] = r.x2[i];
    out[3 * i + 2] = r.w[i];
  }
  return r.size();
}

int64_t orc_line_rule(int64_t n, double* out) {
  Rule1D r = line_rule((int)n);
  for (int i = 0; i < r.size(); i++) {
    out[2 * i] = r.x[i];
    out[2 * i + 1] = r.w[i];
  }
  return r.size();
}

uint64_t orc_pivot_hash(uint64_t seed, uint64_t a, uint64_t b) { return pivot_hash(seed, a, b); }

}  // extern "C"
