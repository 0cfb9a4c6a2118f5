// oracle_core.hpp -- shared internals of the CPU FP64 oracle (test
// infrastructure only; see bem_oracle.h for what is restated from where).
#pragma once
#include <cmath>
#include <complex>
#include <functional>
#include <algorithm>
#include <cstdint>
#include <vector>

namespace orc {

using cd = std::complex<double>;
static constexpr double PI = 3.14159265358979323846264338327950288;
static constexpr double PI2 = 2.0 * PI;
static constexpr double PI4 = 4.0 * PI;
// global.h:53 -- tiny = 10 * machine epsilon of complex<double>
static constexpr double TINY = 10.0 * 2.220446049250313080847263336181640625e-16;
// global.h:43 -- barycentric threshold of the near-singular split
static constexpr double PROJ_EPS = 0.05;

struct V3 {
  double x = 0, y = 0, z = 0;
  V3() = default;
  V3(double a, double b, double c) : x(a), y(b), z(c) {}
  double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }

struct Tri {
  V3 n1, n2, n3;
};

struct Rule2D {  // barycentric (xi1, xi2, w)
  std::vector<double> x1, x2, w;
  int size() const { return (int)w.size(); }
};
struct Rule1D {  // on [-1, 1]
  std::vector<double> x, w;
  int size() const { return (int)w.size(); }
};

Rule2D triangle_rule(int order);
Rule1D line_rule(int n);
uint64_t pivot_hash(uint64_t seed, uint64_t a, uint64_t b);

struct Mesh {
  int64_t n = 0;
  std::vector<Tri> tri;      // cluster order
  std::vector<V3> normal;    // unit normals
  std::vector<V3> colloc;    // centroids
  std::vector<double> area;
  double avgdim = 0;
};
void mesh_prepare(Mesh& m);
// MeshFunctions::reflectTriangles (meshfunctions.cpp:349-380): the mesh
// mirrored in the plane through point with normal (4 x 4 reflection matrix,
// node 1 and node 3 swapped), prepared (normals, centroids, areas)
Mesh reflect_mesh(const Mesh& m, const V3& point, V3 normal);

struct Ops {
  cd L, M, Mt, N;
};

struct OperatorCtx {
  const Mesh* mesh;
  double k;
  Rule2D reg;   // 16-point rule (order 8)
  Rule1D line;  // 5-point Gauss-Legendre
  Rule1D gl16;  // positive half of the 32-point Gauss-Legendre rule
  const Mesh* refl = nullptr;  // impedance plane: the reflected elements, same order
  OperatorCtx(const Mesh* m, double k_, const Mesh* reflected = nullptr);
  // operators of the pair, plus those of the reflected column element when a
  // plane is set (implicitPhiMatrixPlusReflected, boundaryelementsolver.cpp:2042-2050)
  Ops eval(int64_t row, int64_t col) const;
  Ops regular(int64_t row, int64_t col) const;
  // regular rule with the column element taken from another mesh
  // (BemOperatorsReflected, :1516-1554)
  Ops regular_from(int64_t row, const Mesh& cols, int64_t col) const;
  Ops singular(int64_t t) const;
  Ops near_singular(int64_t row, int64_t col) const;
};

struct Coupling {
  cd alpha, alpha_half;
};
Coupling coupling_parameter(int kind, double k);

// Entry generator of the BC-substituted matrices (implicitPhiMatrix2 /
// implicitDPhiMatrix2).
struct EntryGen {
  const OperatorCtx* ops;
  cd alpha, alpha_half;
  const cd* a;
  const cd* b;
  int which;  // 0 phi, 1 dphi
  cd operator()(int64_t row, int64_t col) const;
  void both(int64_t row, int64_t col, cd& phi, cd& dphi) const;
};

// ---- cluster tree / partition ----
struct Box {
  V3 lo{INFINITY, INFINITY, INFINITY}, hi{-INFINITY, -INFINITY, -INFINITY};
  void add(V3 p) {
    for (int i = 0; i < 3; i++) {
      lo[i] = std::min(lo[i], p[i]);
      hi[i] = std::max(hi[i], p[i]);
    }
  }
};
struct Cluster {
  int64_t start = 0, size = 0;
  int64_t son1 = -1, son2 = -1, level = 0;
  bool leaf = false;
  Box box;
};
struct ClusterTree {
  std::vector<Cluster> c;      // c[0] = root
  std::vector<int64_t> perm;   // perm[new] = old
};
ClusterTree build_cluster_tree(const std::vector<V3>& pts, int64_t leaf);

struct BlockInfo {
  int64_t r0, m, c0, n;
  bool adm;
  int64_t rc, cc;  // cluster ids
};
std::vector<BlockInfo> build_partition(const ClusterTree& rt, const ClusterTree& ct,
                                       double eta);
double cluster_distance(const Box& a, const Box& b);
double cluster_diameter(const Box& a);

// ---- H-matrix ----
struct HBlock {
  BlockInfo info;
  int64_t rank = 0;
  std::vector<cd> full;  // m x n col-major
  std::vector<cd> U;     // m x k col-major
  std::vector<cd> s;     // k
  std::vector<cd> V;     // k x n row-major ("VAdjMat" rows)
};

using EntryFn = std::function<cd(int64_t, int64_t)>;

void aca_partial_pivot(HBlock& blk, int64_t max_rank, double tol, const EntryFn& f,
                       uint64_t seed, uint64_t block_id);
void aca_partial_pivot_extra(HBlock& blk, int64_t max_rank, double tol, const EntryFn& f,
                             const std::vector<std::pair<int64_t, int64_t>>& pivots);
std::vector<std::pair<int64_t, int64_t>> normal_filtered_pivots(
    const Mesh& mesh, const BlockInfo& b, double filter_angle, uint64_t seed,
    uint64_t block_id);
void recompress_block(HBlock& blk, int64_t rank, double tol);
// H-LU factorization (hlu.cpp) of an H-matrix given by its blocks in
// partition order: flat leaf lists of L and U (r0, m, c0, n, kind, rank,
// offset; kinds 0 full, 1 low rank, 2 diagonal Q, 3 diagonal R).
void hlu_factor_blocks(const ClusterTree& t, const std::vector<HBlock>& blk, int64_t rank,
                       double tol, std::vector<int64_t>& Ll, std::vector<cd>& Ld,
                       std::vector<int64_t>& Ul, std::vector<cd>& Ud);

// dense complex helpers
void householder_qr(int64_t m, int64_t k, std::vector<cd>& A, std::vector<cd>& Q,
                    std::vector<cd>& R);
void jacobi_svd(int64_t n, std::vector<cd>& A, std::vector<double>& sigma,
                std::vector<cd>& U, std::vector<cd>& V);
int64_t min_rank_for_error(const std::vector<double>& sv, int64_t max_rank, double rel);

}  // namespace orc
