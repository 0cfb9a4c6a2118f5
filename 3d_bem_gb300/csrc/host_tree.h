// host_tree.h -- host-side geometry, cluster tree, block partition and the
// frequency-independent index tables the kernels consume.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "bem_kernels.h"
#include "bem_types.h"

namespace bemgpu {

struct HBox {
  double lo[3], hi[3];
};

struct HCluster {
  int64_t start = 0, size = 0, son1 = -1, son2 = -1, level = 0;
  bool leaf = false;
  HBox box;
};

struct HBlockDesc {
  int64_t r0, m, c0, n;
  bool adm;
  int64_t rc, cc;  // row / column cluster ids
};

// Cluster tree over points (triangle midpoints): bisection of the bounding box
// along its longest side at the half, leaf when size < leaf
// (HMatrix/clustertree.h:262-310), depth-first renumbering
// (clustertree.cpp:265-283). perm[new] = old.
struct HTree {
  std::vector<HCluster> c;
  std::vector<int64_t> perm;
};
HTree build_tree(const std::vector<double>& pts /* n x 3 */, int64_t leaf);

// Block partition (HMatrix/hmatrix.cpp:958-1135): admissible iff
// min(diam) / dist < eta; leaves in the reference's minPartition order.
std::vector<HBlockDesc> build_blocks(const HTree& rows, const HTree& cols, double eta);

// Element geometry in cluster order (global.cpp:903-912, 1285-1290;
// boundaryelements.cpp:37-46).
void prepare_elements(const double* tri_caller, const std::vector<int64_t>& perm,
                      std::vector<Elem>& E, double& avgdim);

// Exactly the device's near_pair() test, in host arithmetic without
// contraction.
bool host_near_pair(const Elem& P, const Elem& Q, double near_r);

// Normal-filtered pivot seeds of one block
// (boundaryelementsolver.cpp:2052-2172), block-relative (row, col) pairs.
void pivot_seeds(const std::vector<Elem>& E, const HBlockDesc& b, double angle, uint64_t seed,
                 uint64_t block_id, std::vector<int32_t>& out);

// Everything the kernels need for one mesh (frequency independent).
struct Layout {
  int64_t N = 0;
  std::vector<HBlockDesc> blocks;
  std::vector<NearBlock> near;
  std::vector<FarBlock> far;
  std::vector<int32_t> far_order;   // launch order (largest first)
  int64_t nbig = 0;                 // leading far_order entries on the 512-thread ACA kernel
  std::vector<NearTile> tiles;
  std::vector<uint32_t> special_bits;
  std::vector<int64_t> sp_entry;
  std::vector<int32_t> sp_row, sp_col;
  std::vector<LeafRows> leaves;
  std::vector<int32_t> list_off, list;
  std::vector<int64_t> piv_off;
  std::vector<int32_t> piv_cnt, piv_rc;
  int64_t near_entries = 0, u_size = 0, v_size = 0, s_size = 0;
};
// E == nullptr for point clouds (no special entries, no pivot seeds).
void build_layout(const HTree& rows, const HTree& cols, const std::vector<Elem>* E,
                  double near_r, double eta, int64_t kcap_default, int64_t max_rank,
                  bool pivots, uint64_t seed, Layout& L);

// Quadrature rule tables of the kernels.
QuadRules make_rules();

// Gauss-Legendre nodes (ascending) and weights on [-1, 1], n <= 64.
void gauss_legendre(int n, double* x, double* w);

}  // namespace bemgpu
