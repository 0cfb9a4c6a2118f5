/*
 * bem_oracle.h -- CPU FP64 restatement of the 3d_BEM Helmholtz H-matrix solve
 * path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the parity checker and the timed
 * CPU baseline. Only the test suite, the smoke check and the CPU-baseline leg
 * of the benchmark load it. The GPU library (libbemgpu) never links, loads or
 * calls anything in this directory.
 *
 * What it restates (reference file:line, paths inside KG93/3d_BEM):
 *   - geometry prep: global.cpp:903-912 (normal, midpoint), global.cpp:1285-1290
 *     (area), boundaryelements.cpp:9-46 (collocation = centroid,
 *     averageTriangleDim = mean(sqrt(area))/2)
 *   - element operators L, M, Mt, N: boundaryelementsolver.cpp:844-894
 *     (BemOperatorsConst), :896-1029 (BemOperatorsSingularPolarInt),
 *     :1387-1514 (BemOperatorsNearSing), global.cpp:955-1228
 *     (projectPointOnTriangleFaster)
 *   - Robin BC substitution: boundaryelementsolver.cpp:2004-2040
 *     (implicitPhiMatrix2 / implicitDPhiMatrix2), :3386-3429 (substitution rule)
 *   - cluster tree: HMatrix/clustertree.h:262-310, clustertree.cpp:114-123,
 *     171-181, 265-283
 *   - block partition / admissibility: HMatrix/hmatrix.cpp:958-1135
 *   - ACA: HMatrix/hmatrix.cpp:471-593 (partialPivotACA), :595-745
 *     (partialPivotACAextra), boundaryelementsolver.cpp:2052-2172 (pivot seeds)
 *   - truncating recompression: HMatrix/hmatrix.cpp:101-140,
 *     golubReinschSVD.cpp:551-585 (minRankforError)
 *   - H-matvec: HMatrix/harithm.cpp:3-28
 *   - H-LU substitutions: HMatrix/harithm.cpp:1314-1412
 *   - GMRES: HMatrix/gmres.h:170-207 (Eigen GMRES, restated from Saad &
 *     Schultz 1986 with Householder-free CGS2 Arnoldi + Givens rotations)
 *   - solve orchestration: boundaryelementsolver.cpp:526-744, :2251-2261
 *   - field evaluation: boundaryelementsolver.cpp:2192-2249, :2263-2353,
 *     :3443-3450 (field.cpp)
 *
 * Deliberate, documented differences from the reference (shared with the GPU
 * library so the two stay comparable):
 *   - random ACA start columns / pivot-seed members (QRandomGenerator::system)
 *     are replaced by a seeded hash (bem_pivot_hash below);
 *   - GMRES starts from x0 = 0 (or the preconditioned RHS) instead of a random
 *     vector; the Krylov method is the same.
 *
 * Parity pinning: the reference cannot be compiled here (needs Qt 6 and Eigen),
 * and it stores no golden vectors. The oracle is pinned by known-answer tests
 * (closed-form panel integrals, the analytic pulsating sphere, polynomial
 * exactness of the rules) and by the reference's own test designs
 * (Tests/tests.cpp) -- parity against reference outputs is unpinned.
 *
 * Conventions: complex numbers are interleaved (re, im) doubles; matrices are
 * column-major; triangles are 9 doubles (node1 xyz, node2 xyz, node3 xyz).
 */
#ifndef BEM_ORACLE_H
#define BEM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_problem orc_problem;
typedef struct orc_hmatrix orc_hmatrix;

/* Mesh + cluster tree + block partition (triangles reordered internally). */
orc_problem* orc_create(const double* tri, int64_t n, int64_t leaf, double eta);
void orc_destroy(orc_problem* p);
/* One impedance plane (point, normal; normal NULL or zero removes it): every
 * operator evaluation adds the reflected column element's regular-rule
 * operators (implicitPhiMatrixPlusReflected, boundaryelementsolver.cpp:
 * 2042-2050; BemOperatorsReflected :1516-1554; MeshFunctions::reflectTriangles
 * meshfunctions.cpp:349-380). */
void orc_set_plane(orc_problem* p, const double* point, const double* normal);
/* Point sources of the solve's right-hand side (nsrc rows x, y, z, Re w, Im w;
 * nsrc = 0 clears): rhs = sourceTermVector + phi g (boundaryelementsolver.cpp:
 * 578-579, sourceTerm :3431-3441). */
void orc_set_sources(orc_problem* p, const double* src, int64_t nsrc);
int64_t orc_n(const orc_problem* p);
/* perm[new_index] = caller index */
void orc_perm(const orc_problem* p, int64_t* perm);
int64_t orc_num_clusters(const orc_problem* p);
/* per cluster: start, size, son1, son2, level, is_leaf (6 int64) + box (6 doubles) */
void orc_clusters(const orc_problem* p, int64_t* info, double* boxes);
int64_t orc_num_blocks(const orc_problem* p);
/* per block (reference minPartition order): r0, m, c0, n, admissible */
void orc_blocks(const orc_problem* p, int64_t* info);
/* geometry in cluster order */
void orc_geometry(const orc_problem* p, double* normals, double* areas,
                  double* colloc, double* avgdim);

/* Raw operators L, M, Mt, N for (row, col) pairs in cluster order.
 * out: cnt x 4 complex. */
void orc_operators(const orc_problem* p, double k, const int64_t* rows,
                   const int64_t* cols, int64_t cnt, double* out);
/* BC-substituted entries of the phi (RHS) and dPhi (system) matrices.
 * a, b: N complex Robin coefficients (cluster order); coupling 0/1/2 =
 * none / Burton-Miller / Kirkup. */
void orc_entries(const orc_problem* p, double k, int coupling, const double* a,
                 const double* b, const int64_t* rows, const int64_t* cols,
                 int64_t cnt, double* phi, double* dphi);

/* H-matrix assembly (which: 0 = phi via partialPivotACA, 1 = dPhi via
 * partialPivotACAextra). */
orc_hmatrix* orc_hassemble(const orc_problem* p, double k, int coupling,
                           const double* a, const double* b, int which,
                           double tol, int64_t max_rank, uint64_t seed,
                           int nthreads);
void orc_hdestroy(orc_hmatrix* h);
/* y += H x */
void orc_hmatvec(const orc_hmatrix* h, const double* x, double* y);
void orc_hdense(const orc_hmatrix* h, double* out);
/* ranks of admissible blocks, -1 for full blocks */
void orc_hranks(const orc_hmatrix* h, int64_t* ranks);
/* block data: U (m x k col-major), s (k), V (k x n row-major); or full m x n */
int64_t orc_hblock(const orc_hmatrix* h, int64_t b, double* U, double* s, double* V,
                   double* full);
/* Truncating recompression of all admissible blocks (rank cap, rel. tol). */
void orc_hrecompress(orc_hmatrix* h, int64_t rank, double tol);

/* One ACA block with a generic point-cloud Helmholtz kernel (the reference's
 * Tests/tests.h:30-42 design: exp(ikr)/(4 pi r), 1 at r = 0). */
orc_hmatrix* orc_hassemble_points(const double* rowpts, int64_t nr,
                                  const double* colpts, int64_t nc, double k,
                                  int64_t leaf, double eta, double tol,
                                  int64_t max_rank, uint64_t seed,
                                  int64_t* rowperm, int64_t* colperm);

/* GMRES on an H-matrix (unpreconditioned). Returns iterations; x in/out. */
int64_t orc_gmres(const orc_hmatrix* h, const double* b, double* x, double tol,
                  int64_t restart, int64_t maxit, double* rel_resid);

/* Flat block-triangular factors (leaf lists).
 * blocks: per leaf r0, m, c0, n, kind (0 full, 1 low-rank, 2 diag-Q, 3 diag-R),
 * rank, data offset (complex elements). Low-rank data: U (m x k col-major),
 * then V (k x n row-major), singular values folded into U. */
void orc_lower_solve(int64_t n, int64_t nblk, const int64_t* blocks,
                     const double* data, const double* b, double* y);
void orc_upper_solve(int64_t n, int64_t nblk, const int64_t* blocks,
                     const double* data, const double* y, double* x);

/* H-LU factors of an assembled H-matrix (HMatrix(const HMatrix&, rank, tol)
 * + HArithm::LUDecomposition, harithm.cpp:1192-1296; hlu.cpp): flat leaf
 * lists for orc_lower_solve / orc_upper_solve. sizes: L leaves, L data
 * (complex), U leaves, U data. */
typedef struct orc_hlu orc_hlu;
orc_hlu* orc_hlu_factor(const orc_problem* p, const orc_hmatrix* h, int64_t rank, double tol);
void orc_hlu_sizes(const orc_hlu* f, int64_t* sizes4);
void orc_hlu_get(const orc_hlu* f, int64_t* Ll, double* Ld, int64_t* Ul, double* Ud);
void orc_hlu_free(orc_hlu* f);

/* Whole frequency solve with the H-LU preconditioner of rank precond_rank
 * (>= 1; 0 = none): stats gets 9 values, the 9th the factorization time. */
int orc_solve_precond(const orc_problem* p, double freq, double c, double rho, int coupling,
                      const double* a, const double* b, const double* g, int64_t R,
                      double aca_tol, int64_t max_rank, double gmres_tol, int64_t restart,
                      int64_t maxit, uint64_t seed, int nthreads, int64_t precond_rank,
                      double precond_tol, double* phi, double* dphi, double* p_out,
                      double* stats);

/* Whole frequency solve (reference hMatrixSolve, unpreconditioned GMRES).
 * g: N x R complex (column-major, caller order), outputs in caller order.
 * stats: [t_assemble_phi, t_rhs, t_assemble_dphi, t_gmres, iters_max,
 *         rel_resid_max, total_seconds, max_rank] */
int orc_solve(const orc_problem* p, double freq, double c, double rho,
              int coupling, const double* a, const double* b, const double* g,
              int64_t R, double aca_tol, int64_t max_rank, double gmres_tol,
              int64_t restart, int64_t maxit, uint64_t seed, int nthreads,
              double* phi, double* dphi, double* pres, double* stats);

/* Dense reference matrices (small N): both N x N column-major, cluster order. */
void orc_dense(const orc_problem* p, double k, int coupling, const double* a,
               const double* b, double* phi, double* dphi, int nthreads);

/* Field evaluation (calculateFieldSolutionRegular, boundaryelementsolver.cpp:
 * 2263-2316; BemOperatorField :2318-2353; sourcePhiTerm :3443-3450): tri is
 * n x 9 in the caller's order, phi / dphi n x nrhs complex, pts npts x 3,
 * src nsrc x 5 (x, y, z, Re w, Im w); phi_f and p_f (npts x nrhs complex) may
 * be NULL. p_f = i rho 2 pi f phi_f (2 pi at f = 0). plane: NULL or 6 doubles
 * (point, normal) of one impedance plane, whose reflected elements add their
 * terms with the same boundary data (:2305-2311). */
void orc_field(const double* tri, int64_t n, double freq, double c, double rho,
               const double* pts, int64_t npts, const double* phi, const double* dphi,
               int64_t nrhs, const double* src, int64_t nsrc, const double* plane,
               int nthreads, double* phi_f, double* p_f);

/* Quadrature tables used (for cross-checking the GPU library's copy). */
int64_t orc_triangle_rule(int64_t order, double* out /* npts x 3 */);
int64_t orc_line_rule(int64_t n, double* out /* npts x 2 */);

/* Seeded replacement of QRandomGenerator picks; identical in the GPU library. */
uint64_t orc_pivot_hash(uint64_t seed, uint64_t a, uint64_t b);

#ifdef __cplusplus
}
#endif
#endif
