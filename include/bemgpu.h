/*
 * bemgpu.h -- C ABI of the GB300 (sm_103a) Helmholtz BEM hot path.
 *
 * Drop-in boundary for the H-matrix solve of KG93/3d_BEM
 * (BoundaryElementSolver::hMatrixSolve, boundaryelementsolver.cpp:526-744).
 * Every entry point takes plain pointers and sizes, returns a bem_status and
 * never aborts; complex numbers are interleaved (re, im) doubles. Unless
 * stated otherwise, pointers are host pointers and the call copies in / out.
 *
 * Index order: the library renumbers elements by its cluster tree exactly as
 * the reference's ClusterTree constructor reorders the triangles in place
 * (HMatrix/clustertree.h:77-86, clustertree.cpp:265-283); instead of
 * reordering the caller's arrays it returns the permutation
 * (bem_get_permutation). Per-element inputs and outputs of bem_set_bc,
 * bem_solve and bem_sweep are in the caller's order; the matrix-level calls
 * (bem_operators, bem_hmatvec, bem_gmres, bem_get_block) use cluster order,
 * like the reference's HMatrix / HArithm calls.
 */
#ifndef BEMGPU_H
#define BEMGPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t bem_status;
#define BEM_OK 0
#define BEM_EINVAL 1     /* bad argument or call order */
#define BEM_ENOMEM 2     /* device allocation failed */
#define BEM_ENONFINITE 3 /* NaN / Inf detected in inputs or results */
#define BEM_EMAXIT 4     /* iteration cap reached before the tolerance */
#define BEM_EBREAKDOWN 5 /* Krylov breakdown */
#define BEM_ETIMEOUT 6   /* a bounded device wait gave up */
#define BEM_ECUDA 7      /* CUDA runtime error */
#define BEM_ERANK 8      /* an ACA block reached its rank reservation */

typedef struct bem_handle bem_handle;

/* Solver parameters (BemSolverParameters, bemparameters.h:21-34, plus the
 * constants the reference hard-wires: leaf size clustertree.h:146,
 * admissibility constant hmatrix.h:240, GMRES tolerance and restart
 * boundaryelementsolver.cpp:670/692 and gmres.h:170). */
typedef struct bem_config {
  int64_t leaf_size;       /* a cluster is a leaf when size < leaf_size (ref: 50) */
  double eta;              /* admissible iff min(diam)/dist < eta (ref: 3) */
  double aca_tol;          /* acaRelativeError */
  int64_t aca_max_rank;    /* acaMaxRank, 0 = unlimited */
  int64_t rank_reserve;    /* initial device rank reservation per admissible
                              block; blocks whose ACA reaches it get it doubled
                              and are assembled again (aca_max_rank = 0) */
  double gmres_tol;        /* relative residual (ref: 1e-3 * aca_tol) */
  int64_t gmres_restart;   /* ref: 300 */
  int64_t gmres_maxit;     /* total Arnoldi steps allowed */
  int32_t coupling;        /* 0 none, 1 Burton-Miller, 2 Kirkup (BemCoupling) */
  int32_t precision;       /* 0 complex FP64 throughout */
  double wave_speed;       /* c */
  double density;          /* rho (p = i rho omega phi) */
  uint64_t seed;           /* seeds the ACA start columns / pivot members */
  int32_t use_preconditioner; /* usePreconditioner: H-LU left preconditioning */
  int32_t selector;         /* learned quadrature orders (mixed precision):
                              bit 0 (1): per near-field pair, the network
                              (bem_set_selector); bit 1 (2): per ACA entry,
                              the rule table (bem_set_aca_rules) */
  int64_t precond_rank;    /* preconditionerRank (ref default 2) */
  double precond_tol;      /* preconditionerRelError (ref default 0) */
  double recompress_tol;   /* > 0: truncating SVD recompression of every ACA
                              block to this relative error after assembly */
  double selector_guard;   /* pairs whose top class probability is below this
                              get the highest order (guard band) */
  int64_t sweep_workers;   /* bem_sweep: frequencies solved concurrently, each
                              worker on its own stream (0: autotuned) */
  int64_t aca_big_mn;      /* ACA size bin: blocks with m + n >= this get the
                              512-thread kernel (0: the blocks with m + n >=
                              2048 plus the largest ones with m + n >= 512
                              up to half the SM count; or autotuned) */
  double precond_reuse;    /* > 1: a solve keeps the H-LU factors of an earlier
                              frequency f0 while max(f / f0, f0 / f) <= this
                              (frequency sweeps; GMRES still converges to the
                              solution of the current matrix); <= 1: factors
                              rebuilt for every solve, as the reference does */
  int32_t hlu_device;      /* 1: the H-LU factorization runs on the GPU (task
                              program of hlu_gpu.h; needs precond_rank 1..64
                              and leaf_size <= 49, else the host factorization
                              is used); 0: on the host */
  int32_t near_fp64;       /* mixed precision (precision 1) only: 1 = the near
                              field is integrated in FP64 and kept as two
                              floats, the complex-FP32 pool plus its remainder;
                              the inner FP32 GMRES reads the first, the FP64
                              refinement residual both (FP64-accurate near
                              field, for bodies whose hypersingular near field
                              cancels strongly, e.g. fine meshes at low kh) */
} bem_config;

typedef struct bem_solve_info {
  int64_t iterations;      /* max GMRES steps over right-hand sides */
  double rel_residual;     /* max GMRES residual estimate */
  double true_residual;    /* max ||b - A x|| / ||b|| after the solve */
  int64_t max_rank;        /* largest ACA rank of the system matrix */
  int64_t capped_blocks;   /* blocks that hit their rank reservation */
  double t_nearfield;      /* seconds, device-timed; the near field runs beside */
  double t_aca;            /* ACA (both spans start with the assembly) */
  double t_rhs;
  double t_gmres;
  double t_total;
  int32_t status;
  int32_t precond_reused;  /* 1: the solve used factors of an earlier frequency */
  double t_precond;        /* H-LU build (host) including transfers */
} bem_solve_info;

void bem_config_default(bem_config* cfg);

/* Create / destroy a solver handle on the current CUDA device. */
bem_status bem_create(const bem_config* cfg, bem_handle** out);
void bem_destroy(bem_handle* h);
const char* bem_last_error(const bem_handle* h);

/* Mesh: n triangles, 9 doubles each (node1, node2, node3). Builds the cluster
 * tree, the block partition and every frequency-independent index table
 * (ClusterTree(BoundaryElements*) clustertree.h:77-86,
 * HMatrix::populateBlockClusterTree hmatrix.cpp:922,
 * prepareBoundaryElements boundaryelementsolver.cpp:3463). */
bem_status bem_set_mesh(bem_handle* h, const double* tri, int64_t n);
bem_status bem_get_permutation(const bem_handle* h, int64_t* perm /* n, perm[new] = caller */);
/* Partition in the reference's minPartition order: per block r0, m, c0, n,
 * admissible. Pass info = NULL to query the count. */
bem_status bem_get_partition(const bem_handle* h, int64_t* nblocks, int64_t* info);

/* Host-only planning (no GPU needed): the cluster-tree permutation and the
 * partition bem_set_mesh would build for this mesh and configuration
 * (perm: n entries; info: 5 per block, NULL to query *nblocks). */
bem_status bem_plan_mesh(const bem_config* cfg, const double* tri, int64_t n, int64_t* perm,
                         int64_t* nblocks, int64_t* info);

/* Host-only planning of the GPU H-LU factorization (no GPU needed): the task
 * program bem_hlu_build runs on the device for this mesh and configuration
 * (cfg->precond_rank = the rank of every low-rank factor block). stats
 * (nstats <= 24 values): tasks, arena (complex elements), truncation scratch
 * per CTA (complex elements), longest dependency chain (tasks), model cost of
 * the critical path and of all tasks (microseconds), widest truncation,
 * dataflow sweeps usable (1 / 0), tasks per type (GEMM, LMUL, RMUL, QR,
 * TRUNC, COPY, ZERO), dependency entries, scratch of the large truncations
 * (complex elements), tasks per type on the model's critical path. */
bem_status bem_hlu_plan(const bem_config* cfg, const double* tri, int64_t n, double* stats,
                        int64_t nstats);

/* Robin coefficients a, b per element, caller order
 * (calculateBoundaryConditionAndSourceTermVector, :3386-3429). */
bem_status bem_set_bc(bem_handle* h, const double* a, const double* b);
/* Impedance walls: per element the admittance ratio beta = rho c / Z_e
 * (complex, caller order), i.e. the Robin data a = i k beta, b = 1 at every
 * frequency k of a solve or sweep (the wall-impedance section of the
 * reference's solving script, wallimpedancesection.cpp:360-407, with the
 * physical rho c and each solve's own k, where the reference's script reader
 * uses the last frequency's k and (last frequency) x rho). */
bem_status bem_set_bc_impedance(bem_handle* h, const double* beta);

/* Collocation operators L, M, Mt, N for (row, col) pairs in cluster order
 * (BemOperatorsConst, boundaryelementsolver.cpp:844-894); out: count x 4
 * complex. */
bem_status bem_operators(bem_handle* h, double k, const int64_t* rows, const int64_t* cols,
                         int64_t count, double* out);

/* Assemble both BC-substituted H-matrices at one frequency:
 * phi via ACA (HMatrix::assembleBlocks, hmatrix.cpp:793) and dPhi via the
 * seeded ACA (assembleBlocksExtra, hmatrix.cpp:825). */
bem_status bem_assemble(bem_handle* h, double freq);

/* y = (accumulate ? y : 0) + H x for nrhs vectors (N x nrhs, column-major,
 * cluster order); which = 0 phi, 1 dPhi (HArithm::MVM, harithm.cpp:3-28).
 * bem_hmatvec_device takes device pointers and runs on the handle's stream. */
bem_status bem_hmatvec(bem_handle* h, int32_t which, const double* x, double* y, int64_t nrhs,
                       int32_t accumulate);
bem_status bem_hmatvec_device(bem_handle* h, int32_t which, const void* x, void* y,
                              int64_t nrhs, int32_t accumulate);

/* bem_hmatvec_device with an explicit arithmetic for complex-FP32 storage
 * (precision 1): 0 = FP64 products (as bem_hmatvec_device), 1 = FP32 products
 * with compensated FP32 sums (the inner GMRES operator), 2 = two-float
 * products on the FP32 units, FP64-accurate (the refinement residual).
 * Complex-FP64 storage always uses FP64 arithmetic. */
#define BEM_ARITH_FP64 0
#define BEM_ARITH_FP32 1
#define BEM_ARITH_TWOFLOAT 2
bem_status bem_hmatvec_device_ex(bem_handle* h, int32_t which, const void* x, void* y,
                                 int64_t nrhs, int32_t accumulate, int32_t arith);

/* Allocation-free variant of bem_hmatvec_device (no counterpart in the
 * reference). For callers that must not allocate GPU memory during the call:
 * real-time loops whose latency budget forbids allocator calls (cudaMalloc
 * can synchronise the device), and hosts whose GPU memory is handed out by an
 * outside pool that the library must not bypass. x and y are device pointers
 * the caller owns; the per-block projections go to a fixed 32 MiB device
 * array inside the library
 * (2^21 complex-FP64 values: the matrix's total rank reservation times the
 * vectors per pass must fit, or the call returns BEM_EINVAL). The call never
 * calls cudaMalloc / cudaFree. Every call shares that array, so calls that
 * overlap on the GPU (other streams, other handles) race; the first call on
 * each device looks the array up (cudaGetSymbolAddress) and should come before
 * any stream capture; the address is kept per device ordinal for the device's
 * primary context (the CUDA runtime's), so it is not valid across
 * cudaDeviceReset or under another context on the same device. FP64
 * arithmetic on the stored entries and the same kernels and work items as
 * bem_hmatvec_device. */
bem_status bem_hmatvec_noalloc(bem_handle* h, int32_t which, const void* x, void* y,
                               int64_t nrhs, int32_t accumulate);

/* Block data of the assembled matrix `which`, block index in partition
 * order. Admissible: rank returned, U (m x k col-major), s (k), V (k x n
 * row-major) written when non-NULL. Full: *rank = -1, F (m x n col-major). */
bem_status bem_get_block(bem_handle* h, int32_t which, int64_t block, int64_t* rank, double* U,
                         double* s, double* V, double* F);
/* Ranks of all blocks (-1 for full blocks). */
bem_status bem_get_ranks(bem_handle* h, int32_t which, int64_t* ranks);

/* GMRES on the assembled dPhi matrix, nrhs right-hand sides, cluster order
 * (GMRES::gmresSolve, gmres.h:170-180; x0 = the content of x). */
bem_status bem_gmres(bem_handle* h, const double* b, double* x, int64_t nrhs,
                     bem_solve_info* info);

/* H-LU preconditioner of the assembled dPhi matrix: a truncated copy
 * (precond_rank, precond_tol: HMatrix(const HMatrix&, rank, err),
 * hmatrix.cpp:770-776) is factorized on the host like
 * HArithm::LUDecomposition (harithm.cpp:1192-1296) and the factors go to
 * the GPU. bem_solve does this itself when cfg.use_preconditioner is set. */
bem_status bem_hlu_build(bem_handle* h);
/* x = U^{-1} L^{-1} b on the GPU for nrhs vectors (cluster order, host
 * buffers): HArithm::LUSubstitutionSolve (harithm.cpp:1168-1190). */
bem_status bem_hlu_solve(bem_handle* h, const double* b, double* x, int64_t nrhs);
/* Form of the sweeps of the built factors: 1 = dataflow (one driver CTA on
 * the chain of diagonal leaves, helper CTAs applying the off-diagonal leaves
 * as their columns are solved; needs diagonal leaves <= 32 rows and ranks
 * <= 32), 0 = one CTA per right-hand side walking the leaf schedule in the
 * reference's order. Both give the same solve to rounding. */
bem_status bem_hlu_sweep_kind(const bem_handle* h, int32_t* kind);
/* ---- Learned quadrature-order selector (no counterpart in the reference,
 * which integrates every regular pair with one 16-point rule,
 * boundaryelementsolver.cpp:857-893). A 24-64-64-5 ReLU network picks per
 * near-field pair one of the 1, 3, 7, 13, 25-point rules of the same family
 * (trianglequadraturerules.cpp orders 1, 2, 5, 7, 10). ---- */
#define BEM_SEL_NFEAT 24
#define BEM_SEL_NCLASS 5
int64_t bem_sel_nparam(void); /* 6085: W1 24x64, b1, W2 64x64, b2, W3 64x5, b3 */
/* Training data: n pairs (collocation triangle P, source triangle Q, 9
 * doubles each; wavenumber k) -> features (n x 24), label = cheapest class
 * whose L, M, Mt, N are within tol (relative) of the reference (the 64-point
 * product rule on a subdivision of Q; the split-polar near-singular rule when
 * the centroid distance is below near_ratio * sqrt(area Q)), 5 if none; an
 * operator's error is relative to max(|its reference|, floor_rel times the
 * pair's largest operator) (1e-3: per operator; 1: against the largest);
 * err (n x 6, may be NULL): relative errors of the 5 classes and of the
 * plain 16-point rule. Host buffers; runs on the current device. */
bem_status bem_sel_label(const double* ptri, const double* qtri, const double* k, int64_t n,
                         double tol, double near_ratio, double floor_rel, float* feat,
                         uint8_t* label, float* err);
/* FP32 training on device buffers: gradient of the mean softmax cross-entropy
 * (bitwise reproducible) with work = B * 265 floats; an Adam step; FP32
 * logits (B x 5). stream: cudaStream_t or NULL. */
bem_status bem_mlp_grad(const float* params, const float* X, const uint8_t* y, int64_t B,
                        float* grad, float* loss, float* work, void* stream);
bem_status bem_mlp_adam(float* params, const float* grad, float* m, float* v, int64_t step,
                        float lr, float beta1, float beta2, float eps, void* stream);
bem_status bem_mlp_forward(const float* params, const float* X, int64_t B, float* logits,
                           void* stream);
/* BF16 tensor-core inference (host weights, device features): logits
 * (B x 8, padded; may be NULL) and classes. Raw features; mu / sigma
 * normalise them. */
bem_status bem_sel_infer(const float* params, const float* mu, const float* sigma,
                         const float* feat, int64_t B, float* logits, uint8_t* cls,
                         void* stream);
/* Install trained weights in a handle (used when cfg.selector = 1). */
bem_status bem_set_selector(bem_handle* h, const float* params, const float* mu,
                            const float* sigma);
/* Rule table of the ACA entries (cfg.selector bit 1): 12 x 12 classes
 * (0..4 = 1, 3, 7, 13, 25 points), row = bin of log(d / e_max), column = bin
 * of log(k e_max), d the centroid distance, e_max the source's longest edge;
 * axes = {x0, dx, y0, dy} of the bins. Fitted to labels of the same kind as
 * the network's, at the ACA-level tolerance. */
bem_status bem_set_aca_rules(bem_handle* h, const uint8_t* table, const float* axes);
/* After an assembly with the selector: stats[0] quadrature points used,
 * [1] entries re-integrated by the check, [2] entries that fell back to the
 * highest order, [3] regular near-field entries. */
bem_status bem_sel_stats(const bem_handle* h, int64_t* stats);
/* The per-entry classes of the last assembly (near-field entry order). */
bem_status bem_sel_classes(bem_handle* h, uint8_t* cls);

/* Truncating SVD recompression of every admissible block of matrix `which`
 * on the GPU: QR of U and V^T, SVD of the core, smallest rank with relative
 * Frobenius tail < tol, capped at rank (0: no cap). Replaces
 * BlockCluster::compressAdmissibleBlock (HMatrix/hmatrix.cpp:101-140) as
 * applied to every block by HMatrix(const HMatrix&, rank, relError)
 * (hmatrix.cpp:770-776). */
bem_status bem_recompress(bem_handle* h, int32_t which, int64_t rank, double tol);
/* Export a factor (which = 0 L, 1 U) as a flat leaf list: per leaf r0, m,
 * c0, n, kind (0 full, 1 low rank, 2 diagonal Q, 3 diagonal R), rank, data
 * offset; data in complex doubles; sched = the order of leaf applications
 * (>= 0 diagonal leaf, < 0 -(leaf) - 1). Call with NULL arrays to get sizes. */
bem_status bem_hlu_export(const bem_handle* h, int32_t which, int64_t* nleaves, int64_t* leaves,
                          int64_t* ndata, double* data, int64_t* nsched, int32_t* sched);

/* Whole frequency solve (calculateBoundarySolution -> hMatrixSolve ->
 * phiSolutionToSoundPressure): g is n x nrhs (caller order); phi, dphi and p
 * (n x nrhs, caller order) may be NULL. */
bem_status bem_solve(bem_handle* h, double freq, const double* g, int64_t nrhs, double* phi,
                     double* dphi, double* p, bem_solve_info* info);
/* Same with device pointers (inputs already resident in GPU memory). */
bem_status bem_solve_device(bem_handle* h, double freq, const void* g, int64_t nrhs, void* phi,
                            void* dphi, void* p, bem_solve_info* info);

/* Autotuner of the batched sweep at a probe frequency: times the ACA size
 * bin thresholds 256 / 512 / 1024 on one assembly and sweeps of 1, 2, 3, 4
 * concurrent workers; keeps the fastest of each in the handle. tuned (may be
 * NULL) receives {workers, aca_big_mn}. No counterpart in the reference,
 * whose frequency loop is serial (bemsolvercontroller.cpp:63-72). */
bem_status bem_autotune(bem_handle* h, double freq, int64_t nrhs, int64_t* tuned);

/* Frequency sweep (BemSolverController::run, bemsolvercontroller.cpp:49-109):
 * nf frequencies x nrhs right-hand sides; p is n x nrhs x nf (caller order).
 * info may be NULL or hold nf records. The cfg.sweep_workers handles take
 * the frequencies in the order given, each the next one when it is free, so
 * a sweep that lists its most expensive frequencies first ends most evenly;
 * results do not depend on the order or on the worker count. */
bem_status bem_sweep(bem_handle* h, const double* freqs, int64_t nf, const double* g,
                     int64_t nrhs, double* p, bem_solve_info* info);
/* Same with device pointers: g (n x nrhs complex FP64) and p (n x nrhs x nf)
 * in GPU memory. The workers' work follows what the caller enqueued on the
 * handle's stream (bem_stream) before the call, and the handle's stream
 * waits for all of it before the call returns, so events recorded on that
 * stream bracket the whole sweep. */
bem_status bem_sweep_device(bem_handle* h, const double* freqs, int64_t nf, const void* g,
                            int64_t nrhs, void* p, bem_solve_info* info);

/* Resumable frequency sweep: bem_sweep with the controller's per-frequency
 * solved flags (boundariesSolvedAtFrequency, bemsolvercontroller.cpp:61-69,
 * set as each frequency completes). solved (nf bytes, in and out, not NULL):
 * a frequency whose flag is non-zero on entry is skipped, and its slice of p
 * and its info record are left as they are. When a frequency completes, its
 * slice of p and its info record are written, its flag is set to 1 and then
 * done(f, user) runs (done may be NULL), one call at a time over the
 * workers, on a worker's thread. A non-zero return from done stops the
 * sweep: frequencies already running finish and are reported, no new one
 * starts, and the call returns as bem_sweep would (the flags tell which
 * frequencies are solved). A later call with the same flags solves the rest;
 * a frequency's result does not depend on which others were solved with it
 * unless precond_reuse > 1 (factors shared by neighbouring frequencies). */
typedef int (*bem_freq_done_fn)(int64_t f, void* user);
bem_status bem_sweep_resume(bem_handle* h, const double* freqs, int64_t nf, const double* g,
                            int64_t nrhs, double* p, bem_solve_info* info, uint8_t* solved,
                            bem_freq_done_fn done, void* user);

/* Point sources of the boundary solve (BoundaryElementSolver::pointSources):
 * nsrc rows x, y, z, Re w, Im w (nsrc = 0 clears; bem_set_mesh clears too).
 * Every solve adds their source term at each collocation point to the
 * right-hand side, rhs = sourceTermVector + phi g (boundaryelementsolver.cpp:
 * 578-579), with sourceTerm (:3431-3441) as written there, including its
 * division of the radial term by (ikr - 1); bem_field adds the sources'
 * incident field through its own sources argument. */
bem_status bem_set_point_sources(bem_handle* h, const double* src, int64_t nsrc);

/* One impedance plane (BoundaryElements::impedancePlanes with a single entry,
 * the infinite baffle of the solving scripts): the plane through point with
 * the given normal. Every matrix entry then adds the operators of the column
 * element reflected in the plane, integrated with the regular 16-point rule
 * (implicitPhiMatrixPlusReflected / implicitDPhiMatrixPlusReflected,
 * boundaryelementsolver.cpp:2042-2050, via implicitPhiMatrixReflected /
 * implicitDPhiMatrixReflected :1556-1643), on the same block partition; the
 * reflected element is MeshFunctions::reflectTriangles (meshfunctions.cpp:
 * 349-380: mirrored nodes, node 1 and node 3 swapped). bem_field adds the
 * reflected terms as calculateFieldSolutionRegular does (:2305-2311). With a
 * plane the near field ignores selector bit 0 (the learned near-field orders
 * were trained on free-space pairs). normal = NULL or zero removes the plane;
 * bem_set_mesh removes it too. bem_operators keeps returning the free-space
 * operators. Two planes (the reference's reflection matrices, :746-842) are
 * not supported. */
bem_status bem_set_impedance_plane(bem_handle* h, const double* point, const double* normal);

/* Field evaluation (BoundaryElementSolver::calculateFieldSolution,
 * boundaryelementsolver.cpp:2192-2249, as its regular sum
 * calculateFieldSolutionRegular :2263-2316 with BemOperatorField :2318-2353):
 * velocity potential phi_f and sound pressure p_f = i rho 2 pi f phi_f (2 pi
 * in place of 2 pi f at f = 0) at npts observation points pts (npts x 3, e.g.
 * the triangle midpoints of an observation field, ObservationField::
 * calculateTrianglesMidpoints) from a boundary solution phi, dphi (n x nrhs,
 * caller order, as bem_solve returns them). Per element the 7-point triangle
 * rule of order 5 (orderLow, boundaryelementsolver.h:653-654), evaluated in
 * the configured precision. sources: nsrc point sources, rows x, y, z, Re w,
 * Im w, host memory (sourcePhiTerm :3443-3450), added to every column; may be
 * NULL when nsrc = 0. phi_f and p_f (npts x nrhs) may be NULL. The reference's
 * default (hMatFieldSolving, bemparameters.h:29) approximates the same sum
 * with on-the-fly ACA at fieldACARelativeError = 1e-2 (:2397-2570); this call
 * evaluates it without approximation. No impedance plane terms. */
bem_status bem_field(bem_handle* h, double freq, const double* pts, int64_t npts,
                     const double* phi, const double* dphi, int64_t nrhs, const double* sources,
                     int64_t nsrc, double* phi_f, double* p_f);
/* Same with device pointers for pts, phi, dphi, phi_f and p_f (sources stay
 * in host memory); asynchronous on bem_stream. */
bem_status bem_field_device(bem_handle* h, double freq, const void* pts, int64_t npts,
                            const void* phi, const void* dphi, int64_t nrhs,
                            const double* sources, int64_t nsrc, void* phi_f, void* p_f);

/* ---- mesh input and boundary data (host only, no GPU needed) ---- */

/* A GMSH ASCII mesh: format 2.2 as mshReader::readSections reads it
 * (mshreader.cpp:200-376: $Nodes, $Elements with number / type / tags,
 * $PhysicalNames), or format 4.1 (block-structured $Nodes / $Elements; an
 * element's geometric number is its entity tag, its physical number the
 * entity's first physical tag from $Entities). Triangles (type 2) and
 * quadrilaterals (type 3) are kept, other element types skipped. On failure
 * *out is NULL and err (errcap bytes, may be NULL) holds the reason. */
typedef struct bem_msh bem_msh;
bem_status bem_msh_read(const char* path, bem_msh** out, char* err, int64_t errcap);
void bem_msh_free(bem_msh* m);
/* $PhysicalNames entries: dimension, number and name (NUL-terminated, cap bytes). */
int64_t bem_msh_num_physical(const bem_msh* m);
bem_status bem_msh_physical(const bem_msh* m, int64_t i, int32_t* dim, int32_t* tag, char* name,
                            int64_t cap);
/* Element selection (mshReader::sortOutIncludesAndExcludes / elementIsIncluded,
 * mshreader.cpp:22-198, :378-428). include / exclude: lists separated by
 * blanks, commas or semicolons of physical group names (case-insensitive),
 * geometric numbers and ranges "a..b" / "a...b" (open ends allowed). An include
 * list that is empty or only "all" keeps everything except the excluded
 * physical groups and geometric numbers; otherwise it keeps the named physical
 * groups plus the included minus the excluded geometric numbers. Returns the
 * selected triangle and quadrilateral counts (either pointer may be NULL);
 * after bem_msh_read everything is selected. */
bem_status bem_msh_select(bem_msh* m, const char* include, const char* exclude, int64_t* ntri,
                          int64_t* nquad);
/* The selection, in file order: triangles (ntri x 9: node1, node2, node3 xyz),
 * quadrilaterals (nquad x 12) and their physical / geometric numbers. Any
 * pointer may be NULL. */
bem_status bem_msh_elements(const bem_msh* m, double* tri, int32_t* tri_phys, int32_t* tri_geom,
                            double* quad, int32_t* quad_phys, int32_t* quad_geom);
/* global::quadrilateralsToTriangles (global.cpp:841-870): each quadrilateral
 * (12 doubles) becomes two triangles (18 doubles) split along the shorter
 * diagonal, node orders as the reference. */
bem_status bem_quads_to_triangles(const double* quad, int64_t nq, double* tri);
/* Mesh refinement of an Elements section (SolvingScript::refineElements,
 * solvingscriptreader.cpp:1104-1127: edge length = (c / MeshFrequency) / 2,
 * or EdgeLength; ElementSection::refineTriangles / recursiveRefineTriangle,
 * elementSection.cpp:688-800): every triangle whose longest edge exceeds
 * edge_length is bisected at that edge, recursively, in the reference's order
 * and node orders. out (cap x 9, may be NULL to count) receives the triangles,
 * parent (may be NULL) the index of the input triangle each came from; *nout
 * the count (BEM_EINVAL when it exceeds cap). */
bem_status bem_refine_triangles(const double* tri, int64_t n, double edge_length, double* out,
                                int64_t cap, int64_t* nout, int64_t* parent);
/* WallImpedanceSection::setUpValues (SolvingScript/wallimpedancesection.cpp:
 * 308-405): the beta of bem_set_bc_impedance (a = i k beta, b = 1, g = 0) for
 * imp_type 0 reflection factor R (beta = (1 - R) / (1 + R), real part of R),
 * 1 damping d (d / (2 - d)), 2 impedance Z (normalized: 1 / Z, else
 * medium_impedance / Z), 3 admittance Y (normalized: Y, else
 * medium_impedance Y). value and beta are complex (re, im). */
bem_status bem_wall_beta(int32_t imp_type, int32_t normalized, const double* value,
                         double medium_impedance, double* beta);

/* Point-cloud H-matrix with the reference's test kernel exp(ikr)/(4 pi r)
 * (Tests/tests.h:30-42): rows and columns get their own cluster trees.
 * Afterwards which = 0 addresses this matrix in bem_hmatvec / bem_get_block
 * (indices in the two cluster orders, returned through rowperm / colperm). */
bem_status bem_points_assemble(bem_handle* h, const double* rowpts, int64_t nr,
                               const double* colpts, int64_t nc, double k, int64_t* rowperm,
                               int64_t* colperm);

/* Number of kernel launches issued by the library since the handle was
 * created, its sweep workers' included (instrumentation for benchmarks). */
int64_t bem_launch_count(const bem_handle* h);

/* The CUDA stream (cudaStream_t) every kernel of this handle runs on, so a
 * caller can order its own work or record timing events on it. */
void* bem_stream(const bem_handle* h);

#ifdef __cplusplus
}
#endif
#endif
