// capi.cpp -- the solver handle and the extern "C" entry points of bemgpu.h.
//
// Host orchestration of one frequency follows BoundaryElementSolver::
// hMatrixSolve (boundaryelementsolver.cpp:526-744): BC set-up, phi assembly,
// rhs = phi g, dPhi assembly, GMRES, BC back-substitution, p = i rho omega phi.
// Everything after bem_set_mesh runs on the GPU; the host only sequences
// kernels and reads back convergence flags.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <new>
#include <numeric>
#include <cstdio>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>
#include <map>
#include <array>

#include "../../include/bemgpu.h"
#include "bem_kernels.h"
#include "hlu.h"
#include "hlu_solve.h"
#include "hlu_gpu.h"
#include "recompress.h"
#include "selector.h"
#include "host_tree.h"
#include "krylov.h"
#include "field.h"
#include "post.h"

using namespace bemgpu;
using cplx = std::complex<double>;

namespace {

struct BemError {
  bem_status st;
  std::string msg;
};

#define CK(x)                                                                             \
  do {                                                                                    \
    cudaError_t e_ = (x);                                                                 \
    if (e_ != cudaSuccess)                                                                \
      throw BemError{e_ == cudaErrorMemoryAllocation ? BEM_ENOMEM : BEM_ECUDA,            \
                     std::string(#x) + ": " + cudaGetErrorString(e_)};                    \
  } while (0)

void require(bool ok, bem_status st, const char* msg) {
  if (!ok) throw BemError{st, msg};
}

// Device bytes held by the library's buffers. BEM_DEVICE_MEM_CAP (bytes, read
// once) turns any allocation beyond it into the BEM_ENOMEM a failing
// cudaMalloc gives, without taking the GPU's memory (tests of that path).
std::atomic<int64_t> g_device_bytes{0};
int64_t device_mem_cap() {
  static const int64_t cap = [] {
    const char* e = std::getenv("BEM_DEVICE_MEM_CAP");
    return e ? (int64_t)std::atoll(e) : (int64_t)0;
  }();
  return cap;
}

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) {
      cudaFree(p);
      g_device_bytes -= (int64_t)(n * sizeof(T));
    }
    p = nullptr;
    n = 0;
  }
  void ensure(size_t cnt) {
    if (cnt <= n && p) return;
    release();
    size_t c = std::max<size_t>(cnt, 1);
    const int64_t cap = device_mem_cap();
    if (cap > 0 && g_device_bytes + (int64_t)(c * sizeof(T)) > cap)
      throw BemError{BEM_ENOMEM, "device allocation beyond BEM_DEVICE_MEM_CAP"};
    CK(cudaMalloc((void**)&p, c * sizeof(T)));
    n = c;
    g_device_bytes += (int64_t)(c * sizeof(T));
  }
  void upload(const std::vector<T>& v, cudaStream_t s) {
    ensure(v.size());
    if (!v.empty()) CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  }
};

// One H-matrix: near-field entries F, low-rank factors U, V and s, stored as
// complex FP64 (16 bytes) or complex FP32 (8 bytes) per the precision mode.
struct DevHM {
  DBuf<unsigned char> F, U, V, S;
  DBuf<float2> Flo;      // near_fp64: remainders of the FP64 near-field entries
  bool has_lo = false;
  DBuf<int32_t> rank, flags;
  std::vector<int32_t> h_rank, h_flags;
  DBuf<int2> vwork;  // H-matvec pass-V work items (block, first row)
  int64_t nvwork = 0;
  int prec = 0;
  bool assembled = false;
};

struct GmresWS {
  int64_t N = 0;
  int R = 0, m = 0;
  DBuf<double2> Vb, w, H, g, cs, sn, h, y, cpart, bcopy, r, d;
  DBuf<double> npart, hnorm;
  DBuf<GmresState> st;
  std::vector<GmresState> hst;
  std::vector<double> hpart;
};

}  // namespace

struct bem_handle {
  bem_config cfg{};
  std::string err;
  int device = 0;
  // batched sweep: worker handles (own streams and buffers) cloned from this
  // one's mesh / BC / selector state, and what the autotuner chose
  std::vector<bem_handle*> workers;
  uint64_t state_gen = 0, workers_gen = ~0ull;
  int64_t tuned_workers = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;  // second stream for concurrent ACA launches
  cudaStream_t nearst = nullptr;  // near-field assembly, concurrent with ACA
  int nsm = 152;                  // streaming multiprocessors of the device
  cudaEvent_t fork = nullptr, join = nullptr;
  int64_t launches = 0;
  // mesh
  int64_t N = 0;
  bool have_mesh = false, points_mode = false;
  HTree rows, cols;
  std::vector<Elem> E;
  double avgdim = 0, near_r = 0;
  Layout L;
  DBuf<Elem> dE;
  DBuf<ElemF> dEF;
  DBuf<NearBlock> dNear;
  DBuf<FarBlock> dFar;
  DBuf<int32_t> dOrder, dSpRow, dSpCol, dListOff, dList, dPivCnt, dPivRc;
  DBuf<NearTile> dTiles;
  DBuf<uint32_t> dBits;
  DBuf<int64_t> dSpEntry, dPivOff, dPerm;
  DBuf<LeafRows> dLeaves;
  DBuf<double> dRowPts, dColPts;
  // impedance walls (bem_set_bc_impedance): a = i k beta, b = 1
  std::vector<cplx> beta;
  bool impedance = false;
  // boundary conditions (cluster order)
  bool have_bc = false;
  std::vector<cplx> a, b;
  DBuf<BcCoef> dBc;
  DBuf<double2> dA, dB;
  double k = 0;
  DevHM hm[2];
  DBuf<double2> dT;
  DBuf<float2> dTf, dXf;
  GmresWS gw;
  DBuf<double2> dG, dX, dRhs, dIn, dOut1, dOut2, dOut3;
  // H-LU preconditioner: host factors and their device copies
  // learned quadrature-order selector (device blob, per-entry classes, counters)
  DBuf<SelBlob> dSel;
  DBuf<uint8_t> dAcaTab;  // learned rule table of the ACA entries
  float aca_axes[4] = {0, 0, 0, 0};
  bool have_aca_tab = false;
  bool have_selector = false;
  DBuf<uint8_t> dCls;
  DBuf<unsigned long long> dSelCnt;
  unsigned long long sel_stats[3] = {0, 0, 0};
  // truncating recompression scratch (QR copies of U / V^T, cores)
  DBuf<unsigned char> rcA, rcB, rcC;
  DBuf<int64_t> dCoff;
  bool have_hlu = false;
  double mat_freq = 0;  // frequency of the assembled matrices
  double hlu_freq = 0;  // frequency of the matrix the factors came from
  FlatFactor hL, hU;
  DBuf<int32_t> dLs, dUs;
  DBuf<int64_t> dLl, dUl;
  DBuf<unsigned char> dLd, dUd;  // factor data, complex FP64 or FP32 (hlu_prec)
  int hlu_prec = 0;
  DBuf<double2> dP1, dP2;
  // dataflow form of the sweeps (one plan per factor) and its workspace
  struct DfDev {
    DBuf<unsigned char> chunks, rows, erows, cols, diag;
    DBuf<int64_t> slot;
    HluDfDev view;
  } dfL, dfU;
  bool df_ok = false;
  int df_helpers = 32;  // helper CTAs per dataflow sweep (12 while concurrent sweep workers run)
  int hlu_ctas_per_sm = 0;  // > 0: the executor's grid, per SM, below hp_grid (sweep workers)
  std::string df_why;
  DBuf<unsigned char> dfXi, dfAcc, dfEacc;  // factor-type vectors
  DBuf<unsigned char> dfPre, dfFin;
  DBuf<int> dfCtrl, dfErr;
  DBuf<int> dBad;
  DBuf<double2> dNear64[2];  // near_fp64: FP64 near field before the split
  // GPU H-LU factorization (hlu_gpu.h): the task program of the current
  // layout and rank, its device tables, the arena holding the factors, and
  // the truncation scratch
  uint64_t layout_gen = 0;  // bumped whenever the block offsets change
  bool hlu_dev = false;     // the current factors live in the arena
  HluProgram hp;
  bool hp_ok = false;
  uint64_t hp_gen = ~0ull;
  int64_t hp_kc = -1;
  // a sweep worker starts with its parent's program (same layout): valid
  // while layout_gen still equals hp_inherit_gen
  bool hp_inherited = false;
  uint64_t hp_inherit_gen = 0;
  int hp_prec = -1, hp_grid = 0;
  std::string hp_why;
  DBuf<HluTask> dHT;
  DBuf<int32_t> dHSuccOff, dHSucc;
  DBuf<int32_t> dHPendInit, dHQueueInit, dHCtrlInit;  // the executor's state at launch
  DBuf<int32_t> dHPend, dHQueue;
  DBuf<HluTruncPair> dHPairs;
  DBuf<HluQrOut> dHQr;
  DBuf<int> dHCtrl;
  DBuf<unsigned char> dArena, dHScr, dHBig;
  HluDfPlan hpl, hpu;       // sweep plans of the program's factors (structure)
  // impedance plane (bem_set_impedance_plane): point, unit normal and the
  // elements reflected in it (cluster order)
  // point sources of the right-hand side (bem_set_point_sources)
  std::vector<double> src;
  DBuf<double> dSrc;
  bool have_plane = false;
  double plane_p[3] = {0, 0, 0}, plane_n[3] = {0, 0, 0};
  std::vector<Elem> Er;
  DBuf<Elem> dEr;
  DBuf<ElemF> dEFr;
  DBuf<FieldElemF> dFeR;
  // field evaluation (bem_field): element records, coefficients, partial
  // sums, copies of the caller's points / boundary data / sources
  DBuf<FieldElemF> dFe;
  DBuf<unsigned char> dFcoef;
  DBuf<double2> dFpart, dFphi, dFdphi, dFout1, dFout2;
  DBuf<double> dFpts, dFsrc;
  std::vector<double> field_src;
  QuadRules rules{};
  cudaEvent_t ev[10]{};
};

namespace {

bem_status fail(bem_handle* h, const BemError& e) {
  if (h) h->err = e.msg;
  return e.st;
}

template <typename F>
bem_status guarded(bem_handle* h, F&& f) {
  try {
    f();
    if (h) h->err.clear();
    return BEM_OK;
  } catch (const BemError& e) {
    return fail(h, e);
  } catch (const std::bad_alloc&) {
    return fail(h, BemError{BEM_ENOMEM, "host allocation failed"});
  } catch (const std::exception& e) {
    return fail(h, BemError{BEM_EINVAL, e.what()});
  }
}

double elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  return ms * 1e-3;
}

cplx coupling_parameter(int kind, double k) {
  const cplx I(0.0, 1.0);
  const double tiny = 10.0 * 2.220446049250313080847263336181640625e-16;
  if (kind == 0) return 0.0;
  if (kind == 1) return std::fabs(k) < tiny ? I : I / k;
  return I / (k + 1.0);
}

// ACA size bin: the far blocks (sorted by m + n, largest first) with
// m + n >= thr get the 512-thread ACA kernel. thr <= 0: every block with
// m + n >= 2048, and besides them the largest blocks with m + n >= 512 up to
// half the SM count -- the few long rank loops start at once on their own
// SMs while the 128-thread kernel fills the rest (sphere 20,480: 76 blocks,
// ACA 19.5 ms; thresholds 512 / 1024 / 3072: 21.1 / 20.4 / 34.6 ms).
void set_big_mn(bem_handle* h, int64_t thr) {
  Layout& L = h->L;
  const int64_t nf = (int64_t)L.far_order.size();
  auto count = [&](int64_t t) {
    int64_t c = 0;
    while (c < nf && (int64_t)L.far[L.far_order[c]].m + L.far[L.far_order[c]].n >= t) c++;
    return c;
  };
  if (thr > 0) {
    L.nbig = count(thr);
    return;
  }
  L.nbig = std::max(count(4 * ACA_BIG_MN), std::min<int64_t>(count(ACA_BIG_MN), h->nsm / 2));
}

void upload_layout(bem_handle* h) {
  cudaStream_t s = h->stream;
  const Layout& L = h->L;
  h->dNear.upload(L.near, s);
  h->dFar.upload(L.far, s);
  h->dOrder.upload(L.far_order, s);
  h->dTiles.upload(L.tiles, s);
  h->dBits.upload(L.special_bits, s);
  h->dSpEntry.upload(L.sp_entry, s);
  h->dSpRow.upload(L.sp_row, s);
  h->dSpCol.upload(L.sp_col, s);
  h->dLeaves.upload(L.leaves, s);
  h->dListOff.upload(L.list_off, s);
  h->dList.upload(L.list, s);
  h->dPivOff.upload(L.piv_off, s);
  h->dPivCnt.upload(L.piv_cnt, s);
  h->dPivRc.upload(L.piv_rc, s);
  for (auto& m : h->hm) m.assembled = false;
  h->have_hlu = false;
  h->layout_gen++;
}

// storage precision of the matrices: point clouds (test kernel) stay FP64
int storage_prec(const bem_handle* h) { return h->points_mode ? 0 : h->cfg.precision; }

void alloc_hm(bem_handle* h, DevHM& m) {
  const Layout& L = h->L;
  m.prec = storage_prec(h);
  const size_t es = m.prec ? sizeof(float2) : sizeof(double2);
  m.F.ensure(L.near_entries * es);
  m.U.ensure(L.u_size * es);
  m.V.ensure(L.v_size * es);
  m.S.ensure(L.s_size * es);
  m.rank.ensure(L.far.size());
  m.flags.ensure(L.far.size());
}

// Doubles the rank reservation (up to min(m, n) and ACA_MAX_KCAP) of every
// admissible block whose ACA stopped at it in either matrix, and lays the
// low-rank pools out again. Returns whether any block grew.
bool grow_capped(bem_handle* h) {
  Layout& L = h->L;
  const size_t nf = L.far.size();
  if (h->hm[0].h_flags.size() != nf || h->hm[1].h_flags.size() != nf) return false;
  bool grew = false;
  for (size_t i = 0; i < nf; i++) {
    FarBlock& f = L.far[i];
    const int64_t lim = std::min<int64_t>(std::min(f.m, f.n), ACA_MAX_KCAP);
    if ((h->hm[0].h_flags[i] || h->hm[1].h_flags[i]) && f.kcap < lim) {
      f.kcap = (int32_t)std::min<int64_t>(2 * (int64_t)f.kcap, lim);
      grew = true;
    }
  }
  if (!grew) return false;
  L.u_size = L.v_size = L.s_size = 0;
  for (FarBlock& f : L.far) {
    f.uoff = L.u_size;
    f.voff = L.v_size;
    f.soff = L.s_size;
    L.u_size += (int64_t)f.kcap * f.m;
    L.v_size += (int64_t)f.kcap * f.n;
    L.s_size += f.kcap;
  }
  h->dFar.upload(L.far, h->stream);
  h->layout_gen++;
  return true;
}

std::vector<ElemF> make_elemf(const std::vector<Elem>& E) {
  std::vector<ElemF> F(E.size());
  for (size_t i = 0; i < E.size(); i++) {
    const Elem& e = E[i];
    ElemF f{};
    for (int d = 0; d < 3; d++) {
      f.v[d] = (float)(e.n1[d] - e.c[d]);
      f.v[3 + d] = (float)(e.n2[d] - e.c[d]);
      f.v[6 + d] = (float)(e.n3[d] - e.c[d]);
      f.nrm[d] = (float)e.nrm[d];
      f.c_hi[d] = (float)e.c[d];
      f.c_lo[d] = (float)(e.c[d] - (double)f.c_hi[d]);
    }
    f.area = (float)e.area;
    double emax = 0;
    const double* V[3] = {e.n1, e.n2, e.n3};
    for (int q = 0; q < 3; q++) {
      const double* A = V[q];
      const double* B = V[(q + 1) % 3];
      emax = std::max(emax, std::sqrt((B[0] - A[0]) * (B[0] - A[0]) + (B[1] - A[1]) * (B[1] - A[1]) +
                                      (B[2] - A[2]) * (B[2] - A[2])));
    }
    f.emax = (float)emax;
    F[i] = f;
  }
  return F;
}

void set_frequency(bem_handle* h, double k) {
  require(h->have_bc, BEM_EINVAL, "boundary conditions not set (bem_set_bc)");
  const int64_t N = h->N;
  std::vector<BcCoef> bc(N);
  std::vector<double2> av(N), bv(N);
  for (int64_t i = 0; i < N; i++) {
    // impedance walls: a = i k beta (beta = rho c / Z), rescaled per frequency
    const cplx a = h->impedance ? cplx(0.0, k) * h->beta[i] : h->a[i], b = h->b[i];
    BcCoef c{};
    c.subst = std::abs(a) < std::abs(b) ? 1 : 0;
    cplx inv = c.subst ? 1.0 / b : 1.0 / a;
    cplx ratio = c.subst ? a / b : b / a;
    c.inv_main = make_double2(inv.real(), inv.imag());
    c.ratio = make_double2(ratio.real(), ratio.imag());
    c.finv_main = make_float2((float)inv.real(), (float)inv.imag());
    c.fratio = make_float2((float)ratio.real(), (float)ratio.imag());
    bc[i] = c;
    av[i] = make_double2(a.real(), a.imag());
    bv[i] = make_double2(b.real(), b.imag());
  }
  h->dBc.upload(bc, h->stream);
  h->dA.upload(av, h->stream);
  h->dB.upload(bv, h->stream);
  h->k = k;
}

void sync(bem_handle* h) { CK(cudaStreamSynchronize(h->stream)); }

void fetch_ranks(bem_handle* h, DevHM& m) {
  const size_t nf = h->L.far.size();
  m.h_rank.resize(nf);
  m.h_flags.resize(nf);
  if (nf) {
    CK(cudaMemcpyAsync(m.h_rank.data(), m.rank.p, nf * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(m.h_flags.data(), m.flags.p, nf * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  }
  sync(h);
  // pass-V work items of the H-matvec: 16 rows of one block each, so the
  // largest blocks spread over many CTAs. The buffer holds the most items the
  // rank reservations allow, so it is allocated once per layout: growing it
  // with the ranks of a frequency would free the old one, and cudaFree waits
  // for every stream of the device (all sweep workers' queued kernels).
  int64_t most = 0;
  for (const FarBlock& f : h->L.far) most += ((int64_t)f.kcap + 15) / 16;
  m.vwork.ensure((size_t)std::max<int64_t>(most, 1));
  std::vector<int2> vw;
  for (size_t i = 0; i < nf; i++)
    for (int32_t l0 = 0; l0 < m.h_rank[i]; l0 += 16) vw.push_back(make_int2((int)i, l0));
  m.vwork.upload(vw, h->stream);
  m.nvwork = (int64_t)vw.size();
  sync(h);
  m.assembled = true;
  // factors of the previous matrix: dropped, unless they are kept as the
  // preconditioner of nearby frequencies
  if (&m == &h->hm[1] && !(h->cfg.precond_reuse > 1.0)) h->have_hlu = false;
}

AcaArgs aca_args(bem_handle* h, DevHM& m, int which, int extra) {
  AcaArgs a{};
  a.mode = h->points_mode ? 1 : 0;
  a.precision = m.prec;
  a.E = h->dE.p;
  a.EF = h->dEF.p;
  a.Er = h->have_plane && !h->points_mode ? h->dEr.p : nullptr;
  a.EFr = h->have_plane && !h->points_mode ? h->dEFr.p : nullptr;
  a.bc = h->dBc.p;
  a.k = h->k;
  a.near_r = h->near_r;
  cplx al = coupling_parameter(h->cfg.coupling, h->k);
  a.alpha = make_double2(al.real(), al.imag());
  a.kf = (float)h->k;
  a.near_r2f = (float)(h->near_r * h->near_r);
  a.alphaf = make_float2((float)al.real(), (float)al.imag());
  a.which = which;
  a.rowpts = h->dRowPts.p;
  a.colpts = h->dColPts.p;
  a.far = h->dFar.p;
  a.order = h->dOrder.p;
  a.nfar = (int64_t)h->L.far.size();
  a.U = m.U.p;
  a.V = m.V.p;
  a.S = m.S.p;
  a.rank = m.rank.p;
  a.flags = m.flags.p;
  a.tol = h->cfg.aca_tol;
  a.max_rank = (int)h->cfg.aca_max_rank;
  a.seed = h->cfg.seed;
  a.extra = extra;
  a.piv_off = h->dPivOff.p;
  a.piv_cnt = h->dPivCnt.p;
  a.piv_rc = h->dPivRc.p;
  if ((h->cfg.selector & 2) && m.prec == 1 && !h->points_mode) {
    require(h->have_aca_tab, BEM_EINVAL, "ACA rule table not set (bem_set_aca_rules)");
    a.rule_tab = h->dAcaTab.p;
    a.tab_x0 = h->aca_axes[0];
    a.tab_dx = h->aca_axes[1];
    a.tab_y0 = h->aca_axes[2];
    a.tab_dy = h->aca_axes[3];
  }
  return a;
}

// ACA launches of one or more matrices: blocks with m + n >= ACA_BIG_MN run
// with 512-thread CTAs on the side stream while the rest run with 128-thread
// CTAs on the main stream; the main stream waits for both.
void launch_aca_split(bem_handle* h, std::initializer_list<AcaArgs> mats) {
  cudaStream_t s = h->stream, s2 = h->side;
  const int64_t nbig = h->L.nbig, nfar = (int64_t)h->L.far.size();
  CK(cudaEventRecord(h->fork, s));
  CK(cudaStreamWaitEvent(s2, h->fork, 0));
  for (AcaArgs a : mats) {
    AcaArgs big = a, small = a;
    big.nfar = nbig;
    small.order = a.order + nbig;
    small.nfar = nfar - nbig;
    h->launches += launch_aca(big, 512, s2);
    h->launches += launch_aca(small, 128, s);
  }
  CK(cudaEventRecord(h->join, s2));
  CK(cudaStreamWaitEvent(s, h->join, 0));
}

// Truncating recompression of every admissible block of m on the GPU
// (compressAdmissibleBlock, hmatrix.cpp:101-140, as applied by
// HMatrix(const HMatrix&, rank, relError), hmatrix.cpp:770-776).
void recompress(bem_handle* h, DevHM& m, int64_t rank, double tol) {
  require(m.assembled, BEM_EINVAL, "matrix not assembled");
  require(rank >= 0 && tol >= 0 && std::isfinite(tol), BEM_EINVAL, "bad rank / tolerance");
  const Layout& L = h->L;
  const size_t nf = L.far.size();
  if (!nf) return;
  std::vector<int64_t> coff(nf);
  int64_t tot = 0;
  for (size_t i = 0; i < nf; i++) {
    coff[i] = tot;
    tot += 2 * (int64_t)m.h_rank[i] * m.h_rank[i];
  }
  const size_t es = m.prec ? sizeof(float2) : sizeof(double2);
  cudaStream_t s = h->stream;
  h->rcA.ensure(L.u_size * es);
  h->rcB.ensure(L.v_size * es);
  h->rcC.ensure(std::max<int64_t>(tot, 1) * es);
  h->dCoff.upload(coff, s);
  RecompressArgs a{};
  a.precision = m.prec;
  a.far = h->dFar.p;
  a.order = h->dOrder.p;
  a.nfar = (int64_t)nf;
  a.U = m.U.p;
  a.V = m.V.p;
  a.S = m.S.p;
  a.rank = m.rank.p;
  a.wa = h->rcA.p;
  a.wb = h->rcB.p;
  a.wc = h->rcC.p;
  a.coff = h->dCoff.p;
  a.max_rank = rank;
  a.tol = tol;
  h->launches += launch_recompress(a, s);
  CK(cudaGetLastError());
  fetch_ranks(h, m);
}

// both H-matrices at wavenumber k; optional timing events
void assemble(bem_handle* h, double freq, double* t_near, double* t_aca) {
  require(h->have_mesh && !h->points_mode, BEM_EINVAL, "mesh not set (bem_set_mesh)");
  const double k = 2.0 * M_PI * freq / h->cfg.wave_speed;
  require(k > 0 && std::isfinite(k), BEM_EINVAL, "frequency must be positive and finite");
  set_frequency(h, k);
  h->mat_freq = freq;
  for (auto& m : h->hm) alloc_hm(h, m);
  cudaStream_t s = h->stream;
  cplx al = coupling_parameter(h->cfg.coupling, k);
  NearfieldArgs na{};
  na.precision = h->hm[0].prec;
  na.E = h->dE.p;
  na.EF = h->dEF.p;
  na.Er = h->have_plane ? h->dEr.p : nullptr;
  na.EFr = h->have_plane ? h->dEFr.p : nullptr;
  na.bc = h->dBc.p;
  na.blocks = h->dNear.p;
  na.tiles = h->dTiles.p;
  na.ntiles = (int64_t)h->L.tiles.size();
  na.special_bits = h->dBits.p;
  na.sp_entry = h->dSpEntry.p;
  na.sp_row = h->dSpRow.p;
  na.sp_col = h->dSpCol.p;
  na.nspecial = (int64_t)h->L.sp_entry.size();
  na.k = k;
  na.alpha = make_double2(al.real(), al.imag());
  na.phi = h->hm[0].F.p;
  na.dphi = h->hm[1].F.p;
  CK(cudaEventRecord(h->ev[0], s));
  // the near field (FP64-pipe-bound singular rules, FP32 regular rules) runs
  // on its own stream beside the barrier-bound ACA kernels; both write
  // disjoint pools of the same matrices
  cudaStream_t ns = h->nearst;
  CK(cudaStreamWaitEvent(ns, h->ev[0], 0));
  // the learned near-field orders were trained on free-space pairs: with an
  // impedance plane the near field keeps the 16-point rule
  const bool fp64_near = na.precision == 1 && h->cfg.near_fp64;
  const bool learned = (h->cfg.selector & 1) && na.precision == 1 && !h->have_plane && !fp64_near;
  for (auto& m : h->hm) m.has_lo = false;
  if (fp64_near) {  // FP64 quadrature into temporaries, split into hi + lo below
    h->dNear64[0].ensure(std::max<int64_t>(h->L.near_entries, 1));
    h->dNear64[1].ensure(std::max<int64_t>(h->L.near_entries, 1));
    for (auto& m : h->hm) m.Flo.ensure(std::max<int64_t>(h->L.near_entries, 1));
    na.precision = 0;
    na.phi = h->dNear64[0].p;
    na.dphi = h->dNear64[1].p;
  }
  if (learned) {
    require(h->have_selector, BEM_EINVAL, "selector weights not set (bem_set_selector)");
    h->dCls.ensure(h->L.near_entries);
    h->dSelCnt.ensure(3);
    CK(cudaMemsetAsync(h->dSelCnt.p, 0, 3 * sizeof(unsigned long long), ns));
    SelNearArgs ca{};
    ca.blob = h->dSel.p;
    ca.EF = h->dEF.p;
    ca.blocks = na.blocks;
    ca.tiles = na.tiles;
    ca.ntiles = na.ntiles;
    ca.special_bits = na.special_bits;
    ca.k = k;
    ca.guard_prob = (float)h->cfg.selector_guard;
    ca.cls = h->dCls.p;
    launch_sel_near_classes(ca, ns);
    SelNearfieldArgs fa{};
    fa.EF = h->dEF.p;
    fa.bc = h->dBc.p;
    fa.blocks = na.blocks;
    fa.tiles = na.tiles;
    fa.ntiles = na.ntiles;
    fa.special_bits = na.special_bits;
    fa.cls = h->dCls.p;
    fa.k = (float)k;
    fa.alpha = make_float2((float)al.real(), (float)al.imag());
    fa.phi = (float2*)h->hm[0].F.p;
    fa.dphi = (float2*)h->hm[1].F.p;
    fa.check_every = 16;
    fa.check_tol = 1e-6f;
    fa.counters = h->dSelCnt.p;
    launch_sel_nearfield32(fa, ns);
    h->launches += 2 * (na.ntiles > 0);
    na.ntiles = 0;  // the special entries only
  }
  launch_nearfield(na, ns);
  h->launches += (na.ntiles > 0) + (na.nspecial > 0);
  if (fp64_near) {
    for (int q = 0; q < 2; q++) {
      launch_split_twofloat(h->dNear64[q].p, (float2*)h->hm[q].F.p, h->hm[q].Flo.p,
                            h->L.near_entries, ns);
      h->hm[q].has_lo = true;
    }
    h->launches += 2 * (h->L.near_entries > 0);
  }
  if (learned)
    CK(cudaMemcpyAsync(h->sel_stats, h->dSelCnt.p, 3 * sizeof(unsigned long long),
                       cudaMemcpyDeviceToHost, ns));
  CK(cudaEventRecord(h->ev[1], ns));
  launch_aca_split(h, {aca_args(h, h->hm[0], 0, 0), aca_args(h, h->hm[1], 1, 1)});
  CK(cudaEventRecord(h->ev[2], s));
  CK(cudaStreamWaitEvent(s, h->ev[1], 0));  // join the near field
  CK(cudaGetLastError());
  fetch_ranks(h, h->hm[0]);
  fetch_ranks(h, h->hm[1]);
  // The reference's ACA doubles its reservation whenever a block needs more
  // rank (hmatrix.cpp:557-563) and stops only at the tolerance or acaMaxRank:
  // blocks that reached their device reservation get twice the room (kept
  // for later frequencies) and the ACA of both matrices runs again.
  for (int round = 0; round < 8 && h->cfg.aca_max_rank == 0 && grow_capped(h); round++) {
    for (auto& m : h->hm) alloc_hm(h, m);
    launch_aca_split(h, {aca_args(h, h->hm[0], 0, 0), aca_args(h, h->hm[1], 1, 1)});
    CK(cudaEventRecord(h->ev[2], s));
    CK(cudaGetLastError());
    fetch_ranks(h, h->hm[0]);
    fetch_ranks(h, h->hm[1]);
  }
  // overlapping phases: the near field's own span, and the ACA span from the
  // start of assembly to its last block
  if (t_near) *t_near = elapsed(h->ev[0], h->ev[1]);
  if (t_aca) *t_aca = elapsed(h->ev[0], h->ev[2]);
  if (h->cfg.recompress_tol > 0) {
    CK(cudaEventRecord(h->ev[1], s));
    for (auto& m : h->hm) recompress(h, m, 0, h->cfg.recompress_tol);
    CK(cudaEventRecord(h->ev[2], s));
    sync(h);
    if (t_aca) *t_aca += elapsed(h->ev[1], h->ev[2]);
  }
}

// Arithmetic of an H-matvec on complex-FP32 storage.
enum Arith { ARITH_FP64 = 0, ARITH_FP32 = 1, ARITH_TWOFLOAT = 2 };

// y = (acc ? y : 0) + H x. arith applies to complex-FP32 storage: FP64
// products, FP32 products with compensated sums (inner GMRES operator), or
// two-float products on the FP32 units (FP64-accurate refinement residual).
// Complex-FP64 storage always uses FP64 arithmetic.
// gate_flags: optional converged flags of the R right-hand sides (stride
// GATE_STRIDE ints); the launch does no work when all are set (HmvGate).
constexpr int GATE_STRIDE = (int)(sizeof(GmresState) / sizeof(int));
void hmatvec_dev(bem_handle* h, int which, const double2* x, double2* y, int64_t R, int acc,
                 int arith = ARITH_FP64, const int* gate_flags = nullptr) {
  require(which == 0 || which == 1, BEM_EINVAL, "which must be 0 (phi) or 1 (dPhi)");
  DevHM& m = h->hm[which];
  require(m.assembled, BEM_EINVAL, "matrix not assembled");
  const int64_t nrows = h->points_mode ? (int64_t)h->rows.perm.size() : h->N;
  const int64_t ncols = h->points_mode ? (int64_t)h->cols.perm.size() : h->N;
  if (m.prec == 0) arith = ARITH_FP64;
  const int64_t per = arith == ARITH_TWOFLOAT ? 4 : 8;  // vectors per pass
  const size_t words = arith == ARITH_TWOFLOAT ? 2 : 1;  // float2 words per value
  h->dT.ensure(std::max<int64_t>(h->L.s_size, 1) * 8);
  if (arith != ARITH_FP64) {
    h->dTf.ensure(std::max<int64_t>(h->L.s_size, 1) * 8 * words);
    h->dXf.ensure((size_t)ncols * 8 * words);
  }
  for (int64_t r0 = 0; r0 < R; r0 += per) {
    HmvArgs a{};
    a.precision = m.prec;
    a.fp32_math = arith;
    a.nrhs = (int)std::min<int64_t>(per, R - r0);
    a.far = h->dFar.p;
    a.rank = m.rank.p;
    a.nfar = (int64_t)h->L.far.size();
    a.nearb = h->dNear.p;
    a.leaves = h->dLeaves.p;
    a.nleaves = (int64_t)h->L.leaves.size();
    a.list_off = h->dListOff.p;
    a.list = h->dList.p;
    a.U = m.U.p;
    a.V = m.V.p;
    a.S = m.S.p;
    a.F = m.F.p;
    a.x = x + r0 * ncols;
    a.ldx = ncols;
    a.t = h->dT.p;
    a.ldt = std::max<int64_t>(h->L.s_size, 1);
    a.y = y + r0 * nrows;
    a.ldy = nrows;
    a.accumulate = acc;
    a.xf = h->dXf.p;
    a.tf = h->dTf.p;
    a.vwork = m.vwork.p;
    a.nvwork = m.nvwork;
    a.Flo = (arith == ARITH_TWOFLOAT && m.has_lo) ? m.Flo.p : nullptr;
    if (gate_flags) a.gate = HmvGate{gate_flags + r0 * GATE_STRIDE, GATE_STRIDE, (int)a.nrhs};
    h->launches += launch_hmatvec(a, h->stream);
  }
}

void ensure_gmres(bem_handle* h, int R) {
  GmresWS& g = h->gw;
  const int m = (int)std::max<int64_t>(1, std::min(h->cfg.gmres_restart, h->cfg.gmres_maxit));
  if (g.N == h->N && g.R == R && g.m == m) return;
  const int64_t N = h->N;
  const int nct = krylov_num_ctas(N);
  g.Vb.ensure((size_t)(m + 1) * R * N);
  g.w.ensure((size_t)R * N);
  g.bcopy.ensure((size_t)R * N);
  g.H.ensure((size_t)R * m * (m + 1));
  g.g.ensure((size_t)R * (m + 1));
  g.cs.ensure((size_t)R * m);
  g.sn.ensure((size_t)R * m);
  g.h.ensure((size_t)R * (m + 1));
  g.y.ensure((size_t)R * m);
  g.cpart.ensure((size_t)nct * R * (m + 1));
  // norm partials: one per partial-sum CTA, or one per 256 elements (the
  // fused Arnoldi update writes those)
  g.npart.ensure((size_t)std::max<int64_t>(nct, (h->N + 255) / 256) * R);
  g.hnorm.ensure(R);
  g.st.ensure(R);
  g.hst.resize(R);
  g.N = N;
  g.R = R;
  g.m = m;
}

KrylovArgs krylov_args(bem_handle* h, double2* x) {
  GmresWS& g = h->gw;
  KrylovArgs a{};
  a.N = g.N;
  a.R = g.R;
  a.m = g.m;
  a.tol = h->cfg.gmres_tol;
  a.Vb = g.Vb.p;
  a.w = g.w.p;
  a.x = x;
  a.H = g.H.p;
  a.g = g.g.p;
  a.cs = g.cs.p;
  a.sn = g.sn.p;
  a.h = g.h.p;
  a.y = g.y.p;
  a.cpart = g.cpart.p;
  a.npart = g.npart.p;
  a.hnorm = g.hnorm.p;
  a.st = g.st.p;
  return a;
}

bool read_states(bem_handle* h) {
  GmresWS& g = h->gw;
  CK(cudaMemcpyAsync(g.hst.data(), g.st.p, g.R * sizeof(GmresState), cudaMemcpyDeviceToHost, h->stream));
  sync(h);
  for (const auto& s : g.hst)
    if (!s.done) return false;
  return true;
}

// ---- H-LU preconditioner ----

// host copy of a stored pool in its storage type (complex FP64 or FP32),
// left uninitialized before the copy; at() reads one value as complex FP64
struct HostPool {
  std::unique_ptr<unsigned char[]> buf;
  int prec = 0;
  cplx at(int64_t i) const {
    if (prec == 0) {
      const double2 v = reinterpret_cast<const double2*>(buf.get())[i];
      return cplx(v.x, v.y);
    }
    const float2 v = reinterpret_cast<const float2*>(buf.get())[i];
    return cplx(v.x, v.y);
  }
};

void pool_to_host(const DevHM& m, const DBuf<unsigned char>& src, size_t total, HostPool& out,
                  cudaStream_t s) {
  out.prec = m.prec;
  const size_t bytes = total * (m.prec == 0 ? sizeof(double2) : sizeof(float2));
  out.buf.reset(new unsigned char[std::max<size_t>(bytes, 1)]);
  if (!total) return;
  CK(cudaMemcpyAsync(out.buf.get(), src.p, bytes, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
}

template <typename T>
void upload_bytes(DBuf<unsigned char>& d, const std::vector<T>& v, cudaStream_t s) {
  d.ensure(v.size() * sizeof(T));
  if (!v.empty())
    CK(cudaMemcpyAsync(d.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}

// Plans of the dataflow sweeps for both factors; when either factor lacks
// their structure both sweeps stay on the sequential kernel (df_why says why).
void upload_df_plans(bem_handle* h) {
  h->df_ok = false;
  h->df_why.clear();
  HluDfPlan pl, pu;
  const int eb = h->hlu_prec == 0 ? (int)sizeof(double2) : (int)sizeof(float2);
  if (!hlu_df_plan(h->hL, h->N, eb, pl, &h->df_why) ||
      !hlu_df_plan(h->hU, h->N, eb, pu, &h->df_why))
    return;
  cudaStream_t s = h->stream;
  const size_t cs = h->hlu_prec == 0 ? sizeof(double2) : sizeof(float2);
  int64_t nslot = 0;
  int D = 0;
  for (int q = 0; q < 2; q++) {
    const HluDfPlan& p = q ? pu : pl;
    bem_handle::DfDev& d = q ? h->dfU : h->dfL;
    upload_bytes(d.chunks, p.chunks, s);
    upload_bytes(d.rows, p.rows, s);
    upload_bytes(d.erows, p.erows, s);
    upload_bytes(d.cols, p.cols, s);
    d.slot.upload(p.slot, s);
    if (h->hlu_prec == 0) {
      upload_bytes(d.diag, p.diag, s);
    } else {
      std::vector<float2> fd(p.diag.size());
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < (int64_t)fd.size(); i++)
        fd[i] = make_float2((float)p.diag[i].real(), (float)p.diag[i].imag());
      upload_bytes(d.diag, fd, s);
      CK(cudaStreamSynchronize(s));  // fd goes out of scope
    }
    d.view.chunks = (const HluDfChunk*)d.chunks.p;
    d.view.rows = (const HluDfRow*)d.rows.p;
    d.view.erows = (const HluDfRow*)d.erows.p;
    d.view.cols = (const HluDfCol*)d.cols.p;
    d.view.slot = d.slot.p;
    d.view.nslot = p.nslot;
    d.view.diag = d.diag.p;
    d.view.D = p.D();
    nslot = std::max(nslot, p.nslot);
    D = std::max(D, p.D());
  }
  h->dfXi.ensure((size_t)HLU_DF_MAX_R * h->N * cs);
  h->dfAcc.ensure((size_t)HLU_DF_MAX_R * h->N * cs);
  h->dfEacc.ensure((size_t)HLU_DF_MAX_R * h->N * cs);
  h->dfPre.ensure((size_t)std::max<int64_t>(2 * nslot, 1) * cs);  // pre and pre2
  h->dfFin.ensure((size_t)std::max<int64_t>(nslot, 1) * cs);
  h->dfCtrl.ensure((size_t)(4 + 4 * D));
  h->dfErr.ensure(1);
  CK(cudaMemsetAsync(h->dfErr.p, 0, sizeof(int), s));
  h->df_ok = true;
}

// Bound of one dependency wait of the H-LU executor, in SM clock cycles:
// 2 s at 2 GHz, or BEM_HLU_WAIT_US microseconds (tests of the timeout path).
int64_t hlu_wait_cycles() {
  const char* e = std::getenv("BEM_HLU_WAIT_US");
  const double us = e ? std::atof(e) : 0.0;
  return us > 0 ? (int64_t)(us * 2000.0) : (int64_t)4000000000LL;
}

int df_helpers(const bem_handle* h) {
  const char* e = std::getenv("BEM_HLU_HELPERS");
  const int v = e ? std::atoi(e) : 0;
  return v > 0 ? v : h->df_helpers;
}

// nonzero sticky error word of the dataflow sweeps: a wait ran out of time
void check_df_error(bem_handle* h) {
  if (!h->df_ok) return;
  int e = 0;
  CK(cudaMemcpyAsync(&e, h->dfErr.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (e) {
    CK(cudaMemsetAsync(h->dfErr.p, 0, sizeof(int), h->stream));
    throw BemError{BEM_ETIMEOUT, "H-LU sweep: a dataflow wait ran out of time"};
  }
}

// ---- GPU H-LU factorization ----

bool hlu_device_eligible(const bem_handle* h) {
  return h->cfg.hlu_device && !h->points_mode && h->cfg.precond_rank >= 1 &&
         h->cfg.precond_rank <= 64 && h->cfg.leaf_size <= HLU_GPU_MAX_LEAF + 1;
}

// The task program of the current layout and rank, its device tables and the
// structure of the sweeps (leaf lists, dataflow plans); built once per mesh
// (and again after the rank reservations grow).
bool prepare_hlu_program(bem_handle* h) {
  if (h->hp_ok && h->hp_gen == h->layout_gen && h->hp_kc == h->cfg.precond_rank) return true;
  h->hp_ok = false;
  h->hp_prec = -1;
  HluProgram& P = h->hp;
  const bool inherit = h->hp_inherited && h->hp_inherit_gen == h->layout_gen &&
                       h->hp_kc == h->cfg.precond_rank;
  h->hp_inherited = false;
  std::string why;
  if (!inherit && !hlu_gpu_plan(h->rows, h->L, h->cfg.precond_rank, P, &why)) {
    h->hp_why = why;
    return false;
  }
  require(P.tasks.size() < (size_t)INT32_MAX, BEM_EINVAL, "H-LU program too large");
  cudaStream_t s = h->stream;
  h->dHT.upload(P.tasks, s);
  h->dHSuccOff.upload(P.succ_off, s);
  h->dHSucc.upload(P.succ.empty() ? std::vector<int32_t>{0} : P.succ, s);
  {
    std::vector<int32_t> pend(P.tasks.size());
    for (size_t i = 0; i < P.tasks.size(); i++) pend[i] = P.dep_off[i + 1] - P.dep_off[i];
    h->dHPendInit.upload(pend, s);
  }
  h->dHQueueInit.upload(P.queue_init, s);
  h->dHCtrlInit.upload(std::vector<int32_t>{0, 0, 0, 0, P.nready0, 0, 0, 0}, s);
  h->dHPend.ensure(P.tasks.size());
  h->dHQueue.ensure(P.tasks.size());
  h->dHPairs.upload(P.pairs, s);
  h->dHQr.upload(P.qr, s);
  h->dHCtrl.ensure(8);
  sync(h);
  h->hp_gen = h->layout_gen;
  h->hp_kc = h->cfg.precond_rank;
  h->hp_ok = true;
  return true;
}

// Arena (zeroed once, so padding never holds stale bits), per-CTA scratch for
// the executor's grid and the large truncations' regions, per precision.
void prepare_hlu_arena(bem_handle* h, int prec) {
  const HluProgram& P = h->hp;
  if (h->hp_prec == prec) return;
  const size_t es = prec ? sizeof(float2) : sizeof(double2);
  const int occ = hlu_exec_occupancy(prec);
  require(occ >= 1, BEM_ECUDA, "H-LU executor: its CTA does not fit an SM");
  // CTAs per SM of the executor (all that fit, at most 4; BEM_HLU_CTAS_PER_SM
  // caps it lower, leaving SM room to concurrent sweep workers' kernels)
  int cap = 4;
  if (const char* e = std::getenv("BEM_HLU_CTAS_PER_SM"))
    if (std::atoi(e) >= 1) cap = std::min(4, std::atoi(e));
  h->hp_grid = h->nsm * std::min(occ, cap);
  h->dArena.release();
  h->dHScr.release();
  h->dHBig.release();
  h->dArena.ensure((size_t)P.arena * es);
  CK(cudaMemsetAsync(h->dArena.p, 0, (size_t)P.arena * es, h->stream));
  h->dHScr.ensure((size_t)h->hp_grid * P.scratch * es);
  h->dHBig.ensure((size_t)std::max<int64_t>(P.big_scratch, 1) * es);
  // sweep plans: the staging offsets of their late leaves depend on the
  // element size of the factors
  h->hpl = HluDfPlan();
  h->hpu = HluDfPlan();
  if (P.df_ok) {
    std::string w;
    const bool ok = hlu_df_plan_structure(P.L, h->N, (int)es, h->hpl, &w) &&
                    hlu_df_plan_structure(P.U, h->N, (int)es, h->hpu, &w);
    require(ok, BEM_EINVAL, "H-LU program: sweep plan");
  }
  h->hp_prec = prec;
}

// The dataflow sweeps of the program's factors: plans uploaded without their
// apply matrices, which the QR tasks write into the arena at the plans'
// offsets.
void upload_df_plans_device(bem_handle* h) {
  h->df_ok = false;
  h->df_why = h->hp.df_why;
  if (!h->hp.df_ok) return;
  cudaStream_t s = h->stream;
  const size_t cs = h->hlu_prec == 0 ? sizeof(double2) : sizeof(float2);
  int64_t nslot = 0;
  int D = 0;
  for (int q = 0; q < 2; q++) {
    const HluDfPlan& p = q ? h->hpu : h->hpl;
    bem_handle::DfDev& d = q ? h->dfU : h->dfL;
    upload_bytes(d.chunks, p.chunks, s);
    upload_bytes(d.rows, p.rows, s);
    upload_bytes(d.erows, p.erows, s);
    upload_bytes(d.cols, p.cols, s);
    d.slot.upload(p.slot, s);
    d.view.chunks = (const HluDfChunk*)d.chunks.p;
    d.view.rows = (const HluDfRow*)d.rows.p;
    d.view.erows = (const HluDfRow*)d.erows.p;
    d.view.cols = (const HluDfCol*)d.cols.p;
    d.view.slot = d.slot.p;
    d.view.nslot = p.nslot;
    d.view.diag = h->dArena.p + (size_t)(q ? h->hp.rinv_base : h->hp.qh_base) * cs;
    d.view.D = p.D();
    nslot = std::max(nslot, p.nslot);
    D = std::max(D, p.D());
  }
  h->dfXi.ensure((size_t)HLU_DF_MAX_R * h->N * cs);
  h->dfAcc.ensure((size_t)HLU_DF_MAX_R * h->N * cs);
  h->dfEacc.ensure((size_t)HLU_DF_MAX_R * h->N * cs);
  h->dfPre.ensure((size_t)std::max<int64_t>(2 * nslot, 1) * cs);  // pre and pre2
  h->dfFin.ensure((size_t)std::max<int64_t>(nslot, 1) * cs);
  h->dfCtrl.ensure((size_t)(4 + 4 * D));
  h->dfErr.ensure(1);
  CK(cudaMemsetAsync(h->dfErr.p, 0, sizeof(int), s));
  h->df_ok = true;
}

// H-LU of the truncated copy of the assembled dPhi matrix, on the GPU: one
// launch of the task program (loads of the near-field blocks and truncations
// of the ACA blocks to the preconditioner rank, then the factorization); the
// factors stay in the arena. Returns false, keeping no factors, when a pivot
// is zero or a value is not finite (the solve then runs unpreconditioned, as
// on the host path); a dependency wait that runs out is BEM_ETIMEOUT.
// Summary of one traced factorization: makespan, busy time per task type,
// the measured critical path (longest chain of start-to-end times along the
// dependencies) and the time tasks waited for their dependencies.
void hlu_trace_summary(const HluProgram& P, const DBuf<unsigned long long>& tr, int grid,
                       double tol, const char* path) {
  const size_t nt = P.tasks.size();
  std::vector<unsigned long long> t(3 * nt);
  CK(cudaMemcpy(t.data(), tr.p, t.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  unsigned long long t0 = ~0ull, t1 = 0;
  for (size_t i = 0; i < nt; i++) {
    t0 = std::min(t0, t[3 * i]);
    t1 = std::max(t1, t[3 * i + 2]);
  }
  double busy[8] = {}, wait[8] = {}, mx[8] = {};
  int64_t cnt[8] = {};
  std::vector<double> fin(nt, 0.0);
  std::vector<int32_t> pred(nt, -1);
  int64_t last = 0;
  for (size_t i = 0; i < nt; i++) {
    const int ty = P.tasks[i].type & 7;
    const double d = 1e-3 * (double)(t[3 * i + 2] - t[3 * i + 1]);
    busy[ty] += d;
    mx[ty] = std::max(mx[ty], d);
    wait[ty] += 1e-3 * (double)(t[3 * i + 1] - t[3 * i]);
    cnt[ty]++;
    double best = 0;
    for (int32_t k = P.dep_off[i]; k < P.dep_off[i + 1]; k++)
      if (fin[P.deps[k]] > best) {
        best = fin[P.deps[k]];
        pred[i] = P.deps[k];
      }
    fin[i] = best + d;
    if (fin[i] > fin[last]) last = (int64_t)i;
  }
  int64_t path_cnt[8] = {}, path_loads = 0;
  double path_t[8] = {}, path_load_t = 0;
  std::vector<int64_t> chain;
  for (int64_t i = last; i >= 0; i = pred[i]) {
    const int ty = P.tasks[i].type & 7;
    const double d = 1e-3 * (double)(t[3 * i + 2] - t[3 * i + 1]);
    path_cnt[ty]++;
    path_t[ty] += d;
    chain.push_back(i);
    if (ty == HT_TRUNC && P.tasks[i].x1 == 1 && P.pairs[P.tasks[i].x0].rank_idx >= 0) {
      path_loads++;
      path_load_t += d;
    }
  }
  FILE* f = std::fopen(path, "w");
  if (!f) return;
  const char* nm[8] = {"gemm", "lmul", "rmul", "qr", "trunc", "copy", "zero", "?"};
  std::fprintf(f, "tasks %zu grid %d makespan_us %.1f critical_path_us %.1f\n", nt, grid,
               1e-3 * (double)(t1 - t0), fin[last]);
  for (int k = 0; k < 7; k++)
    std::fprintf(f, "%-6s n %9lld busy_us %12.1f avg_us %8.2f max_us %9.1f wait_us %12.1f "
                 "path_n %6lld path_us %10.1f\n", nm[k], (long long)cnt[k], busy[k],
                 cnt[k] ? busy[k] / cnt[k] : 0.0, mx[k], wait[k], (long long)path_cnt[k], path_t[k]);
  std::fprintf(f, "path loads n %lld us %.1f\n", (long long)path_loads, path_load_t);
  // truncations by the executor's path (column bound q for kt): subspace with
  // the sides in shared memory / in scratch, dense small, range finder, QR
  {
    const char* cn[5] = {"sub_smem", "sub_glob", "small", "range", "qr"};
    int64_t cc[5] = {}, cp[5] = {};
    double cb[5] = {}, cpt[5] = {};
    std::vector<char> on_path(nt, 0);
    for (int64_t i : chain) on_path[i] = 1;
    for (size_t i = 0; i < nt; i++) {
      const HluTask& k = P.tasks[i];
      if ((k.type & 7) != HT_TRUNC) continue;
      const int64_t m = k.m, n = k.n, kt = k.q, kc = P.kc;
      const int64_t subb = hlu_sub_buffers(m, n, kt);
      int c;
      if (kc <= 2 && !(tol > 0) && subb <= HLU_SMEM_ELEMS)
        c = subb + (m + n) * kt <= HLU_SMEM_ELEMS ? 0 : 1;
      else if (m <= 32 && n <= 32)
        c = 2;
      else if (kc <= 8 && !(tol > 0) && kt > kc + 6 && m > kc + 6 && n > kc + 6)
        c = 3;
      else
        c = 4;
      const double d = 1e-3 * (double)(t[3 * i + 2] - t[3 * i + 1]);
      cc[c]++;
      cb[c] += d;
      if (on_path[i]) {
        cp[c]++;
        cpt[c] += d;
      }
    }
    for (int c = 0; c < 5; c++)
      std::fprintf(f, "trunc %-8s n %9lld busy_us %12.1f avg_us %8.2f path_n %6lld path_us %10.1f\n",
                   cn[c], (long long)cc[c], cb[c], cc[c] ? cb[c] / cc[c] : 0.0, (long long)cp[c],
                   cpt[c]);
  }
  {  // the most frequent GEMM shapes (m, n, q, ops) with their mean time
    std::map<std::array<int, 4>, std::pair<int64_t, double>> shp;
    for (size_t i = 0; i < nt; i++) {
      const HluTask& k = P.tasks[i];
      if ((k.type & 7) != HT_GEMM) continue;
      auto& e = shp[{k.m, k.n, k.q, k.flags & 15}];
      e.first++;
      e.second += 1e-3 * (double)(t[3 * i + 2] - t[3 * i + 1]);
    }
    std::vector<std::pair<std::array<int, 4>, std::pair<int64_t, double>>> v(shp.begin(), shp.end());
    std::sort(v.begin(), v.end(), [](const auto& a, const auto& b) { return a.second.second > b.second.second; });
    for (size_t r = 0; r < std::min<size_t>(12, v.size()); r++)
      std::fprintf(f, "gemm m %d n %d q %d ops %d n %lld busy_us %.1f avg_us %.2f\n", v[r].first[0],
                   v[r].first[1], v[r].first[2], v[r].first[3], (long long)v[r].second.first,
                   v[r].second.second, v[r].second.second / v[r].second.first);
  }
  std::sort(chain.begin(), chain.end(), [&](int64_t a, int64_t b) {
    return t[3 * a + 2] - t[3 * a + 1] > t[3 * b + 2] - t[3 * b + 1];
  });
  for (size_t r = 0; r < std::min<size_t>(15, chain.size()); r++) {
    const HluTask& k = P.tasks[chain[r]];
    std::fprintf(f, "path %s m %d n %d q %d pairs %d us %.1f\n", nm[k.type & 7], k.m, k.n, k.q,
                 k.x1, 1e-3 * (double)(t[3 * chain[r] + 2] - t[3 * chain[r] + 1]));
  }
  // the slowest tasks
  std::vector<size_t> ord(nt);
  std::iota(ord.begin(), ord.end(), 0);
  std::partial_sort(ord.begin(), ord.begin() + std::min<size_t>(20, nt), ord.end(),
                    [&](size_t a, size_t b) {
                      return t[3 * a + 2] - t[3 * a + 1] > t[3 * b + 2] - t[3 * b + 1];
                    });
  for (size_t r = 0; r < std::min<size_t>(20, nt); r++) {
    const HluTask& k = P.tasks[ord[r]];
    std::fprintf(f, "slow %s m %d n %d q %d pairs %d us %.1f\n", nm[k.type & 7], k.m, k.n, k.q,
                 k.x1, 1e-3 * (double)(t[3 * ord[r] + 2] - t[3 * ord[r] + 1]));
  }
  std::fclose(f);
}

bool build_hlu_device(bem_handle* h) {
  DevHM& m = h->hm[1];
  const HluProgram& P = h->hp;
  prepare_hlu_arena(h, m.prec);
  cudaStream_t s = h->stream;
  const size_t nt = P.tasks.size();
  CK(cudaMemcpyAsync(h->dHPend.p, h->dHPendInit.p, nt * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(h->dHQueue.p, h->dHQueueInit.p, nt * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(h->dHCtrl.p, h->dHCtrlInit.p, 8 * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
  HluExecArgs a{};
  a.precision = m.prec;
  a.arena = h->dArena.p;
  a.F = m.F.p;
  a.U = m.U.p;
  a.V = m.V.p;
  a.S = m.S.p;
  a.rank = m.rank.p;
  a.tasks = h->dHT.p;
  a.ntasks = (int32_t)P.tasks.size();
  a.succ_off = h->dHSuccOff.p;
  a.succ = h->dHSucc.p;
  a.pairs = h->dHPairs.p;
  a.qr = h->dHQr.p;
  a.pending = h->dHPend.p;
  a.queue = h->dHQueue.p;
  a.ctrl = h->dHCtrl.p;
  a.scratch = h->dHScr.p;
  a.scratch_per_cta = P.scratch;
  a.big_scratch = h->dHBig.p;
  a.kc = P.kc;
  a.tol = h->cfg.precond_tol;
  a.wait_cycles = hlu_wait_cycles();
  {  // power iterations of the truncations' range finder (default 0: on the
     // pencil the factors precondition as well as with one iteration)
    const char* e = std::getenv("BEM_HLU_RANGE_POWER");
    a.range_power = e && *e ? (std::atoi(e) > 0 ? 1 : 0) : 0;
  }
  // BEM_HLU_TRACE=<file>: per-task timestamps, summarised into the file
  const char* trace_path = std::getenv("BEM_HLU_TRACE");
  DBuf<unsigned long long> trace;
  if (trace_path && *trace_path) {
    trace.ensure(3 * P.tasks.size());
    CK(cudaMemsetAsync(trace.p, 0, 3 * P.tasks.size() * sizeof(unsigned long long), s));
    a.trace = trace.p;
  }
  const int grid = h->hlu_ctas_per_sm > 0 ? std::min(h->hp_grid, h->nsm * h->hlu_ctas_per_sm)
                                          : h->hp_grid;  // scratch holds hp_grid CTAs
  const int nl = launch_hlu_exec(a, grid, s);
  require(nl > 0, BEM_ECUDA, "H-LU executor: launch refused");
  h->launches += nl;
  CK(cudaGetLastError());
  launch_hlu_finite_check(h->dArena.p, P.arena, m.prec, h->dHCtrl.p + 3, h->nsm, s);
  h->launches++;
  int ctrl[4] = {0, 0, 0, 0};
  CK(cudaMemcpyAsync(ctrl, h->dHCtrl.p, sizeof(ctrl), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (a.trace) hlu_trace_summary(P, trace, grid, h->cfg.precond_tol, trace_path);
  if (ctrl[1])
    throw BemError{BEM_ETIMEOUT, "H-LU factorization: a task dependency wait ran out of time"};
  if (ctrl[2] || ctrl[3]) return false;
  h->hlu_prec = m.prec;
  h->hL = P.L;
  h->hU = P.U;
  h->dLs.upload(P.L.schedule, s);
  h->dLl.upload(P.L.leaves, s);
  h->dUs.upload(P.U.schedule, s);
  h->dUl.upload(P.U.leaves, s);
  upload_df_plans_device(h);
  CK(cudaStreamSynchronize(s));
  h->hlu_dev = true;
  h->have_hlu = true;
  h->hlu_freq = h->mat_freq;
  return true;
}

// Truncated copy of the assembled dPhi matrix (HMatrix(const HMatrix&, rank,
// err), hmatrix.cpp:770-776) factorized on the host; factors uploaded.
// Returns false, keeping no factors, when they hold NaN or Inf: the solve
// then runs unpreconditioned (LUPair.first.hasNan() ...,
// boundaryelementsolver.cpp:661-668).
bool build_hlu(bem_handle* h) {
  h->have_hlu = false;
  h->hlu_dev = false;
  require(h->hm[1].assembled && !h->points_mode, BEM_EINVAL, "system matrix not assembled");
  if (hlu_device_eligible(h) && prepare_hlu_program(h)) return build_hlu_device(h);
  require(h->cfg.leaf_size <= HLU_MAX_LEAF + 1, BEM_EINVAL,
          "the preconditioner needs leaf_size <= 513");
  DevHM& m = h->hm[1];
  const Layout& L = h->L;
  cudaStream_t s = h->stream;
  HostPool F, U, V, S;
  pool_to_host(m, m.F, L.near_entries, F, s);
  pool_to_host(m, m.U, L.u_size, U, s);
  pool_to_host(m, m.V, L.v_size, V, s);
  pool_to_host(m, m.S, L.s_size, S, s);
  const size_t nb = L.blocks.size();
  std::vector<InBlock> in(nb);
  size_t ni = 0, fi = 0;
  std::vector<int64_t> far_of(nb, -1), near_of(nb, -1);
  for (size_t i = 0; i < nb; i++) (L.blocks[i].adm ? far_of[i] = fi++ : near_of[i] = ni++);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < (int64_t)nb; i++) {
    const HBlockDesc& b = L.blocks[i];
    InBlock& ib = in[i];
    if (!b.adm) {
      const NearBlock& nbk = L.near[near_of[i]];
      ib.F.resize(b.m * b.n);
      for (int64_t e = 0; e < b.m * b.n; e++) ib.F[e] = F.at(nbk.off + e);
      continue;
    }
    const FarBlock& fb = L.far[far_of[i]];
    const int64_t k = m.h_rank[far_of[i]];
    ib.lowrank = true;
    ib.k = k;
    ib.A.resize(b.m * k);
    ib.B.resize(b.n * k);
    for (int64_t l = 0; l < k; l++) {
      const cplx sl = S.at(fb.soff + l);
      for (int64_t r = 0; r < b.m; r++) ib.A[l * b.m + r] = U.at(fb.uoff + l * b.m + r) * sl;
      for (int64_t c = 0; c < b.n; c++) ib.B[l * b.n + c] = V.at(fb.voff + l * b.n + c);
    }
    rk_truncate(b.m, b.n, ib.k, ib.A, ib.B, h->cfg.precond_rank, h->cfg.precond_tol);
  }
  hlu_factor(h->rows, L.blocks, in, h->cfg.precond_rank, h->cfg.precond_tol, h->hL, h->hU);
  for (const FlatFactor* f : {&h->hL, &h->hU})
    for (const cplx& v : f->data)
      if (!std::isfinite(v.real()) || !std::isfinite(v.imag())) return false;
  // every leaf the sweep kernel reads stays inside the vectors, the data pool
  // and its shared-memory staging
  for (const FlatFactor* f : {&h->hL, &h->hU}) {
    const int64_t nd = (int64_t)f->data.size();
    for (int64_t i = 0; i < f->nleaves(); i++) {
      const int64_t* lv = &f->leaves[7 * i];
      const int64_t r0 = lv[0], mm = lv[1], c0 = lv[2], nn = lv[3], kind = lv[4], k = lv[5];
      require(kind != 1 || k <= HLU_MAX_RANK, BEM_EINVAL,
              "preconditioner rank exceeds 512 (set precond_rank)");
      require(kind < 2 || mm <= HLU_MAX_LEAF, BEM_EINVAL, "diagonal leaf exceeds 512 rows");
      const int64_t size = kind == 1 ? (mm + nn) * k : mm * nn;
      require(r0 >= 0 && c0 >= 0 && mm >= 0 && nn >= 0 && r0 + mm <= h->N && c0 + nn <= h->N &&
                  lv[6] >= 0 && lv[6] + size <= nd,
              BEM_EINVAL, "H-LU leaf out of range");
    }
    for (int32_t op : f->schedule)
      require((op >= 0 ? op : -(int64_t)op - 1) < f->nleaves(), BEM_EINVAL,
              "H-LU schedule out of range");
  }
  // the factors are applied in the system matrix's storage precision
  h->hlu_prec = m.prec;
  auto up = [&](const FlatFactor& f, DBuf<int32_t>& ds, DBuf<int64_t>& dl,
                DBuf<unsigned char>& dd) {
    ds.upload(f.schedule, s);
    dl.upload(f.leaves, s);
    if (h->hlu_prec == 0) {
      dd.ensure(f.data.size() * sizeof(double2));
      if (!f.data.empty())
        CK(cudaMemcpyAsync(dd.p, f.data.data(), f.data.size() * sizeof(double2),
                           cudaMemcpyHostToDevice, s));
    } else {
      std::vector<float2> fd(f.data.size());
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < (int64_t)fd.size(); i++)
        fd[i] = make_float2((float)f.data[i].real(), (float)f.data[i].imag());
      dd.ensure(fd.size() * sizeof(float2));
      if (!fd.empty())
        CK(cudaMemcpyAsync(dd.p, fd.data(), fd.size() * sizeof(float2), cudaMemcpyHostToDevice, s));
      CK(cudaStreamSynchronize(s));  // fd goes out of scope
    }
  };
  up(h->hL, h->dLs, h->dLl, h->dLd);
  up(h->hU, h->dUs, h->dUl, h->dUd);
  upload_df_plans(h);
  CK(cudaStreamSynchronize(s));
  h->have_hlu = true;
  h->hlu_freq = h->mat_freq;
  return true;
}

// factor data (which = 0 L, 1 U): the arena on the device path (the leaf
// offsets of the program's leaf lists point into it), else the uploads of the
// host factors
const void* hlu_data(const bem_handle* h, int which) {
  if (h->hlu_dev) return h->dArena.p;
  return which ? h->dUd.p : h->dLd.p;
}

// mean driver phase times of a traced lower sweep: wait for R(i), corner,
// solve, hand-over to the next chunk (appended to path)
void df_trace_summary(bem_handle* h, const DBuf<unsigned long long>& tr, int R, const char* path) {
  const int D = h->dfL.view.D;
  std::vector<unsigned long long> t(4 * (size_t)D);
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(t.data(), tr.p, t.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  double ph[4] = {};
  for (int i = 0; i + 1 < D; i++) {
    ph[0] += 1e-3 * (double)(t[4 * i + 1] - t[4 * i]);
    ph[1] += 1e-3 * (double)(t[4 * i + 2] - t[4 * i + 1]);
    ph[2] += 1e-3 * (double)(t[4 * i + 3] - t[4 * i + 2]);
    ph[3] += 1e-3 * (double)(t[4 * (i + 1)] - t[4 * i + 3]);
  }
  FILE* f = std::fopen(path, "a");
  if (!f) return;
  const double n = D > 1 ? (double)(D - 1) : 1.0;
  std::fprintf(f, "df L sweep: chunks %d R %d total_us %.1f per chunk us: wait %.3f corner %.3f "
               "solve %.3f handover %.3f\n", D, R, 1e-3 * (double)(t[4 * (D - 1) + 3] - t[0]),
               ph[0] / n, ph[1] / n, ph[2] / n, ph[3] / n);
  // the wait by corner kind (device factors: the program's plan): none,
  // full, low rank, low rank with a prefix (R(i) then waits for C(i - 2))
  if (h->hlu_dev && (int)h->hpl.chunks.size() == D + 1) {
    double wsum[4] = {}, late[4] = {};
    int64_t cnt[4] = {};
    for (int i = 1; i + 1 < D; i++) {
      const HluDfChunk& c = h->hpl.chunks[i];
      const int kind = c.corner < 0 ? 0 : (!(c.cflags & 1) ? 1 : ((c.cflags & 2) ? 3 : 2));
      wsum[kind] += 1e-3 * (double)(t[4 * i + 1] - t[4 * i]);
      late[kind] += (double)(h->hpl.chunks[i + 1].rbeg - c.rbeg);
      cnt[kind]++;
    }
    const char* nm[4] = {"none", "full", "lowrank", "lowrank+pre"};
    for (int k = 0; k < 4; k++)
      if (cnt[k])
        std::fprintf(f, "  corner %-11s chunks %6lld wait_us %.3f late_entries %.2f\n", nm[k],
                     (long long)cnt[k], wsum[k] / cnt[k], late[k] / cnt[k]);
  }
  std::fclose(f);
}

// w := U^{-1} L^{-1} w for R device vectors (LUPrecondidionedHMatrixWrapper's
// two substitutions, gmres.h:134-147)
void apply_precond(bem_handle* h, double2* w, int R, const int* gate_flags = nullptr) {
  const int64_t N = h->N;
  cudaStream_t s = h->stream;
  if (h->df_ok) {  // dataflow sweeps: w -> dP2 -> w, up to 8 vectors per launch
    h->dP2.ensure((size_t)std::min(R, HLU_DF_MAX_R) * N);
    HluDfWork ws{h->dfXi.p, h->dfAcc.p, h->dfEacc.p, h->dfPre.p, h->dfFin.p, h->dfCtrl.p, h->dfErr.p};
    if (const char* e = std::getenv("BEM_DF_WAIT_US"))  // tests of the timeout path
      if (std::atof(e) > 0) ws.wait_ns = (unsigned long long)(std::atof(e) * 1000.0);
    const int hp = df_helpers(h);
    // BEM_DF_TRACE=<file>: the lower sweep's driver phases of this
    // application, summarised into the file (profiling)
    const char* trace_path = std::getenv("BEM_DF_TRACE");
    DBuf<unsigned long long> trace;
    if (trace_path && *trace_path) {
      trace.ensure(4 * (size_t)h->dfL.view.D);
      ws.trace = trace.p;
    }
    for (int r0 = 0; r0 < R; r0 += HLU_DF_MAX_R) {
      const int rc = std::min(HLU_DF_MAX_R, R - r0);
      double2* wr = w + (size_t)r0 * N;
      const HmvGate gate = gate_flags ? HmvGate{gate_flags + r0 * GATE_STRIDE, GATE_STRIDE, rc}
                                      : HmvGate{nullptr, 0, 0};
      h->launches += launch_hlu_df(h->dfL.view, h->dLl.p, hlu_data(h, 0), h->hlu_prec, wr, h->dP2.p,
                                   N, rc, ws, hp, s, gate);
      HluDfWork wu = ws;
      wu.trace = nullptr;
      h->launches += launch_hlu_df(h->dfU.view, h->dUl.p, hlu_data(h, 1), h->hlu_prec, h->dP2.p, wr,
                                   N, rc, wu, hp, s, gate);
    }
    if (ws.trace) df_trace_summary(h, trace, R, trace_path);
    return;
  }
  h->dP1.ensure((size_t)R * N);
  h->dP2.ensure((size_t)R * N);
  CK(cudaMemcpyAsync(h->dP1.p, w, (size_t)R * N * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  h->launches += launch_hlu_sweep(h->dLs.p, (int)h->hL.schedule.size(), h->dLl.p, hlu_data(h, 0),
                                  h->hlu_prec, h->dP1.p, h->dP2.p, N, R, 0, s);
  h->launches += launch_hlu_sweep(h->dUs.p, (int)h->hU.schedule.size(), h->dUl.p, hlu_data(h, 1),
                                  h->hlu_prec, h->dP2.p, w, N, R, 1, s);
}

bool use_precond(const bem_handle* h) { return h->cfg.use_preconditioner && h->have_hlu; }

struct GmresResult {
  int64_t iters = 0;
  double resid = 0;
  bool converged = false;
};

// Restarted GMRES for R right-hand sides on the dPhi matrix (device b, x;
// x holds the initial guess). f32 selects the FP32-arithmetic operator.
// estimate_ok: stop when the Arnoldi residual estimates of all right-hand
// sides meet tol, without the explicit residual of the updated x (one more
// operator product and preconditioner application); for the inner solves of
// the refinement, whose outer step measures the true residual in FP64.
GmresResult gmres_core(bem_handle* h, const double2* b, double2* x, int R, double tol,
                       int64_t maxit, bool f32, bool x_zero = false, bool estimate_ok = false) {
  ensure_gmres(h, R);
  GmresWS& g = h->gw;
  const int64_t N = h->N;
  cudaStream_t s = h->stream;
  KrylovArgs a = krylov_args(h, x);
  a.tol = tol;
  // with the H-LU preconditioner the iteration runs on (LU)^{-1} A x =
  // (LU)^{-1} b and the tolerance applies to that residual, as in
  // GMRES::gmresLUPreconditionedSolve (gmres.h:191-207)
  const bool pc = use_precond(h);
  CK(cudaMemcpyAsync(g.bcopy.p, b, (size_t)R * N * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  if (pc) apply_precond(h, g.bcopy.p, R);
  CK(cudaMemcpyAsync(g.w.p, g.bcopy.p, (size_t)R * N * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  krylov_restart(a, 1, s);  // measures ||b||
  h->launches += 2;
  int64_t total = 0;
  bool first = true;
  while (true) {
    if (first && x_zero) {  // r = b: skip the product with the zero guess
      CK(cudaMemcpyAsync(g.w.p, g.bcopy.p, (size_t)R * N * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    } else {
      hmatvec_dev(h, 1, x, g.w.p, R, 0, f32);
      if (pc) apply_precond(h, g.w.p, R);
      krylov_residual(g.bcopy.p, g.w.p, (int64_t)R * N, s);
      h->launches++;
    }
    first = false;
    krylov_restart(a, 0, s);
    h->launches += 2;
    if (read_states(h) || total >= maxit) break;
    // the operator products of an Arnoldi step are gated by the converged
    // flags: the steps run past convergence before the next host check
    // (every 8 steps) do no work
    const int* done_flags = &g.st.p[0].done;
    bool conv = false;
    for (int j = 0; j < g.m; j++) {
      hmatvec_dev(h, 1, g.Vb.p + (int64_t)j * R * N, g.w.p, R, 0, f32, done_flags);
      if (pc) apply_precond(h, g.w.p, R, done_flags);
      h->launches += krylov_orthogonalize(a, j, s);
      total++;
      const bool last = (j == g.m - 1) || total >= maxit;
      if (((j + 1) % 8 == 0) || last) {
        if (read_states(h)) {
          conv = true;
          break;
        }
      }
      if (total >= maxit) break;
    }
    krylov_update(a, s);
    h->launches += 2;
    if (conv && estimate_ok) break;
  }
  CK(cudaGetLastError());
  GmresResult res;
  res.converged = true;
  for (const auto& st : g.hst) {
    res.iters = std::max<int64_t>(res.iters, st.iters);
    res.resid = std::max(res.resid, st.resid);
    res.converged = res.converged && st.done;
  }
  return res;
}

// per-RHS 2-norms of R device vectors of length N
std::vector<double> norms(bem_handle* h, const double2* v, int R) {
  GmresWS& g = h->gw;
  const int nct = krylov_num_ctas(h->N);
  g.npart.ensure((size_t)nct * R);
  krylov_norm_partials(v, h->N, R, g.npart.p, h->stream);
  h->launches++;
  g.hpart.resize((size_t)nct * R);
  CK(cudaMemcpyAsync(g.hpart.data(), g.npart.p, g.hpart.size() * sizeof(double),
                     cudaMemcpyDeviceToHost, h->stream));
  sync(h);
  std::vector<double> out(R, 0.0);
  for (int c = 0; c < nct; c++)
    for (int r = 0; r < R; r++) out[r] += g.hpart[(size_t)c * R + r];
  for (auto& v2 : out) v2 = std::sqrt(v2);
  return out;
}

// Solve dPhi x = b for R right-hand sides (device b, x; x = initial guess).
// precision 0: GMRES with the complex-FP64 operator (GMRES::gmresSolve,
// gmres.h:170-180). precision 1: FP64 iterative refinement -- the residual
// b - A x uses FP64 arithmetic on the stored complex-FP32 operator, each
// correction comes from GMRES on the FP32-arithmetic operator.
void gmres_dev(bem_handle* h, const double2* b, double2* x, int R, bem_solve_info* info,
               bool x_zero = false) {
  require(h->hm[1].assembled, BEM_EINVAL, "system matrix not assembled");
  const double tol = h->cfg.gmres_tol;
  const int64_t maxit = h->cfg.gmres_maxit;
  bem_solve_info loc{};
  if (h->hm[1].prec == 0) {
    GmresResult r = gmres_core(h, b, x, R, tol, maxit, false, x_zero);
    loc.iterations = r.iters;
    loc.rel_residual = loc.true_residual = r.resid;
    loc.status = r.converged ? BEM_OK : BEM_EMAXIT;
    if (use_precond(h)) {  // r.resid is the preconditioned residual
      GmresWS& g = h->gw;
      g.r.ensure((size_t)R * h->N);
      hmatvec_dev(h, 1, x, g.r.p, R, 0);
      krylov_residual(b, g.r.p, (int64_t)R * h->N, h->stream);
      h->launches++;
      const std::vector<double> bn = norms(h, b, R), rn = norms(h, g.r.p, R);
      loc.true_residual = 0;
      for (int q = 0; q < R; q++)
        loc.true_residual = std::max(loc.true_residual, bn[q] > 0 ? rn[q] / bn[q] : 0.0);
    }
  } else {
    GmresWS& g = h->gw;
    const int64_t N = h->N;
    cudaStream_t s = h->stream;
    ensure_gmres(h, R);
    g.r.ensure((size_t)R * N);
    g.d.ensure((size_t)R * N);
    const std::vector<double> bn = norms(h, b, R);
    int64_t total = 0;
    double rel = 0, inner_res = 0;
    for (int outer = 0; outer < 30; outer++) {
      // r = b - A x with FP64 arithmetic on the stored operator
      if (outer == 0 && x_zero) {
        CK(cudaMemcpyAsync(g.r.p, b, (size_t)R * N * sizeof(double2), cudaMemcpyDeviceToDevice, s));
      } else {
        hmatvec_dev(h, 1, x, g.r.p, R, 0, ARITH_TWOFLOAT);
        krylov_residual(b, g.r.p, (int64_t)R * N, s);
        h->launches++;
      }
      const std::vector<double> rn = norms(h, g.r.p, R);
      rel = 0;
      for (int q = 0; q < R; q++) rel = std::max(rel, bn[q] > 0 ? rn[q] / bn[q] : 0.0);
      if (rel < tol || total >= maxit) break;
      // the correction only has to gain the missing digits, but FP32
      // products cap what one inner solve can deliver at about 1e-6
      const double inner_tol = std::max(1e-6, 0.3 * tol / rel);
      CK(cudaMemsetAsync(g.d.p, 0, (size_t)R * N * sizeof(double2), s));
      GmresResult ir = gmres_core(h, g.r.p, g.d.p, R, inner_tol, maxit - total, true, true, true);
      total += ir.iters;
      inner_res = ir.resid;
      krylov_axpy(x, g.d.p, (int64_t)R * N, s);
      h->launches++;
    }
    loc.iterations = total;
    loc.rel_residual = inner_res;
    loc.true_residual = rel;
    loc.status = rel < tol ? BEM_OK : BEM_EMAXIT;
  }
  if (info) {
    info->iterations = loc.iterations;
    info->rel_residual = loc.rel_residual;
    info->true_residual = loc.true_residual;
    info->status = loc.status;
  }
}

void fill_rank_info(bem_handle* h, bem_solve_info* info) {
  if (!info) return;
  int64_t mr = 0, capped = 0;
  for (int w = 0; w < 2; w++) {
    const DevHM& m = h->hm[w];
    for (size_t i = 0; i < m.h_rank.size(); i++) {
      if (w == 1) mr = std::max<int64_t>(mr, m.h_rank[i]);
      capped += m.h_flags[i] ? 1 : 0;
    }
  }
  info->max_rank = mr;
  info->capped_blocks = capped;
}

// One frequency, all R right-hand sides; g / outputs are device pointers in
// caller order.
void solve_dev(bem_handle* h, double freq, const double2* g_caller, int64_t R, double2* phi,
               double2* dphi, double2* p, bem_solve_info* info) {
  require(R >= 1, BEM_EINVAL, "nrhs must be >= 1");
  const int64_t N = h->N;
  cudaStream_t s = h->stream;
  auto t0 = std::chrono::steady_clock::now();
  bem_solve_info loc{};
  assemble(h, freq, &loc.t_nearfield, &loc.t_aca);
  const auto t_asm = std::chrono::steady_clock::now();
  if (h->cfg.use_preconditioner) {
    const double r = h->hlu_freq > 0 ? std::max(freq / h->hlu_freq, h->hlu_freq / freq) : 0.0;
    if (h->have_hlu && h->cfg.precond_reuse > 1.0 && r > 0 && r <= h->cfg.precond_reuse) {
      loc.precond_reused = 1;
    } else {
      const auto tp = std::chrono::steady_clock::now();
      build_hlu(h);  // non-finite factors: continue without the preconditioner
      loc.t_precond = std::chrono::duration<double>(std::chrono::steady_clock::now() - tp).count();
    }
  }
  const auto t_pc = std::chrono::steady_clock::now();
  h->dG.ensure((size_t)R * N);
  h->dRhs.ensure((size_t)R * N);
  h->dX.ensure((size_t)R * N);
  launch_gather(g_caller, h->dG.p, h->dPerm.p, N, (int)R, s);
  h->launches++;
  CK(cudaEventRecord(h->ev[3], s));
  // rhs = source term + phi * g  (boundaryelementsolver.cpp:578-579)
  hmatvec_dev(h, 0, h->dG.p, h->dRhs.p, R, 0, ARITH_TWOFLOAT);  // FP64-accurate, FP32 units
  if (!h->src.empty()) {
    const cplx al = coupling_parameter(h->cfg.coupling, h->k);
    h->launches += launch_source_rhs(h->dE.p, N, h->dSrc.p, (int)(h->src.size() / 5), h->k,
                                     make_double2(al.real(), al.imag()), h->dRhs.p, (int)R, s);
  }
  CK(cudaEventRecord(h->ev[4], s));
  if (use_precond(h)) {  // initial guess (LU)^{-1} rhs (boundaryelementsolver.cpp:688)
    CK(cudaMemcpyAsync(h->dX.p, h->dRhs.p, (size_t)R * N * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    apply_precond(h, h->dX.p, (int)R);
    gmres_dev(h, h->dRhs.p, h->dX.p, (int)R, &loc, false);
  } else {
    CK(cudaMemsetAsync(h->dX.p, 0, (size_t)R * N * sizeof(double2), s));
    gmres_dev(h, h->dRhs.p, h->dX.p, (int)R, &loc, true);
  }
  CK(cudaEventRecord(h->ev[5], s));
  const auto t_gm = std::chrono::steady_clock::now();
  const double omega = 2.0 * M_PI * freq;
  double2 pfac = make_double2(0.0, h->cfg.density * omega);
  launch_backsub(h->dX.p, h->dG.p, h->dA.p, h->dB.p, h->dBc.p, h->dPerm.p, N, (int)R, pfac, phi,
                 dphi, p, s);
  h->launches++;
  h->dBad.ensure(1);
  CK(cudaMemsetAsync(h->dBad.p, 0, sizeof(int), s));
  h->launches += launch_finite_check(h->dX.p, R * N, h->dBad.p, s);
  int bad = 0;
  CK(cudaMemcpyAsync(&bad, h->dBad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  sync(h);
  if (use_precond(h)) check_df_error(h);
  loc.t_rhs = elapsed(h->ev[3], h->ev[4]);
  loc.t_gmres = elapsed(h->ev[4], h->ev[5]);
  loc.t_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (std::getenv("BEM_SOLVE_TRACE")) {  // host wall times of the steps (profiling)
    auto sec = [&](std::chrono::steady_clock::time_point t) {
      return std::chrono::duration<double>(t - t0).count();
    };
    std::fprintf(stderr,
                 "solve h %p f %.2f wall: assembled %.4f precond %.4f gmres %.4f total %.4f | "
                 "device: nearfield %.4f aca %.4f rhs %.4f gmres %.4f iters %lld\n",
                 (void*)h, freq, sec(t_asm), sec(t_pc), sec(t_gm), loc.t_total, loc.t_nearfield,
                 loc.t_aca, loc.t_rhs, loc.t_gmres, (long long)loc.iterations);
  }
  fill_rank_info(h, &loc);
  if (bad) loc.status = BEM_ENONFINITE;
  if (info) *info = loc;
  if (bad) throw BemError{BEM_ENONFINITE, "non-finite values in the solution"};
}

void copy_in(bem_handle* h, DBuf<double2>& d, const double* src, size_t cnt) {
  d.ensure(cnt);
  CK(cudaMemcpyAsync(d.p, src, cnt * sizeof(double2), cudaMemcpyHostToDevice, h->stream));
}

void copy_out(bem_handle* h, double* dst, const double2* src, size_t cnt) {
  if (!dst) return;
  CK(cudaMemcpyAsync(dst, src, cnt * sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
}

// ---- batched frequency sweep ----

// A worker gets the parent's mesh, layout, BCs and selector weights (host
// copies plus its own device uploads), so it can solve any frequency alone.
void clone_state(bem_handle* c, bem_handle* p) {
  c->rows = p->rows;
  c->cols = p->cols;
  c->N = p->N;
  c->E = p->E;
  c->avgdim = p->avgdim;
  c->near_r = p->near_r;
  c->L = p->L;
  c->points_mode = false;
  c->dE.upload(c->E, c->stream);
  c->dEF.upload(make_elemf(c->E), c->stream);
  c->dPerm.upload(c->rows.perm, c->stream);
  upload_layout(c);
  c->have_mesh = true;
  c->a = p->a;
  c->b = p->b;
  c->beta = p->beta;
  c->impedance = p->impedance;
  c->have_bc = p->have_bc;
  c->src = p->src;
  if (!c->src.empty()) c->dSrc.upload(c->src, c->stream);
  c->have_plane = p->have_plane;
  if (p->have_plane) {
    for (int d = 0; d < 3; d++) {
      c->plane_p[d] = p->plane_p[d];
      c->plane_n[d] = p->plane_n[d];
    }
    c->Er = p->Er;
    c->dEr.upload(c->Er, c->stream);
    c->dEFr.upload(make_elemf(c->Er), c->stream);
  }
  c->have_aca_tab = p->have_aca_tab;
  if (p->have_aca_tab) {
    c->dAcaTab.ensure(ACA_TAB_N * ACA_TAB_N);
    CK(cudaMemcpyAsync(c->dAcaTab.p, p->dAcaTab.p, ACA_TAB_N * ACA_TAB_N, cudaMemcpyDeviceToDevice,
                       c->stream));
    for (int i = 0; i < 4; i++) c->aca_axes[i] = p->aca_axes[i];
  }
  if (p->hp_ok && p->hp_gen == p->layout_gen) {  // the parent's H-LU program fits this layout
    c->hp = p->hp;
    c->hp_kc = p->hp_kc;
    c->hp_inherited = true;
    c->hp_inherit_gen = c->layout_gen;
  }
  c->have_selector = false;
  if (p->have_selector) {
    c->dSel.ensure(1);
    CK(cudaMemcpyAsync(c->dSel.p, p->dSel.p, sizeof(SelBlob), cudaMemcpyDeviceToDevice, c->stream));
    c->have_selector = true;
  }
  sync(c);
}

// nw worker handles beside h, cloned from h's current state
void ensure_workers(bem_handle* h, int nw) {
  CK(cudaSetDevice(h->device));
  if (h->workers_gen != h->state_gen) {
    for (bem_handle* w : h->workers) bem_destroy(w);
    h->workers.clear();
    h->workers_gen = h->state_gen;
  }
  while ((int)h->workers.size() < nw) {
    bem_config c = h->cfg;
    c.sweep_workers = 1;
    bem_handle* w = nullptr;
    const bem_status st = bem_create(&c, &w);
    require(st == BEM_OK && w, st == BEM_OK ? BEM_ECUDA : st, "could not create a sweep worker");
    h->workers.push_back(w);
    try {
      clone_state(w, h);
    } catch (...) {
      bem_destroy(w);
      h->workers.pop_back();
      throw;
    }
  }
}

// Frequencies idx[0..n) of a sweep on W handles (h and W - 1 workers), one
// host thread per handle, each on its own stream; a handle that is free takes
// the next frequency of idx (a shared counter: the sweep ends at most one
// solve after the average load instead of with the heaviest share of a fixed
// split; each frequency's result is the same on every handle). With H-LU
// factor reuse each handle takes a fixed contiguous block of ascending
// frequencies instead. p (caller order, n_freq slices) gets each frequency's pressure.
// With device pointers (gd, pd non-null) instead of g / p: every worker reads
// gd and writes its frequencies' slices of pd directly; the workers' streams
// start after the work already on h's stream and h's stream waits for them.
// on_done (host buffers only; may be null) runs after each frequency's slice
// of p and its info record are written, one call at a time across the
// handles; a true return stops the sweep before the next frequency of every
// handle (the ones running finish and are reported).
void run_sweep(bem_handle* h, int W, const double* freqs, const int64_t* idx, int64_t n,
               const double* g, int64_t nrhs, double* p, bem_solve_info* info,
               bem_status& worst, const double2* gd = nullptr, double2* pd = nullptr,
               const std::function<bool(int64_t)>* on_done = nullptr) {
  require(h->have_mesh && h->have_bc && !h->points_mode, BEM_EINVAL,
          "mesh and boundary conditions must be set");
  W = (int)std::max<int64_t>(1, std::min<int64_t>(W, n));
  ensure_workers(h, W - 1);
  std::vector<bem_handle*> hs{h};
  for (int w = 0; w + 1 < W; w++) hs.push_back(h->workers[w]);
  // A lone solve is fastest with 32 helpers per dataflow sweep and the
  // executor on every CTA an SM holds (4). Concurrent workers share the SMs
  // (each helper holds a whole SM's registers; an executor grid of 4 per SM
  // fills the GPU while its critical path leaves most CTAs waiting). On the
  // 81,920-triangle pencil with 6 workers: 32 / 16 / 12 / 8 helpers measured
  // 0.51 / 0.48 / 0.46 / 0.47 s per frequency (executor at 4 per SM); with
  // 12 helpers, the executor at 4 / 2 / 1 per SM 0.465 / 0.397 / 0.390 s.
  for (bem_handle* x : hs) {
    x->df_helpers = W > 1 ? 12 : 32;
    x->hlu_ctas_per_sm = W > 1 ? 1 : 0;
  }
  struct Restore {
    bem_handle* h;
    ~Restore() {
      h->df_helpers = 32;
      h->hlu_ctas_per_sm = 0;
    }
  } restore{h};
  const size_t cnt = (size_t)h->N * nrhs;
  const bool dev = gd != nullptr;
  cudaEvent_t e0 = nullptr;
  std::vector<cudaEvent_t> ew(W, nullptr);
  if (dev) {
    CK(cudaEventCreateWithFlags(&e0, cudaEventDisableTiming));
    for (auto& e : ew) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    CK(cudaEventRecord(e0, h->stream));
  }
  std::vector<bem_status> st(W, BEM_OK), wst(W, BEM_OK);
  std::atomic<bool> stop{false};
  std::atomic<int64_t> next{0};
  std::mutex done_mu;
  const bool blocks = h->cfg.use_preconditioner && h->cfg.precond_reuse > 1.0;
  // the k-th position of handle w's share of idx, or n when it has none left
  auto claim = [&](int w, int64_t k) -> int64_t {
    if (stop.load(std::memory_order_acquire)) return n;
    if (!blocks) return std::min<int64_t>(n, next.fetch_add(1));
    const int64_t i = n * w / W + k;
    return i < n * (w + 1) / W ? i : n;
  };
  auto body = [&](int w) {
    bem_handle* x = hs[w];
    st[w] = guarded(x, [&] {
      CK(cudaSetDevice(h->device));
      if (dev) {
        CK(cudaStreamWaitEvent(x->stream, e0, 0));
        for (int64_t k = 0, i; (i = claim(w, k)) < n; k++) {
          const int64_t f = idx[i];
          bem_solve_info loc{};
          solve_dev(x, freqs[f], gd, nrhs, nullptr, nullptr, pd + cnt * f, &loc);
          if (info) info[f] = loc;
          if (loc.status != BEM_OK) wst[w] = loc.status;
        }
        CK(cudaEventRecord(ew[w], x->stream));
        return;
      }
      copy_in(x, x->dIn, g, cnt);
      x->dOut3.ensure(cnt);
      // with factor reuse, each handle takes a contiguous block of the
      // (sorted) frequencies, so its consecutive solves are close
      for (int64_t k = 0, i; (i = claim(w, k)) < n; k++) {
        const int64_t f = idx[i];
        bem_solve_info loc{};
        solve_dev(x, freqs[f], x->dIn.p, nrhs, nullptr, nullptr, x->dOut3.p, &loc);
        copy_out(x, p + 2 * cnt * f, x->dOut3.p, cnt);
        sync(x);
        if (info) info[f] = loc;
        if (loc.status != BEM_OK) wst[w] = loc.status;
        if (on_done) {
          std::lock_guard<std::mutex> lk(done_mu);
          if ((*on_done)(f)) stop.store(true, std::memory_order_release);
        }
      }
    });
  };
  if (W == 1) {
    body(0);
  } else {
    std::vector<std::thread> th;
    for (int w = 1; w < W; w++) th.emplace_back(body, w);
    body(0);
    for (auto& t : th) t.join();
  }
  if (dev) {
    for (int w = 0; w < W; w++)
      if (st[w] == BEM_OK) CK(cudaStreamWaitEvent(h->stream, ew[w], 0));
    CK(cudaEventDestroy(e0));
    for (auto& e : ew) CK(cudaEventDestroy(e));
  }
  for (int w = 0; w < W; w++) {
    if (st[w] != BEM_OK) throw BemError{st[w], "sweep worker: " + hs[w]->err};
    if (wst[w] != BEM_OK) worst = wst[w];
  }
}

// Wall-clock rate (frequencies per second) of W workers on nrep * W copies of
// a probe frequency (distinct by 1e-6 relative, so nothing is reused).
double probe_rate(bem_handle* h, int W, double freq, int64_t nrhs, int nrep) {
  const int64_t n = (int64_t)W * nrep;
  std::vector<double> fr(n);
  std::vector<int64_t> idx(n);
  for (int64_t i = 0; i < n; i++) {
    fr[i] = freq * (1.0 + 1e-6 * (double)(i + 1));
    idx[i] = i;
  }
  std::vector<double> g(2 * (size_t)h->N * nrhs, 0.0), p(2 * (size_t)h->N * nrhs * n);
  for (size_t i = 0; i < (size_t)h->N * nrhs; i++) g[2 * i] = 1.0;
  bem_status worst = BEM_OK;
  const auto t0 = std::chrono::steady_clock::now();
  run_sweep(h, W, fr.data(), idx.data(), n, g.data(), nrhs, p.data(), nullptr, worst);
  const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return (double)n / dt;
}

void autotune(bem_handle* h, double freq, int64_t nrhs) {
  require(h->have_mesh && h->have_bc && !h->points_mode, BEM_EINVAL,
          "mesh and boundary conditions must be set");
  require(freq > 0 && std::isfinite(freq) && nrhs >= 1, BEM_EINVAL, "bad probe");
  // ACA size bin: the threshold with the shortest ACA phase (best of two)
  int64_t best_thr = h->cfg.aca_big_mn;
  double best_t = 1e300;
  for (int64_t thr : {0, 256, 512, 1024, 2048}) {  // 0: the size rule of set_big_mn
    set_big_mn(h, thr);
    double t = 1e300;
    for (int rep = 0; rep < 2; rep++) {
      double tn = 0, ta = 0;
      assemble(h, freq * (1.0 + 1e-6 * (rep + 1)), &tn, &ta);
      t = std::min(t, ta);
    }
    if (t < best_t) {
      best_t = t;
      best_thr = thr;
    }
  }
  set_big_mn(h, best_thr);
  h->cfg.aca_big_mn = best_thr;
  h->state_gen++;  // workers must take the tuned layout
  // workers: warm every candidate handle once, then time 1..4 of them
  const int maxw = 4;
  probe_rate(h, maxw, freq, nrhs, 1);
  int best_w = 1;
  double best_r = 0;
  for (int W = 1; W <= maxw; W++) {
    const double r = probe_rate(h, W, freq, nrhs, 2);
    if (r > best_r * 1.03) {  // a worker must earn its memory
      best_r = r;
      best_w = W;
    }
  }
  h->tuned_workers = best_w;
}

}  // namespace

extern "C" {

void bem_config_default(bem_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->leaf_size = 32;
  c->eta = 2.0;
  c->aca_tol = 1e-4;
  c->aca_max_rank = 0;
  c->rank_reserve = 96;
  c->gmres_tol = 1e-8;
  c->gmres_restart = 300;
  c->gmres_maxit = 1000;
  c->coupling = 2;
  c->precision = 0;
  c->wave_speed = 343.0;
  c->density = 1.2;
  c->seed = 1234;
  c->use_preconditioner = 0;
  c->precond_rank = 2;
  c->precond_tol = 0.0;
  c->selector = 0;
  c->selector_guard = 0.9;
  c->sweep_workers = 0;
  c->aca_big_mn = 0;
  c->precond_reuse = 0.0;
  c->hlu_device = 1;
  c->near_fp64 = 0;
}

bem_status bem_create(const bem_config* cfg, bem_handle** out) {
  if (!out) return BEM_EINVAL;
  *out = nullptr;
  bem_handle* h = new (std::nothrow) bem_handle();
  if (!h) return BEM_ENOMEM;
  bem_status st = guarded(h, [&] {
    if (cfg) h->cfg = *cfg;
    else bem_config_default(&h->cfg);
    require(h->cfg.leaf_size >= 2, BEM_EINVAL, "leaf_size must be >= 2");
    require(h->cfg.eta > 0, BEM_EINVAL, "eta must be positive");
    require(h->cfg.aca_tol >= 0, BEM_EINVAL, "aca_tol must be >= 0");
    require(h->cfg.rank_reserve >= 1 && h->cfg.rank_reserve <= ACA_MAX_KCAP, BEM_EINVAL,
            "rank_reserve must be in [1, 512]");
    require(h->cfg.gmres_restart >= 1 && h->cfg.gmres_maxit >= 1, BEM_EINVAL,
            "gmres_restart and gmres_maxit must be >= 1");
    require(h->cfg.coupling >= 0 && h->cfg.coupling <= 2, BEM_EINVAL, "coupling must be 0, 1 or 2");
    require(h->cfg.precision == 0 || h->cfg.precision == 1, BEM_EINVAL,
            "precision must be 0 (complex FP64) or 1 (mixed)");
    require(h->cfg.wave_speed > 0, BEM_EINVAL, "wave_speed must be positive");
    require(h->cfg.sweep_workers >= 0 && h->cfg.sweep_workers <= 16, BEM_EINVAL,
            "sweep_workers must be 0 (auto) .. 16");
    require(h->cfg.aca_big_mn >= 0, BEM_EINVAL, "aca_big_mn must be >= 0");
    require(h->cfg.precond_reuse >= 0 && std::isfinite(h->cfg.precond_reuse), BEM_EINVAL,
            "precond_reuse must be finite and >= 0");
    require(h->cfg.hlu_device == 0 || h->cfg.hlu_device == 1, BEM_EINVAL,
            "hlu_device must be 0 or 1");
    require(h->cfg.near_fp64 == 0 || h->cfg.near_fp64 == 1, BEM_EINVAL,
            "near_fp64 must be 0 or 1");
    CK(cudaGetDevice(&h->device));
    CK(cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, h->device));
    // the near-field stream at the highest priority: its short, FP64-bound
    // blocks go first while the ACA blocks fill the remaining slots
    int prio_low = 0, prio_high = 0;
    CK(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
    CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithPriority(&h->nearst, cudaStreamNonBlocking, prio_high));
    CK(cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&h->join, cudaEventDisableTiming));
    for (auto& e : h->ev) CK(cudaEventCreate(&e));
    h->rules = make_rules();
    nearfield_upload_rules(h->rules, h->stream);
    aca_upload_rules(h->rules, h->stream);
    CK(cudaGetLastError());
    sync(h);
  });
  if (st != BEM_OK) {
    bem_destroy(h);
    return st;
  }
  *out = h;
  return BEM_OK;
}

void bem_destroy(bem_handle* h) {
  if (!h) return;
  for (bem_handle* w : h->workers) bem_destroy(w);
  h->workers.clear();
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->side) cudaStreamSynchronize(h->side);
  if (h->nearst) cudaStreamSynchronize(h->nearst);
  for (auto& e : h->ev)
    if (e) cudaEventDestroy(e);
  if (h->fork) cudaEventDestroy(h->fork);
  if (h->join) cudaEventDestroy(h->join);
  cudaStream_t s = h->stream, s2 = h->side, s3 = h->nearst;
  delete h;  // device buffers are released by their destructors
  if (s) cudaStreamDestroy(s);
  if (s2) cudaStreamDestroy(s2);
  if (s3) cudaStreamDestroy(s3);
}

const char* bem_last_error(const bem_handle* h) { return h ? h->err.c_str() : "null handle"; }

bem_status bem_set_mesh(bem_handle* h, const double* tri, int64_t n) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(tri != nullptr && n >= 1, BEM_EINVAL, "mesh needs at least one triangle");
    for (int64_t i = 0; i < 9 * n; i++)
      require(std::isfinite(tri[i]), BEM_ENONFINITE, "non-finite vertex coordinate");
    std::vector<double> mids(3 * n);
    for (int64_t i = 0; i < n; i++)
      for (int d = 0; d < 3; d++)
        mids[3 * i + d] = ((tri[9 * i + d] + tri[9 * i + 3 + d]) + tri[9 * i + 6 + d]) / 3.0;
    h->rows = build_tree(mids, h->cfg.leaf_size);
    h->cols = h->rows;
    h->N = n;
    prepare_elements(tri, h->rows.perm, h->E, h->avgdim);
    h->have_plane = false;  // a plane belongs to the mesh it was set for
    h->src.clear();
    for (const Elem& e : h->E)
      require(e.area > 0 && std::isfinite(e.nrm[0]), BEM_EINVAL, "degenerate (zero-area) triangle");
    h->near_r = 4.0 * h->avgdim;
    build_layout(h->rows, h->cols, &h->E, h->near_r, h->cfg.eta, h->cfg.rank_reserve,
                 h->cfg.aca_max_rank, true, h->cfg.seed, h->L);
    h->points_mode = false;
    h->dE.upload(h->E, h->stream);
    h->dEF.upload(make_elemf(h->E), h->stream);
    h->dPerm.upload(h->rows.perm, h->stream);
    set_big_mn(h, h->cfg.aca_big_mn);
    upload_layout(h);
    h->have_mesh = true;
    h->have_bc = false;
    h->state_gen++;
    sync(h);
  });
}

bem_status bem_plan_mesh(const bem_config* cfg, const double* tri, int64_t n, int64_t* perm,
                         int64_t* nblocks, int64_t* info) {
  return guarded(nullptr, [&] {
    bem_config c;
    if (cfg) c = *cfg;
    else bem_config_default(&c);
    require(tri != nullptr && n >= 1 && nblocks != nullptr, BEM_EINVAL, "bad arguments");
    require(c.leaf_size >= 2 && c.eta > 0, BEM_EINVAL, "bad configuration");
    std::vector<double> mids(3 * n);
    for (int64_t i = 0; i < n; i++)
      for (int d = 0; d < 3; d++)
        mids[3 * i + d] = ((tri[9 * i + d] + tri[9 * i + 3 + d]) + tri[9 * i + 6 + d]) / 3.0;
    HTree t = build_tree(mids, c.leaf_size);
    std::vector<HBlockDesc> blocks = build_blocks(t, t, c.eta);
    if (perm) std::memcpy(perm, t.perm.data(), n * sizeof(int64_t));
    if (info)
      for (size_t i = 0; i < blocks.size(); i++) {
        int64_t* o = info + 5 * i;
        o[0] = blocks[i].r0;
        o[1] = blocks[i].m;
        o[2] = blocks[i].c0;
        o[3] = blocks[i].n;
        o[4] = blocks[i].adm ? 1 : 0;
      }
    *nblocks = (int64_t)blocks.size();
  });
}

bem_status bem_hlu_plan(const bem_config* cfg, const double* tri, int64_t n, double* stats,
                        int64_t nstats) {
  return guarded(nullptr, [&] {
    bem_config c;
    if (cfg) c = *cfg;
    else bem_config_default(&c);
    require(tri != nullptr && n >= 1 && stats != nullptr && nstats >= 1, BEM_EINVAL,
            "bad arguments");
    require(c.leaf_size >= 2 && c.eta > 0, BEM_EINVAL, "bad configuration");
    for (int64_t i = 0; i < 9 * n; i++)
      require(std::isfinite(tri[i]), BEM_ENONFINITE, "non-finite vertex coordinate");
    std::vector<double> mids(3 * n);
    for (int64_t i = 0; i < n; i++)
      for (int d = 0; d < 3; d++)
        mids[3 * i + d] = ((tri[9 * i + d] + tri[9 * i + 3 + d]) + tri[9 * i + 6 + d]) / 3.0;
    HTree t = build_tree(mids, c.leaf_size);
    std::vector<Elem> E;
    double avgdim = 0;
    prepare_elements(tri, t.perm, E, avgdim);
    Layout L;
    build_layout(t, t, &E, 4.0 * avgdim, c.eta, c.rank_reserve, c.aca_max_rank, false, c.seed, L);
    HluProgram P;
    std::string why;
    require(hlu_gpu_plan(t, L, c.precond_rank, P, &why), BEM_EINVAL,
            ("H-LU program: " + why).c_str());
    int64_t ndeps = (int64_t)P.deps.size();
    const double v[24] = {(double)P.tasks.size(), (double)P.arena, (double)P.scratch,
                          (double)P.levels, P.cost_path, P.cost_total, (double)P.max_kt,
                          P.df_ok ? 1.0 : 0.0, (double)P.counts[0], (double)P.counts[1],
                          (double)P.counts[2], (double)P.counts[3], (double)P.counts[4],
                          (double)P.counts[5], (double)P.counts[6], (double)ndeps,
                          (double)P.big_scratch, (double)P.path_counts[0],
                          (double)P.path_counts[1], (double)P.path_counts[2],
                          (double)P.path_counts[3], (double)P.path_counts[4],
                          (double)P.path_counts[5], (double)P.path_counts[6]};
    for (int64_t i = 0; i < std::min<int64_t>(nstats, 24); i++) stats[i] = v[i];
  });
}

bem_status bem_get_permutation(const bem_handle* h, int64_t* perm) {
  if (!h || !perm || !h->have_mesh) return BEM_EINVAL;
  std::memcpy(perm, h->rows.perm.data(), h->rows.perm.size() * sizeof(int64_t));
  return BEM_OK;
}

bem_status bem_get_partition(const bem_handle* h, int64_t* nblocks, int64_t* info) {
  if (!h || !nblocks || !(h->have_mesh || h->points_mode)) return BEM_EINVAL;
  *nblocks = (int64_t)h->L.blocks.size();
  if (info)
    for (size_t i = 0; i < h->L.blocks.size(); i++) {
      const HBlockDesc& b = h->L.blocks[i];
      int64_t* o = info + 5 * i;
      o[0] = b.r0;
      o[1] = b.m;
      o[2] = b.c0;
      o[3] = b.n;
      o[4] = b.adm ? 1 : 0;
    }
  return BEM_OK;
}

bem_status bem_set_bc(bem_handle* h, const double* a, const double* b) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(h->have_mesh && !h->points_mode, BEM_EINVAL, "mesh not set (bem_set_mesh)");
    require(a && b, BEM_EINVAL, "a and b are required");
    const int64_t N = h->N;
    h->a.resize(N);
    h->b.resize(N);
    for (int64_t i = 0; i < N; i++) {
      const int64_t o = h->rows.perm[i];
      cplx av(a[2 * o], a[2 * o + 1]), bv(b[2 * o], b[2 * o + 1]);
      require(std::isfinite(av.real()) && std::isfinite(av.imag()) && std::isfinite(bv.real()) &&
                  std::isfinite(bv.imag()),
              BEM_ENONFINITE, "non-finite Robin coefficient");
      // the reference only warns when both are tiny (:3425-3428); dividing by
      // them would produce NaN, so reject it
      const double tiny = 10.0 * 2.220446049250313080847263336181640625e-16;
      require(!(std::abs(av) < tiny && std::abs(bv) < tiny), BEM_EINVAL,
              "Robin coefficients a and b are both zero for an element");
      h->a[i] = av;
      h->b[i] = bv;
    }
    h->impedance = false;
    h->have_hlu = false;  // factors of another operator
    h->have_bc = true;
    h->state_gen++;
  });
}

bem_status bem_set_bc_impedance(bem_handle* h, const double* beta) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(h->have_mesh && !h->points_mode, BEM_EINVAL, "mesh not set (bem_set_mesh)");
    require(beta, BEM_EINVAL, "beta is required");
    const int64_t N = h->N;
    h->beta.resize(N);
    h->a.assign(N, cplx(0.0, 0.0));
    h->b.assign(N, cplx(1.0, 0.0));
    for (int64_t i = 0; i < N; i++) {
      const int64_t o = h->rows.perm[i];
      const cplx bv(beta[2 * o], beta[2 * o + 1]);
      require(std::isfinite(bv.real()) && std::isfinite(bv.imag()), BEM_ENONFINITE,
              "non-finite wall admittance");
      h->beta[i] = bv;
    }
    h->impedance = true;
    h->have_hlu = false;  // factors of another operator
    h->have_bc = true;
    h->state_gen++;
  });
}

bem_status bem_set_point_sources(bem_handle* h, const double* src, int64_t nsrc) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(h->have_mesh && !h->points_mode, BEM_EINVAL, "mesh not set (bem_set_mesh)");
    require(nsrc >= 0 && nsrc <= (1 << 20) && (nsrc == 0 || src), BEM_EINVAL, "bad sources");
    for (int64_t i = 0; i < 5 * nsrc; i++)
      require(std::isfinite(src[i]), BEM_ENONFINITE, "non-finite point source");
    h->src.assign(src, src + 5 * nsrc);
    if (nsrc > 0) h->dSrc.upload(h->src, h->stream);
    h->state_gen++;
    sync(h);
  });
}

bem_status bem_set_impedance_plane(bem_handle* h, const double* point, const double* normal) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(h->have_mesh && !h->points_mode, BEM_EINVAL, "mesh not set (bem_set_mesh)");
    double nn = 0;
    if (normal)
      for (int d = 0; d < 3; d++) nn += normal[d] * normal[d];
    h->have_hlu = false;  // factors of another operator
    h->state_gen++;
    if (!normal || nn == 0.0) {  // no plane
      h->have_plane = false;
      return;
    }
    require(point && std::isfinite(nn), BEM_EINVAL, "plane point and normal required");
    for (int d = 0; d < 3; d++)
      require(std::isfinite(point[d]), BEM_EINVAL, "non-finite plane point");
    // MeshFunctions::reflectTriangles (meshfunctions.cpp:349-380): every node
    // x -> x - 2 (n . x + d) n with the unit normal n and d = -n . point; node 1
    // and node 3 swap so the reflected element keeps its orientation
    const double inv = 1.0 / std::sqrt(nn);
    double n[3], dd = 0;
    for (int d = 0; d < 3; d++) {
      n[d] = normal[d] * inv;
      dd -= n[d] * point[d];
    }
    const int64_t N = h->N;
    std::vector<double> tri((size_t)9 * N);
    const auto reflect = [&](const double* x, double* out) {
      const double t = n[0] * x[0] + n[1] * x[1] + n[2] * x[2] + dd;
      for (int d = 0; d < 3; d++) out[d] = x[d] - 2.0 * t * n[d];
    };
    for (int64_t i = 0; i < N; i++) {
      const Elem& e = h->E[i];
      reflect(e.n3, &tri[9 * i]);
      reflect(e.n2, &tri[9 * i + 3]);
      reflect(e.n1, &tri[9 * i + 6]);
    }
    std::vector<int64_t> ident(N);
    for (int64_t i = 0; i < N; i++) ident[i] = i;
    double avg = 0;
    prepare_elements(tri.data(), ident, h->Er, avg);
    for (int d = 0; d < 3; d++) {
      h->plane_p[d] = point[d];
      h->plane_n[d] = n[d];
    }
    h->dEr.upload(h->Er, h->stream);
    h->dEFr.upload(make_elemf(h->Er), h->stream);
    h->have_plane = true;
    sync(h);
  });
}

bem_status bem_operators(bem_handle* h, double k, const int64_t* rows, const int64_t* cols,
                         int64_t count, double* out) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(h->have_mesh && !h->points_mode, BEM_EINVAL, "mesh not set");
    require(count >= 0 && (count == 0 || (rows && cols && out)), BEM_EINVAL, "bad arguments");
    for (int64_t i = 0; i < count; i++)
      require(rows[i] >= 0 && rows[i] < h->N && cols[i] >= 0 && cols[i] < h->N, BEM_EINVAL,
              "index out of range");
    if (count == 0) return;
    DBuf<int64_t> dr, dc;
    DBuf<double2> dout;
    dr.ensure(count);
    dc.ensure(count);
    dout.ensure(4 * count);
    CK(cudaMemcpyAsync(dr.p, rows, count * 8, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(dc.p, cols, count * 8, cudaMemcpyHostToDevice, h->stream));
    launch_operators(h->dE.p, dr.p, dc.p, count, k, h->near_r, dout.p, h->stream);
    h->launches++;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, dout.p, 4 * count * sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
    sync(h);
  });
}

bem_status bem_assemble(bem_handle* h, double freq) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] { assemble(h, freq, nullptr, nullptr); });
}

bem_status bem_hmatvec(bem_handle* h, int32_t which, const double* x, double* y, int64_t nrhs,
                       int32_t accumulate) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(x && y && nrhs >= 1, BEM_EINVAL, "bad arguments");
    const int64_t nr = h->points_mode ? (int64_t)h->rows.perm.size() : h->N;
    const int64_t nc = h->points_mode ? (int64_t)h->cols.perm.size() : h->N;
    copy_in(h, h->dIn, x, (size_t)nc * nrhs);
    h->dOut1.ensure((size_t)nr * nrhs);
    if (accumulate)
      CK(cudaMemcpyAsync(h->dOut1.p, y, (size_t)nr * nrhs * sizeof(double2), cudaMemcpyHostToDevice, h->stream));
    hmatvec_dev(h, which, h->dIn.p, h->dOut1.p, nrhs, accumulate);
    CK(cudaGetLastError());
    copy_out(h, y, h->dOut1.p, (size_t)nr * nrhs);
    sync(h);
  });
}

// ---- selector data generation and training (no handle; stream NULL = default) ----

int64_t bem_sel_nparam(void) { return SEL_NPARAM; }

bem_status bem_sel_label(const double* ptri, const double* qtri, const double* k, int64_t n,
                         double tol, double near_ratio, double floor_rel, float* feat,
                         uint8_t* label, float* err) {
  return guarded(nullptr, [&] {
    require(n >= 0 && (n == 0 || (ptri && qtri && k && feat && label)), BEM_EINVAL,
            "bad arguments");
    require(tol > 0 && near_ratio >= 0 && floor_rel >= 0, BEM_EINVAL,
            "bad tolerance / near ratio / error floor");
    const int64_t chunk = 1 << 18;
    DBuf<Elem> dP, dQ;
    DBuf<double> dk;
    DBuf<float> df, de;
    DBuf<uint8_t> dl;
    std::vector<Elem> EP, EQ;
    for (int64_t o = 0; o < n; o += chunk) {
      const int64_t m = std::min(chunk, n - o);
      std::vector<int64_t> id(m);
      for (int64_t i = 0; i < m; i++) id[i] = i;
      double avg;
      prepare_elements(ptri + 9 * o, id, EP, avg);
      prepare_elements(qtri + 9 * o, id, EQ, avg);
      for (int64_t i = 0; i < m; i++)
        require(std::isfinite(k[o + i]) && k[o + i] > 0 && EQ[i].area > 0 && EP[i].area > 0,
                BEM_EINVAL, "degenerate pair or wavenumber");
      dP.upload(EP, 0);
      dQ.upload(EQ, 0);
      dk.ensure(m);
      CK(cudaMemcpy(dk.p, k + o, m * sizeof(double), cudaMemcpyHostToDevice));
      df.ensure(m * SEL_NF);
      dl.ensure(m);
      if (err) de.ensure(m * 6);
      launch_sel_label(dP.p, dQ.p, dk.p, m, tol, near_ratio, floor_rel, df.p, dl.p,
                       err ? de.p : nullptr, 0);
      CK(cudaGetLastError());
      CK(cudaMemcpy(feat + o * SEL_NF, df.p, m * SEL_NF * sizeof(float), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(label + o, dl.p, m, cudaMemcpyDeviceToHost));
      if (err) CK(cudaMemcpy(err + o * 6, de.p, m * 6 * sizeof(float), cudaMemcpyDeviceToHost));
    }
  });
}

bem_status bem_mlp_grad(const float* params, const float* X, const uint8_t* y, int64_t B,
                        float* grad, float* loss, float* work, void* stream) {
  return guarded(nullptr, [&] {
    require(params && X && y && grad && loss && work && B >= 1, BEM_EINVAL, "bad arguments");
    launch_mlp_grad(params, X, y, B, grad, loss, work, (cudaStream_t)stream);
    CK(cudaGetLastError());
  });
}

bem_status bem_mlp_adam(float* params, const float* grad, float* m, float* v, int64_t step,
                        float lr, float beta1, float beta2, float eps, void* stream) {
  return guarded(nullptr, [&] {
    require(params && grad && m && v && step >= 1, BEM_EINVAL, "bad arguments");
    launch_mlp_adam(params, grad, m, v, step, lr, beta1, beta2, eps, (cudaStream_t)stream);
    CK(cudaGetLastError());
  });
}

bem_status bem_mlp_forward(const float* params, const float* X, int64_t B, float* logits,
                           void* stream) {
  return guarded(nullptr, [&] {
    require(params && X && logits && B >= 0, BEM_EINVAL, "bad arguments");
    launch_mlp_forward(params, X, B, logits, (cudaStream_t)stream);
    CK(cudaGetLastError());
  });
}

bem_status bem_sel_infer(const float* params, const float* mu, const float* sigma,
                         const float* feat, int64_t B, float* logits, uint8_t* cls,
                         void* stream) {
  return guarded(nullptr, [&] {
    require(params && mu && sigma && feat && cls && B >= 0, BEM_EINVAL, "bad arguments");
    SelBlob b;
    sel_make_blob(params, mu, sigma, b);
    DBuf<SelBlob> db;
    db.ensure(1);
    cudaStream_t s = (cudaStream_t)stream;
    CK(cudaMemcpyAsync(db.p, &b, sizeof(SelBlob), cudaMemcpyHostToDevice, s));
    launch_sel_infer_rows(db.p, feat, B, logits, cls, s);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
  });
}

bem_status bem_set_selector(bem_handle* h, const float* params, const float* mu,
                            const float* sigma) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(params && mu && sigma, BEM_EINVAL, "bad arguments");
    for (int i = 0; i < SEL_NPARAM; i++)
      require(std::isfinite(params[i]), BEM_ENONFINITE, "non-finite selector weights");
    SelBlob b;
    sel_make_blob(params, mu, sigma, b);
    h->dSel.ensure(1);
    CK(cudaMemcpyAsync(h->dSel.p, &b, sizeof(SelBlob), cudaMemcpyHostToDevice, h->stream));
    sync(h);
    h->have_selector = true;
    h->state_gen++;
  });
}

bem_status bem_set_aca_rules(bem_handle* h, const uint8_t* table, const float* axes) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(table && axes, BEM_EINVAL, "bad arguments");
    for (int i = 0; i < ACA_TAB_N * ACA_TAB_N; i++)
      require(table[i] < SEL_C, BEM_EINVAL, "rule-table classes must be 0..4");
    require(std::isfinite(axes[0]) && std::isfinite(axes[2]) && axes[1] > 0 && axes[3] > 0,
            BEM_EINVAL, "bad rule-table axes");
    h->dAcaTab.ensure(ACA_TAB_N * ACA_TAB_N);
    CK(cudaMemcpyAsync(h->dAcaTab.p, table, ACA_TAB_N * ACA_TAB_N, cudaMemcpyHostToDevice,
                       h->stream));
    for (int i = 0; i < 4; i++) h->aca_axes[i] = axes[i];
    sync(h);
    h->have_aca_tab = true;
    h->state_gen++;
  });
}

bem_status bem_sel_stats(const bem_handle* h, int64_t* stats) {
  if (!h || !stats) return BEM_EINVAL;
  for (int i = 0; i < 3; i++) stats[i] = (int64_t)h->sel_stats[i];
  stats[3] = h->L.near_entries - (int64_t)h->L.sp_entry.size();  // selector-governed entries
  return BEM_OK;
}

bem_status bem_sel_classes(bem_handle* h, uint8_t* cls) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(cls, BEM_EINVAL, "bad arguments");
    require(h->dCls.n >= (size_t)h->L.near_entries && h->L.near_entries > 0, BEM_EINVAL,
            "no selector classes (assemble with cfg.selector = 1 first)");
    CK(cudaMemcpyAsync(cls, h->dCls.p, h->L.near_entries, cudaMemcpyDeviceToHost, h->stream));
    sync(h);
  });
}

bem_status bem_recompress(bem_handle* h, int32_t which, int64_t rank, double tol) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(which == 0 || which == 1, BEM_EINVAL, "which must be 0 (phi) or 1 (dPhi)");
    recompress(h, h->hm[which], rank, tol);
  });
}

bem_status bem_hlu_build(bem_handle* h) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(build_hlu(h), BEM_ENONFINITE, "non-finite values in the H-LU factors");
  });
}

bem_status bem_hlu_solve(bem_handle* h, const double* b, double* x, int64_t nrhs) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(b && x && nrhs >= 1, BEM_EINVAL, "bad arguments");
    require(h->have_hlu, BEM_EINVAL, "preconditioner not built (bem_hlu_build)");
    copy_in(h, h->dIn, b, (size_t)h->N * nrhs);
    apply_precond(h, h->dIn.p, (int)nrhs);
    CK(cudaGetLastError());
    copy_out(h, x, h->dIn.p, (size_t)h->N * nrhs);
    sync(h);
    check_df_error(h);
  });
}

bem_status bem_hlu_sweep_kind(const bem_handle* hc, int32_t* kind) {
  if (!hc) return BEM_EINVAL;
  bem_handle* h = const_cast<bem_handle*>(hc);
  return guarded(h, [&] {
    require(kind != nullptr, BEM_EINVAL, "bad arguments");
    require(h->have_hlu, BEM_EINVAL, "preconditioner not built (bem_hlu_build)");
    *kind = h->df_ok ? 1 : 0;
  });
}

bem_status bem_hlu_export(const bem_handle* hc, int32_t which, int64_t* nleaves, int64_t* leaves,
                          int64_t* ndata, double* data, int64_t* nsched, int32_t* sched) {
  if (!hc) return BEM_EINVAL;
  bem_handle* h = const_cast<bem_handle*>(hc);
  return guarded(h, [&] {
    require(which == 0 || which == 1, BEM_EINVAL, "which must be 0 (L) or 1 (U)");
    require(h->have_hlu, BEM_EINVAL, "preconditioner not built (bem_hlu_build)");
    const FlatFactor& f = which ? h->hU : h->hL;
    if (h->hlu_dev) {  // leaves packed in order, data gathered from the arena
      const int64_t nl = f.nleaves();
      std::vector<int64_t> lv(f.leaves);
      int64_t tot = 0;
      for (int64_t i = 0; i < nl; i++) {
        const int64_t* L = &f.leaves[7 * i];
        tot += L[4] == 1 ? (L[1] + L[3]) * L[5] : L[1] * L[3];
      }
      if (nleaves) *nleaves = nl;
      if (ndata) *ndata = tot;
      if (nsched) *nsched = (int64_t)f.schedule.size();
      if (sched) std::memcpy(sched, f.schedule.data(), f.schedule.size() * sizeof(int32_t));
      if (leaves || data) {
        std::vector<unsigned char> host;
        const size_t es = h->hlu_prec ? sizeof(float2) : sizeof(double2);
        if (data) {
          host.resize((size_t)h->hp.arena * es);
          CK(cudaMemcpyAsync(host.data(), h->dArena.p, host.size(), cudaMemcpyDeviceToHost,
                             h->stream));
          CK(cudaStreamSynchronize(h->stream));
        }
        int64_t o = 0;
        for (int64_t i = 0; i < nl; i++) {
          int64_t* L = &lv[7 * i];
          const int64_t cnt = L[4] == 1 ? (L[1] + L[3]) * L[5] : L[1] * L[3];
          if (data)
            for (int64_t e = 0; e < cnt; e++) {
              if (h->hlu_prec) {
                const float2 v = reinterpret_cast<const float2*>(host.data())[L[6] + e];
                data[2 * (o + e)] = v.x;
                data[2 * (o + e) + 1] = v.y;
              } else {
                const double2 v = reinterpret_cast<const double2*>(host.data())[L[6] + e];
                data[2 * (o + e)] = v.x;
                data[2 * (o + e) + 1] = v.y;
              }
            }
          L[6] = o;
          o += cnt;
        }
        if (leaves) std::memcpy(leaves, lv.data(), lv.size() * sizeof(int64_t));
      }
      return;
    }
    if (nleaves) *nleaves = f.nleaves();
    if (ndata) *ndata = (int64_t)f.data.size();
    if (nsched) *nsched = (int64_t)f.schedule.size();
    if (leaves) std::memcpy(leaves, f.leaves.data(), f.leaves.size() * sizeof(int64_t));
    if (data) std::memcpy(data, f.data.data(), f.data.size() * sizeof(double2));
    if (sched) std::memcpy(sched, f.schedule.data(), f.schedule.size() * sizeof(int32_t));
  });
}

bem_status bem_hmatvec_device(bem_handle* h, int32_t which, const void* x, void* y, int64_t nrhs,
                              int32_t accumulate) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(x && y && nrhs >= 1, BEM_EINVAL, "bad arguments");
    hmatvec_dev(h, which, (const double2*)x, (double2*)y, nrhs, accumulate);
    CK(cudaGetLastError());
  });
}

bem_status bem_hmatvec_device_ex(bem_handle* h, int32_t which, const void* x, void* y,
                                 int64_t nrhs, int32_t accumulate, int32_t arith) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(x && y && nrhs >= 1, BEM_EINVAL, "bad arguments");
    require(arith >= 0 && arith <= 2, BEM_EINVAL, "arith must be 0, 1 or 2");
    hmatvec_dev(h, which, (const double2*)x, (double2*)y, nrhs, accumulate, arith);
    CK(cudaGetLastError());
  });
}

// Allocation-free H-matvec: same kernels and arithmetic as bem_hmatvec_device
// with fp64 products, but the projections t live in the library's fixed
// device array (hmatvec.cu) instead of the handle's allocated buffer, and
// nothing on this path allocates GPU memory.
bem_status bem_hmatvec_noalloc(bem_handle* h, int32_t which, const void* x, void* y,
                               int64_t nrhs, int32_t accumulate) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(which == 0 || which == 1, BEM_EINVAL, "which must be 0 (phi) or 1 (dPhi)");
    require(x && y && nrhs >= 1, BEM_EINVAL, "bad arguments");
    DevHM& m = h->hm[which];
    require(m.assembled, BEM_EINVAL, "matrix not assembled");
    const int64_t nrows = h->points_mode ? (int64_t)h->rows.perm.size() : h->N;
    const int64_t ncols = h->points_mode ? (int64_t)h->cols.perm.size() : h->N;
    const int64_t ldt = std::max<int64_t>(h->L.s_size, 1);
    const int64_t cap = hmatvec_noalloc_capacity();
    require(ldt <= cap, BEM_EINVAL,
            "bem_hmatvec_noalloc: the matrix's rank reservation exceeds the fixed scratch "
            "(2^21 complex values); use bem_hmatvec_device");
    double2* t = nullptr;
    CK(hmatvec_noalloc_scratch(&t));
    const int64_t chunk = std::min<int64_t>(8, cap / ldt);
    const double2* xd = (const double2*)x;
    double2* yd = (double2*)y;
    for (int64_t r0 = 0; r0 < nrhs; r0 += chunk) {
      HmvArgs a{};
      a.precision = m.prec;
      a.fp32_math = 0;
      a.nrhs = (int)std::min<int64_t>(chunk, nrhs - r0);
      a.far = h->dFar.p;
      a.rank = m.rank.p;
      a.nfar = (int64_t)h->L.far.size();
      a.nearb = h->dNear.p;
      a.leaves = h->dLeaves.p;
      a.nleaves = (int64_t)h->L.leaves.size();
      a.list_off = h->dListOff.p;
      a.list = h->dList.p;
      a.U = m.U.p;
      a.V = m.V.p;
      a.S = m.S.p;
      a.F = m.F.p;
      a.vwork = m.vwork.p;  // (block, 16-row) work items of pass V: handle-owned, no allocation
      a.nvwork = m.nvwork;
      a.x = xd + r0 * ncols;
      a.ldx = ncols;
      a.t = t;
      a.ldt = ldt;
      a.y = yd + r0 * nrows;
      a.ldy = nrows;
      a.accumulate = accumulate;
      h->launches += launch_hmatvec(a, h->stream);
    }
    CK(cudaGetLastError());
  });
}

bem_status bem_get_block(bem_handle* h, int32_t which, int64_t block, int64_t* rank, double* U,
                         double* s, double* V, double* F) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(which == 0 || which == 1, BEM_EINVAL, "which must be 0 or 1");
    DevHM& m = h->hm[which];
    require(m.assembled, BEM_EINVAL, "matrix not assembled");
    require(block >= 0 && block < (int64_t)h->L.blocks.size(), BEM_EINVAL, "block out of range");
    // map partition index -> near / far index
    int64_t nearI = 0, farI = 0;
    for (int64_t i = 0; i < block; i++) (h->L.blocks[i].adm ? farI : nearI)++;
    const HBlockDesc& b = h->L.blocks[block];
    const size_t es = m.prec ? sizeof(float2) : sizeof(double2);
    // copy `cnt` stored complex numbers starting at element `off` into dst
    // (complex FP64), widening complex-FP32 storage
    auto fetch = [&](double* dst, const DBuf<unsigned char>& src, int64_t off, int64_t cnt) {
      std::vector<unsigned char> tmp(cnt * es);
      if (cnt > 0)
        CK(cudaMemcpyAsync(tmp.data(), src.p + off * es, cnt * es, cudaMemcpyDeviceToHost, h->stream));
      sync(h);
      for (int64_t i = 0; i < cnt; i++) {
        if (m.prec) {
          const float* f = reinterpret_cast<const float*>(tmp.data()) + 2 * i;
          dst[2 * i] = f[0];
          dst[2 * i + 1] = f[1];
        } else {
          const double* d = reinterpret_cast<const double*>(tmp.data()) + 2 * i;
          dst[2 * i] = d[0];
          dst[2 * i + 1] = d[1];
        }
      }
    };
    if (b.adm) {
      const FarBlock& fb = h->L.far[farI];
      const int k = m.h_rank[farI];
      if (rank) *rank = k;
      if (U) fetch(U, m.U, fb.uoff, (int64_t)k * b.m);
      if (V) fetch(V, m.V, fb.voff, (int64_t)k * b.n);
      if (s) fetch(s, m.S, fb.soff, k);
    } else {
      const NearBlock& nb = h->L.near[nearI];
      if (rank) *rank = -1;
      if (F) fetch(F, m.F, nb.off, (int64_t)b.m * b.n);
    }
    sync(h);
  });
}

bem_status bem_get_ranks(bem_handle* h, int32_t which, int64_t* ranks) {
  if (!h || !ranks) return BEM_EINVAL;
  return guarded(h, [&] {
    require(which == 0 || which == 1, BEM_EINVAL, "which must be 0 or 1");
    DevHM& m = h->hm[which];
    require(m.assembled, BEM_EINVAL, "matrix not assembled");
    int64_t fi = 0;
    for (size_t i = 0; i < h->L.blocks.size(); i++)
      ranks[i] = h->L.blocks[i].adm ? m.h_rank[fi++] : -1;
  });
}

bem_status bem_gmres(bem_handle* h, const double* b, double* x, int64_t nrhs, bem_solve_info* info) {
  if (!h) return BEM_EINVAL;
  bem_solve_info loc{};
  bem_status st = guarded(h, [&] {
    require(b && x && nrhs >= 1, BEM_EINVAL, "bad arguments");
    require(!h->points_mode, BEM_EINVAL, "GMRES needs the BEM system matrix");
    const int64_t N = h->N;
    copy_in(h, h->dRhs, b, (size_t)N * nrhs);
    copy_in(h, h->dX, x, (size_t)N * nrhs);
    gmres_dev(h, h->dRhs.p, h->dX.p, (int)nrhs, &loc);
    copy_out(h, x, h->dX.p, (size_t)N * nrhs);
    sync(h);
  });
  if (info) *info = loc;
  return st != BEM_OK ? st : loc.status;
}

namespace {

// ---- field evaluation ----

// Element chunks of the field sum: enough CTAs for about eight per SM, chunks
// of at least 512 elements.
int field_split(const bem_handle* h, int64_t M) {
  const int64_t bx = (M + FIELD_PTS - 1) / FIELD_PTS;
  const int64_t want = (8LL * h->nsm + bx - 1) / bx;
  const int64_t most = std::max<int64_t>(1, h->N / 512);
  return (int)std::max<int64_t>(1, std::min<int64_t>({want, most, 256}));
}

// calculateFieldSolution (boundaryelementsolver.cpp:2192-2249) on device
// buffers: pts M x 3, phi / dphi N x R (caller order), src nsrc x 5 on the
// host; phi_f / p_f M x R (either may be null).
void field_dev(bem_handle* h, double freq, const double* pts, int64_t M, const double2* phi,
               const double2* dphi, int64_t R, const double* src, int64_t nsrc, double2* phi_f,
               double2* p_f) {
  require(h->have_mesh && !h->points_mode, BEM_EINVAL, "mesh not set");
  require(std::isfinite(freq) && freq >= 0, BEM_EINVAL, "frequency must be >= 0");
  require(M >= 0 && R >= 1 && R <= (1 << 20) && nsrc >= 0 && nsrc <= (1 << 20), BEM_EINVAL,
          "bad sizes");
  require(phi && dphi && (M == 0 || pts) && (nsrc == 0 || src), BEM_EINVAL, "bad arguments");
  if (M == 0) return;
  const int64_t N = h->N;
  const int prec = h->cfg.precision != 0 ? 1 : 0;
  const double k = 2.0 * M_PI * freq / h->cfg.wave_speed;
  // sound pressure i rho 2 pi f phi; 2 pi at f = 0 (:2236-2243)
  const double2 pfac = make_double2(0.0, h->cfg.density * 2.0 * M_PI * (freq != 0 ? freq : 1.0));
  cudaStream_t s = h->stream;
  if (nsrc > 0) {
    // staged through the handle's pageable copy, so the caller's array may be
    // reused as soon as the call returns even when it is pinned
    h->field_src.assign(src, src + 5 * nsrc);
    h->dFsrc.upload(h->field_src, s);
  }
  if (prec == 1) h->dFe.ensure((size_t)N);
  h->dFcoef.ensure((size_t)N * R * (prec == 1 ? sizeof(FieldCoefF) : sizeof(FieldCoef)));
  const int S = field_split(h, M);
  // with an impedance plane the reflected elements add a second set of S
  // partial sums with the same coefficients (:2305-2311)
  const int passes = h->have_plane ? 2 : 1;
  h->dFpart.ensure((size_t)passes * S * R * M);
  h->launches += launch_field_prep(h->dE.p, h->dPerm.p, N, phi, dphi, (int)R, prec, h->dFe.p,
                                   h->dFcoef.p, s);
  h->launches += launch_field_sum(h->dE.p, h->dFe.p, h->dFcoef.p, N, (int)R, pts, M, k, prec, S,
                                  h->dFpart.p, s);
  if (h->have_plane) {
    if (prec == 1) {
      h->dFeR.ensure((size_t)N);
      h->launches += launch_field_prep(h->dEr.p, nullptr, N, nullptr, nullptr, 0, prec,
                                       h->dFeR.p, nullptr, s);
    }
    h->launches += launch_field_sum(h->dEr.p, h->dFeR.p, h->dFcoef.p, N, (int)R, pts, M, k, prec,
                                    S, h->dFpart.p + (size_t)S * R * M, s);
  }
  h->launches += launch_field_finish(h->dFpart.p, passes * S, M, (int)R, pts,
                                     nsrc ? h->dFsrc.p : nullptr, (int)nsrc, k, pfac, phi_f, p_f,
                                     s);
  CK(cudaGetLastError());
}

}  // namespace

bem_status bem_field(bem_handle* h, double freq, const double* pts, int64_t npts,
                     const double* phi, const double* dphi, int64_t nrhs, const double* sources,
                     int64_t nsrc, double* phi_f, double* p_f) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(h->have_mesh && !h->points_mode, BEM_EINVAL, "mesh not set");
    require(phi && dphi && nrhs >= 1 && npts >= 0 && (npts == 0 || pts), BEM_EINVAL,
            "bad arguments");
    if (npts == 0) return;
    const size_t cn = (size_t)h->N * nrhs, cm = (size_t)npts * nrhs;
    h->dFpts.ensure((size_t)npts * 3);
    CK(cudaMemcpyAsync(h->dFpts.p, pts, (size_t)npts * 3 * sizeof(double), cudaMemcpyHostToDevice,
                       h->stream));
    copy_in(h, h->dFphi, phi, cn);
    copy_in(h, h->dFdphi, dphi, cn);
    if (phi_f) h->dFout1.ensure(cm);
    if (p_f) h->dFout2.ensure(cm);
    field_dev(h, freq, h->dFpts.p, npts, h->dFphi.p, h->dFdphi.p, nrhs, sources, nsrc,
              phi_f ? h->dFout1.p : nullptr, p_f ? h->dFout2.p : nullptr);
    copy_out(h, phi_f, h->dFout1.p, cm);
    copy_out(h, p_f, h->dFout2.p, cm);
    sync(h);
  });
}

bem_status bem_field_device(bem_handle* h, double freq, const void* pts, int64_t npts,
                            const void* phi, const void* dphi, int64_t nrhs,
                            const double* sources, int64_t nsrc, void* phi_f, void* p_f) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    field_dev(h, freq, (const double*)pts, npts, (const double2*)phi, (const double2*)dphi, nrhs,
              sources, nsrc, (double2*)phi_f, (double2*)p_f);
  });
}

bem_status bem_solve_device(bem_handle* h, double freq, const void* g, int64_t nrhs, void* phi,
                            void* dphi, void* p, bem_solve_info* info) {
  if (!h) return BEM_EINVAL;
  bem_solve_info loc{};
  bem_status st = guarded(h, [&] {
    require(g != nullptr, BEM_EINVAL, "g is required");
    solve_dev(h, freq, (const double2*)g, nrhs, (double2*)phi, (double2*)dphi, (double2*)p, &loc);
  });
  if (info) *info = loc;
  return st != BEM_OK ? st : loc.status;
}

bem_status bem_solve(bem_handle* h, double freq, const double* g, int64_t nrhs, double* phi,
                     double* dphi, double* p, bem_solve_info* info) {
  if (!h) return BEM_EINVAL;
  bem_solve_info loc{};
  bem_status st = guarded(h, [&] {
    require(h->have_mesh && !h->points_mode, BEM_EINVAL, "mesh not set");
    require(g != nullptr && nrhs >= 1, BEM_EINVAL, "bad arguments");
    const int64_t N = h->N;
    const size_t cnt = (size_t)N * nrhs;
    copy_in(h, h->dIn, g, cnt);
    h->dOut1.ensure(cnt);
    h->dOut2.ensure(cnt);
    h->dOut3.ensure(cnt);
    solve_dev(h, freq, h->dIn.p, nrhs, phi ? h->dOut1.p : nullptr, dphi ? h->dOut2.p : nullptr,
              p ? h->dOut3.p : nullptr, &loc);
    copy_out(h, phi, h->dOut1.p, cnt);
    copy_out(h, dphi, h->dOut2.p, cnt);
    copy_out(h, p, h->dOut3.p, cnt);
    sync(h);
  });
  if (info) *info = loc;
  return st != BEM_OK ? st : loc.status;
}

bem_status bem_autotune(bem_handle* h, double freq, int64_t nrhs, int64_t* tuned) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    autotune(h, freq, nrhs);
    if (tuned) {
      tuned[0] = h->tuned_workers;
      tuned[1] = h->cfg.aca_big_mn;
    }
  });
}

namespace {
// bem_sweep / bem_sweep_resume: the frequencies whose solved flag is zero
// (all of them without flags), sorted ascending under factor reuse.
bem_status sweep_host(bem_handle* h, const double* freqs, int64_t nf, const double* g,
                      int64_t nrhs, double* p, bem_solve_info* info, uint8_t* solved,
                      bem_freq_done_fn done, void* user) {
  if (!h) return BEM_EINVAL;
  bem_status worst = BEM_OK;
  bem_status st = guarded(h, [&] {
    require(freqs && g && p && nf >= 1 && nrhs >= 1, BEM_EINVAL, "bad arguments");
    for (int64_t f = 0; f < nf; f++)
      require(freqs[f] > 0 && std::isfinite(freqs[f]), BEM_EINVAL, "frequencies must be positive");
    std::vector<int64_t> idx;
    for (int64_t i = 0; i < nf; i++)
      if (!solved || !solved[i]) idx.push_back(i);
    if (idx.empty()) return;
    const int64_t n = (int64_t)idx.size();
    int W = (int)h->cfg.sweep_workers;
    if (W == 0) {  // autotuned once per handle, on long sweeps only
      if (h->tuned_workers == 0 && n >= 16) {
        std::vector<double> sorted;
        for (int64_t i : idx) sorted.push_back(freqs[i]);
        std::sort(sorted.begin(), sorted.end());
        autotune(h, sorted[n / 2], nrhs);
      }
      W = h->tuned_workers > 0 ? (int)h->tuned_workers : 1;
    }
    // interleave cheap and expensive frequencies over the workers; with
    // factor reuse, frequencies go in ascending order
    if (h->cfg.use_preconditioner && h->cfg.precond_reuse > 1.0)
      std::stable_sort(idx.begin(), idx.end(),
                       [&](int64_t x, int64_t y) { return freqs[x] < freqs[y]; });
    std::function<bool(int64_t)> on_done = [&](int64_t f) {
      solved[f] = 1;
      return done != nullptr && done(f, user) != 0;
    };
    run_sweep(h, W, freqs, idx.data(), n, g, nrhs, p, info, worst, nullptr, nullptr,
              solved ? &on_done : nullptr);
  });
  return st != BEM_OK ? st : worst;
}
}  // namespace

bem_status bem_sweep(bem_handle* h, const double* freqs, int64_t nf, const double* g, int64_t nrhs,
                     double* p, bem_solve_info* info) {
  return sweep_host(h, freqs, nf, g, nrhs, p, info, nullptr, nullptr, nullptr);
}

bem_status bem_sweep_resume(bem_handle* h, const double* freqs, int64_t nf, const double* g,
                            int64_t nrhs, double* p, bem_solve_info* info, uint8_t* solved,
                            bem_freq_done_fn done, void* user) {
  if (!solved) return BEM_EINVAL;
  return sweep_host(h, freqs, nf, g, nrhs, p, info, solved, done, user);
}

bem_status bem_sweep_device(bem_handle* h, const double* freqs, int64_t nf, const void* g,
                            int64_t nrhs, void* p, bem_solve_info* info) {
  if (!h) return BEM_EINVAL;
  bem_status worst = BEM_OK;
  bem_status st = guarded(h, [&] {
    require(freqs && g && p && nf >= 1 && nrhs >= 1, BEM_EINVAL, "bad arguments");
    for (int64_t f = 0; f < nf; f++)
      require(freqs[f] > 0 && std::isfinite(freqs[f]), BEM_EINVAL, "frequencies must be positive");
    int W = (int)h->cfg.sweep_workers;
    if (W == 0) W = h->tuned_workers > 0 ? (int)h->tuned_workers : 1;
    std::vector<int64_t> idx(nf);
    for (int64_t i = 0; i < nf; i++) idx[i] = i;
    if (h->cfg.use_preconditioner && h->cfg.precond_reuse > 1.0)
      std::stable_sort(idx.begin(), idx.end(),
                       [&](int64_t x, int64_t y) { return freqs[x] < freqs[y]; });
    run_sweep(h, W, freqs, idx.data(), nf, nullptr, nrhs, nullptr, info, worst,
              (const double2*)g, (double2*)p);
  });
  return st != BEM_OK ? st : worst;
}

bem_status bem_points_assemble(bem_handle* h, const double* rowpts, int64_t nr,
                               const double* colpts, int64_t nc, double k, int64_t* rowperm,
                               int64_t* colperm) {
  if (!h) return BEM_EINVAL;
  return guarded(h, [&] {
    require(rowpts && colpts && nr >= 1 && nc >= 1, BEM_EINVAL, "bad arguments");
    std::vector<double> rp(rowpts, rowpts + 3 * nr), cp(colpts, colpts + 3 * nc);
    h->rows = build_tree(rp, h->cfg.leaf_size);
    h->cols = build_tree(cp, h->cfg.leaf_size);
    build_layout(h->rows, h->cols, nullptr, 0.0, h->cfg.eta, h->cfg.rank_reserve,
                 h->cfg.aca_max_rank, false, h->cfg.seed, h->L);
    std::vector<double> rps(3 * nr), cps(3 * nc);
    for (int64_t i = 0; i < nr; i++)
      for (int d = 0; d < 3; d++) rps[3 * i + d] = rp[3 * h->rows.perm[i] + d];
    for (int64_t i = 0; i < nc; i++)
      for (int d = 0; d < 3; d++) cps[3 * i + d] = cp[3 * h->cols.perm[i] + d];
    h->dRowPts.upload(rps, h->stream);
    h->dColPts.upload(cps, h->stream);
    upload_layout(h);
    h->points_mode = true;
    h->have_mesh = false;
    h->N = nr;
    h->k = k;
    for (auto& q : h->hm) q.has_lo = false;  // point clouds: FP64 storage, no remainders
    DevHM& m = h->hm[0];
    alloc_hm(h, m);
    launch_points_nearfield(h->dNear.p, (int64_t)h->L.near.size(), h->dTiles.p,
                            (int64_t)h->L.tiles.size(), h->dRowPts.p, h->dColPts.p, k,
                            (double2*)m.F.p, h->stream);
    AcaArgs a = aca_args(h, m, 0, 0);
    a.mode = 1;
    h->launches++;
    launch_aca_split(h, {a});
    CK(cudaGetLastError());
    fetch_ranks(h, m);
    h->hm[1].assembled = false;
    if (rowperm) std::memcpy(rowperm, h->rows.perm.data(), nr * sizeof(int64_t));
    if (colperm) std::memcpy(colperm, h->cols.perm.data(), nc * sizeof(int64_t));
  });
}

int64_t bem_launch_count(const bem_handle* h) {
  if (!h) return 0;
  int64_t c = h->launches;
  for (const bem_handle* w : h->workers) c += w->launches;  // the sweep workers' kernels
  return c;
}

void* bem_stream(const bem_handle* h) { return h ? (void*)h->stream : nullptr; }

}  // extern "C"
