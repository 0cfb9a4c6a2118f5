/*
 * bemgpu.hpp -- C++ facade over the C ABI (bemgpu.h) with the names of the
 * reference's call surface, in standard-library types instead of Eigen/Qt:
 *
 *   HMatrix                          HMatrix/hmatrix.h (assembleBlocks,
 *                                    assembleBlocksExtra: one assembly of
 *                                    both BC-substituted matrices)
 *   HArithm::MVM(y, H, x)            HMatrix/harithm.h:32 (y += H x)
 *   HArithm::LUDecomposition(H)      HMatrix/harithm.h:216 (factors kept on
 *                                    the GPU; the H-matrix stays intact)
 *   HArithm::LUSubstitutionSolve     HMatrix/harithm.cpp:1168-1190
 *   GMRES::gmresSolve(A, x0, b, tol) HMatrix/gmres.h:170
 *   BoundaryElementSolver            boundaryelementsolver.h
 *     ::calculateBoundarySolution()  -> hMatrixSolve() (:526-744)
 *     ::getPhiSolution() / getDPhiSolution() / getSoundPressure()
 *   BemSolverController              bemsolvercontroller.cpp:49-109 (the
 *     ::run() / requestStop()        frequency loop, per-frequency solved
 *     ::isBoundarySolvedAtFreq(i)    flags; a stopped run resumes)
 *
 * Header-only; link libbemgpu.so. Every call that fails throws bemgpu::Error
 * with the status and the handle's message. Complex vectors are
 * std::vector<std::complex<double>> (an Eigen::VectorXcd maps onto the same
 * memory: Eigen::Map<VectorXcd>(v.data(), v.size())).
 */
#ifndef BEMGPU_HPP
#define BEMGPU_HPP

#include <atomic>
#include <complex>
#include <exception>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "bemgpu.h"

namespace bemgpu {

using cplx = std::complex<double>;
using CVec = std::vector<cplx>;

class Error : public std::runtime_error {
 public:
  Error(bem_status st, const std::string& msg) : std::runtime_error(msg), status(st) {}
  bem_status status;
};

// BemSolverParameters (bemparameters.h:21-34) with the constants the
// reference hard-wires as fields (leaf size, admissibility, restart)
struct BemSolverParameters {
  double acaRelativeError = 1e-3;
  long acaMaxRank = 0;
  bool usePreconditioner = false;
  long preconditionerRank = 2;
  double preconditionerRelError = 0.0;
  int couplingParameter = 2;  // 0 none, 1 Burton-Miller, 2 Kirkup
  double gmresRelativeError = -1.0;  // < 0: 1e-3 * acaRelativeError (:670, :692)
  long leafSize = 50;
  double eta = 3.0;
  long gmresRestart = 300;
  long gmresMaxIterations = 1000;
  bool mixedPrecision = false;  // complex-FP32 storage with FP64 refinement
  long sweepWorkers = 1;        // frequencies solved concurrently by a sweep
};

namespace detail {
inline void check(bem_status st, const bem_handle* h, const char* what) {
  if (st != BEM_OK) throw Error(st, std::string(what) + ": " + bem_last_error(h));
}
struct HandleDeleter {
  void operator()(bem_handle* h) const { bem_destroy(h); }
};
}  // namespace detail

using Handle = std::shared_ptr<bem_handle>;

inline Handle make_handle(const BemSolverParameters& p, double c, double rho) {
  bem_config cfg;
  bem_config_default(&cfg);
  cfg.leaf_size = p.leafSize;
  cfg.eta = p.eta;
  cfg.aca_tol = p.acaRelativeError;
  cfg.aca_max_rank = p.acaMaxRank;
  cfg.gmres_tol = p.gmresRelativeError > 0 ? p.gmresRelativeError : 1e-3 * p.acaRelativeError;
  cfg.gmres_restart = p.gmresRestart;
  cfg.gmres_maxit = p.gmresMaxIterations;
  cfg.coupling = p.couplingParameter;
  cfg.precision = p.mixedPrecision ? 1 : 0;
  cfg.wave_speed = c;
  cfg.density = rho;
  cfg.use_preconditioner = p.usePreconditioner ? 1 : 0;
  cfg.precond_rank = p.preconditionerRank;
  cfg.precond_tol = p.preconditionerRelError;
  cfg.sweep_workers = p.sweepWorkers;
  bem_handle* h = nullptr;
  const bem_status st = bem_create(&cfg, &h);
  if (st != BEM_OK) throw Error(st, "bem_create failed");
  return Handle(h, detail::HandleDeleter());
}

// Host-only planning (no GPU): the cluster-tree permutation and the block
// partition (r0, m, c0, n, admissible) in the reference's minPartition order.
inline void planMesh(const std::vector<double>& triangles, const BemSolverParameters& p,
                     std::vector<int64_t>& perm, std::vector<int64_t>& blocks) {
  bem_config cfg;
  bem_config_default(&cfg);
  cfg.leaf_size = p.leafSize;
  cfg.eta = p.eta;
  const int64_t n = (int64_t)triangles.size() / 9;
  perm.assign(n, 0);
  int64_t nb = 0;
  bem_status st = bem_plan_mesh(&cfg, triangles.data(), n, perm.data(), &nb, nullptr);
  if (st != BEM_OK) throw Error(st, "bem_plan_mesh failed");
  blocks.assign(5 * nb, 0);
  st = bem_plan_mesh(&cfg, triangles.data(), n, perm.data(), &nb, blocks.data());
  if (st != BEM_OK) throw Error(st, "bem_plan_mesh failed");
}

// One assembled H-matrix of a handle (which = 0 phi, 1 dPhi), indices in
// cluster order like the reference's HMatrix.
class HMatrix {
 public:
  HMatrix(Handle h, int which, int64_t rows) : h_(std::move(h)), which_(which), rows_(rows) {}
  int64_t rows() const { return rows_; }
  int64_t cols() const { return rows_; }
  int which() const { return which_; }
  bem_handle* handle() const { return h_.get(); }

 private:
  Handle h_;
  int which_;
  int64_t rows_;
};

struct HArithm {
  // y += H x (harithm.h:32)
  static void MVM(CVec& y, const HMatrix& H, const CVec& x) {
    if ((int64_t)x.size() != H.cols() || (int64_t)y.size() != H.rows())
      throw Error(BEM_EINVAL, "HArithm::MVM: dimension mismatch");
    detail::check(bem_hmatvec(H.handle(), H.which(), reinterpret_cast<const double*>(x.data()),
                              reinterpret_cast<double*>(y.data()), 1, 1),
                  H.handle(), "bem_hmatvec");
  }
  // H-LU of the (truncated copy of the) system matrix; the factors live in
  // the handle (the reference returns the pair of factor H-matrices)
  static void LUDecomposition(const HMatrix& H) {
    if (H.which() != 1) throw Error(BEM_EINVAL, "LUDecomposition: the system matrix (dPhi)");
    detail::check(bem_hlu_build(H.handle()), H.handle(), "bem_hlu_build");
  }
  // x = U^{-1} L^{-1} b with the factors of LUDecomposition
  static CVec LUSubstitutionSolve(const HMatrix& H, const CVec& b) {
    CVec x(b.size());
    detail::check(bem_hlu_solve(H.handle(), reinterpret_cast<const double*>(b.data()),
                                reinterpret_cast<double*>(x.data()), 1),
                  H.handle(), "bem_hlu_solve");
    return x;
  }
};

struct GMRES {
  // GMRES on the dPhi matrix from x0 (gmres.h:170-180); tolerance and
  // restart come from the handle's parameters
  static CVec gmresSolve(const HMatrix& A, const CVec& x0, const CVec& b,
                         bem_solve_info* info = nullptr) {
    CVec x = x0;
    bem_solve_info loc{};
    const bem_status st =
        bem_gmres(A.handle(), reinterpret_cast<const double*>(b.data()),
                  reinterpret_cast<double*>(x.data()), 1, info ? info : &loc);
    if (st != BEM_OK && st != BEM_EMAXIT) detail::check(st, A.handle(), "bem_gmres");
    return x;
  }
};

// BoundaryElementSolver for one frequency: triangles (n x 9, node 1, 2, 3),
// the Robin data a phi + b dphi/dn = g per element (caller order)
class BoundaryElementSolver {
 public:
  BoundaryElementSolver(const std::vector<double>& triangles, const CVec& a, const CVec& b,
                        const CVec& g, double frequency, const BemSolverParameters& params,
                        double c = 343.0, double rho = 1.2)
      : n_((int64_t)triangles.size() / 9), freq_(frequency), g_(g) {
    if ((int64_t)a.size() != n_ || (int64_t)b.size() != n_ || (int64_t)g.size() != n_)
      throw Error(BEM_EINVAL, "BoundaryElementSolver: one a, b, g per triangle");
    h_ = make_handle(params, c, rho);
    detail::check(bem_set_mesh(h_.get(), triangles.data(), n_), h_.get(), "bem_set_mesh");
    std::vector<double> ad(2 * n_), bd(2 * n_);
    for (int64_t i = 0; i < n_; i++) {
      ad[2 * i] = a[i].real();
      ad[2 * i + 1] = a[i].imag();
      bd[2 * i] = b[i].real();
      bd[2 * i + 1] = b[i].imag();
    }
    detail::check(bem_set_bc(h_.get(), ad.data(), bd.data()), h_.get(), "bem_set_bc");
  }

  // calculateBoundarySolution -> hMatrixSolve -> phiSolutionToSoundPressure
  void calculateBoundarySolution() {
    phi_.assign(n_, 0.0);
    dphi_.assign(n_, 0.0);
    p_.assign(n_, 0.0);
    const bem_status st = bem_solve(
        h_.get(), freq_, reinterpret_cast<const double*>(g_.data()), 1,
        reinterpret_cast<double*>(phi_.data()), reinterpret_cast<double*>(dphi_.data()),
        reinterpret_cast<double*>(p_.data()), &info_);
    if (st != BEM_OK && st != BEM_EMAXIT) detail::check(st, h_.get(), "bem_solve");
  }
  void hMatrixSolve() { calculateBoundarySolution(); }

  const CVec& getPhiSolution() const { return phi_; }
  const CVec& getDPhiSolution() const { return dphi_; }
  const CVec& getSoundPressure() const { return p_; }
  const bem_solve_info& info() const { return info_; }
  // the assembled matrices of the last solve (phi: which 0, dPhi: 1)
  HMatrix hMatrix(int which) const { return HMatrix(h_, which, n_); }
  bem_handle* handle() const { return h_.get(); }

 private:
  Handle h_;
  int64_t n_;
  double freq_;
  CVec g_, phi_, dphi_, p_;
  bem_solve_info info_{};
};

// BemSolverController (bemsolvercontroller.cpp:49-109): the frequency loop of
// one mesh with the boundariesSolvedAtFrequency flags. run() solves every
// frequency not flagged yet (sweepWorkers at a time), flags each one as it
// completes and calls boundarySolvedForFreqIndex(i) (the reference's signal
// of that name; a place to save the result). After requestStop() the run
// ends once the frequencies in flight are done, in place of the reference's
// QThread::terminate (:211-227); a later run() solves the rest.
class BemSolverController {
 public:
  BemSolverController(const std::vector<double>& triangles, const CVec& a, const CVec& b,
                      const CVec& g, const std::vector<double>& frequencies,
                      const BemSolverParameters& params, double c = 343.0, double rho = 1.2)
      : n_((int64_t)triangles.size() / 9), freqs_(frequencies) {
    if ((int64_t)a.size() != n_ || (int64_t)b.size() != n_ || (int64_t)g.size() != n_)
      throw Error(BEM_EINVAL, "BemSolverController: one a, b, g per triangle");
    if (freqs_.empty()) throw Error(BEM_EINVAL, "BemSolverController: no frequencies");
    h_ = make_handle(params, c, rho);
    detail::check(bem_set_mesh(h_.get(), triangles.data(), n_), h_.get(), "bem_set_mesh");
    std::vector<double> ad(2 * n_), bd(2 * n_);
    g_.resize(2 * n_);
    for (int64_t i = 0; i < n_; i++) {
      ad[2 * i] = a[i].real();
      ad[2 * i + 1] = a[i].imag();
      bd[2 * i] = b[i].real();
      bd[2 * i + 1] = b[i].imag();
      g_[2 * i] = g[i].real();
      g_[2 * i + 1] = g[i].imag();
    }
    detail::check(bem_set_bc(h_.get(), ad.data(), bd.data()), h_.get(), "bem_set_bc");
    p_.assign(2 * n_ * freqs_.size(), 0.0);
    solved_.assign(freqs_.size(), 0);
    infos_.assign(freqs_.size(), bem_solve_info{});
  }

  void run() {
    stop_ = false;
    hook_error_ = nullptr;
    const bem_status st =
        bem_sweep_resume(h_.get(), freqs_.data(), (int64_t)freqs_.size(), g_.data(), 1,
                         p_.data(), infos_.data(), solved_.data(), &on_done, this);
    if (hook_error_) std::rethrow_exception(hook_error_);
    if (st != BEM_OK && st != BEM_EMAXIT) detail::check(st, h_.get(), "bem_sweep_resume");
  }
  void requestStop() { stop_ = true; }

  std::size_t numFrequencies() const { return freqs_.size(); }
  bool isBoundarySolvedAtFreq(std::size_t i) const { return solved_.at(i) != 0; }
  // sound pressure on the elements at frequency i (caller order)
  CVec getSoundPressure(std::size_t i) const {
    if (!isBoundarySolvedAtFreq(i)) throw Error(BEM_EINVAL, "frequency not solved yet");
    const double* q = p_.data() + 2 * n_ * i;
    CVec out(n_);
    for (int64_t e = 0; e < n_; e++) out[e] = cplx(q[2 * e], q[2 * e + 1]);
    return out;
  }
  const bem_solve_info& info(std::size_t i) const { return infos_.at(i); }

  std::function<void(std::size_t)> boundarySolvedForFreqIndex;

 private:
  static int on_done(int64_t f, void* user) {  // one call at a time
    auto* c = static_cast<BemSolverController*>(user);
    try {
      if (c->boundarySolvedForFreqIndex) c->boundarySolvedForFreqIndex((std::size_t)f);
    } catch (...) {
      c->hook_error_ = std::current_exception();
      return 1;
    }
    return c->stop_.load() ? 1 : 0;
  }

  Handle h_;
  int64_t n_;
  std::vector<double> freqs_, g_, p_;
  std::vector<uint8_t> solved_;
  std::vector<bem_solve_info> infos_;
  std::atomic<bool> stop_{false};
  std::exception_ptr hook_error_;
};

}  // namespace bemgpu

#endif
