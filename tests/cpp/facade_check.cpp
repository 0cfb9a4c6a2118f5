// Exercises the C++ facade (include/bemgpu.hpp) the way the reference's
// callers would: planning (host only), or a full BoundaryElementSolver solve
// plus HArithm::MVM, HArithm::LUDecomposition / LUSubstitutionSolve and
// GMRES::gmresSolve on its matrices. Input: a binary file of n x 9 doubles.
// Output: plain text lines the test compares with the Python path.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "bemgpu.hpp"

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  const std::string mode = argv[1];
  std::ifstream f(argv[2], std::ios::binary | std::ios::ate);
  const std::streamsize bytes = f.tellg();
  f.seekg(0);
  std::vector<double> tri(bytes / sizeof(double));
  f.read(reinterpret_cast<char*>(tri.data()), bytes);
  const int64_t n = (int64_t)tri.size() / 9;
  bemgpu::BemSolverParameters par;
  par.leafSize = 32;
  par.eta = 2.0;
  try {
    if (mode == "plan") {
      std::vector<int64_t> perm, blocks;
      bemgpu::planMesh(tri, par, perm, blocks);
      long long ps = 0;
      for (int64_t i = 0; i < n; i++) ps += (long long)(i + 1) * perm[i];
      std::printf("n %lld blocks %lld perm_checksum %lld\n", (long long)n,
                  (long long)(blocks.size() / 5), ps);
      return 0;
    }
    par.acaRelativeError = 1e-6;
    par.gmresRelativeError = 1e-10;
    if (mode == "sweep") {  // BemSolverController: stop after two frequencies, then resume
      par.sweepWorkers = 2;
      const bemgpu::CVec a(n, 0.0), b(n, 1.0), g(n, 1.0);
      const std::vector<double> fr = {200.0, 300.0, 400.0, 500.0, 600.0};
      bemgpu::BemSolverController c(tri, a, b, g, fr, par, 343.0, 1.2);
      int done = 0;
      c.boundarySolvedForFreqIndex = [&](std::size_t) {
        if (++done == 2) c.requestStop();
      };
      c.run();
      int first = 0;
      for (std::size_t i = 0; i < fr.size(); i++) first += c.isBoundarySolvedAtFreq(i);
      c.run();
      std::printf("first_run %d second_run %d\n", first, done - first);
      for (std::size_t i = 0; i < fr.size(); i++) {
        double pn = 0;
        for (const auto& v : c.getSoundPressure(i)) pn += std::norm(v);
        std::printf("f%zu %.15e status%zu %d\n", i, std::sqrt(pn), i, c.info(i).status);
      }
      return 0;
    }
    par.usePreconditioner = mode == "solve_precond";
    const bemgpu::CVec a(n, 0.0), b(n, 1.0), g(n, 1.0);
    bemgpu::BoundaryElementSolver s(tri, a, b, g, 300.0, par, 343.0, 1.2);
    s.calculateBoundarySolution();
    const bemgpu::CVec& p = s.getSoundPressure();
    double pn = 0;
    for (const auto& v : p) pn += std::norm(v);
    std::printf("status %d iterations %lld pnorm %.15e p0 %.15e %.15e\n", s.info().status,
                (long long)s.info().iterations, std::sqrt(pn), p[0].real(), p[0].imag());
    // the matrix-level calls of the reference on the assembled system matrix
    bemgpu::HMatrix A = s.hMatrix(1);
    bemgpu::CVec x(n), y(n, 0.0);
    for (int64_t i = 0; i < n; i++) x[i] = bemgpu::cplx(std::cos(0.1 * i), std::sin(0.2 * i));
    bemgpu::HArithm::MVM(y, A, x);  // y += A x
    bemgpu::CVec x2 = bemgpu::GMRES::gmresSolve(A, bemgpu::CVec(n, 0.0), y);
    double e = 0, xn = 0;
    for (int64_t i = 0; i < n; i++) {
      e += std::norm(x2[i] - x[i]);
      xn += std::norm(x[i]);
    }
    std::printf("gmres_rel_err %.3e\n", std::sqrt(e / xn));
    bemgpu::HArithm::LUDecomposition(A);
    bemgpu::CVec z = bemgpu::HArithm::LUSubstitutionSolve(A, y);
    e = 0;
    for (int64_t i = 0; i < n; i++) e += std::norm(z[i] - x[i]);
    std::printf("hlu_rel_err %.3e\n", std::sqrt(e / xn));
  } catch (const bemgpu::Error& err) {
    std::printf("error %d %s\n", (int)err.status, err.what());
    return 1;
  }
  return 0;
}
