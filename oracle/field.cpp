// field.cpp -- CPU FP64 restatement of the field evaluation (test
// infrastructure only: the parity checker of bem_field).
//
// Restates BoundaryElementSolver::calculateFieldSolutionRegular
// (boundaryelementsolver.cpp:2263-2316): at every observation point the sum of
// the point-source terms (sourcePhiTerm, :3443-3450) plus, per boundary
// element j, Mk_j phi_j - Lk_j dphi_j with Mk, Lk from BemOperatorField
// (:2318-2353) -- the 7-point triangle rule of order 5 (orderLow,
// boundaryelementsolver.h:653-654), Lk = A sum w G, Mk = A sum w dG/dr rnq,
// G = exp(ikr) / (4 pi r), dG/dr = (G / r)(ikr - 1), rnq = -((p - q) . n_q) / r.
// Sound pressure: i rho 2 pi f phi, with 2 pi in place of 2 pi f at f = 0
// (calculateFieldSolution, :2232-2244). k = 2 pi f / c (:2199). With one
// impedance plane the reflected elements add the same terms with the same
// boundary data (:2305-2311).
#include "bem_oracle.h"
#include "oracle_core.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace orc;

extern "C" void orc_field(const double* tri, int64_t n, double freq, double c, double rho,
                          const double* pts, int64_t npts, const double* phi, const double* dphi,
                          int64_t nrhs, const double* src, int64_t nsrc, const double* plane,
                          int nthreads, double* phi_f, double* p_f) {
  Mesh m;
  m.tri.resize(n);
  for (int64_t i = 0; i < n; i++) {
    const double* t = tri + 9 * i;
    m.tri[i] = Tri{V3(t[0], t[1], t[2]), V3(t[3], t[4], t[5]), V3(t[6], t[7], t[8])};
  }
  mesh_prepare(m);
  std::vector<const Mesh*> parts{&m};
  Mesh mirrored;
  if (plane && (plane[3] != 0 || plane[4] != 0 || plane[5] != 0)) {
    mirrored = reflect_mesh(m, V3(plane[0], plane[1], plane[2]), V3(plane[3], plane[4], plane[5]));
    parts.push_back(&mirrored);
  }
  const Rule2D rule = triangle_rule(5);
  const double k = PI2 * freq / c;
  const cd ik(0.0, k);
  const cd pfac = freq != 0.0 ? cd(0.0, rho * PI2 * freq) : cd(0.0, rho * PI2);
  const cd* ph = reinterpret_cast<const cd*>(phi);
  const cd* dph = reinterpret_cast<const cd*>(dphi);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t f = 0; f < npts; f++) {
    const V3 p(pts[3 * f], pts[3 * f + 1], pts[3 * f + 2]);
    cd s0 = 0.0;
    for (int64_t q = 0; q < nsrc; q++) {  // sourcePhiTerm
      const double* sq = src + 5 * q;
      const double r = norm(V3(sq[0], sq[1], sq[2]) - p);
      s0 += cd(sq[3], sq[4]) * std::exp(ik * r) / (PI4 * r);
    }
    std::vector<cd> acc(nrhs, s0);
    for (const Mesh* g : parts)
    for (int64_t j = 0; j < n; j++) {  // BemOperatorField
      const Tri& t = g->tri[j];
      const V3 nq = g->normal[j];
      cd Lk = 0.0, Mk = 0.0;
      for (int i = 0; i < rule.size(); i++) {
        const double a1 = rule.x1[i], a2 = rule.x2[i], a3 = 1.0 - a2 - a1;
        const V3 qp = (a1 * t.n1 + a2 * t.n2) + a3 * t.n3;
        const V3 rv = p - qp;
        const double r = norm(rv);
        const double rnq = -dot(rv, nq) / r;
        const cd ikr = ik * r;
        const cd G = std::exp(ikr) / (PI4 * r);
        Lk += rule.w[i] * G;
        Mk += rule.w[i] * ((G / r) * (ikr - 1.0)) * rnq;
      }
      Lk *= g->area[j];
      Mk *= g->area[j];
      for (int64_t r = 0; r < nrhs; r++) acc[r] += Mk * ph[r * n + j] - Lk * dph[r * n + j];
    }
    for (int64_t r = 0; r < nrhs; r++) {
      const cd v = acc[r];
      if (phi_f) {
        phi_f[2 * (r * npts + f)] = v.real();
        phi_f[2 * (r * npts + f) + 1] = v.imag();
      }
      if (p_f) {
        const cd pv = pfac * v;
        p_f[2 * (r * npts + f)] = pv.real();
        p_f[2 * (r * npts + f) + 1] = pv.imag();
      }
    }
  }
}
