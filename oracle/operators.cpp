// operators.cpp -- oracle restatement of the collocation operators L, M, Mt, N
// and the Robin-BC substitution (test infrastructure only).
#include "oracle_core.hpp"

#include <stdexcept>

namespace orc {

// ---------------------------------------------------------------------------
// Quadrature tables.
// Symmetric triangle rules of Dunavant (1985), degree d, in the point order of
// trianglequadraturerules.cpp (orders n = 1, 2, 5, 7, 8, 10 at :17-27, :47-57,
// :74-90, :91-110, :134-163). Values are the published ones as the reference
// tabulates them; the weights sum to 1 and are multiplied by the area later.
// ---------------------------------------------------------------------------
Rule1D gauss_legendre(int n);

namespace {
void push(Rule2D& r, double x1, double x2, double w) {
  r.x1.push_back(x1);
  r.x2.push_back(x2);
  r.w.push_back(w);
}

Rule2D rule_from_rows(const double* rows, int n) {
  Rule2D r;
  for (int i = 0; i < n; i++) push(r, rows[3 * i], rows[3 * i + 1], rows[3 * i + 2]);
  return r;
}
}  // namespace

Rule2D triangle_rule(int order) {
  if (order <= 1) {
    static const double t[] = {0.33333333333333, 0.33333333333333, 1.0};
    return rule_from_rows(t, 1);
  }
  if (order == 2) {
    static const double t[] = {0.16666666666667, 0.16666666666667, 0.33333333333333,
                               0.16666666666667, 0.66666666666667, 0.33333333333333,
                               0.66666666666667, 0.16666666666667, 0.33333333333333};
    return rule_from_rows(t, 3);
  }
  if (order == 5) {
    static const double t[] = {
        0.33333333333333, 0.33333333333333, 0.22500000000000,
        0.47014206410511, 0.47014206410511, 0.13239415278851,
        0.47014206410511, 0.05971587178977, 0.13239415278851,
        0.05971587178977, 0.47014206410511, 0.13239415278851,
        0.10128650732346, 0.10128650732346, 0.12593918054483,
        0.10128650732346, 0.79742698535309, 0.12593918054483,
        0.79742698535309, 0.10128650732346, 0.12593918054483};
    return rule_from_rows(t, 7);
  }
  if (order == 7) {
    static const double t[] = {
        0.33333333333333, 0.33333333333333, -0.14957004446768,
        0.26034596607904, 0.26034596607904, 0.17561525743321,
        0.26034596607904, 0.47930806784192, 0.17561525743321,
        0.47930806784192, 0.26034596607904, 0.17561525743321,
        0.06513010290222, 0.06513010290222, 0.05334723560884,
        0.06513010290222, 0.86973979419557, 0.05334723560884,
        0.86973979419557, 0.06513010290222, 0.05334723560884,
        0.31286549600487, 0.63844418856981, 0.07711376089026,
        0.63844418856981, 0.04869031542532, 0.07711376089026,
        0.04869031542532, 0.31286549600487, 0.07711376089026,
        0.63844418856981, 0.31286549600487, 0.07711376089026,
        0.31286549600487, 0.04869031542532, 0.07711376089026,
        0.04869031542532, 0.63844418856981, 0.07711376089026};
    return rule_from_rows(t, 13);
  }
  if (order == 8) {
    static const double t[] = {
        0.33333333333333, 0.33333333333333, 0.14431560767779,
        0.45929258829272, 0.45929258829272, 0.09509163426728,
        0.45929258829272, 0.08141482341455, 0.09509163426728,
        0.08141482341455, 0.45929258829272, 0.09509163426728,
        0.17056930775176, 0.17056930775176, 0.10321737053472,
        0.17056930775176, 0.65886138449648, 0.10321737053472,
        0.65886138449648, 0.17056930775176, 0.10321737053472,
        0.05054722831703, 0.05054722831703, 0.03245849762320,
        0.05054722831703, 0.89890554336594, 0.03245849762320,
        0.89890554336594, 0.05054722831703, 0.03245849762320,
        0.26311282963464, 0.72849239295540, 0.02723031417443,
        0.72849239295540, 0.00839477740996, 0.02723031417443,
        0.00839477740996, 0.26311282963464, 0.02723031417443,
        0.72849239295540, 0.26311282963464, 0.02723031417443,
        0.26311282963464, 0.00839477740996, 0.02723031417443,
        0.00839477740996, 0.72849239295540, 0.02723031417443};
    return rule_from_rows(t, 16);
  }
  if (order == 10) {
    // weights are tabulated halved in the source and doubled there
    static const double t[] = {
        0.333333333333333, 0.333333333333333, 0.045408995191377,
        0.028844733232685, 0.485577633383657, 0.018362978878233,
        0.485577633383657, 0.485577633383657, 0.018362978878233,
        0.485577633383657, 0.028844733232685, 0.018362978878233,
        0.781036849029926, 0.109481575485037, 0.022660529717764,
        0.109481575485037, 0.109481575485037, 0.022660529717764,
        0.109481575485037, 0.781036849029926, 0.022660529717764,
        0.141707219414880, 0.307939838764121, 0.036378958422710,
        0.307939838764121, 0.550352941820999, 0.036378958422710,
        0.550352941820999, 0.141707219414880, 0.036378958422710,
        0.307939838764121, 0.141707219414880, 0.036378958422710,
        0.550352941820999, 0.307939838764121, 0.036378958422710,
        0.141707219414880, 0.550352941820999, 0.036378958422710,
        0.025003534762686, 0.246672560639903, 0.014163621265528,
        0.246672560639903, 0.728323904597411, 0.014163621265528,
        0.728323904597411, 0.025003534762686, 0.014163621265528,
        0.246672560639903, 0.025003534762686, 0.014163621265528,
        0.728323904597411, 0.246672560639903, 0.014163621265528,
        0.025003534762686, 0.728323904597411, 0.014163621265528,
        0.009540815400299, 0.066803251012200, 0.004710833481867,
        0.066803251012200, 0.923655933587500, 0.004710833481867,
        0.923655933587500, 0.009540815400299, 0.004710833481867,
        0.066803251012200, 0.009540815400299, 0.004710833481867,
        0.923655933587500, 0.066803251012200, 0.004710833481867,
        0.009540815400299, 0.923655933587500, 0.004710833481867};
    Rule2D r = rule_from_rows(t, 25);
    for (auto& w : r.w) w *= 2.0;
    return r;
  }
  if (order >= 15) {
    // 64-point conical product rule: Gauss-Jacobi(1,0) in xi1 times
    // Gauss-Legendre in xi2 on [0, 1 - xi1] (same construction as the
    // reference's n = 15 table, computed here to full double precision).
    Rule1D gl = gauss_legendre(8);
    // Gauss-Jacobi nodes for weight (1-u) on [0, 1]: roots of P_8^(1,0)(2u-1)
    // found by Newton on the three-term recurrence.
    const int n = 8;
    std::vector<double> u(n), wu(n);
    for (int i = 0; i < n; i++) {
      double x = std::cos(PI * (i + 0.75) / (n + 0.5));  // initial guess on [-1,1]
      for (int it = 0; it < 100; it++) {
        // Jacobi P_n^(a,b) with a = 1, b = 0 via recurrence
        double a = 1.0, b = 0.0;
        double p0 = 1.0, p1 = 0.5 * (a - b + (a + b + 2.0) * x);
        double pn = p1, pnm1 = p0;
        for (int kk = 2; kk <= n; kk++) {
          double k2 = 2.0 * kk + a + b;
          double c1 = 2.0 * kk * (kk + a + b) * (k2 - 2.0);
          double c2 = (k2 - 1.0) * (a * a - b * b);
          double c3 = (k2 - 2.0) * (k2 - 1.0) * k2;
          double c4 = 2.0 * (kk + a - 1.0) * (kk + b - 1.0) * k2;
          double pk = ((c2 + c3 * x) * pn - c4 * pnm1) / c1;
          pnm1 = pn;
          pn = pk;
        }
        // derivative: d/dx P_n^(a,b) = 0.5 (n + a + b + 1) P_{n-1}^(a+1,b+1)
        double a2 = a + 1.0, b2 = b + 1.0;
        double q0 = 1.0, q1 = 0.5 * (a2 - b2 + (a2 + b2 + 2.0) * x);
        double qn = (n - 1 == 0) ? q0 : q1, qnm1 = q0;
        for (int kk = 2; kk <= n - 1; kk++) {
          double k2 = 2.0 * kk + a2 + b2;
          double c1 = 2.0 * kk * (kk + a2 + b2) * (k2 - 2.0);
          double c2 = (k2 - 1.0) * (a2 * a2 - b2 * b2);
          double c3 = (k2 - 2.0) * (k2 - 1.0) * k2;
          double c4 = 2.0 * (kk + a2 - 1.0) * (kk + b2 - 1.0) * k2;
          double qk = ((c2 + c3 * x) * qn - c4 * qnm1) / c1;
          qnm1 = qn;
          qn = qk;
        }
        double dp = 0.5 * (n + a + b + 1.0) * qn;
        double dx = pn / dp;
        x -= dx;
        if (std::fabs(dx) < 1e-16) break;
      }
      u[i] = 0.5 * (1.0 + x);  // weight (1-x) on [-1,1] maps to weight (1-u) on [0,1]
    }
    // Weights by solving the moment equations sum_i wu_i u_i^j = int_0^1 (1-u) u^j du
    // is ill-conditioned; use the closed form via Lagrange basis integration with
    // the 8-point Gauss-Legendre rule of degree 15 on [0,1] (exact for degree <= 15).
    for (int i = 0; i < n; i++) {
      double acc = 0.0;
      for (int q = 0; q < gl.size(); q++) {
        double t = 0.5 * (gl.x[q] + 1.0);
        double li = 1.0;
        for (int j = 0; j < n; j++)
          if (j != i) li *= (t - u[j]) / (u[i] - u[j]);
        acc += 0.5 * gl.w[q] * li * (1.0 - t);
      }
      wu[i] = acc;
    }
    Rule2D r;
    // u is the collapsed coordinate measured from the edge xi1 = 0 towards the
    // vertex xi1 = 1, so xi1 = u and the Jacobian (1 - u) is in wu.
    for (int i = 0; i < n; i++)
      for (int j = 0; j < gl.size(); j++) {
        double v = 0.5 * (gl.x[j] + 1.0);
        push(r, u[i], (1.0 - u[i]) * v, 2.0 * wu[i] * 0.5 * gl.w[j]);
      }
    return r;
  }
  throw std::runtime_error("triangle_rule: unsupported order");
}

// Gauss-Legendre nodes/weights on [-1, 1] by Newton iteration on the Legendre
// recurrence (the reference tabulates the same rules, linequadraturerules.cpp:8-121).
Rule1D gauss_legendre(int n) {
  Rule1D r;
  r.x.resize(n);
  r.w.resize(n);
  for (int i = 0; i < n; i++) {
    double x = std::cos(PI * (i + 0.75) / (n + 0.5));
    double dp = 0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = x;
      for (int k = 2; k <= n; k++) {
        double pk = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = pk;
      }
      if (n == 1) { p1 = x; p0 = 1.0; }
      dp = n * (x * p1 - p0) / (x * x - 1.0);
      double dx = p1 / dp;
      x -= dx;
      if (std::fabs(dx) < 1e-17) break;
    }
    // recompute derivative at the converged node
    double p0 = 1.0, p1 = x;
    for (int k = 2; k <= n; k++) {
      double pk = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = pk;
    }
    dp = (n == 1) ? 1.0 : n * (x * p1 - p0) / (x * x - 1.0);
    r.x[n - 1 - i] = x;  // ascending order
    r.w[n - 1 - i] = 2.0 / ((1.0 - x * x) * dp * dp);
  }
  if (n == 1) {
    r.x[0] = 0.0;
    r.w[0] = 2.0;
  }
  return r;
}

Rule1D line_rule(int n) {
  if (n <= 5) return gauss_legendre(n < 1 ? 1 : n);
  return gauss_legendre(32);
}

// splitmix64 finaliser over (seed, a, b): the seeded stand-in for the
// reference's QRandomGenerator::system() picks (hmatrix.cpp:508,
// boundaryelementsolver.cpp:2156-2158).
uint64_t pivot_hash(uint64_t seed, uint64_t a, uint64_t b) {
  uint64_t z = seed ^ (a * 0x9E3779B97F4A7C15ull) ^ (b * 0xC2B2AE3D27D4EB4Full);
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// ---------------------------------------------------------------------------
// Geometry: normalVectorOfTriangle / midpointOfTriangle (global.cpp:903-912),
// areaOfTriangle (global.cpp:1285-1290), averageTriangleDim
// (boundaryelements.cpp:37-46).
// ---------------------------------------------------------------------------
void mesh_prepare(Mesh& m) {
  m.n = (int64_t)m.tri.size();
  m.normal.resize(m.n);
  m.colloc.resize(m.n);
  m.area.resize(m.n);
  double acc = 0;
  for (int64_t i = 0; i < m.n; i++) {
    const Tri& t = m.tri[i];
    V3 c = cross(t.n2 - t.n1, t.n3 - t.n1);
    double cn = norm(c);
    m.normal[i] = V3(c.x / cn, c.y / cn, c.z / cn);
    V3 s = (t.n1 + t.n2) + t.n3;
    m.colloc[i] = V3(s.x / 3.0, s.y / 3.0, s.z / 3.0);
    m.area[i] = norm(cross(t.n1 - t.n2, t.n1 - t.n3)) / 2.0;
    acc += std::sqrt(m.area[i]);
  }
  m.avgdim = m.n > 0 ? acc / m.n / 2.0 : 0.0;
}

Mesh reflect_mesh(const Mesh& m, const V3& point, V3 normal) {
  const double nn = norm(normal);
  normal = V3(normal.x / nn, normal.y / nn, normal.z / nn);
  const double d = -dot(normal, point);
  double R[3][4];
  for (int i = 0; i < 3; i++) {
    for (int j = 0; j < 3; j++) R[i][j] = (i == j ? 1.0 : 0.0) - 2.0 * normal[i] * normal[j];
    R[i][3] = -2.0 * normal[i] * d;
  }
  const auto apply = [&](const V3& x) {
    V3 y;
    for (int i = 0; i < 3; i++) y[i] = R[i][0] * x.x + R[i][1] * x.y + R[i][2] * x.z + R[i][3];
    return y;
  };
  Mesh r;
  r.tri.resize(m.tri.size());
  for (size_t i = 0; i < m.tri.size(); i++)
    r.tri[i] = Tri{apply(m.tri[i].n3), apply(m.tri[i].n2), apply(m.tri[i].n1)};
  mesh_prepare(r);
  return r;
}

OperatorCtx::OperatorCtx(const Mesh* m, double k_, const Mesh* reflected)
    : mesh(m), k(k_), refl(reflected) {
  reg = triangle_rule(8);  // orderRegular = 8 (boundaryelementsolver.h:655-660)
  line = line_rule(5);     // orderLineQuadrature = 5 (:662-664)
  Rule1D g32 = gauss_legendre(32);
  for (int i = 16; i < 32; i++) {  // positive abscissas, ascending
    gl16.x.push_back(g32.x[i]);
    gl16.w.push_back(g32.w[i]);
  }
}

// BemOperatorsConst dispatch (boundaryelementsolver.cpp:844-856).
Ops OperatorCtx::eval(int64_t row, int64_t col) const {
  Ops o;
  if (row == col) o = singular(row);
  else if (norm(mesh->colloc[row] - mesh->colloc[col]) < 4.0 * mesh->avgdim)
    o = near_singular(row, col);
  else o = regular(row, col);
  if (refl) {
    const Ops r = regular_from(row, *refl, col);
    o.L += r.L;
    o.M += r.M;
    o.Mt += r.Mt;
    o.N += r.N;
  }
  return o;
}

namespace {
// the integrand shared by the regular and near-singular rules
// (boundaryelementsolver.cpp:872-887 and :1486-1500)
inline void accumulate(Ops& o, double w, V3 p, V3 q, V3 np, V3 nq, double upNq, double k) {
  const cd I(0.0, 1.0);
  V3 rv = p - q;
  double rr = dot(rv, rv);
  double r = std::sqrt(rr);
  double rnq = -dot(rv, nq) / r;
  double rnp = dot(rv, np) / r;
  cd ikr = I * k * r;
  cd G = std::exp(ikr) / (PI4 * r);
  o.L += w * G;
  cd dG = (G / r) * (ikr - 1.0);
  o.M += w * dG * rnq;
  o.Mt += w * dG * rnp;
  cd d2G = (G / rr) * (2.0 - 2.0 * ikr - k * k * rr);
  o.N += w * (dG * (-(upNq + rnp * rnq) / r) + d2G * rnp * rnq);
}
}  // namespace

// Regular 16-point rule (boundaryelementsolver.cpp:857-893).
Ops OperatorCtx::regular(int64_t row, int64_t col) const { return regular_from(row, *mesh, col); }

Ops OperatorCtx::regular_from(int64_t row, const Mesh& cm, int64_t col) const {
  Ops o{};
  const Tri& t = cm.tri[col];
  V3 p = mesh->colloc[row], np = mesh->normal[row], nq = cm.normal[col];
  double upNq = dot(np, nq);
  for (int i = 0; i < reg.size(); i++) {
    double a1 = reg.x1[i], a2 = reg.x2[i], a3 = 1.0 - a2 - a1;
    V3 q = (a1 * t.n1) + (a2 * t.n2) + (a3 * t.n3);
    accumulate(o, reg.w[i], p, q, np, nq, upNq, k);
  }
  double A = cm.area[col];
  o.L *= A;
  o.M *= A;
  o.Mt *= A;
  o.N *= A;
  return o;
}

// Singular (i == j) polar integration (boundaryelementsolver.cpp:896-1029):
// split at the collocation point into three sub-triangles, integrate the
// angle with the 32-point Gauss-Legendre rule (16 symmetric pairs) and the
// radius analytically.
Ops OperatorCtx::singular(int64_t ti) const {
  const cd I(0.0, 1.0);
  const Tri& t = mesh->tri[ti];
  V3 c = mesh->colloc[ti];
  const V3 sub[3][2] = {{t.n1, t.n2}, {t.n2, t.n3}, {t.n3, t.n1}};
  cd Lsum = 0, Nsum = 0;
  for (int s = 0; s < 3; s++) {
    V3 P1 = sub[s][0], P2 = sub[s][1];
    V3 cs = c - P1, bs = c - P2, as = P2 - P1;
    double b2 = dot(bs, bs), c2 = dot(cs, cs), a2 = dot(as, as);
    double b = std::sqrt(b2), cc = std::sqrt(c2);
    if (cc < b) std::swap(cc, b);
    double A = std::acos((b2 + c2 - a2) / (2.0 * b * cc));
    double B = std::atan((b * std::sin(A)) / (cc - b * std::cos(A)));
    double half = 0.5 * A;
    cd Ls = 0, Ns = 0;
    for (int i = 0; i < gl16.size(); i++) {
      double th1 = gl16.x[i] * half + half;
      double th2 = -gl16.x[i] * half + half;
      double r1 = cc * std::sin(B) / std::sin(th1 + B);
      double r2 = cc * std::sin(B) / std::sin(th2 + B);
      cd e1 = std::exp(I * k * r1), e2 = std::exp(I * k * r2);
      Ls += gl16.w[i] * (e1 + e2);
      Ns += gl16.w[i] * (e1 / r1 + e2 / r2);
    }
    Lsum += Ls * half;
    Nsum += Ns * half;
  }
  cd LT = Lsum / PI2;
  cd NT = Nsum / PI4;
  Ops o{};
  o.L = (I / (2.0 * k)) * (1.0 - LT);
  o.N = (I * k / 2.0) - NT;
  return o;
}

// projectPointOnTriangleFaster (global.cpp:955-1228): closest point of a
// triangle to p, classified as interior / node / side with the 0.05
// barycentric threshold. The region-by-region minimisation is D. Eberly's
// published point-to-triangle distance algorithm ("Distance Between Point and
// Triangle in 3D", Geometric Tools), as in the reference.
enum Region { IN_INTERIOR, ON_NODE1, ON_NODE2, ON_NODE3, ON_SIDE21, ON_SIDE32, ON_SIDE13 };

static std::pair<V3, Region> project_point(const Tri& tr, V3 point) {
  V3 diff = tr.n1 - point;
  V3 e0 = tr.n2 - tr.n1, e1 = tr.n3 - tr.n1;
  double a00 = dot(e0, e0), a01 = dot(e0, e1), a11 = dot(e1, e1);
  double b0 = dot(diff, e0), b1 = dot(diff, e1);
  double det = std::max(a00 * a11 - a01 * a01, 0.0);
  double s = a01 * b1 - a11 * b0;
  double t = a01 * b0 - a00 * b1;
  if (s + t <= det) {
    if (s < 0.0) {
      if (t < 0.0) {  // region 4
        if (b0 < 0.0) {
          t = 0.0;
          s = (-b0 >= a00) ? 1.0 : -b0 / a00;
        } else {
          s = 0.0;
          if (b1 >= 0.0) t = 0.0;
          else if (-b1 >= a11) t = 1.0;
          else t = -b1 / a11;
        }
      } else {  // region 3
        s = 0.0;
        if (b1 >= 0.0) t = 0.0;
        else if (-b1 >= a11) t = 1.0;
        else t = -b1 / a11;
      }
    } else if (t < 0.0) {  // region 5
      t = 0.0;
      if (b0 >= 0.0) s = 0.0;
      else if (-b0 >= a00) s = 1.0;
      else s = -b0 / a00;
    } else {  // region 0
      s /= det;
      t /= det;
    }
  } else {
    if (s < 0.0) {  // region 2
      double tmp0 = a01 + b0, tmp1 = a11 + b1;
      if (tmp1 > tmp0) {
        double numer = tmp1 - tmp0, denom = a00 - 2.0 * a01 + a11;
        if (numer >= denom) { s = 1.0; t = 0.0; }
        else { s = numer / denom; t = 1.0 - s; }
      } else {
        s = 0.0;
        if (tmp1 <= 0.0) t = 1.0;
        else if (b1 >= 0.0) t = 0.0;
        else t = -b1 / a11;
      }
    } else if (t < 0.0) {  // region 6
      double tmp0 = a01 + b1, tmp1 = a00 + b0;
      if (tmp1 > tmp0) {
        double numer = tmp1 - tmp0, denom = a00 - 2.0 * a01 + a11;
        if (numer >= denom) { t = 1.0; s = 0.0; }
        else { t = numer / denom; s = 1.0 - t; }
      } else {
        t = 0.0;
        if (tmp1 <= 0.0) s = 1.0;
        else if (b0 >= 0.0) s = 0.0;
        else s = -b0 / a00;
      }
    } else {  // region 1
      double numer = a11 + b1 - a01 - b0;
      if (numer <= 0.0) { s = 0.0; t = 1.0; }
      else {
        double denom = a00 - 2.0 * a01 + a11;
        if (numer >= denom) { s = 1.0; t = 0.0; }
        else { s = numer / denom; t = 1.0 - s; }
      }
    }
  }
  double c1 = 1.0 - s - t, c2 = s, c3 = t;
  int sig = (c1 > PROJ_EPS) + (c2 > PROJ_EPS) + (c3 > PROJ_EPS);
  Region reg;
  if (sig == 3) {
    reg = IN_INTERIOR;
  } else if (sig == 2) {
    if (c1 > PROJ_EPS && c2 > PROJ_EPS) {
      reg = ON_SIDE21; c1 += c3 / 2.0; c2 += c3 / 2.0; c3 = 0.0;
    } else if (c1 > PROJ_EPS && c3 > PROJ_EPS) {
      reg = ON_SIDE13; c1 += c2 / 2.0; c3 += c2 / 2.0; c2 = 0.0;
    } else {
      reg = ON_SIDE32; c2 += c1 / 2.0; c3 += c1 / 2.0; c1 = 0.0;
    }
  } else {
    if (c1 > PROJ_EPS) { reg = ON_NODE1; c1 = 1; c2 = 0; c3 = 0; }
    else if (c2 > PROJ_EPS) { reg = ON_NODE2; c1 = 0; c2 = 1; c3 = 0; }
    else { reg = ON_NODE3; c1 = 0; c2 = 0; c3 = 1; }
  }
  return {(c1 * tr.n1) + (c2 * tr.n2) + (c3 * tr.n3), reg};
}

// Near-singular split-polar rule (boundaryelementsolver.cpp:1387-1514).
Ops OperatorCtx::near_singular(int64_t row, int64_t col) const {
  Ops o{};
  V3 p = mesh->colloc[row], np = mesh->normal[row], nq = mesh->normal[col];
  double upNq = dot(np, nq);
  const Tri& d = mesh->tri[col];
  auto pr = project_point(d, p);
  V3 P = pr.first;
  Tri sub[3];
  int ns = 0;
  switch (pr.second) {
    case IN_INTERIOR:
      sub[0] = {P, d.n1, d.n2}; sub[1] = {P, d.n2, d.n3}; sub[2] = {P, d.n3, d.n1}; ns = 3;
      break;
    case ON_NODE1: sub[0] = d; ns = 1; break;
    case ON_NODE2: sub[0] = {d.n2, d.n3, d.n1}; ns = 1; break;
    case ON_NODE3: sub[0] = {d.n3, d.n1, d.n2}; ns = 1; break;
    case ON_SIDE21: sub[0] = {P, d.n3, d.n1}; sub[1] = {P, d.n2, d.n3}; ns = 2; break;
    case ON_SIDE32: sub[0] = {P, d.n3, d.n1}; sub[1] = {P, d.n1, d.n2}; ns = 2; break;
    case ON_SIDE13: sub[0] = {P, d.n1, d.n2}; sub[1] = {P, d.n2, d.n3}; ns = 2; break;
  }
  for (int s = 0; s < ns; s++) {
    const Tri& ct = sub[s];
    V3 s13 = ct.n3 - ct.n1, s23 = ct.n3 - ct.n2, s12 = ct.n2 - ct.n1;
    double q13 = dot(s13, s13), q23 = dot(s23, s23), q12 = dot(s12, s12);
    double l13 = std::sqrt(q13), l23 = std::sqrt(q23), l12 = std::sqrt(q12);
    double angP = std::acos((q13 + q12 - q23) / (2.0 * l13 * l12));
    double ang2 = std::acos((q23 + q12 - q13) / (2.0 * l23 * l12));
    V3 e0 = (1.0 / l12) * s12;
    V3 t1 = s13 - dot(e0, s13) * e0;
    V3 e1 = (1.0 / norm(t1)) * t1;
    Ops acc{};
    for (int i = 0; i < line.size(); i++) {
      double th = (angP + line.x[i] * angP) / 2.0;
      double rmax = l12 * std::sin(ang2) / std::sin(th + ang2);
      for (int j = 0; j < line.size(); j++) {
        double rs = (rmax + line.x[j] * rmax) / 2.0;
        double x = rs * std::cos(th), y = rs * std::sin(th);
        V3 q = ct.n1 + (x * e0) + (y * e1);
        double w = rmax / 2.0 * rs * line.w[i] * line.w[j];
        accumulate(acc, w, p, q, np, nq, upNq, k);
      }
    }
    double f = angP / 2.0;
    o.L += f * acc.L;
    o.M += f * acc.M;
    o.Mt += f * acc.Mt;
    o.N += f * acc.N;
  }
  return o;
}

// Coupling parameter (boundaryelementsolver.cpp:36-59, bemparameters.h:16).
Coupling coupling_parameter(int kind, double k) {
  const cd I(0.0, 1.0);
  Coupling c{};
  if (kind == 0) c.alpha = 0.0;
  else if (kind == 1) c.alpha = (std::fabs(k) < TINY) ? I : I / k;
  else c.alpha = I / (k + 1.0);
  c.alpha_half = c.alpha / 2.0;
  return c;
}

// implicitPhiMatrix2 / implicitDPhiMatrix2 (boundaryelementsolver.cpp:2004-2040)
// with substituteDPhiWithPhi = |a| < |b| (:3423).
void EntryGen::both(int64_t row, int64_t col, cd& phi, cd& dphi) const {
  Ops o = ops->eval(row, col);
  double on = (row == col) ? 1.0 : 0.0;
  cd X = o.L + alpha * o.Mt + on * alpha_half;
  cd Y = o.M + alpha * o.N - on * 0.5;
  if (std::abs(a[col]) < std::abs(b[col])) {
    phi = -X / b[col];
    dphi = -a[col] / b[col] * X - Y;
  } else {
    phi = Y / a[col];
    dphi = X + b[col] / a[col] * Y;
  }
}

cd EntryGen::operator()(int64_t row, int64_t col) const {
  cd p, d;
  both(row, col, p, d);
  return which == 0 ? p : d;
}

}  // namespace orc
