"""Field evaluation on the GPU (bem_field: calculateFieldSolution,
boundaryelementsolver.cpp:2192-2249, as the regular sum :2263-2316 with
BemOperatorField :2318-2353 and sourcePhiTerm :3443-3450) against the oracle.

Tolerances (norm-wise relative over all points and columns): FP64 mode 1e-11;
mixed precision (FP32 integrand, FP64 accumulation per 128 elements) 2e-5.
"""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

RHO, C = 1.2041, 343.0


def box_case(meshes, R=5, npts=700, seed=3):
    tri = meshes.box(n_target=1200, seed=7)  # 0.3 x 0.2 x 0.4 m, corner at the origin
    n = tri.shape[0]
    rng = np.random.default_rng(seed)
    phi = rng.standard_normal((n, R)) + 1j * rng.standard_normal((n, R))
    dphi = rng.standard_normal((n, R)) + 1j * rng.standard_normal((n, R))
    pts = rng.uniform(-0.4, 0.8, (npts, 3))  # inside, outside and near the box
    src = [[0.15, 0.1, 0.2, 1.0 + 0.5j], [-0.3, 0.4, 0.1, -0.25j]]
    return tri, phi, dphi, pts, src


def solver(bem, tri, precision):
    s = bem.Solver(precision=precision, wave_speed=C, density=RHO)
    s.set_mesh(tri)
    return s


@pytest.mark.parametrize("precision,tol", [(0, 1e-11), (1, 2e-5)])
@pytest.mark.parametrize("freq", [0.0, 900.0])
def test_field_matches_oracle(bem, meshes, orc, precision, tol, freq):
    tri, phi, dphi, pts, src = box_case(meshes)
    s = solver(bem, tri, precision)
    pf, pp = s.field(freq, pts, phi, dphi, src)
    of, op = orc.field(tri, freq, pts, phi, dphi, sources=src, c=C, rho=RHO)
    assert rel(pf, of) < tol
    assert rel(pp, op) < tol
    for r in range(phi.shape[1]):  # every column of both passes (4 + 1)
        assert rel(pf[:, r], of[:, r]) < tol
    # deterministic: partial sums are added in a fixed order
    pf2, _ = s.field(freq, pts, phi, dphi, src)
    assert np.array_equal(pf, pf2)


def test_field_device_entry_matches_host(bem, meshes):
    torch = pytest.importorskip("torch")
    tri, phi, dphi, pts, src = box_case(meshes, R=2, npts=300)
    s = solver(bem, tri, 1)
    pf, pp = s.field(500.0, pts, phi, dphi, src)
    dpts = torch.from_numpy(pts).to("cuda")
    dphi_ = torch.from_numpy(np.asfortranarray(phi).T.copy()).to("cuda")   # R x n = n x R col-major
    ddphi = torch.from_numpy(np.asfortranarray(dphi).T.copy()).to("cuda")
    of = torch.zeros((2, 300), dtype=torch.complex128, device="cuda")
    op = torch.zeros((2, 300), dtype=torch.complex128, device="cuda")
    s.field_device(500.0, dpts.data_ptr(), 300, dphi_.data_ptr(), ddphi.data_ptr(), 2,
                   of.data_ptr(), op.data_ptr(), sources=src)
    torch.cuda.synchronize()
    assert np.array_equal(of.cpu().numpy().T, pf)
    assert np.array_equal(op.cpu().numpy().T, pp)


def test_field_linearity_at_scale(bem, meshes):
    """Size-independent property at 200k points (many element chunks per
    point block is not the regime here; many point blocks is): the field is
    linear in the boundary data."""
    tri, phi, dphi, _, _ = box_case(meshes, R=2)
    rng = np.random.default_rng(11)
    pts = rng.uniform(-1.0, 1.4, (200_000, 3))
    s = solver(bem, tri, 1)
    f1, _ = s.field(700.0, pts, phi[:, 0], dphi[:, 0])
    f2, _ = s.field(700.0, pts, phi[:, 1], dphi[:, 1])
    a, b = 0.7 - 0.2j, -1.3 + 0.4j
    f12, _ = s.field(700.0, pts, a * phi[:, 0] + b * phi[:, 1], a * dphi[:, 0] + b * dphi[:, 1])
    assert rel(f12[:, 0], a * f1[:, 0] + b * f2[:, 0]) < 1e-5
    assert np.isfinite(f12).all()


def test_field_after_solve_pulsating_sphere(bem, meshes, orc):
    """Solve, then field: outside a sphere with uniform normal velocity
    p(r) = p(a) (a / r) exp(ik(r - a)); the GPU field of the GPU solution also
    matches the oracle's field of the same boundary data."""
    a = 1.0
    tri = meshes.icosphere(4, a)
    n = tri.shape[0]
    f = 200.0
    k = 2 * np.pi * f / C
    s = bem.Solver(precision=1, aca_tol=1e-5, gmres_tol=1e-8, wave_speed=C, density=RHO)
    s.set_mesh(tri)
    s.set_bc(np.zeros(n), np.ones(n))
    phi, dphi, p, info = s.solve(f, np.ones(n))
    assert info["status"] == 0
    r = np.array([1.2, 2.0, 5.0, 10.0])
    pts = np.column_stack([r * 0.48, r * 0.6, r * 0.64])
    pf, pp = s.field(f, pts, phi, dphi)
    pa = RHO * C * (1j * k * a) / (1j * k * a - 1)
    ex = pa * (a / r) * np.exp(1j * k * (r - a))
    assert (np.abs(pp[:, 0] - ex) / np.abs(ex)).max() < 0.02
    _, op = orc.field(tri, f, pts, phi, dphi, c=C, rho=RHO)
    assert rel(pp, op) < 2e-5


def test_field_facade_observation_fields(bem, meshes):
    """BoundaryElementSolver.calculateFieldSolution fills every observation
    field at its triangle midpoints."""
    tri = meshes.icosphere(3, 0.5)
    n = tri.shape[0]
    be = bem.BoundaryElements(tri, np.zeros(n), np.ones(n), np.ones(n))
    par = bem.BemSolverParameters(acaRelativeError=1e-4)
    sol = bem.BoundaryElementSolver(be, 300.0, bemSolverParameters=par)
    sol.calculateBoundarySolution()
    plane = meshes.icosphere(1, 2.0)  # a spherical observation surface
    sol.observationFields = [bem.ObservationField(plane), bem.ObservationField(plane[:7])]
    sol.calculateFieldSolution()
    mid = sol.observationFields[0].calculateTrianglesMidpoints()
    ref_f, ref_p = sol._solver().field(300.0, mid, be.phiSolution, be.dPhiSolution)
    assert np.array_equal(sol.observationFields[0].soundPressure, ref_p[:, 0])
    assert np.array_equal(sol.observationFields[1].phiSolution, ref_f[:7, 0])
    sol.close()


def test_field_edge_cases(bem, meshes):
    tri, phi, dphi, pts, _ = box_case(meshes, R=1, npts=5)
    s = solver(bem, tri, 1)
    pf, pp = s.field(100.0, np.zeros((0, 3)), phi, dphi)
    assert pf.shape == (0, 1) and pp.shape == (0, 1)
    with pytest.raises(bem.BemError):
        s.field(-1.0, pts, phi, dphi)
    with pytest.raises(bem.BemError):
        s.field(float("nan"), pts, phi, dphi)
    fresh = bem.Solver()
    with pytest.raises(bem.BemError):  # no mesh
        fresh.field(100.0, pts, phi, dphi)
    # one point, one element chunk: a single observation point still works
    one, _ = s.field(100.0, pts[:1], phi, dphi)
    many, _ = s.field(100.0, pts, phi, dphi)
    assert rel(one[0], many[0]) < 1e-6
