"""One impedance plane on the GPU (bem_set_impedance_plane): every entry adds
the reflected element's regular-rule operators on the same partition
(implicitPhiMatrixPlusReflected, boundaryelementsolver.cpp:2042-2050), and the
field adds the reflected terms (:2305-2311). Checked against the oracle (whose
half-space matrices equal the folded mirrored full-space ones, test_oracle),
against the GPU's own full-space solve of body + mirror image, and for state
handling (removal, sweep workers)."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

POINT, NORMAL = [0.0, 0.0, 0.0], [0.0, 0.0, 1.0]


def body(meshes, sub=3):
    tri = meshes.icosphere(sub, 0.5)
    tri[:, 2::3] += 0.7  # sphere above the plane z = 0, gap 0.2 m
    return tri


def mirror(tri):
    nrm = np.asarray(NORMAL) / np.linalg.norm(NORMAL)
    R = lambda x: x - 2.0 * (x @ nrm)[:, None] * nrm
    return np.hstack([R(tri[:, 6:9]), R(tri[:, 3:6]), R(tri[:, 0:3])])


def solver(bem, tri, precision, plane=True, **cfg):
    s = bem.Solver(**{"aca_tol": 1e-5, "gmres_tol": 1e-9, "precision": precision, **cfg})
    s.set_mesh(tri)
    n = tri.shape[0]
    s.set_bc(np.zeros(n), np.ones(n))
    if plane:
        s.set_impedance_plane(POINT, NORMAL)
    return s


@pytest.mark.parametrize("precision,tol", [(0, 1e-6), (1, 2e-5)])
def test_half_space_solve_vs_oracle(bem, meshes, orc, precision, tol):
    tri = body(meshes)
    n = tri.shape[0]
    s = solver(bem, tri, precision)
    phi, dphi, p, info = s.solve(400.0, np.ones(n))
    assert info["status"] == 0 and info["true_residual"] < 1e-8
    P = orc.Problem(tri, 32, 2.0)
    P.set_plane(POINT, NORMAL)
    po, dpo, ppo, st = P.solve(400.0, 343.0, 1.2, 2, np.zeros(n), np.ones(n), np.ones(n),
                               1e-5, 1e-9, seed=s.config.seed)
    assert rel(p[:, 0], ppo[:, 0]) < tol
    # the rigid plane matters: the free-space pressures differ by more than 5 %
    _, _, pf, _ = solver(bem, tri, precision, plane=False).solve(400.0, np.ones(n))
    assert rel(pf[:, 0], p[:, 0]) > 0.05


def test_half_space_equals_mirrored_full_space(bem, meshes):
    tri = body(meshes)
    n = tri.shape[0]
    _, _, p_half, _ = solver(bem, tri, 1).solve(400.0, np.ones(n))
    full = np.vstack([tri, mirror(tri)])
    _, _, p_full, _ = solver(bem, full, 1, plane=False).solve(400.0, np.ones(2 * n))
    # both are H-matrix approximations (ACA 1e-5) of the same discrete system
    assert rel(p_half[:, 0], p_full[:n, 0]) < 1e-4
    assert rel(p_full[:n, 0], p_full[n:, 0]) < 1e-4  # symmetric image


def test_plane_removal_and_workers(bem, meshes):
    tri = body(meshes, 2)
    n = tri.shape[0]
    g = np.ones(n)
    s = solver(bem, tri, 1, sweep_workers=2)
    _, _, p1, _ = s.solve(300.0, g)
    s.set_impedance_plane()  # removed
    _, _, p0, _ = s.solve(300.0, g)
    _, _, pf, _ = solver(bem, tri, 1, plane=False).solve(300.0, g)
    assert np.array_equal(p0, pf)
    s.set_impedance_plane(POINT, NORMAL)
    _, _, p1b, _ = s.solve(300.0, g)
    assert np.array_equal(p1, p1b)
    # concurrent sweep workers get the plane too
    P, info = s.sweep(np.array([300.0, 450.0]), g)
    assert np.array_equal(P[:, :, 0], p1)
    _, _, p450, _ = s.solve(450.0, g)
    assert np.array_equal(P[:, :, 1], p450)
    # a new mesh drops the plane
    s.set_mesh(tri)
    s.set_bc(np.zeros(n), np.ones(n))
    _, _, p2, _ = s.solve(300.0, g)
    assert np.array_equal(p2, pf)


def test_half_space_field_vs_oracle(bem, meshes, orc):
    tri = body(meshes)
    n = tri.shape[0]
    s = solver(bem, tri, 1, wave_speed=343.0, density=1.2041)
    phi, dphi, p, _ = s.solve(400.0, np.ones(n))
    rng = np.random.default_rng(8)
    pts = np.column_stack([rng.uniform(-3, 3, 400), rng.uniform(-3, 3, 400),
                           rng.uniform(0.05, 3, 400)])
    pf, pp = s.field(400.0, pts, phi, dphi)
    of, op = orc.field(tri, 400.0, pts, phi, dphi, c=343.0, rho=1.2041, plane=(POINT, NORMAL))
    assert rel(pf, of) < 2e-5 and rel(pp, op) < 2e-5
    # on the plane the reflected terms double the free-space contribution's
    # image: the field differs from the one without the plane
    s.set_impedance_plane()
    pf0, _ = s.field(400.0, pts, phi, dphi)
    assert rel(pf0, pf) > 0.05


@pytest.mark.parametrize("coupling", [0, 2])
def test_point_sources_vs_oracle(bem, meshes, orc, coupling):
    """bem_set_point_sources: rhs = sourceTermVector + phi g with the
    reference's sourceTerm; a box with Robin walls and two sources, alone and
    with a driven face, against the oracle."""
    tri = meshes.box(n_target=1200, seed=4)
    n = tri.shape[0]
    rng = np.random.default_rng(12)
    a = 0.3j * rng.random(n)
    b = np.ones(n, complex)
    g = np.where(rng.random(n) < 0.2, 1.0, 0.0) + 0j
    src = [[0.6, 0.1, 0.2, 1.0 + 0.5j], [-0.4, -0.3, 0.5, 0.7j]]
    s = bem.Solver(aca_tol=1e-5, gmres_tol=1e-10, precision=1, coupling=coupling)
    s.set_mesh(tri)
    s.set_bc(a, b)
    s.set_point_sources(src)
    phi, dphi, p, info = s.solve(700.0, g)
    P = orc.Problem(tri, 32, 2.0)
    P.set_sources(src)
    po, dpo, ppo, st = P.solve(700.0, 343.0, 1.2, coupling, a, b, g, 1e-5, 1e-10,
                               seed=s.config.seed)
    assert rel(phi[:, 0], po[:, 0]) < 2e-5
    s.set_point_sources()
    _, _, p0, _ = s.solve(700.0, g)
    assert rel(p0[:, 0], p[:, 0]) > 1e-2  # the sources matter


def test_rank_reservation_grows(bem, meshes):
    """The reference's ACA doubles its reservation until the tolerance is met
    (hmatrix.cpp:557-563): a handle created with a reservation of 4 ends with
    no capped block and the pressures of the default reservation; a user rank
    cap (acaMaxRank) still limits the ranks."""
    tri = body(meshes)
    n = tri.shape[0]
    g = np.ones(n)
    _, _, p96, i96 = solver(bem, tri, 1).solve(400.0, g)
    s4 = solver(bem, tri, 1, rank_reserve=4)
    _, _, p4, i4 = s4.solve(400.0, g)
    assert i96["capped_blocks"] == 0 and i4["capped_blocks"] == 0
    assert i4["max_rank"] == i96["max_rank"]
    assert rel(p4[:, 0], p96[:, 0]) < 1e-12
    _, _, p4b, _ = s4.solve(400.0, g)  # the grown reservation is kept
    assert np.array_equal(p4b, p4)
    # a user rank cap (acaMaxRank) is a limit, not a reservation to grow
    capped = solver(bem, tri, 1, rank_reserve=4, aca_max_rank=4)
    _, _, pc, ic = capped.solve(400.0, g)
    assert ic["max_rank"] <= 4 and rel(pc[:, 0], p96[:, 0]) > 1e-6
