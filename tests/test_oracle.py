"""CPU tests of the oracle: it is pinned against independent known answers
before it is trusted as the checker of the GPU kernels."""
import os

import numpy as np
import pytest

from conftest import rel

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "operators.npz")


def test_triangle_rules_exact_for_polynomials(orc):
    # Dunavant degree-8 rule (16 pts): exact for x^a y^b, a + b <= 8, on the
    # reference triangle (area 1/2): int x^a y^b = a! b! / (a + b + 2)!
    from math import factorial
    for order, deg in [(1, 1), (2, 2), (5, 5), (7, 7), (8, 8), (10, 10), (15, 14)]:
        r = orc.triangle_rule(order)
        assert abs(r[:, 2].sum() - 1.0) < 1e-12, order
        for a in range(deg + 1):
            for b in range(deg + 1 - a):
                exact = factorial(a) * factorial(b) / factorial(a + b + 2)
                approx = 0.5 * np.sum(r[:, 2] * r[:, 0] ** a * r[:, 1] ** b)
                assert abs(approx - exact) < 2e-12 + 1e-9 * exact, (order, a, b)


def test_line_rules(orc):
    for n in (1, 2, 3, 4, 5, 32):
        r = orc.line_rule(n)
        x, w = np.polynomial.legendre.leggauss(n)
        assert np.allclose(r[:, 0], x, atol=1e-15) and np.allclose(r[:, 1], w, atol=1e-15)


def test_operators_against_golden(orc):
    z = np.load(GOLDEN)
    P = orc.Problem(z["tri"], 32, 2.0)
    inv = np.argsort(P.perm)
    pairs, kinds = z["pairs"], z["kinds"]
    for a, k in enumerate(z["ks"]):
        ops = P.operators(k, inv[pairs[:, 0]], inv[pairs[:, 1]])
        ref = z["vals"][a]
        scale = np.abs(ref).max(axis=0)
        reg = kinds == 0
        # 16-point rule at distance >= 4 * averageTriangleDim
        assert (np.abs(ops[reg] - ref[reg]) / scale).max() < 1e-6
        # the reference's 5 x 5 split-polar rule on adjacent panels
        assert (np.abs(ops[~reg] - ref[~reg]) / scale).max() < 5e-2
    idx = z["self_idx"]
    ops = P.operators(1e-5, inv[idx], inv[idx])
    assert np.abs(ops[:, 0].real - z["self_laplace"]).max() < 1e-9
    assert np.all(ops[:, 1] == 0) and np.all(ops[:, 2] == 0)  # flat panel: M = Mt = 0


def test_pulsating_sphere_analytic(orc, meshes):
    """Uniform normal velocity on a sphere: p = rho c v ika / (ika - 1)."""
    tri = meshes.icosphere(3, 1.0)
    P = orc.Problem(tri, 32, 2.0)
    n = P.n
    f, c, rho = 200.0, 343.0, 1.2
    k = 2 * np.pi * f / c
    a, b, g = np.zeros(n), np.ones(n), np.ones(n)
    phi, dphi, p, st = P.solve(f, c, rho, 2, a, b, g, 1e-4, 1e-8)
    pa = rho * c * (1j * k) / (1j * k - 1)
    assert st["rel_resid"] < 1e-8
    assert np.abs(p[:, 0] - pa).max() / abs(pa) < 0.03  # O(h^2) discretisation error
    assert np.allclose(dphi[:, 0], 1.0)


def test_hmatrix_vs_dense_solution(orc, meshes):
    tri = meshes.icosphere(3, 1.0)
    P = orc.Problem(tri, 32, 2.0)
    n = P.n
    f, c, rho = 200.0, 343.0, 1.2
    k = 2 * np.pi * f / c
    a, b, g = np.zeros(n), np.ones(n), np.ones(n)
    perm = P.perm
    Dphi, Ddphi = P.dense(k, 2, a[perm], b[perm])
    x = np.linalg.solve(Ddphi, Dphi @ g[perm])
    pd = np.zeros(n, complex)
    pd[perm] = 1j * rho * 2 * np.pi * f * x
    for tol in (1e-4, 1e-6):
        _, _, p, st = P.solve(f, c, rho, 2, a, b, g, tol, 1e-3 * tol)
        assert rel(p[:, 0], pd) < 20 * tol


def test_point_cloud_aca_reference_design(orc):
    """Tests/tests.cpp:27-43 design: 300 random points, k = 150, tol 1e-3."""
    rng = np.random.default_rng(7)
    X = rng.uniform(-1, 1, (300, 3))
    Y = rng.uniform(-1, 1, (300, 3))
    H, rp, cp = orc.hassemble_points(X, Y, 150.0, 32, 3.0, 1e-3)
    Xs, Ys = X[rp], Y[cp]
    d = np.linalg.norm(Xs[:, None] - Ys[None], axis=2)
    with np.errstate(divide="ignore", invalid="ignore"):
        A = np.where(d == 0, 1.0, np.exp(1j * 150 * d) / (4 * np.pi * d))
    D = H.dense()
    assert rel(D, A) < 2e-3
    x = rng.standard_normal(300) + 1j * rng.standard_normal(300)
    tiny = 10 * np.finfo(float).eps
    assert rel(H.matvec(x), D @ x) < tiny * 10


def test_recompression_truncates(orc, meshes):
    tri = meshes.icosphere(3, 1.0)
    P = orc.Problem(tri, 32, 2.0)
    n = P.n
    k = 2 * np.pi * 200 / 343
    a, b = np.zeros(n), np.ones(n)
    H = P.hassemble(k, 2, a, b, 1, 1e-6)
    D0 = H.dense()
    r0 = H.ranks()
    H.recompress(0, 1e-4)
    r1 = H.ranks()
    assert np.all(r1[r0 >= 0] <= r0[r0 >= 0])
    assert rel(H.dense(), D0) < 1e-3
    H.recompress(2, 0.0)
    assert r1.max() >= 2 and H.ranks().max() <= 2


def _random_block_triangular(n, leaf, rng, lower):
    """Flat leaf lists of a random block-triangular matrix on a binary
    cluster split (diag leaves Q (unitary) or R (upper), off-diagonal full or
    low-rank), plus its dense form."""
    blocks, data = [], []
    D = np.zeros((n, n), complex)

    def add(r0, m, c0, nn, kind, arr):
        off = sum(x.size for x in data)
        rank = 0
        if kind == 1:
            U, V = arr
            rank = U.shape[1]
            data.append(np.asfortranarray(U).ravel(order="F"))
            data.append(np.ascontiguousarray(V).ravel())
            D[r0:r0 + m, c0:c0 + nn] = U @ V
        else:
            data.append(np.asfortranarray(arr).ravel(order="F"))
            D[r0:r0 + m, c0:c0 + nn] = arr
        blocks.append([r0, m, c0, nn, kind, rank, off])

    def rec(s, m):
        if m <= leaf:
            A = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
            Q, R = np.linalg.qr(A + 4 * np.eye(m))
            add(s, m, s, m, 2 if lower else 3, Q if lower else R)
            return
        m1 = m // 2
        m2 = m - m1
        rec(s, m1)
        rec(s + m1, m2)
        if lower:
            r0, mm, c0, nn = s + m1, m2, s, m1
        else:
            r0, mm, c0, nn = s, m1, s + m1, m2
        if rng.random() < 0.5:
            add(r0, mm, c0, nn, 0, 0.1 * (rng.standard_normal((mm, nn)) + 1j * rng.standard_normal((mm, nn))))
        else:
            kk = 3
            add(r0, mm, c0, nn, 1, (0.1 * rng.standard_normal((mm, kk)) + 0j,
                                    rng.standard_normal((kk, nn)) + 0j))

    rec(0, n)
    return np.array(blocks, np.int64), np.concatenate(data), D


def test_block_triangular_solves(orc):
    rng = np.random.default_rng(3)
    n = 150
    Lb, Ld, LD = _random_block_triangular(n, 20, rng, True)
    Ub, Ud, UD = _random_block_triangular(n, 20, rng, False)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    # L is block lower triangular with unitary diagonal blocks Q: the leaf
    # solve applies Q^H (harithm.cpp:1324-1327)
    diagQ = np.zeros((n, n), complex)
    for r0, m, c0, nn, kind, rank, off in Lb:
        if kind == 2:
            diagQ[r0:r0 + m, c0:c0 + nn] = LD[r0:r0 + m, c0:c0 + nn]
    y = orc.lower_solve(n, Lb, Ld, b)
    assert rel(LD @ y, b) < 1e-12
    x = orc.upper_solve(n, Ub, Ud, y)
    assert rel(UD @ x, y) < 1e-12


def _monopole_data(tri, k):
    """Boundary data of a unit monopole at the origin: phi and dphi/dn at the
    element centroids (normals from the node order, as the reference)."""
    c = (tri[:, 0:3] + tri[:, 3:6] + tri[:, 6:9]) / 3.0
    nrm = np.cross(tri[:, 3:6] - tri[:, 0:3], tri[:, 6:9] - tri[:, 0:3])
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    r = np.linalg.norm(c, axis=1)
    phi = np.exp(1j * k * r) / (4 * np.pi * r)
    dphi = phi * (1j * k - 1 / r) * np.sum(nrm * c, 1) / r
    return phi, dphi


def test_field_reproduces_monopole(orc, meshes):
    """Kirchhoff-Helmholtz representation (calculateFieldSolutionRegular):
    exterior monopole data give the monopole outside the surface (O(h^2)
    faceting error) and zero inside."""
    tri = meshes.icosphere(3, 0.5)
    f = 400.0
    k = 2 * np.pi * f / 343.0
    phi, dphi = _monopole_data(tri, k)
    out = np.array([[1.0, 0, 0], [0, 1.5, 0.3], [2, 2, 2], [-0.4, 0.7, -0.9]])
    inside = np.array([[0.1, 0.05, 0.0], [0.0, -0.2, 0.1]])
    pf, pp = orc.field(tri, f, np.vstack([out, inside]), phi, dphi)
    r = np.linalg.norm(out, axis=1)
    ex = np.exp(1j * k * r) / (4 * np.pi * r)
    assert (np.abs(pf[:4, 0] - ex) / np.abs(ex)).max() < 0.01
    assert np.abs(pf[4:, 0]).max() < 0.01 * np.abs(ex).max()
    # sound pressure i rho 2 pi f phi (calculateFieldSolution :2236-2243)
    assert np.allclose(pp, 1j * 1.2041 * 2 * np.pi * f * pf, rtol=1e-14, atol=0)


def test_field_point_sources(orc, meshes):
    """sourcePhiTerm: with zero boundary data the field is the point sources'
    w exp(ikr) / (4 pi r), summed; at f = 0 the pressure factor is 2 pi."""
    tri = meshes.icosphere(1, 0.5)
    n = tri.shape[0]
    pts = np.array([[1.0, 0.2, 0.0], [0.3, -2.0, 0.5]])
    src = [[0, 0, 0, 1.0], [0.1, 0.2, -0.1, 0.5 - 2j]]
    for f in (250.0, 0.0):
        k = 2 * np.pi * f / 343.0
        pf, pp = orc.field(tri, f, pts, np.zeros(n), np.zeros(n), sources=src)
        ex = 0
        for s in src:
            r = np.linalg.norm(pts - np.array(s[:3]).real, axis=1)
            ex = ex + s[3] * np.exp(1j * k * r) / (4 * np.pi * r)
        assert rel(pf[:, 0], ex) < 1e-14
        fac = 2 * np.pi * (f if f else 1.0)
        assert np.allclose(pp[:, 0], 1j * 1.2041 * fac * pf[:, 0], rtol=1e-14, atol=0)


def test_field_matches_vectorised_restatement(orc, meshes):
    """The oracle's loop against an independent numpy evaluation of the same
    sum (7-point rule of order 5, BemOperatorField :2318-2353), two columns."""
    tri = meshes.icosphere(1, 0.7)
    n = tri.shape[0]
    rng = np.random.default_rng(5)
    phi = rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2))
    dphi = rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2))
    pts = rng.uniform(-2, 2, (7, 3))
    f = 700.0
    k = 2 * np.pi * f / 343.0
    pf, _ = orc.field(tri, f, pts, phi, dphi)
    rule = orc.triangle_rule(5)
    assert rule.shape == (7, 3)
    n1, n2, n3 = tri[:, 0:3], tri[:, 3:6], tri[:, 6:9]
    cr = np.cross(n2 - n1, n3 - n1)
    area = np.linalg.norm(cr, axis=1) / 2
    nq = cr / np.linalg.norm(cr, axis=1)[:, None]
    q = (rule[:, 0, None, None] * n1 + rule[:, 1, None, None] * n2
         + (1 - rule[:, 0] - rule[:, 1])[:, None, None] * n3)      # 7 x n x 3
    rv = pts[:, None, None, :] - q[None]                           # P x 7 x n x 3
    r = np.linalg.norm(rv, axis=-1)
    G = np.exp(1j * k * r) / (4 * np.pi * r)
    rnq = -np.sum(rv * nq[None, None], -1) / r
    w = rule[:, 2][None, :, None]
    Lk = (w * G).sum(1) * area
    Mk = (w * G / r * (1j * k * r - 1) * rnq).sum(1) * area
    ref = Mk @ phi - Lk @ dphi
    assert rel(pf, ref) < 1e-13


def test_field_pulsating_sphere(orc, meshes):
    """Solve then field: p(r) = p(a) (a / r) exp(ik(r - a)) outside a sphere
    with uniform normal velocity."""
    a = 1.0
    tri = meshes.icosphere(3, a)
    P = orc.Problem(tri, 32, 2.0)
    n = P.n
    f, c, rho = 200.0, 343.0, 1.2
    k = 2 * np.pi * f / c
    phi, dphi, p, st = P.solve(f, c, rho, 2, np.zeros(n), np.ones(n), np.ones(n), 1e-4, 1e-8)
    r = np.array([1.5, 2.0, 4.0])
    pts = np.column_stack([r * 0.6, r * 0.0, r * 0.8])
    _, pp = orc.field(tri, f, pts, phi[:, 0], dphi[:, 0], c=c, rho=rho)
    pa = rho * c * (1j * k * a) / (1j * k * a - 1)
    ex = pa * (a / r) * np.exp(1j * k * (r - a))
    assert np.abs(pp[:, 0] - ex).max() / abs(pa) < 0.03


def _mirror(tri, point, normal):
    """MeshFunctions::reflectTriangles: mirrored nodes, node 1 and node 3 swapped."""
    nrm = np.asarray(normal, float) / np.linalg.norm(normal)
    d = -nrm @ np.asarray(point, float)
    R = lambda x: x - 2.0 * (x @ nrm + d)[:, None] * nrm
    return np.hstack([R(tri[:, 6:9]), R(tri[:, 3:6]), R(tri[:, 0:3])])


def _caller(D, perm):
    out = np.empty_like(D)
    out[np.ix_(perm, perm)] = D
    return out


def test_half_space_equals_mirrored_full_space(orc, meshes):
    """One impedance plane (implicitPhiMatrixPlusReflected): the half-space
    matrices equal the free-space matrices of the body plus its mirror image,
    folded onto the body's elements (mirror far enough that no mirrored pair
    is near-singular, so both use the regular rule)."""
    tri = meshes.icosphere(2, 0.5)
    tri[:, 2::3] += 0.9
    n = tri.shape[0]
    point, normal = [0.0, 0.0, 0.0], [0.0, 0.0, 2.0]
    full = np.vstack([tri, _mirror(tri, point, normal)])
    rng = np.random.default_rng(2)
    a = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    k = 2 * np.pi * 300.0 / 343.0
    P = orc.Problem(tri)
    P.set_plane(point, normal)
    F = orc.Problem(full)
    hp, hd = P.dense(k, 2, a[P.perm], b[P.perm])
    a2, b2 = np.concatenate([a, a]), np.concatenate([b, b])
    fp, fd = F.dense(k, 2, a2[F.perm], b2[F.perm])
    for H, Fm in ((hp, fp), (hd, fd)):
        Hc, Fc = _caller(H, P.perm), _caller(Fm, F.perm)
        assert rel(Hc, Fc[:n, :n] + Fc[:n, n:]) < 1e-13
    # removing the plane gives the free-space matrices back
    P.set_plane()
    fp1, _ = orc.Problem(tri).dense(k, 2, a[P.perm], b[P.perm])
    hp1, _ = P.dense(k, 2, a[P.perm], b[P.perm])
    assert np.array_equal(hp1, fp1)


def test_half_space_field_equals_mirrored_data(orc, meshes):
    tri = meshes.icosphere(1, 0.5)
    tri[:, 2::3] += 0.8
    n = tri.shape[0]
    rng = np.random.default_rng(6)
    phi = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    dphi = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    pts = np.column_stack([rng.uniform(-2, 2, 9), rng.uniform(-2, 2, 9), rng.uniform(0.1, 3, 9)])
    plane = ([0.0, 0.0, 0.0], [0.0, 0.0, 1.0])
    f_half, _ = orc.field(tri, 500.0, pts, phi, dphi, plane=plane)
    full = np.vstack([tri, _mirror(tri, *plane)])
    f_full, _ = orc.field(full, 500.0, pts, np.concatenate([phi, phi]),
                          np.concatenate([dphi, dphi]))
    assert rel(f_half, f_full) < 1e-13


def test_point_source_rhs_kelvin_image(orc, meshes):
    """rhs = sourceTermVector + phi g (boundaryelementsolver.cpp:578-579): a
    unit point source at distance 2 from a sound-soft unit sphere (phi = 0,
    a = 1, b = 0, g = 0) at 1 Hz is the Laplace problem whose exact normal
    derivative comes from the Kelvin image (-a/d at a^2/d). Without coupling
    the source term is the plain Green's function; flat-panel discretisation
    error ~1 %."""
    tri = meshes.icosphere(4, 1.0)
    n = tri.shape[0]
    c = (tri[:, 0:3] + tri[:, 3:6] + tri[:, 6:9]) / 3
    nrm = np.cross(tri[:, 3:6] - tri[:, 0:3], tri[:, 6:9] - tri[:, 0:3])
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]

    def grad(y, w):
        r = c - y
        return -w * r / (4 * np.pi * np.linalg.norm(r, axis=1)[:, None] ** 3)

    exact = np.sum((grad(np.array([0, 0, 2.0]), 1.0) + grad(np.array([0, 0, 0.5]), -0.5)) * nrm, 1)
    P = orc.Problem(tri, 32, 2.0)
    P.set_sources([[0, 0, 2.0, 1.0]])
    phi, dphi, p, st = P.solve(1.0, 343.0, 1.2, 0, np.ones(n), np.zeros(n), np.zeros(n),
                               1e-6, 1e-10)
    assert np.abs(phi).max() == 0.0
    assert rel(dphi[:, 0], exact) < 0.02
    # clearing the sources gives the zero solution back
    P.set_sources()
    _, dphi0, _, _ = P.solve(1.0, 343.0, 1.2, 0, np.ones(n), np.zeros(n), np.zeros(n), 1e-6, 1e-10)
    assert np.abs(dphi0).max() == 0.0
