"""CPU checks of the quadrature-order selector's test oracle and data
pipeline: the oracle's analytic gradient against central differences, its
BF16 rounding, the seeded pair generator and the convergence of the labels'
reference rule."""
import importlib

import numpy as np

from oracle import mlp


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = mlp.init(1)
    X = rng.standard_normal((40, mlp.NF))
    y = rng.integers(0, mlp.C, 40)
    g = mlp.grad(p, X, y)
    assert g.shape == (mlp.NPARAM,) == (6085,)
    idx = np.concatenate([rng.choice(mlp.NPARAM, 60, replace=False),
                          np.arange(mlp.NPARAM - 5, mlp.NPARAM)])
    fd = mlp.grad_fd(p, X, y, idx)
    assert np.allclose(g[idx], fd, rtol=1e-5, atol=1e-8)


def test_oracle_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.0e-3, 65504.0], np.float32)
    r = mlp.bf16(x)
    # bf16 keeps 8 significant bits; ties go to even
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.0078125)
    assert np.all(np.abs(r - x) <= np.abs(x) * 2.0 ** -8)


def test_pair_generator_is_seeded_and_covers_the_ranges():
    sd = importlib.import_module("3d_bem_gb300.selector_data")
    P1, Q1, k1, d1 = sd.pairs(3000, seed=7)
    P2, Q2, k2, d2 = sd.pairs(3000, seed=7)
    assert np.array_equal(P1, P2) and np.array_equal(k1, k2)
    assert P1.shape == (3000, 9) and Q1.shape == (3000, 9)
    assert (d1 < 3).mean() > 0.6 and d1.max() < 10 and d1.min() >= 0
    h = np.sqrt(0.5 * np.linalg.norm(np.cross(Q1[:, 3:6] - Q1[:, :3], Q1[:, 6:] - Q1[:, :3]),
                                     axis=1))
    kh = k1 * h
    assert kh.min() >= 0.01 * (1 - 1e-9) and kh.max() <= 1.5 * (1 + 1e-9)
    c = Q1.reshape(-1, 3, 3).mean(1)
    e = np.linalg.norm(Q1[:, 3:6] - Q1[:, :3], axis=1)
    assert np.isfinite(c).all() and (e > 0).all()


def test_label_reference_rule_is_converged(orc):
    """The labels' reference (64-point collapsed Gauss-Legendre product rule on
    an 8- or 4-fold subdivision) agrees with the oracle's 64-point
    Gauss-Jacobi conical rule (order 15) on the same subdivisions, from one
    source size on (closer pairs use the split-polar rule), and with the
    plain 64-point rules on far pairs."""
    from oracle import selector_ref as sr
    sd = importlib.import_module("3d_bem_gb300.selector_data")
    P, Q, k, dh = sd.pairs(400, seed=3)
    a = sr.label_reference(P, Q, k)
    b = np.where((dh < 3)[:, None],
                 sr.ops(P, Q, k, sr.subdivided(orc.triangle_rule(15), 8)),
                 sr.ops(P, Q, k, sr.subdivided(orc.triangle_rule(15), 4)))
    e = sr.rel_err(a, b)
    assert e[dh >= 1].max() < 1e-9
    far = dh > 5
    c = sr.ops(P[far], Q[far], k[far], orc.triangle_rule(15))
    assert sr.rel_err(a[far], c).max() < 1e-8
    rules = {o: orc.triangle_rule(o) for o in sr.CLASS_ORDERS + (sr.PLAIN_ORDER,)}
    err, lab = sr.errors_and_labels(P, Q, k, rules, 1e-7, ref=a)
    # the error falls with the order, and far pairs pass with some rule
    assert np.median(err[:, 0]) > np.median(err[:, 2]) > np.median(err[:, 4])
    assert (lab[dh > 5] <= 4).mean() > 0.99
