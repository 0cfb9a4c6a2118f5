"""Truncating SVD recompression on the GPU (BlockCluster::compressAdmissibleBlock,
HMatrix/hmatrix.cpp:101-140) against the oracle's restatement applied to the
oracle's own ACA blocks (identical pivots, so the same input blocks)."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu
FREQ = 200.0


def setup(bem, meshes, sub=3, **cfg):
    tri = meshes.icosphere(sub, 1.0)
    s = bem.Solver(**{"aca_tol": 1e-6, "gmres_tol": 1e-9, **cfg})
    s.set_mesh(tri)
    n = tri.shape[0]
    s.set_bc(np.zeros(n), np.ones(n))
    return tri, s


def block_errors(info, D1, D2):
    out = []
    for r0, m, c0, n, adm in info:
        if adm:
            A = D1[r0:r0 + m, c0:c0 + n]
            B = D2[r0:r0 + m, c0:c0 + n]
            out.append(np.linalg.norm(A - B) / max(np.linalg.norm(B), 1e-300))
    return np.array(out)


@pytest.mark.parametrize("tol", [1e-3, 1e-5])
def test_recompress_vs_oracle(bem, meshes, orc, tol):
    tri, s = setup(bem, meshes)
    n = tri.shape[0]
    k = 2 * np.pi * FREQ / 343
    a, b = np.zeros(n), np.ones(n)
    P = orc.Problem(tri, 32, 2.0)
    s.assemble(FREQ)
    info = s.partition()
    adm = info[:, 4] == 1
    for which in (0, 1):
        H = P.hassemble(k, 2, a, b, which, 1e-6, seed=s.config.seed)
        D0, H0 = s.dense(which, info), H.dense()
        r0, ro0 = s.ranks(which), H.ranks()
        e0 = block_errors(info, D0, H0)  # ACA inputs: equal pivots -> ~1e-15
        s.recompress(which, 0, tol)
        H.recompress(0, tol)
        rg, ro = s.ranks(which), H.ranks()
        assert np.all(rg[adm] <= r0[adm]) and np.all(rg[adm] >= np.minimum(r0[adm], 1))
        assert rg[adm].sum() < r0[adm].sum()
        # the same smallest ranks, up to blocks whose singular value sits on the cut
        assert np.mean(rg[adm] == ro[adm]) > 0.97
        assert np.all(np.abs(rg[adm] - ro[adm]) <= 1)
        D1 = s.dense(which, info)
        # every block keeps its relative Frobenius tail below tol
        assert block_errors(info, D1, D0).max() < 1.01 * tol
        # blocks whose ACA inputs agree and whose truncated ranks agree: the
        # same best approximation as the oracle's; the others differ by about
        # their ACA inputs' difference
        eq = ((rg == ro) & (r0 == ro0))[adm] & (e0 < 1e-12)
        assert eq.mean() > 0.9
        e = block_errors(info, D1, H.dense())
        assert e[eq].max() < 1e-8
        assert e.max() < 1e-5


def test_recompress_rank_cap_and_noop(bem, meshes):
    tri, s = setup(bem, meshes)
    s.assemble(FREQ)
    info = s.partition()
    adm = info[:, 4] == 1
    r0 = s.ranks(1)
    D0 = s.dense(1, info)
    s.recompress(1, 0, 0.0)  # no cap, no tolerance: untouched (hmatrix.cpp:108)
    assert np.array_equal(s.ranks(1), r0)
    assert np.array_equal(s.dense(1, info), D0)
    s.recompress(1, 2, 0.0)
    r = s.ranks(1)
    assert r[adm].max() <= 2 and r0[adm].max() > 2
    # rank-2 truncation is the best rank-2 approximation: error <= ACA-level tail
    e = block_errors(info, s.dense(1, info), D0)
    assert np.isfinite(e).all()
    with pytest.raises(bem.BemError):
        s.recompress(1, -1, 0.1)


def test_recompress_mixed_precision(bem, meshes):
    tri, s = setup(bem, meshes, precision=1, aca_tol=1e-5)
    s.assemble(FREQ)
    info = s.partition()
    adm = info[:, 4] == 1
    r0 = s.ranks(1)
    D0 = s.dense(1, info)
    s.recompress(1, 0, 1e-4)
    r1 = s.ranks(1)
    assert r1[adm].sum() < r0[adm].sum()
    assert block_errors(info, s.dense(1, info), D0).max() < 1.05e-4


@pytest.mark.parametrize("precision", [0, 1])
def test_solve_with_recompression(bem, meshes, precision):
    tri, s0 = setup(bem, meshes, precision=precision, aca_tol=1e-5, gmres_tol=1e-10)
    _, s1 = setup(bem, meshes, precision=precision, aca_tol=1e-5, gmres_tol=1e-10,
                  recompress_tol=1e-5)
    n = tri.shape[0]
    g = np.ones(n, complex)
    _, _, p0, i0 = s0.solve(FREQ, g)
    _, _, p1, i1 = s1.solve(FREQ, g)
    assert i0["status"] == 0 and i1["status"] == 0
    adm = s0.partition()[:, 4] == 1
    assert s1.ranks(1)[adm].sum() < s0.ranks(1)[adm].sum()
    assert rel(p1, p0) < 2e-5
