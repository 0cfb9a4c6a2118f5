"""H-LU preconditioner: the host factorization (HArithm::LUDecomposition,
HMatrix/harithm.cpp:1192-1296) checked against the dense system matrix, the
GPU forward/backward block-triangular solves (harithm.cpp:1314-1340,
:1386-1412) against the oracle's leaf-by-leaf restatement, and the
preconditioned GMRES (GMRES::gmresLUPreconditionedSolve, HMatrix/gmres.h:191-207)
against the unpreconditioned solve."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu
FREQ = 200.0


def setup(bem, meshes, sub=3, precision=0, **cfg):
    tri = meshes.icosphere(sub, 1.0)
    s = bem.Solver(**{"aca_tol": 1e-6, "gmres_tol": 1e-9, "precision": precision, **cfg})
    s.set_mesh(tri)
    n = tri.shape[0]
    s.set_bc(np.zeros(n), np.ones(n))
    return tri, s


def dense_factor(n, leaves, data):
    D = np.zeros((n, n), complex)
    for r0, m, c0, nn, kind, k, off in leaves:
        if kind == 1:
            U = data[off:off + m * k].reshape(k, m).T
            V = data[off + m * k:off + m * k + k * nn].reshape(k, nn)
            D[r0:r0 + m, c0:c0 + nn] = U @ V
        else:
            D[r0:r0 + m, c0:c0 + nn] = data[off:off + m * nn].reshape(nn, m).T
    return D


def check_structure(n, leaves, data, sched, lower):
    # every leaf scheduled once; the diagonal leaves tile the diagonal
    ops = [int(o) if o >= 0 else -int(o) - 1 for o in sched]
    assert sorted(ops) == list(range(len(leaves)))
    diag = leaves[leaves[:, 4] >= 2]
    assert (diag[:, 0] == diag[:, 2]).all() and (diag[:, 1] == diag[:, 3]).all()
    assert diag[:, 1].sum() == n
    assert (diag[:, 4] == (2 if lower else 3)).all()
    off = leaves[leaves[:, 4] < 2]
    if lower:
        assert (off[:, 2] + off[:, 3] <= off[:, 0]).all()
    else:
        assert (off[:, 0] + off[:, 1] <= off[:, 2]).all()
    for r0, m, c0, nn, kind, k, o in diag:
        B = data[o:o + m * m].reshape(m, m).T
        if lower:
            assert np.abs(B.conj().T @ B - np.eye(m)).max() < 1e-12
        else:
            assert np.abs(np.tril(B, -1)).max() == 0


def test_hlu_factors_reproduce_matrix(bem, meshes):
    """Untruncated (rank 0, tolerance 1e-12) factors: L U = A to the truncation."""
    tri, s = setup(bem, meshes, 3, precond_rank=0, precond_tol=1e-12)
    n = tri.shape[0]
    s.assemble(FREQ)
    s.hlu_build()
    Ll, Ld, Ls = s.hlu_export(0)
    Ul, Ud, Us = s.hlu_export(1)
    check_structure(n, Ll, Ld, Ls, True)
    check_structure(n, Ul, Ud, Us, False)
    A = s.dense(1)
    LU = dense_factor(n, Ll, Ld) @ dense_factor(n, Ul, Ud)
    assert np.linalg.norm(LU - A) / np.linalg.norm(A) < 1e-9
    # and the GPU solve inverts it
    rng = np.random.default_rng(5)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    z = s.hlu_solve(s.hmatvec(1, x))
    assert rel(z, x) < 1e-7


@pytest.mark.parametrize("rank", [2, 8])
def test_hlu_solve_vs_oracle(bem, meshes, orc, rank):
    tri, s = setup(bem, meshes, 3, precond_rank=rank)
    n = tri.shape[0]
    s.assemble(FREQ)
    s.hlu_build()
    Ll, Ld, _ = s.hlu_export(0)
    Ul, Ud, _ = s.hlu_export(1)
    assert Ll[Ll[:, 4] == 1, 5].max() <= rank and Ul[Ul[:, 4] == 1, 5].max() <= rank
    rng = np.random.default_rng(rank)
    B = rng.standard_normal((n, 3)) + 1j * rng.standard_normal((n, 3))
    X = s.hlu_solve(B)
    for q in range(3):
        y = orc.lower_solve(n, Ll, Ld, B[:, q])
        x = orc.upper_solve(n, Ul, Ud, y)
        assert rel(X[:, q], x) < 1e-12, q


def test_hlu_solve_edge_cases(bem, meshes):
    tri, s = setup(bem, meshes, 2, precond_rank=2)
    with pytest.raises(bem.BemError):
        s.hlu_solve(np.ones(tri.shape[0]))  # not built
    s.assemble(FREQ)
    with pytest.raises(bem.BemError):
        s.hlu_export(0)
    s.hlu_build()
    n = tri.shape[0]
    assert np.array_equal(s.hlu_solve(np.zeros(n)), np.zeros(n))
    s.assemble(FREQ * 1.5)  # reassembly drops the factors of the old matrix
    with pytest.raises(bem.BemError):
        s.hlu_solve(np.ones(n))


@pytest.mark.parametrize("precision", [0, 1])
def test_preconditioned_solve(bem, meshes, precision):
    tri, s0 = setup(bem, meshes, 3, precision=precision)
    _, s1 = setup(bem, meshes, 3, precision=precision, use_preconditioner=1, precond_rank=2)
    n = tri.shape[0]
    c = tri.reshape(-1, 3, 3).mean(axis=1)
    g = np.stack([np.ones(n), c[:, 2]], axis=1).astype(complex)
    phi0, _, _, i0 = s0.solve(FREQ, g)
    phi1, _, _, i1 = s1.solve(FREQ, g)
    assert i1["status"] == 0 and i0["status"] == 0
    assert i1["t_precond"] > 0
    assert i1["true_residual"] < 1e-8
    assert i1["iterations"] < i0["iterations"], (i0["iterations"], i1["iterations"])
    assert rel(phi1, phi0) < 1e-7


def test_facade_preconditioner(bem, meshes):
    tri = meshes.icosphere(3, 1.0)
    n = tri.shape[0]
    out = []
    for pc in (False, True):
        be = bem.BoundaryElements(tri, np.zeros(n, complex), np.ones(n, complex),
                                  np.ones(n, complex))
        par = bem.BemSolverParameters(acaRelativeError=1e-5, usePreconditioner=pc)
        sol = bem.BoundaryElementSolver(be, FREQ, bemSolverParameters=par)
        sol.calculateBoundarySolution()
        out.append(be.phiSolution)
    assert rel(out[1], out[0]) < 1e-6


def test_hlu_solve_fp32_factors_vs_oracle(bem, meshes, orc):
    """Mixed precision stores the factors in complex FP32 and sweeps in FP32
    arithmetic: the result is the oracle's FP64 solve with the same factors
    to FP32 accuracy."""
    tri, s = setup(bem, meshes, 3, precision=1, precond_rank=2)
    n = tri.shape[0]
    s.assemble(FREQ)
    s.hlu_build()
    Ll, Ld, _ = s.hlu_export(0)
    Ul, Ud, _ = s.hlu_export(1)
    rng = np.random.default_rng(9)
    B = rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2))
    X = s.hlu_solve(B)
    for q in range(2):
        x = orc.upper_solve(n, Ul, Ud, orc.lower_solve(n, Ll, Ld, B[:, q]))
        assert rel(X[:, q], x) < 1e-4, q


def oracle_solve(orc, s, n, B):
    Ll, Ld, _ = s.hlu_export(0)
    Ul, Ud, _ = s.hlu_export(1)
    return np.stack([orc.upper_solve(n, Ul, Ud, orc.lower_solve(n, Ll, Ld, B[:, q]))
                     for q in range(B.shape[1])], axis=1)


def test_dataflow_sweep_many_rhs_and_helpers(bem, meshes, orc, monkeypatch):
    """The dataflow sweep (default for leaf 32, rank <= 32): 11 right-hand
    sides take two launches (8 + 3); the result matches the oracle's
    leaf-by-leaf solve, and is bitwise the same for any number of helper
    blocks (each sum has one fixed order)."""
    tri, s = setup(bem, meshes, 3, precond_rank=4)
    n = tri.shape[0]
    s.assemble(FREQ)
    s.hlu_build()
    assert s.hlu_sweep_kind() == 1
    rng = np.random.default_rng(4)
    B = rng.standard_normal((n, 11)) + 1j * rng.standard_normal((n, 11))
    X = s.hlu_solve(B)
    assert rel(X, oracle_solve(orc, s, n, B)) < 1e-12
    for h in ("1", "3", "150"):
        monkeypatch.setenv("BEM_HLU_HELPERS", h)
        assert np.array_equal(s.hlu_solve(B), X), h


def test_sequential_sweep_for_large_leaves(bem, meshes, orc):
    """Diagonal leaves above 32 rows (leaf_size 64) keep the sequential
    sweep; it matches the oracle too."""
    tri, s = setup(bem, meshes, 3, precond_rank=2, leaf_size=64)
    n = tri.shape[0]
    s.assemble(FREQ)
    s.hlu_build()
    assert s.hlu_sweep_kind() == 0
    rng = np.random.default_rng(6)
    B = rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2))
    assert rel(s.hlu_solve(B), oracle_solve(orc, s, n, B)) < 1e-12


def test_factor_reuse_over_a_sweep(bem, meshes):
    """precond_reuse = 1.3: a sweep keeps the H-LU factors while the frequency
    stays within 1.3x of the one they were built at, and rebuilds them past
    it; every pressure is the solution of its own matrix (GMRES on
    (LU)^-1 A x = (LU)^-1 b with the residual of the current A)."""
    tri = meshes.icosphere(3, 1.0)
    n = tri.shape[0]
    freqs = np.array([200.0, 220.0, 250.0, 270.0, 300.0])
    g = np.ones(n)
    out = {}
    for reuse in (0.0, 1.3):
        s = bem.Solver(aca_tol=1e-6, gmres_tol=1e-10, precision=1, use_preconditioner=1,
                       precond_rank=2, precond_reuse=reuse, sweep_workers=1)
        s.set_mesh(tri)
        s.set_bc(np.zeros(n), np.ones(n))
        out[reuse] = s.sweep(freqs, g)
        s.close()
    (p0, i0), (p1, i1) = out[0.0], out[1.3]
    assert [i["precond_reused"] for i in i0] == [0, 0, 0, 0, 0]
    assert [i["precond_reused"] for i in i1] == [0, 1, 1, 0, 1]
    assert all(i["status"] == 0 and i["true_residual"] < 1e-9 for i in i0 + i1)
    assert rel(p1, p0) < 1e-7



# ---- H-LU factorization on the GPU (task program, hlu_gpu.h) ----

@pytest.mark.parametrize("precision", [0, 1])
def test_device_factors_match_host_and_oracle(bem, meshes, orc, precision):
    """Rank-2 factors from the GPU task program against the host
    factorization of the same matrix and the oracle's restatement
    (HArithm::LUDecomposition, harithm.cpp:1192-1296) of the oracle's own
    assembly: the three approximate A equally well and differ by less than
    the truncation error."""
    tri = meshes.icosphere(3, 1.0)
    n = tri.shape[0]
    prods, errs = {}, {}
    for dev in (1, 0):
        _, s = setup(bem, meshes, 3, precision=precision, precond_rank=2, hlu_device=dev)
        s.assemble(FREQ)
        s.hlu_build()
        Ll, Ld, Ls = s.hlu_export(0)
        Ul, Ud, Us = s.hlu_export(1)
        if precision == 0:  # Q unitary to FP64 rounding
            check_structure(n, Ll, Ld, Ls, True)
            check_structure(n, Ul, Ud, Us, False)
        A = s.dense(1)
        prods[dev] = dense_factor(n, Ll, Ld) @ dense_factor(n, Ul, Ud)
        errs[dev] = rel(prods[dev], A)
        s.close()
    P = orc.Problem(tri, 32, 2.0)
    k = 2 * np.pi * FREQ / 343.0
    H = P.hassemble(k, 2, np.zeros(n), np.ones(n), 1, 1e-6)
    Ll, Ld, Ul, Ud = P.hlu(H, 2)
    Ao = H.dense()
    LUo = dense_factor(n, Ll, Ld) @ dense_factor(n, Ul, Ud)
    err_o = rel(LUo, Ao)
    for e in (errs[0], errs[1], err_o):
        assert 1e-4 < e < 5e-3, (errs, err_o)
    assert errs[1] < 1.1 * errs[0] and errs[1] < 1.1 * err_o
    assert rel(prods[1], prods[0]) < 1e-3
    # the oracle's cluster order is the library's (same tree), so the
    # factor products compare entry by entry
    assert rel(prods[1], LUo) < 1e-3


@pytest.mark.parametrize("sub", [2, 3])
def test_device_factors_exact_at_full_rank(bem, meshes, orc, sub):
    """At rank 64 with a 1e-14 truncation the GPU factors reproduce the
    matrix (L U = A to 1e-9), as the oracle's do."""
    tri, s = setup(bem, meshes, sub, precond_rank=64, precond_tol=1e-14)
    n = tri.shape[0]
    s.assemble(FREQ)
    s.hlu_build()
    Ll, Ld, Ls = s.hlu_export(0)
    Ul, Ud, Us = s.hlu_export(1)
    check_structure(n, Ll, Ld, Ls, True)
    check_structure(n, Ul, Ud, Us, False)
    A = s.dense(1)
    assert rel(dense_factor(n, Ll, Ld) @ dense_factor(n, Ul, Ud), A) < 1e-9
    rng = np.random.default_rng(sub)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    assert rel(s.hlu_solve(s.hmatvec(1, x)), x) < 1e-7


def test_device_factorization_wait_limit(bem, meshes, monkeypatch):
    """A dependency wait of the factorization kernel that runs out (a limit
    of a few nanoseconds, which the dependencies cannot meet) ends the launch
    with BEM_ETIMEOUT; no task is left running and the handle stays usable."""
    tri, s = setup(bem, meshes, 3, precond_rank=2)
    s.assemble(FREQ)
    monkeypatch.setenv("BEM_HLU_WAIT_US", "0.001")
    with pytest.raises(bem.BemError) as ei:
        s.hlu_build()
    assert ei.value.status == bem.BEM_ETIMEOUT
    monkeypatch.delenv("BEM_HLU_WAIT_US")
    s.hlu_build()
    n = tri.shape[0]
    rng = np.random.default_rng(2)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    assert rel(s.hlu_solve(s.hmatvec(1, x)), x) < 1e-2


def test_dataflow_sweep_wait_limit(bem, meshes, monkeypatch):
    """A wait of the dataflow sweep that runs out (a limit of a nanosecond,
    which no dependency can meet) ends the launch: every block gives up and
    returns, the call reports BEM_ETIMEOUT, and with the normal limit the same
    handle gives the same solution as before, bitwise."""
    tri, s = setup(bem, meshes, 3, precond_rank=2)
    n = tri.shape[0]
    s.assemble(FREQ)
    s.hlu_build()
    assert s.hlu_sweep_kind() == 1
    rng = np.random.default_rng(5)
    B = rng.standard_normal((n, 3)) + 1j * rng.standard_normal((n, 3))
    X = s.hlu_solve(B)
    monkeypatch.setenv("BEM_DF_WAIT_US", "0.001")
    with pytest.raises(bem.BemError) as ei:
        s.hlu_solve(B)
    assert ei.value.status == bem.BEM_ETIMEOUT
    monkeypatch.delenv("BEM_DF_WAIT_US")
    assert np.array_equal(s.hlu_solve(B), X)
