"""Mixed precision against the complex-FP64 oracle on an ill-conditioned
body: the pencil (cylinder with a conical tip, Robin impedance walls, Kirkup
coupling, H-LU preconditioned GMRES as BoundaryElementSolver::hMatrixSolve,
boundaryelementsolver.cpp:526-744) with 5,120 triangles.

The pencil amplifies any perturbation of the operator by its conditioning
(~1e2 at low frequency), so it separates the two error sources of the mixed
arm: complex-FP32 storage of the near field (the cancelling hypersingular
entries), which the FP64 near-field residual removes, and the ACA
approximation itself, which both arms share at a given tolerance."""
import os

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu
C0, RHO = 343.0, 1.2


@pytest.fixture(scope="module")
def pencil(meshes):
    tri = meshes.pencil(n_target=5120)
    n = tri.shape[0]
    return tri, meshes.pencil_rhs(tri)[:, :3], meshes.wall_admittance(n)


def gpu_solve(bem, tri, g, beta, freqs, **cfg):
    s = bem.Solver(**{"gmres_tol": 1e-10, "wave_speed": C0, "density": RHO,
                      "use_preconditioner": 1, "precond_rank": 2, "gmres_maxit": 1000,
                      "sweep_workers": 1, **cfg})
    s.set_mesh(tri)
    s.set_bc_impedance(beta)
    out = [s.solve(f, g, want=("p",))[2] for f in freqs]
    s.close()
    return out


def oracle_solve(orc, tri, g, beta, freqs, aca, gmres_tol):
    n = tri.shape[0]
    P = orc.Problem(tri, 32, 2.0)
    out = []
    for f in freqs:
        k = 2 * np.pi * f / C0
        out.append(P.solve(f, C0, RHO, 2, 1j * k * beta, np.ones(n), g, aca, gmres_tol,
                           nthreads=os.cpu_count() or 1, precond_rank=2, maxit=2000)[2])
    return out


def err(p, q):
    return max(rel(p[:, r], q[:, r]) for r in range(q.shape[1]))


def test_mixed_within_1e5_of_converged_fp64_oracle(bem, orc, pencil):
    """Mixed arm (complex-FP32 operator in GMRES, FP64 near field in the
    refinement residual) at ACA 1e-6 against the oracle's FP64 solve at ACA
    1e-7: relative surface-pressure error <= 1e-5 per right-hand side."""
    tri, g, beta = pencil
    freqs = (1000.0, 8000.0)
    mixed = gpu_solve(bem, tri, g, beta, freqs, precision=1, near_fp64=1, aca_tol=1e-6)
    ref = oracle_solve(orc, tri, g, beta, freqs, 1e-7, 1e-12)
    errs = [err(pm, po) for pm, po in zip(mixed, ref)]
    assert max(errs) <= 1e-5, errs


def test_fp64_near_field_removes_the_storage_error(bem, orc, pencil):
    """At the same ACA tolerance (1e-5) the plain complex-FP64 GPU arm equals
    the oracle's solve; the mixed arm differs from it by the ACA
    approximations of its FP32 entries, and at 200 Hz by the complex-FP32
    rounding of the near field, which the FP64 near-field residual removes."""
    tri, g, beta = pencil
    freqs = (200.0,)
    plain = gpu_solve(bem, tri, g, beta, freqs, precision=0, aca_tol=1e-5)
    ref = oracle_solve(orc, tri, g, beta, freqs, 1e-5, 1e-10)
    assert err(plain[0], ref[0]) < 1e-7
    m32 = gpu_solve(bem, tri, g, beta, freqs, precision=1, aca_tol=1e-5)
    m64 = gpu_solve(bem, tri, g, beta, freqs, precision=1, near_fp64=1, aca_tol=1e-5)
    e32, e64 = err(m32[0], ref[0]), err(m64[0], ref[0])
    assert e64 < 0.6 * e32, (e32, e64)
    assert e64 < 1e-4, (e32, e64)


def test_near_fp64_ignored_in_fp64_mode(bem, pencil):
    """near_fp64 only changes the mixed arm: the complex-FP64 arm already
    holds its near field in FP64 and gives the same pressures bitwise."""
    tri, g, beta = pencil
    a = gpu_solve(bem, tri, g[:, :1], beta, (1000.0,), precision=0, aca_tol=1e-4)
    b = gpu_solve(bem, tri, g[:, :1], beta, (1000.0,), precision=0, aca_tol=1e-4, near_fp64=1)
    assert np.array_equal(a[0], b[0])
