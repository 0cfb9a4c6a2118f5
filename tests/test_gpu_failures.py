"""Failure paths of the solve, made on the host without faulting the GPU: an
iteration cap GMRES reaches (BEM_EMAXIT, the reference's GMRES stops at its
maximum iteration count, HMatrix/gmres.h:204-205), a device allocation that
fails (BEM_ENOMEM, through the library's allocation cap standing in for a
failing cudaMalloc), and ACA blocks whose residual vanishes after the first
step (the tiny-pivot break of BlockCluster::partialPivotACA, hmatrix.cpp:
524-545). After each failure the handle stays usable."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, rel

pytestmark = pytest.mark.gpu


def test_gmres_iteration_cap(bem, meshes):
    tri = meshes.icosphere(3, 1.0)
    n = tri.shape[0]
    s = bem.Solver(aca_tol=1e-6, gmres_tol=1e-12, gmres_maxit=2)
    s.set_mesh(tri)
    s.set_bc(np.zeros(n), np.ones(n))
    phi, _, p, info = s.solve(300.0, np.ones(n))
    assert info["status"] == bem.BEM_EMAXIT
    assert info["iterations"] <= 2 and np.isfinite(p).all()
    # the same handle solves again (and stops at the cap again)
    _, _, p2, info2 = s.solve(310.0, np.ones(n))
    assert info2["status"] == bem.BEM_EMAXIT and np.isfinite(p2).all()
    s.close()


def test_allocation_failure_reports_enomem():
    """A child process with a 64 MB cap on the library's device allocations:
    assembling the 5,120-triangle sphere needs more, the call returns
    BEM_ENOMEM, and a smaller mesh on a fresh handle still solves."""
    code = r'''
import importlib, sys, numpy as np
sys.path.insert(0, sys.argv[1])
bem = importlib.import_module("3d_bem_gb300")
meshes = importlib.import_module("3d_bem_gb300.meshes")
tri = meshes.icosphere(4, 1.0); n = tri.shape[0]
s = bem.Solver(aca_tol=1e-5, gmres_tol=1e-8)
s.set_mesh(tri); s.set_bc(np.zeros(n), np.ones(n))
try:
    s.solve(300.0, np.ones(n))
    print("NO_ERROR")
except bem.BemError as e:
    print("STATUS", e.status)
s.close()
tri = meshes.icosphere(1, 1.0); n = tri.shape[0]
s = bem.Solver(aca_tol=1e-5, gmres_tol=1e-8)
s.set_mesh(tri); s.set_bc(np.zeros(n), np.ones(n))
_, _, p, info = s.solve(300.0, np.ones(n))
print("SMALL", info["status"], bool(np.isfinite(p).all()))
'''
    env = dict(os.environ, BEM_DEVICE_MEM_CAP=str(64 << 20))
    r = subprocess.run([sys.executable, "-c", code, ROOT], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.split("\n")
    assert f"STATUS {2}" in lines, r.stdout  # BEM_ENOMEM
    assert "SMALL 0 True" in lines, r.stdout


def test_aca_vanishing_residual(bem):
    """Column points within 1e-9 of one location: every admissible block has
    numerical rank 4 at most (the point and the first-order terms of the
    three jitter directions), so the next ACA step finds a residual at
    rounding level and stops there (no division by a vanishing pivot); the
    H-matvec equals the dense product."""
    rng = np.random.default_rng(3)
    rows = rng.uniform(-1, 1, (300, 3))
    cols = np.tile(np.array([[5.0, 0.3, -0.2]]), (200, 1)) + 1e-9 * rng.standard_normal((200, 3))
    s = bem.Solver(aca_tol=1e-10, precision=0)
    k = 2.0
    rp, cp = s.points_assemble(rows, cols, k)
    ranks = s.ranks(0)
    info = s.partition()
    far = info[:, 4] == 1
    assert far.any() and ranks[far].max() <= 4
    x = rng.standard_normal(200) + 1j * rng.standard_normal(200)
    y = s.hmatvec(0, x)
    R = rows[rp][:, None, :] - cols[cp][None, :, :]
    r = np.linalg.norm(R, axis=2)
    D = np.exp(1j * k * r) / (4 * np.pi * r)
    assert rel(y, D @ x) < 1e-9
    s.close()
