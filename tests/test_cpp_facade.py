"""The C++ facade (include/bemgpu.hpp: BoundaryElementSolver, HMatrix,
HArithm::MVM / LUDecomposition / LUSubstitutionSolve, GMRES::gmresSolve, the
names of the reference's call surface) compiles against the public headers,
links libbemgpu.so and gives the results of the Python path: host-only
planning here, a full solve on the GPU."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "facade_check.cpp")


@pytest.fixture(scope="module")
def facade_bin(bem, tmp_path_factory):
    lib = bem.build()
    out = str(tmp_path_factory.mktemp("facade") / "facade_check")
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           SRC, "-o", out, "-L", libdir, "-lbemgpu", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def run(binary, mode, tri, tmp_path):
    path = str(tmp_path / "tri.bin")
    np.ascontiguousarray(tri, np.float64).tofile(path)
    r = subprocess.run([binary, mode, path], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    vals = {}
    for line in r.stdout.strip().split("\n"):
        toks = line.split()
        for i in range(0, len(toks) - 1, 2):
            vals[toks[i]] = toks[i + 1]
    return r.stdout, vals


def test_facade_plan_matches_python(bem, meshes, facade_bin, tmp_path):
    tri = meshes.icosphere(3)
    out, vals = run(facade_bin, "plan", tri, tmp_path)
    perm, info = bem.plan_mesh(tri, bem.default_config(leaf_size=32, eta=2.0))
    assert int(vals["n"]) == tri.shape[0]
    assert int(vals["blocks"]) == info.shape[0]
    assert int(vals["perm_checksum"]) == int(((np.arange(len(perm)) + 1) * perm).sum())


@pytest.mark.gpu
@pytest.mark.parametrize("precond", [False, True])
def test_facade_solve_matches_python(bem, meshes, facade_bin, tmp_path, precond):
    tri = meshes.icosphere(2)
    n = tri.shape[0]
    out, vals = run(facade_bin, "solve_precond" if precond else "solve", tri, tmp_path)
    assert int(vals["status"]) == 0, out
    s = bem.Solver(leaf_size=32, eta=2.0, aca_tol=1e-6, gmres_tol=1e-10,
                   use_preconditioner=int(precond), wave_speed=343.0, density=1.2)
    s.set_mesh(tri)
    s.set_bc(np.zeros(n), np.ones(n))
    _, _, p, _ = s.solve(300.0, np.ones(n))
    s.close()
    assert abs(float(vals["pnorm"]) - np.linalg.norm(p)) < 1e-9 * np.linalg.norm(p)
    line = [l for l in out.split("\n") if l.startswith("status")][0].split()
    p0 = complex(float(line[line.index("p0") + 1]), float(line[line.index("p0") + 2]))
    assert abs(p0 - p[0, 0]) < 1e-9 * abs(p[0, 0])
    assert float(vals["gmres_rel_err"]) < 1e-6
    assert float(vals["hlu_rel_err"]) < 0.2  # rank-2 preconditioner, not a solver


def test_facade_controller_compiles(facade_bin):
    """BemSolverController is in the header the fixture compiled (-Wall
    -Werror); the GPU test below runs it."""
    assert os.path.exists(facade_bin)


@pytest.mark.gpu
def test_facade_controller_stops_and_resumes(bem, meshes, facade_bin, tmp_path):
    """BemSolverController (bemsolvercontroller.cpp:49-109): a run stopped
    after two completed frequencies (two workers, so two or three are
    flagged), a second run that solves only the rest, and pressures equal to
    the Python sweep of the same frequencies."""
    tri = meshes.icosphere(2)
    n = tri.shape[0]
    out, vals = run(facade_bin, "sweep", tri, tmp_path)
    first, second = int(vals["first_run"]), int(vals["second_run"])
    assert 2 <= first <= 3 and first + second == 5, out
    s = bem.Solver(leaf_size=32, eta=2.0, aca_tol=1e-6, gmres_tol=1e-10, wave_speed=343.0,
                   density=1.2, sweep_workers=2)
    s.set_mesh(tri)
    s.set_bc(np.zeros(n), np.ones(n))
    p, _ = s.sweep([200.0, 300.0, 400.0, 500.0, 600.0], np.ones(n))
    s.close()
    for i in range(5):
        assert int(vals[f"status{i}"]) == 0, out
        ref = np.linalg.norm(p[:, 0, i])
        assert abs(float(vals[f"f{i}"]) - ref) < 1e-9 * ref, (i, out)
