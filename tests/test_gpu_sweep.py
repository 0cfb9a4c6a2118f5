"""Batched frequency sweep (BemSolverController::run, bemsolvercontroller.cpp:
49-78, whose frequency loop is serial): concurrent workers give the same
pressures as the sequential sweep and as single solves; the autotuner picks
valid settings; the box-with-piston sweep (closed box, piston + random
patches) stays finite and solves every frequency."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


def box_solver(bem, meshes, n_target=1200, **cfg):
    tri = meshes.box(n_target=n_target, seed=7)
    n = tri.shape[0]
    s = bem.Solver(**{"aca_tol": 1e-5, "gmres_tol": 1e-10, "precision": 1, **cfg})
    s.set_mesh(tri)
    s.set_bc(np.zeros(n), np.ones(n))
    return tri, s


def test_concurrent_sweep_matches_sequential(bem, meshes):
    tri, s1 = box_solver(bem, meshes, sweep_workers=1)
    _, s3 = box_solver(bem, meshes, sweep_workers=3)
    g = meshes.box_piston_rhs(tri, patches=1)
    freqs = meshes.log_frequencies(7, 100.0, 1500.0)
    p1, i1 = s1.sweep(freqs, g)
    p3, i3 = s3.sweep(freqs, g)
    assert all(i["status"] == 0 for i in i1 + i3)
    # each frequency runs the same deterministic kernels on its worker
    assert np.array_equal(p1, p3)
    # and a single solve at one of the frequencies agrees
    _, _, p, _ = s1.solve(freqs[4], g)
    assert rel(p, p1[:, :, 4]) < 1e-12
    # a second sweep on the same handle reuses the workers
    p3b, _ = s3.sweep(freqs[::-1], g)
    assert np.array_equal(p3b[:, :, ::-1], p3)


def test_workers_follow_new_boundary_conditions(bem, meshes):
    tri, s = box_solver(bem, meshes, sweep_workers=2)
    n = tri.shape[0]
    g = np.ones(n)
    freqs = np.array([200.0, 300.0])
    p_a, _ = s.sweep(freqs, g)
    s.set_bc(np.ones(n), np.zeros(n))  # Dirichlet now: workers must be rebuilt
    p_b, _ = s.sweep(freqs, g)
    ref = bem.Solver(aca_tol=1e-5, gmres_tol=1e-10, precision=1, sweep_workers=1)
    ref.set_mesh(tri)
    ref.set_bc(np.ones(n), np.zeros(n))
    p_r, _ = ref.sweep(freqs, g)
    assert np.array_equal(p_b, p_r)
    assert rel(p_a, p_b) > 1e-3


def test_autotune(bem, meshes):
    tri, s = box_solver(bem, meshes, sweep_workers=0)
    n = tri.shape[0]
    g = np.ones(n)
    _, _, p0, _ = s.solve(500.0, g)
    t = s.autotune(500.0, 1)
    assert 1 <= t["workers"] <= 4 and t["aca_big_mn"] in (0, 256, 512, 1024, 2048)
    # the ACA size bin changes thread counts, not the approximation's accuracy
    _, _, p1, _ = s.solve(500.0, g)
    assert rel(p1, p0) < 1e-6
    p, info = s.sweep(np.array([400.0, 500.0, 600.0]), g)
    assert rel(p[:, :, 1], p1) < 1e-12 and all(i["status"] == 0 for i in info)


def test_box_piston_sweep(bem, meshes):
    tri, s = box_solver(bem, meshes, n_target=2000, sweep_workers=0)
    g = meshes.box_piston_rhs(tri)
    freqs = meshes.log_frequencies(16, 50.0, 2000.0)
    p, info = s.sweep(freqs, g)
    assert p.shape == (tri.shape[0], 4, 16)
    assert np.isfinite(p).all()
    assert all(i["status"] == 0 and i["true_residual"] < 1e-9 for i in info)
    # the pressure on the piston grows with frequency (radiation loading)
    on = g[:, 0] != 0
    amp = np.abs(p[on, 0, :]).mean(0)
    assert amp[-1] > amp[0]


def test_impedance_walls_match_robin_data(bem, meshes):
    """bem_set_bc_impedance (a = i k beta, b = 1 at every frequency) solves
    exactly what per-frequency Robin data a, b would."""
    tri = meshes.box(n_target=1200, seed=5)
    n = tri.shape[0]
    beta = meshes.wall_admittance(n, seed=3)
    g = np.ones(n)
    freqs = np.array([300.0, 700.0])
    s = bem.Solver(aca_tol=1e-5, gmres_tol=1e-10, precision=1, sweep_workers=2)
    s.set_mesh(tri)
    s.set_bc_impedance(beta)
    p, info = s.sweep(freqs, g)
    assert all(i["status"] == 0 for i in info)
    for q, f in enumerate(freqs):
        r = bem.Solver(aca_tol=1e-5, gmres_tol=1e-10, precision=1)
        r.set_mesh(tri)
        k = 2 * np.pi * f / 343.0
        r.set_bc(1j * k * beta, np.ones(n))
        _, _, pr, _ = r.solve(f, g)
        assert np.array_equal(p[:, :, q], pr)


def test_device_sweep_with_preconditioner_matches_solves(bem, meshes):
    """bem_sweep_device: concurrent workers with the GPU H-LU preconditioner
    (each worker starts from the parent's task program) read g and write p in
    GPU memory; the pressures equal single device solves bitwise, and events
    on the handle's stream bracket the whole sweep."""
    import torch
    tri = meshes.pencil(n_target=1280)
    n = tri.shape[0]
    g = meshes.pencil_rhs(tri)[:, :3]
    beta = meshes.wall_admittance(n)
    cfg = dict(aca_tol=1e-5, gmres_tol=1e-10, wave_speed=343.0, density=1.2, precision=1,
               use_preconditioner=1, precond_rank=2, near_fp64=1)
    freqs = np.array([400.0, 900.0, 2500.0, 6000.0, 1500.0])
    R = g.shape[1]
    gd = torch.from_numpy(np.ascontiguousarray(g.T)).to("cuda")  # n x R column-major
    s = bem.Solver(sweep_workers=3, **cfg)
    s.set_mesh(tri)
    s.set_bc_impedance(beta)
    s.solve(700.0, g)  # the parent's task program, then inherited by the workers
    p = torch.zeros((freqs.size, R, n), dtype=torch.complex128, device="cuda")
    stream = torch.cuda.ExternalStream(bem.lib().bem_stream(s._h))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    infos = s.sweep_device(freqs, gd.data_ptr(), R, p.data_ptr())
    e1.record(stream)
    torch.cuda.synchronize()
    assert e0.elapsed_time(e1) > 0
    assert all(i["status"] == 0 for i in infos)
    ref = bem.Solver(sweep_workers=1, **cfg)
    ref.set_mesh(tri)
    ref.set_bc_impedance(beta)
    for k, f in enumerate(freqs):
        q = torch.zeros((R, n), dtype=torch.complex128, device="cuda")
        ref.solve_device(float(f), gd.data_ptr(), R, 0, 0, q.data_ptr())
        torch.cuda.synchronize()
        assert torch.equal(q, p[k]), f
    s.close()
    ref.close()


def test_checkpointed_sweep_resumes(bem, meshes, tmp_path):
    """Checkpoint / resume (the controller's per-frequency solved flags,
    bemsolvercontroller.cpp:61-69): a checkpointed sweep stopped after 3 of 7
    frequencies leaves those (and the one another worker was finishing) on
    disk; a new handle over the same inputs loads them, solves only the rest
    and gives the pressures of an uninterrupted sweep bitwise. A checkpoint
    of a different sweep is refused."""
    import os

    tri, s = box_solver(bem, meshes, sweep_workers=2)
    g = meshes.box_piston_rhs(tri, patches=1)
    freqs = meshes.log_frequencies(7, 100.0, 1500.0)
    ref, iref = s.sweep(freqs, g)
    d = str(tmp_path / "ck")
    s._stop_after = 3
    s.sweep(freqs, g, checkpoint=d)
    first = {f: os.stat(os.path.join(d, f)).st_mtime_ns
             for f in os.listdir(d) if f.startswith("freq_")}
    assert 3 <= len(first) <= 4, sorted(first)
    s.close()
    _, s2 = box_solver(bem, meshes, sweep_workers=2)
    p, infos = s2.sweep(freqs, g, checkpoint=d)
    assert np.array_equal(p, ref)
    assert all(i["status"] == 0 and i["iterations"] == r["iterations"]
               for i, r in zip(infos, iref))
    files = {f: os.stat(os.path.join(d, f)).st_mtime_ns
             for f in os.listdir(d) if f.startswith("freq_")}
    assert len(files) == 7
    assert all(files[f] == t for f, t in first.items())  # loaded, not solved again
    # a finished checkpoint solves nothing and returns the same pressures
    p2, _ = s2.sweep(freqs, g, checkpoint=d)
    assert np.array_equal(p2, ref)
    with pytest.raises(ValueError):
        s2.sweep(freqs, 2.0 * g, checkpoint=d)
    s2.close()
