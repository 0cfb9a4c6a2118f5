#!/usr/bin/env python
"""Benchmark of the Helmholtz H-matrix BEM solve on one GB300.

Workload (the configuration the headline metric is quoted on): pulsating
sphere, radius 1 m, icosphere with 20,480 flat triangles, uniform normal
velocity (a = 0, b = 1, g = 1), c = 343 m/s, rho = 1.2, f = 1.5 kHz, leaf 32,
eta = 2, ACA tol 1e-5, GMRES tol 1e-10, Kirkup coupling, complex FP64.

A step is one complete frequency solve: near-field quadrature, ACA assembly of
both H-matrices, right-hand side, GMRES, BC back-substitution and pressure.
Consecutive steps use distinct frequencies 1500 * (1 + 0.002 i) Hz so nothing
is reused between steps; every step's working set (GBs of H-matrix data) is
far larger than the 129 MB L2, so no explicit flush is needed.

  value : freq-solves/s with g resident in GPU memory (bem_solve_device)
  e2e   : freq-solves/s through bem_solve with host buffers (g copied in, p
          copied out inside the timed region)

``--impl reference`` times the CPU restatement of the reference path (the
oracle: FP64 C++/OpenMP, all host cores) on the same workload.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FREQ = 1500.0
C0, RHO = 343.0, 1.2
ACA_TOL, GMRES_TOL = 1e-5, 1e-10
SUBDIV = 5  # 20 * 4**5 = 20,480 triangles
METRIC = "freq-solves/sec (H-matrix Helmholtz BEM solve, <=1e-5 rel. surface-pressure error)"
UNIT = "freq-solves/s"


def workload_config(extra=None):
    cfg = {"workload": "pulsating sphere r=1 m, icosphere 20,480 triangles, f=1.5 kHz",
           "n_elements": 20480, "freq_hz": FREQ, "aca_tol": ACA_TOL, "gmres_tol": GMRES_TOL,
           "leaf_size": 32, "eta": 2.0, "coupling": "Kirkup", "bc": "Neumann v=1",
           "nrhs": 1, "precision": "complex fp64",
           "l2": "working set (H-matrix, GBs) >> 129 MB L2; no flush needed"}
    if extra:
        cfg.update(extra)
    return cfg


def freqs(count, offset=0):
    return [FREQ * (1.0 + 0.002 * (offset + i)) for i in range(count)]


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def matvec_bytes(info, ranks, n, R=1, elem=16):
    """Algorithmic bytes of one H-matvec: stored entries once, plus each
    block's x segment and the y read-modify-write per block row."""
    near = info[:, 4] == 0
    far = ~near
    m, nn = info[:, 1], info[:, 3]
    k = np.where(far, ranks, 0)
    mat = (m[near] * nn[near]).sum() * elem + ((m[far] + nn[far]) * k[far]).sum() * elem \
        + k[far].sum() * elem
    vec = R * (nn.sum() * elem + 2 * n * elem)
    return int(mat + vec)


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    pkg = importlib.import_module("3d_bem_gb300")
    meshes = importlib.import_module("3d_bem_gb300.meshes")
    pkg.build()
    tri = meshes.icosphere(SUBDIV, 1.0)
    n = tri.shape[0]
    s = pkg.Solver(aca_tol=ACA_TOL, gmres_tol=GMRES_TOL, wave_speed=C0, density=RHO)
    s.set_mesh(tri)
    s.set_bc(np.zeros(n), np.ones(n))
    stream = torch.cuda.ExternalStream(pkg.lib().bem_stream(s._h))
    g = torch.ones(n, dtype=torch.complex128, device="cuda")
    p = torch.zeros(n, dtype=torch.complex128, device="cuda")
    for f in freqs(args.warmup, 1000 + rank * 100):
        s.solve_device(f, g.data_ptr(), 1, 0, 0, p.data_ptr())
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clk = Clocks(local)
    clk.start()
    l0 = s.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    infos = []
    e0.record(stream)
    for f in freqs(args.steps, rank * 100):
        infos.append(s.solve_device(f, g.data_ptr(), 1, 0, 0, p.data_ptr()))
    e1.record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clocks = clk.stop()
    launches = s.launch_count() - l0
    ms = e0.elapsed_time(e1)
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * args.steps / (ms / 1e3)

    # accuracy of the last solve against the analytic monopole (the fixed
    # discretisation error of this mesh) and the converged GMRES residual
    k = 2 * np.pi * freqs(args.steps, rank * 100)[-1] / C0
    pa = RHO * C0 * (1j * k) / (1j * k - 1)
    ph = p.cpu().numpy()
    analytic_err = float(np.abs(ph - pa).max() / abs(pa))

    # end-to-end through the host-buffer API (pinned host memory)
    gh = torch.ones(n, dtype=torch.complex128).pin_memory()
    ph_host = torch.zeros(n, dtype=torch.complex128).pin_memory()
    K2 = max(1, args.steps // 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for f in freqs(K2, 500 + rank * 100):
        _, _, pp, _ = s.solve(f, gh.numpy(), want=("p",))
    torch.cuda.synchronize()
    e2e = K2 / (time.perf_counter() - t0)

    # roofline of the H-matvec kernels (the GMRES inner operator), timed with
    # events on the library's stream over repeated applications
    info_part = s.partition()
    ranks = s.ranks(1)
    B = matvec_bytes(info_part, ranks, n)
    x = torch.randn(n, dtype=torch.complex128, device="cuda")
    y = torch.zeros(n, dtype=torch.complex128, device="cuda")
    reps = 50
    for _ in range(3):
        pkg.lib().bem_hmatvec_device(s._h, 1, x.data_ptr(), y.data_ptr(), 1, 0)
    h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    h0.record(stream)
    for _ in range(reps):
        pkg.lib().bem_hmatvec_device(s._h, 1, x.data_ptr(), y.data_ptr(), 1, 0)
    h1.record(stream)
    torch.cuda.synchronize()
    mv_ms = h0.elapsed_time(h1) / reps
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    achieved = B / (mv_ms * 1e-3) / 1e9

    phase = {key: float(np.mean([i[key] for i in infos]))
             for key in ("t_nearfield", "t_aca", "t_rhs", "t_gmres", "t_total")}
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128 (fp64)",
        "data": "synthetic (seeded icosphere; analytic monopole as accuracy check)",
        "config": workload_config({"parallelism": f"replicas{ws}" if ws > 1 else "single-gpu"}),
        "e2e": {"value": round(e2e, 4), "unit": UNIT, "h2d_bytes_per_step": n * 16,
                "d2h_bytes_per_step": n * 16},
        "roofline": {"kernel": "hmatvec (V pass + U pass)", "bound": "hbm",
                     "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "traffic": None,
                     "bytes_per_launch": B, "ms_per_launch": round(mv_ms, 4),
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback"},
        "gpu_launches": int(launches),
        "phases_s": {k2: round(v, 5) for k2, v in phase.items()},
        "gmres_iterations": int(max(i["iterations"] for i in infos)),
        "true_residual": float(max(i["true_residual"] for i in infos)),
        "max_rank": int(max(i["max_rank"] for i in infos)),
        "analytic_rel_err": round(analytic_err, 5),
        "clocks": clocks,
    }
    if not args.no_cpu_baseline and rank == 0 and ws == 1:
        line["cpu_baseline"] = cpu_baseline_sample(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    s.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def cpu_solve_once(tri, f, nthreads):
    import oracle
    oracle.build()
    P = oracle.Problem(tri, 32, 2.0)
    n = tri.shape[0]
    t0 = time.perf_counter()
    _, _, p, st = P.solve(f, C0, RHO, 2, np.zeros(n), np.ones(n), np.ones(n), ACA_TOL,
                          GMRES_TOL, nthreads=nthreads)
    return time.perf_counter() - t0, st


def cpu_baseline_sample(args):
    """The oracle (FP64 C++/OpenMP restatement of the reference path) on all
    host cores, one full frequency solve of the same workload."""
    meshes = importlib.import_module("3d_bem_gb300.meshes")
    tri = meshes.icosphere(SUBDIV, 1.0)
    cores = os.cpu_count() or 1
    dt, st = cpu_solve_once(tri, FREQ, cores)
    return {"value": round(1.0 / dt, 5), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"one full frequency solve of the same workload ({dt:.1f} s; "
                      f"GMRES iterations {int(st['iters'])})"}


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    meshes = importlib.import_module("3d_bem_gb300.meshes")
    tri = meshes.icosphere(SUBDIV, 1.0)
    cores = os.cpu_count() or 1
    # each step is one full frequency solve; bounded to a few minutes total
    budget = float(os.environ.get("BEM_REF_BUDGET_S", "240"))
    times = []
    t_start = time.perf_counter()
    for f in freqs(args.steps):
        dt, st = cpu_solve_once(tri, f, cores)
        times.append(dt)
        if time.perf_counter() - t_start + dt > budget:
            break
    value = len(times) / sum(times)
    line = {
        "metric": METRIC, "value": round(value, 5), "unit": UNIT, "n_gpus": ws,
        "steps": len(times), "warmup": 0, "ms_per_step": round(1e3 * sum(times) / len(times), 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128 (fp64)", "data": "synthetic (seeded icosphere)",
        "config": workload_config({"parallelism": "cpu-openmp"}),
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 5), "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{len(times)} full frequency solve(s) of the workload; "
                                   "the reference itself needs Qt 6 + Eigen and cannot be "
                                   "built here, so its CPU path is the oracle restatement"},
        "e2e": {"value": round(value, 5), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
