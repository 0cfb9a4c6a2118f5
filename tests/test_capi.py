"""CPU checks of the C-ABI library: it builds, loads, exports every symbol the
public header declares, and its host-only planning matches the oracle."""
import ctypes as ct
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "bemgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(bem_[a-z_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(bem):
    L = bem.lib()
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
    assert sorted(bem.EXPORTS) == syms


def test_config_default_is_host_only(bem):
    c = bem.default_config()
    assert c.leaf_size == 32 and c.eta == 2.0 and c.coupling == 2 and c.gmres_restart == 300


@pytest.mark.parametrize("sub,leaf,eta", [(2, 32, 2.0), (3, 32, 2.0), (3, 50, 3.0), (4, 32, 2.0)])
def test_plan_matches_oracle(bem, meshes, orc, sub, leaf, eta):
    tri = meshes.icosphere(sub)
    perm, info = bem.plan_mesh(tri, bem.default_config(leaf_size=leaf, eta=eta))
    P = orc.Problem(tri, leaf, eta)
    assert np.array_equal(perm, P.perm)
    assert np.array_equal(info, P.blocks())


def test_plan_box_and_pencil(bem, meshes, orc):
    for tri in (meshes.box(n_target=1200), meshes.pencil(n_target=2000)):
        perm, info = bem.plan_mesh(tri)
        P = orc.Problem(tri, 32, 2.0)
        assert np.array_equal(perm, P.perm)
        assert np.array_equal(info, P.blocks())
        # partition covers the matrix exactly once
        n = tri.shape[0]
        assert (info[:, 1] * info[:, 3]).sum() == n * n


def test_plan_single_triangle(bem):
    tri = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], float)
    perm, info = bem.plan_mesh(tri)
    assert perm.tolist() == [0]
    assert info.tolist() == [[0, 1, 0, 1, 0]]


def test_plan_rejects_bad_input(bem):
    L = bem.lib()
    nb = ct.c_int64()
    assert L.bem_plan_mesh(None, None, 0, None, ct.byref(nb), None) == bem.BEM_EINVAL


def test_hlu_plan_program(bem, meshes):
    """The GPU H-LU task program is built on the host alone: every task type
    appears, dependencies are fewer than a handful per task, the sweeps'
    dataflow form applies to its factors, and the program refuses what the
    executor cannot hold (rank above 64, diagonal leaves above 48 rows)."""
    tri = meshes.icosphere(3)
    st = bem.hlu_plan(tri, bem.default_config(precond_rank=2))
    assert st["tasks"] > 1000 and st["dataflow_sweeps"] == 1.0
    for k in ("gemm", "lmul", "qr", "trunc", "copy", "zero"):
        assert st[k] > 0, k
    assert st["qr"] == 55  # one per leaf cluster (diagonal leaf)
    assert st["levels"] < st["tasks"] and st["dep_entries"] < 4 * st["tasks"]
    assert st["cost_path_us"] < st["cost_total_us"]
    big = bem.hlu_plan(tri, bem.default_config(precond_rank=64))
    assert big["tasks"] == st["tasks"] and big["arena_elems"] > st["arena_elems"]
    with pytest.raises(bem.BemError):
        bem.hlu_plan(tri, bem.default_config(precond_rank=65))
    with pytest.raises(bem.BemError):
        bem.hlu_plan(tri, bem.default_config(precond_rank=2, leaf_size=64))
