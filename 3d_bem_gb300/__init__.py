"""GB300-native Helmholtz boundary-element hot path (ctypes host layer).

The compute runs in ``libbemgpu.so`` (CUDA, sm_103a) behind the C ABI declared
in ``include/bemgpu.h``.  This module loads that library and mirrors the call
surface of KG93/3d_BEM's H-matrix solve:

* :class:`BoundaryElementSolver` -- ``calculateBoundarySolution`` /
  ``hMatrixSolve`` (boundaryelementsolver.cpp:12, :526-744),
* :class:`HMatrix` with :meth:`HArithm.MVM` (HMatrix/harithm.cpp:3-28),
* :meth:`GMRES.gmresSolve` (HMatrix/gmres.h:170-180),

plus :class:`Solver`, a thin handle wrapper used by the tests and the benchmark.
There is no CPU fallback: if the library is missing or no CUDA device is
present, every call raises :class:`BemError`.
"""
from __future__ import annotations

import ctypes as ct
import hashlib
import json
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libbemgpu.so")

BEM_OK, BEM_EINVAL, BEM_ENOMEM, BEM_ENONFINITE, BEM_EMAXIT = 0, 1, 2, 3, 4
BEM_EBREAKDOWN, BEM_ETIMEOUT, BEM_ECUDA, BEM_ERANK = 5, 6, 7, 8
STATUS_NAMES = {0: "OK", 1: "EINVAL", 2: "ENOMEM", 3: "ENONFINITE", 4: "EMAXIT",
                5: "EBREAKDOWN", 6: "ETIMEOUT", 7: "ECUDA", 8: "ERANK"}

# the C-ABI symbols declared in include/bemgpu.h
EXPORTS = [
    "bem_config_default", "bem_create", "bem_destroy", "bem_last_error", "bem_set_mesh",
    "bem_plan_mesh", "bem_hlu_plan",
    "bem_get_permutation", "bem_get_partition", "bem_set_bc", "bem_operators",
    "bem_assemble", "bem_hmatvec", "bem_hmatvec_device", "bem_get_block", "bem_get_ranks",
    "bem_gmres", "bem_solve", "bem_solve_device", "bem_sweep", "bem_sweep_device",
    "bem_sweep_resume",
    "bem_points_assemble",
    "bem_launch_count", "bem_stream", "bem_hmatvec_noalloc", "bem_hmatvec_device_ex",
    "bem_hlu_build", "bem_hlu_solve", "bem_hlu_export", "bem_hlu_sweep_kind", "bem_recompress",
    "bem_sel_nparam", "bem_sel_label", "bem_mlp_grad", "bem_mlp_adam", "bem_mlp_forward",
    "bem_sel_infer", "bem_set_selector", "bem_sel_stats", "bem_sel_classes", "bem_autotune",
    "bem_set_aca_rules", "bem_set_bc_impedance", "bem_field", "bem_field_device",
    "bem_msh_read", "bem_msh_free", "bem_msh_num_physical", "bem_msh_physical", "bem_msh_select",
    "bem_msh_elements", "bem_quads_to_triangles", "bem_wall_beta", "bem_set_impedance_plane",
    "bem_set_point_sources", "bem_refine_triangles",
]
BEM_ARITH_FP64, BEM_ARITH_FP32, BEM_ARITH_TWOFLOAT = 0, 1, 2


class BemError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class Config(ct.Structure):
    _fields_ = [("leaf_size", ct.c_int64), ("eta", ct.c_double), ("aca_tol", ct.c_double),
                ("aca_max_rank", ct.c_int64), ("rank_reserve", ct.c_int64),
                ("gmres_tol", ct.c_double), ("gmres_restart", ct.c_int64),
                ("gmres_maxit", ct.c_int64), ("coupling", ct.c_int32),
                ("precision", ct.c_int32), ("wave_speed", ct.c_double),
                ("density", ct.c_double), ("seed", ct.c_uint64),
                ("use_preconditioner", ct.c_int32), ("selector", ct.c_int32),
                ("precond_rank", ct.c_int64), ("precond_tol", ct.c_double),
                ("recompress_tol", ct.c_double), ("selector_guard", ct.c_double),
                ("sweep_workers", ct.c_int64), ("aca_big_mn", ct.c_int64),
                ("precond_reuse", ct.c_double), ("hlu_device", ct.c_int32),
                ("near_fp64", ct.c_int32)]


# bem_freq_done_fn: int (*)(int64_t f, void* user)
FREQ_DONE_FN = ct.CFUNCTYPE(ct.c_int, ct.c_int64, ct.c_void_p)


def _write_atomic(path, data: bytes):
    """Write a file under a temporary name, then rename it into place, so a
    reader sees either nothing or the whole file."""
    tmp = f"{path}.tmp{os.getpid()}"
    with open(tmp, "wb") as fh:
        fh.write(data)
        fh.flush()
        os.fsync(fh.fileno())
    os.replace(tmp, path)


def _npz_bytes(**arrays) -> bytes:
    import io
    b = io.BytesIO()
    np.savez(b, **arrays)
    return b.getvalue()


class SolveInfo(ct.Structure):
    _fields_ = [("iterations", ct.c_int64), ("rel_residual", ct.c_double),
                ("true_residual", ct.c_double), ("max_rank", ct.c_int64),
                ("capped_blocks", ct.c_int64), ("t_nearfield", ct.c_double),
                ("t_aca", ct.c_double), ("t_rhs", ct.c_double), ("t_gmres", ct.c_double),
                ("t_total", ct.c_double), ("status", ct.c_int32), ("precond_reused", ct.c_int32),
                ("t_precond", ct.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# ---- sweep checkpoints (per-frequency files of a resumable sweep) ----
def checkpoint_open(path: str, manifest: dict) -> list[str]:
    """Create the checkpoint directory of a sweep, or check that it belongs
    to the same sweep (ValueError otherwise). Returns the per-frequency file
    names."""
    os.makedirs(path, exist_ok=True)
    mpath = os.path.join(path, "manifest.json")
    if os.path.exists(mpath):
        with open(mpath) as fh:
            if json.load(fh) != manifest:
                raise ValueError(f"{path} holds a checkpoint of a different sweep")
    else:
        _write_atomic(mpath, json.dumps(manifest).encode())
    return [f"freq_{i:05d}.npz" for i in range(len(manifest["freqs"]))]


def _info_record(info: SolveInfo) -> np.ndarray:
    return np.array(tuple(getattr(info, k) for k, _ in SolveInfo._fields_),
                    dtype=[(k, np.dtype(t)) for k, t in SolveInfo._fields_])


def checkpoint_write(path: str, name: str, p_slice, freq: float, info: SolveInfo):
    """One completed frequency: its pressures (n x R) and info record."""
    _write_atomic(os.path.join(path, name),
                  _npz_bytes(p=np.ascontiguousarray(p_slice), freq=np.float64(freq),
                             info=_info_record(info)))


def checkpoint_load(path: str, names, p, infos) -> np.ndarray:
    """The completed frequencies of a checkpoint into p[:, :, i] and
    infos[i]; returns the solved flags (uint8 per frequency)."""
    solved = np.zeros(len(names), np.uint8)
    for i, name in enumerate(names):
        f = os.path.join(path, name)
        if not os.path.exists(f):
            continue
        with np.load(f) as z:
            p[:, :, i] = z["p"]
            rec = z["info"][()]
            for k, _ in SolveInfo._fields_:
                setattr(infos[i], k, rec[k].item())
        solved[i] = 1
    return solved



_lib = None


def build(force: bool = False) -> str:
    """Compile libbemgpu.so in-tree (nvcc, sm_103a)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_bemgpu_build", os.path.join(_HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def lib():
    """Load libbemgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise BemError(BEM_EINVAL, f"{LIB_PATH} is missing: build the CUDA library first "
                                   "(python 3d_bem_gb300/build.py)")
    L = ct.CDLL(LIB_PATH)
    vp, i64, i32, dbl = ct.c_void_p, ct.c_int64, ct.c_int32, ct.c_double
    P = ct.POINTER
    L.bem_config_default.argtypes = [P(Config)]
    L.bem_config_default.restype = None
    L.bem_create.argtypes = [P(Config), P(vp)]
    L.bem_destroy.argtypes = [vp]
    L.bem_destroy.restype = None
    L.bem_last_error.argtypes = [vp]
    L.bem_last_error.restype = ct.c_char_p
    L.bem_set_mesh.argtypes = [vp, vp, i64]
    L.bem_plan_mesh.argtypes = [P(Config), vp, i64, vp, P(i64), vp]
    L.bem_hlu_plan.argtypes = [P(Config), vp, i64, vp, i64]
    L.bem_get_permutation.argtypes = [vp, vp]
    L.bem_get_partition.argtypes = [vp, P(i64), vp]
    L.bem_set_bc.argtypes = [vp, vp, vp]
    L.bem_operators.argtypes = [vp, dbl, vp, vp, i64, vp]
    L.bem_assemble.argtypes = [vp, dbl]
    L.bem_hmatvec.argtypes = [vp, i32, vp, vp, i64, i32]
    L.bem_hmatvec_device.argtypes = [vp, i32, vp, vp, i64, i32]
    L.bem_hmatvec_noalloc.argtypes = [vp, i32, vp, vp, i64, i32]
    L.bem_hmatvec_device_ex.argtypes = [vp, i32, vp, vp, i64, i32, i32]
    L.bem_get_block.argtypes = [vp, i32, i64, P(i64), vp, vp, vp, vp]
    L.bem_get_ranks.argtypes = [vp, i32, vp]
    L.bem_gmres.argtypes = [vp, vp, vp, i64, P(SolveInfo)]
    L.bem_solve.argtypes = [vp, dbl, vp, i64, vp, vp, vp, P(SolveInfo)]
    L.bem_solve_device.argtypes = [vp, dbl, vp, i64, vp, vp, vp, P(SolveInfo)]
    L.bem_sweep.argtypes = [vp, vp, i64, vp, i64, vp, vp]
    L.bem_sweep_device.argtypes = [vp, vp, i64, vp, i64, vp, vp]
    L.bem_sweep_resume.argtypes = [vp, vp, i64, vp, i64, vp, vp, vp, FREQ_DONE_FN, vp]
    L.bem_points_assemble.argtypes = [vp, vp, i64, vp, i64, dbl, vp, vp]
    L.bem_recompress.argtypes = [vp, i32, i64, dbl]
    L.bem_sel_nparam.argtypes = []
    L.bem_sel_nparam.restype = i64
    L.bem_sel_label.argtypes = [vp, vp, vp, i64, dbl, dbl, dbl, vp, vp, vp]
    L.bem_mlp_grad.argtypes = [vp, vp, vp, i64, vp, vp, vp, vp]
    L.bem_mlp_adam.argtypes = [vp, vp, vp, vp, i64, ct.c_float, ct.c_float, ct.c_float,
                               ct.c_float, vp]
    L.bem_mlp_forward.argtypes = [vp, vp, i64, vp, vp]
    L.bem_sel_infer.argtypes = [vp, vp, vp, vp, i64, vp, vp, vp]
    L.bem_set_selector.argtypes = [vp, vp, vp, vp]
    L.bem_sel_stats.argtypes = [vp, vp]
    L.bem_sel_classes.argtypes = [vp, vp]
    L.bem_autotune.argtypes = [vp, dbl, i64, vp]
    L.bem_set_aca_rules.argtypes = [vp, vp, vp]
    L.bem_set_bc_impedance.argtypes = [vp, vp]
    L.bem_field.argtypes = [vp, dbl, vp, i64, vp, vp, i64, vp, i64, vp, vp]
    L.bem_msh_read.argtypes = [ct.c_char_p, P(vp), ct.c_char_p, i64]
    L.bem_msh_free.argtypes = [vp]
    L.bem_msh_free.restype = None
    L.bem_msh_num_physical.argtypes = [vp]
    L.bem_msh_num_physical.restype = i64
    L.bem_msh_physical.argtypes = [vp, i64, P(i32), P(i32), ct.c_char_p, i64]
    L.bem_msh_select.argtypes = [vp, ct.c_char_p, ct.c_char_p, P(i64), P(i64)]
    L.bem_msh_elements.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.bem_quads_to_triangles.argtypes = [vp, i64, vp]
    L.bem_wall_beta.argtypes = [i32, i32, vp, dbl, vp]
    L.bem_set_impedance_plane.argtypes = [vp, vp, vp]
    L.bem_set_point_sources.argtypes = [vp, vp, i64]
    L.bem_refine_triangles.argtypes = [vp, i64, dbl, vp, i64, P(i64), vp]
    L.bem_field_device.argtypes = [vp, dbl, vp, i64, vp, vp, i64, vp, i64, vp, vp]
    L.bem_hlu_build.argtypes = [vp]
    L.bem_hlu_solve.argtypes = [vp, vp, vp, i64]
    L.bem_hlu_export.argtypes = [vp, i32, P(i64), vp, P(i64), vp, P(i64), vp]
    L.bem_hlu_sweep_kind.argtypes = [vp, P(i32)]
    L.bem_launch_count.argtypes = [vp]
    L.bem_launch_count.restype = i64
    L.bem_stream.argtypes = [vp]
    L.bem_stream.restype = vp
    for name in EXPORTS:
        f = getattr(L, name)
        if f.restype is ct.c_int:  # default restype: status codes are int32
            f.restype = ct.c_int32
    _lib = L
    return L


def default_config(**overrides) -> Config:
    c = Config()
    lib().bem_config_default(ct.byref(c))
    for k, v in overrides.items():
        setattr(c, k, v)
    return c


def plan_mesh(tri, config: Config | None = None):
    """Host-only cluster-tree permutation and partition (no GPU needed)."""
    tri = np.ascontiguousarray(tri, dtype=np.float64).reshape(-1, 9)
    cfg = config if config is not None else default_config()
    n = tri.shape[0]
    perm = np.zeros(n, np.int64)
    nb = ct.c_int64()
    st = lib().bem_plan_mesh(ct.byref(cfg), _ptr(tri), n, _ptr(perm), ct.byref(nb), None)
    if st != BEM_OK:
        raise BemError(st, "bem_plan_mesh failed")
    info = np.zeros((nb.value, 5), np.int64)
    st = lib().bem_plan_mesh(ct.byref(cfg), _ptr(tri), n, _ptr(perm), ct.byref(nb), _ptr(info))
    if st != BEM_OK:
        raise BemError(st, "bem_plan_mesh failed")
    return perm, info


HLU_PLAN_KEYS = ("tasks", "arena_elems", "scratch_elems", "levels", "cost_path_us",
                 "cost_total_us", "max_trunc_width", "dataflow_sweeps", "gemm", "lmul",
                 "rmul", "qr", "trunc", "copy", "zero", "dep_entries", "big_scratch_elems",
                 "path_gemm", "path_lmul", "path_rmul", "path_qr", "path_trunc", "path_copy",
                 "path_zero")


def hlu_plan(tri, config: Config | None = None) -> dict:
    """Host-only statistics of the GPU H-LU task program for a mesh (no GPU
    needed): task counts, arena size, critical path of the cost model."""
    tri = np.ascontiguousarray(tri, dtype=np.float64).reshape(-1, 9)
    cfg = config if config is not None else default_config()
    out = np.zeros(len(HLU_PLAN_KEYS))
    st = lib().bem_hlu_plan(ct.byref(cfg), _ptr(tri), tri.shape[0], _ptr(out), out.size)
    if st != BEM_OK:
        raise BemError(st, "bem_hlu_plan failed")
    return dict(zip(HLU_PLAN_KEYS, out.tolist()))


def _ptr(a: np.ndarray):
    return ct.c_void_p(a.ctypes.data) if a is not None else None


def _c128(a, n=None):
    a = np.asarray(a, dtype=np.complex128)
    return np.asfortranarray(a) if a.ndim == 2 else np.ascontiguousarray(a)


SELECTOR_WEIGHTS = os.path.join(_HERE, "selector_weights.npz")
SEL_NFEAT, SEL_NCLASS = 24, 5
SEL_RULE_POINTS = (1, 3, 7, 13, 25)


def load_selector_weights(path: str = SELECTOR_WEIGHTS) -> dict:
    if not os.path.exists(path):
        raise BemError(BEM_EINVAL, f"no trained selector weights at {path} "
                       "(train them with 3d_bem_gb300/selector_train.py)")
    z = np.load(path)
    return {k: z[k] for k in z.files}


def _status(st, what):
    if st != BEM_OK:
        raise BemError(st, what)


def sel_label(ptri, qtri, k, tol=1e-7, near_ratio=1.0, want_err=False, floor_rel=1e-3):
    """Features (n x 24), labels (n) and optionally the per-rule errors (n x 6)
    of n pairs, computed on the GPU (bem_sel_label)."""
    ptri = np.ascontiguousarray(ptri, np.float64).reshape(-1, 9)
    qtri = np.ascontiguousarray(qtri, np.float64).reshape(-1, 9)
    k = np.ascontiguousarray(k, np.float64).ravel()
    n = k.size
    feat = np.zeros((n, SEL_NFEAT), np.float32)
    lab = np.zeros(n, np.uint8)
    err = np.zeros((n, 6), np.float32) if want_err else None
    _status(lib().bem_sel_label(_ptr(ptri), _ptr(qtri), _ptr(k), n, tol, near_ratio, floor_rel,
                                _ptr(feat), _ptr(lab), _ptr(err)), "bem_sel_label")
    return (feat, lab, err) if want_err else (feat, lab)


class Solver:
    """One GPU solver handle (mesh, BCs, assembled H-matrices, GMRES state)."""

    def __init__(self, config: Config | None = None, **overrides):
        L = lib()
        self.config = config if config is not None else default_config(**overrides)
        h = ct.c_void_p()
        st = L.bem_create(ct.byref(self.config), ct.byref(h))
        if st != BEM_OK:
            raise BemError(st, "bem_create failed (is a CUDA device visible?)")
        self._h = h
        self.n = 0
        self.rows = 0
        self._inputs = {}  # digests of what was set, for sweep checkpoints
        if self.config.selector:
            self.set_selector()

    def close(self):
        if getattr(self, "_h", None):
            lib().bem_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def _note(self, key, *arrays):
        d = hashlib.sha256()
        for x in arrays:
            x = np.ascontiguousarray(x)
            d.update(str((x.dtype.str, x.shape)).encode())
            d.update(x.tobytes())
        self._inputs[key] = d.hexdigest()

    def fingerprint(self) -> str:
        """Digest of the configuration and of every input set on this
        handle (mesh, boundary conditions, sources, plane, selector)."""
        d = hashlib.sha256(bytes(self.config))
        for k in sorted(self._inputs):
            d.update(f"{k}={self._inputs[k]};".encode())
        return d.hexdigest()

    def _check(self, st, what=""):
        if st != BEM_OK:
            msg = lib().bem_last_error(self._h)
            raise BemError(st, f"{what}: {msg.decode() if msg else ''}")
        return st

    # ---- mesh / BC ----
    def set_mesh(self, tri: np.ndarray):
        tri = np.ascontiguousarray(tri, dtype=np.float64).reshape(-1, 9)
        self._check(lib().bem_set_mesh(self._h, _ptr(tri), tri.shape[0]), "bem_set_mesh")
        # a new mesh drops the boundary conditions, sources and plane
        for k in ("bc", "sources", "plane"):
            self._inputs.pop(k, None)
        self._note("mesh", tri)
        self.n = tri.shape[0]
        self.rows = self.n  # rows of the assembled matrices

    @property
    def permutation(self) -> np.ndarray:
        p = np.zeros(self.n, np.int64)
        self._check(lib().bem_get_permutation(self._h, _ptr(p)), "bem_get_permutation")
        return p

    def partition(self) -> np.ndarray:
        nb = ct.c_int64()
        self._check(lib().bem_get_partition(self._h, ct.byref(nb), None), "bem_get_partition")
        info = np.zeros((nb.value, 5), np.int64)
        self._check(lib().bem_get_partition(self._h, ct.byref(nb), _ptr(info)), "bem_get_partition")
        return info

    def set_bc_impedance(self, beta):
        """Impedance walls: a = i k beta (beta = rho c / Z per element), b = 1."""
        beta = np.ascontiguousarray(np.asarray(beta, np.complex128).ravel())
        self._check(lib().bem_set_bc_impedance(self._h, _ptr(beta)), "bem_set_bc_impedance")
        self._note("bc", np.array([1]), beta)

    def set_bc(self, a, b):
        a = _c128(a)
        b = _c128(b)
        self._check(lib().bem_set_bc(self._h, _ptr(a), _ptr(b)), "bem_set_bc")
        self._note("bc", np.array([0]), a, b)

    # ---- operators / matrices ----
    def operators(self, k, rows, cols) -> np.ndarray:
        rows = np.ascontiguousarray(rows, np.int64)
        cols = np.ascontiguousarray(cols, np.int64)
        out = np.zeros((rows.size, 4), np.complex128)
        self._check(lib().bem_operators(self._h, k, _ptr(rows), _ptr(cols), rows.size, _ptr(out)),
                    "bem_operators")
        return out

    def assemble(self, freq: float):
        self._check(lib().bem_assemble(self._h, freq), "bem_assemble")

    def hmatvec(self, which: int, x, y=None, accumulate: bool = False) -> np.ndarray:
        x = _c128(x)
        R = 1 if x.ndim == 1 else x.shape[1]
        rows = self.rows or x.shape[0]
        if y is None:  # one row per row of the matrix (point clouds: rectangular)
            out = np.zeros((rows,) if x.ndim == 1 else (rows, R), np.complex128, order="F")
        else:
            out = _c128(y).copy(order="F")
            if out.shape[0] != rows:
                raise BemError(BEM_EINVAL, "hmatvec: y needs one row per matrix row")
        self._check(lib().bem_hmatvec(self._h, which, _ptr(x), _ptr(out), R, int(accumulate)),
                    "bem_hmatvec")
        return out

    def set_selector(self, weights=None):
        """Install trained selector weights (a dict / npz with params, mu,
        sigma; default: the package's ``selector_weights.npz``)."""
        w = load_selector_weights() if weights is None else weights
        prm = np.ascontiguousarray(w["params"], np.float32)
        mu = np.ascontiguousarray(w["mu"], np.float32)
        sg = np.ascontiguousarray(w["sigma"], np.float32)
        self._check(lib().bem_set_selector(self._h, _ptr(prm), _ptr(mu), _ptr(sg)),
                    "bem_set_selector")
        self._note("selector", prm, mu, sg)
        if "aca_table" in w:
            tab = np.ascontiguousarray(w["aca_table"], np.uint8)
            axes = np.ascontiguousarray(w["aca_axes"], np.float32)
            self._check(lib().bem_set_aca_rules(self._h, _ptr(tab), _ptr(axes)),
                        "bem_set_aca_rules")
            self._note("aca_rules", tab, axes)

    def sel_stats(self) -> dict:
        st = np.zeros(4, np.int64)
        self._check(lib().bem_sel_stats(self._h, _ptr(st)), "bem_sel_stats")
        return {"points": int(st[0]), "checked": int(st[1]), "fallback": int(st[2]),
                "regular_entries": int(st[3])}

    def sel_classes(self) -> np.ndarray:
        info = self.partition()
        near = info[info[:, 4] == 0]
        cls = np.zeros(int((near[:, 1] * near[:, 3]).sum()), np.uint8)
        self._check(lib().bem_sel_classes(self._h, _ptr(cls)), "bem_sel_classes")
        return cls

    def autotune(self, freq: float, nrhs: int = 1) -> dict:
        """Tune the batched sweep (workers, ACA size bin) at a probe frequency."""
        out = np.zeros(2, np.int64)
        self._check(lib().bem_autotune(self._h, freq, nrhs, _ptr(out)), "bem_autotune")
        return {"workers": int(out[0]), "aca_big_mn": int(out[1])}

    def recompress(self, which: int, rank: int = 0, tol: float = 0.0):
        """Truncating SVD recompression of every admissible block on the GPU."""
        self._check(lib().bem_recompress(self._h, which, rank, tol), "bem_recompress")

    def hlu_build(self):
        """H-LU factors of the assembled system matrix (HArithm::LUDecomposition)."""
        self._check(lib().bem_hlu_build(self._h), "bem_hlu_build")

    def hlu_solve(self, b) -> np.ndarray:
        """x = U^-1 L^-1 b on the GPU, cluster order (HArithm::LUSubstitutionSolve)."""
        b = _c128(b)
        R = 1 if b.ndim == 1 else b.shape[1]
        x = np.zeros_like(b)
        self._check(lib().bem_hlu_solve(self._h, _ptr(b), _ptr(x), R), "bem_hlu_solve")
        return x

    def hlu_sweep_kind(self) -> int:
        """1: dataflow sweeps (driver + helper CTAs), 0: sequential sweeps."""
        k = ct.c_int32()
        self._check(lib().bem_hlu_sweep_kind(self._h, ct.byref(k)), "bem_hlu_sweep_kind")
        return k.value

    def hlu_export(self, which: int):
        """Flat factor ``which`` (0 L, 1 U): (leaves n x 7, data, schedule)."""
        nl, nd, ns = ct.c_int64(), ct.c_int64(), ct.c_int64()
        self._check(lib().bem_hlu_export(self._h, which, ct.byref(nl), None, ct.byref(nd), None,
                                         ct.byref(ns), None), "bem_hlu_export")
        leaves = np.zeros((nl.value, 7), np.int64)
        data = np.zeros(nd.value, np.complex128)
        sched = np.zeros(ns.value, np.int32)
        self._check(lib().bem_hlu_export(self._h, which, ct.byref(nl), _ptr(leaves), ct.byref(nd),
                                         _ptr(data), ct.byref(ns), _ptr(sched)), "bem_hlu_export")
        return leaves, data, sched

    def ranks(self, which: int) -> np.ndarray:
        r = np.zeros(self.partition().shape[0], np.int64)
        self._check(lib().bem_get_ranks(self._h, which, _ptr(r)), "bem_get_ranks")
        return r

    def block(self, which: int, i: int, info_row):
        r0, m, c0, n, adm = [int(v) for v in info_row]
        rank = ct.c_int64()
        if adm:
            self._check(lib().bem_get_block(self._h, which, i, ct.byref(rank), None, None, None,
                                            None), "bem_get_block")
            k = rank.value
            U = np.zeros((k, m), np.complex128)
            s = np.zeros(k, np.complex128)
            V = np.zeros((k, n), np.complex128)
            self._check(lib().bem_get_block(self._h, which, i, ct.byref(rank), _ptr(U), _ptr(s),
                                            _ptr(V), None), "bem_get_block")
            return U.T.copy(), s, V
        F = np.zeros((n, m), np.complex128)
        self._check(lib().bem_get_block(self._h, which, i, ct.byref(rank), None, None, None,
                                        _ptr(F)), "bem_get_block")
        return F.T.copy()

    def dense(self, which: int, info=None) -> np.ndarray:
        """Expand the assembled H-matrix (tests only; O(N^2) memory)."""
        info = self.partition() if info is None else info
        nr = int((info[:, 0] + info[:, 1]).max())
        nc = int((info[:, 2] + info[:, 3]).max())
        D = np.zeros((nr, nc), np.complex128)
        for i, row in enumerate(info):
            r0, m, c0, n, adm = [int(v) for v in row]
            blk = self.block(which, i, row)
            if adm:
                U, s, V = blk
                D[r0:r0 + m, c0:c0 + n] = (U * s) @ V
            else:
                D[r0:r0 + m, c0:c0 + n] = blk
        return D

    def gmres(self, b, x0=None):
        b = _c128(b)
        R = 1 if b.ndim == 1 else b.shape[1]
        x = np.zeros_like(b) if x0 is None else _c128(x0).copy()
        info = SolveInfo()
        st = lib().bem_gmres(self._h, _ptr(b), _ptr(x), R, ct.byref(info))
        if st not in (BEM_OK, BEM_EMAXIT):
            self._check(st, "bem_gmres")
        return x, info.as_dict()

    def solve(self, freq: float, g, want=("phi", "dphi", "p")):
        g = np.asarray(g, np.complex128)
        g = np.asfortranarray(g.reshape(self.n or g.shape[0], -1))
        R = g.shape[1]
        outs = {k: (np.zeros((self.n, R), np.complex128, order="F") if k in want else None)
                for k in ("phi", "dphi", "p")}
        info = SolveInfo()
        st = lib().bem_solve(self._h, freq, _ptr(g), R, _ptr(outs["phi"]), _ptr(outs["dphi"]),
                             _ptr(outs["p"]), ct.byref(info))
        if st not in (BEM_OK, BEM_EMAXIT):
            self._check(st, "bem_solve")
        return outs["phi"], outs["dphi"], outs["p"], info.as_dict()

    def solve_device(self, freq: float, g_ptr: int, R: int, phi_ptr=0, dphi_ptr=0, p_ptr=0):
        info = SolveInfo()
        st = lib().bem_solve_device(self._h, freq, ct.c_void_p(g_ptr), R,
                                    ct.c_void_p(phi_ptr) if phi_ptr else None,
                                    ct.c_void_p(dphi_ptr) if dphi_ptr else None,
                                    ct.c_void_p(p_ptr) if p_ptr else None, ct.byref(info))
        if st not in (BEM_OK, BEM_EMAXIT):
            self._check(st, "bem_solve_device")
        return info.as_dict()

    def sweep(self, freqs, g, checkpoint: str | None = None):
        """Frequency sweep: pressures n x R x nf (caller order) and the
        per-frequency infos.

        checkpoint: a directory. Each frequency is written there as it
        completes (``freq_<index>.npz``: its pressures and info), beside a
        manifest of the sweep (frequencies, right-hand sides and the handle's
        :meth:`fingerprint`). A call with the same directory and the same
        sweep loads the completed frequencies and solves only the others,
        as the controller's per-frequency solved flags do
        (bemsolvercontroller.cpp:61-69); a directory of a different sweep
        raises ValueError."""
        freqs = np.ascontiguousarray(freqs, np.float64)
        g = np.asfortranarray(np.asarray(g, np.complex128).reshape(self.n, -1))
        R = g.shape[1]
        p = np.zeros((self.n, R, freqs.size), np.complex128, order="F")
        infos = (SolveInfo * freqs.size)()
        if checkpoint is None:
            st = lib().bem_sweep(self._h, _ptr(freqs), freqs.size, _ptr(g), R, _ptr(p), infos)
        else:
            st = self._sweep_checkpointed(freqs, g, p, infos, checkpoint)
        if st not in (BEM_OK, BEM_EMAXIT):
            self._check(st, "bem_sweep")
        return p, [i.as_dict() for i in infos]

    _stop_after = None  # tests: stop a checkpointed sweep after this many frequencies

    def _sweep_checkpointed(self, freqs, g, p, infos, path):
        key = hashlib.sha256()
        for x in (freqs, g):
            key.update(np.ascontiguousarray(x).tobytes())
        key.update(self.fingerprint().encode())
        names = checkpoint_open(path, {"n": self.n, "R": int(g.shape[1]),
                                       "freqs": freqs.tolist(), "key": key.hexdigest()})
        solved = checkpoint_load(path, names, p, infos)
        count, failed = [0], []

        def done(i, _user):
            try:
                checkpoint_write(path, names[i], p[:, :, i], freqs[i], infos[i])
            except Exception as e:  # stop the sweep; raised below
                failed.append(e)
                return 1
            count[0] += 1
            return int(self._stop_after is not None and count[0] >= self._stop_after)

        cb = FREQ_DONE_FN(done)
        st = lib().bem_sweep_resume(self._h, _ptr(freqs), freqs.size, _ptr(g), g.shape[1],
                                    _ptr(p), infos, _ptr(solved), cb, None)
        if failed:
            raise failed[0]
        return st

    def sweep_device(self, freqs, g_ptr: int, R: int, p_ptr: int):
        """bem_sweep with device pointers: g (n x R complex FP64, caller order)
        and p (n x R per frequency, nf slices) in GPU memory. Returns the
        per-frequency infos."""
        freqs = np.ascontiguousarray(freqs, np.float64)
        infos = (SolveInfo * freqs.size)()
        st = lib().bem_sweep_device(self._h, _ptr(freqs), freqs.size, ct.c_void_p(g_ptr), R,
                                    ct.c_void_p(p_ptr), infos)
        if st not in (BEM_OK, BEM_EMAXIT):
            self._check(st, "bem_sweep_device")
        return [i.as_dict() for i in infos]

    def set_point_sources(self, sources=None):
        """Point sources of the right-hand side: rows (x, y, z, complex weight);
        None clears them."""
        src = _sources(sources)
        self._check(lib().bem_set_point_sources(self._h, _ptr(src) if src.shape[0] else None,
                                                src.shape[0]), "bem_set_point_sources")
        self._note("sources", src)

    def set_impedance_plane(self, point=None, normal=None):
        """One infinite rigid plane (impedance plane); None removes it."""
        if normal is None:
            self._check(lib().bem_set_impedance_plane(self._h, None, None),
                        "bem_set_impedance_plane")
            self._inputs.pop("plane", None)
            return
        p = np.ascontiguousarray(point, np.float64).reshape(3)
        n = np.ascontiguousarray(normal, np.float64).reshape(3)
        self._check(lib().bem_set_impedance_plane(self._h, _ptr(p), _ptr(n)),
                    "bem_set_impedance_plane")
        self._note("plane", p, n)

    def field(self, freq: float, pts, phi, dphi, sources=None):
        """Velocity potential and sound pressure (npts x R each) at the
        observation points ``pts`` from a boundary solution phi, dphi (n x R,
        caller order); ``sources``: rows (x, y, z, complex weight)."""
        pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
        phi = np.asarray(phi, np.complex128)
        n = self.n or phi.shape[0]
        phi = np.asfortranarray(phi.reshape(n, -1))
        dphi = np.asfortranarray(np.asarray(dphi, np.complex128).reshape(n, -1))
        R = phi.shape[1]
        src = _sources(sources)
        pf = np.zeros((pts.shape[0], R), np.complex128, order="F")
        pp = np.zeros((pts.shape[0], R), np.complex128, order="F")
        self._check(lib().bem_field(self._h, freq, _ptr(pts), pts.shape[0], _ptr(phi), _ptr(dphi),
                                    R, _ptr(src) if src.shape[0] else None, src.shape[0],
                                    _ptr(pf), _ptr(pp)), "bem_field")
        return pf, pp

    def field_device(self, freq: float, pts_ptr: int, npts: int, phi_ptr: int, dphi_ptr: int,
                     R: int, phi_f_ptr=0, p_f_ptr=0, sources=None):
        """bem_field_device on raw device pointers (asynchronous on the
        handle's stream)."""
        src = _sources(sources)
        self._check(lib().bem_field_device(
            self._h, freq, ct.c_void_p(pts_ptr), npts, ct.c_void_p(phi_ptr),
            ct.c_void_p(dphi_ptr), R, _ptr(src) if src.shape[0] else None, src.shape[0],
            ct.c_void_p(phi_f_ptr) if phi_f_ptr else None,
            ct.c_void_p(p_f_ptr) if p_f_ptr else None), "bem_field_device")

    def points_assemble(self, rowpts, colpts, k):
        rowpts = np.ascontiguousarray(rowpts, np.float64)
        colpts = np.ascontiguousarray(colpts, np.float64)
        rp = np.zeros(rowpts.shape[0], np.int64)
        cp = np.zeros(colpts.shape[0], np.int64)
        self._check(lib().bem_points_assemble(self._h, _ptr(rowpts), rowpts.shape[0],
                                              _ptr(colpts), colpts.shape[0], k, _ptr(rp),
                                              _ptr(cp)), "bem_points_assemble")
        self.rows = rowpts.shape[0]
        return rp, cp

    def launch_count(self) -> int:
        return int(lib().bem_launch_count(self._h))


def _sources(sources) -> np.ndarray:
    """Point sources (x, y, z, complex weight) as the C-ABI's nsrc x 5 rows."""
    if sources is None or len(sources) == 0:
        return np.zeros((0, 5))
    s = np.asarray(sources, np.complex128).reshape(-1, 4)
    return np.ascontiguousarray(np.column_stack([s[:, :3].real, s[:, 3].real, s[:, 3].imag]))


# ---------------------------------------------------------------------------
# Mesh input and boundary data (host only)
# ---------------------------------------------------------------------------
class MshFile:
    """A GMSH ASCII mesh (formats 2.2 and 4.1) read by the library
    (bem_msh_read); :meth:`select` applies the reference's include / exclude
    lists."""

    def __init__(self, path):
        err = ct.create_string_buffer(512)
        h = ct.c_void_p()
        st = lib().bem_msh_read(os.fsencode(path), ct.byref(h), err, 512)
        if st != BEM_OK:
            raise BemError(st, f"bem_msh_read: {err.value.decode(errors='replace')}")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().bem_msh_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def physical_names(self) -> list:
        """[(dim, number, name)] from $PhysicalNames."""
        out = []
        name = ct.create_string_buffer(256)
        d, t = ct.c_int32(), ct.c_int32()
        for i in range(lib().bem_msh_num_physical(self._h)):
            _raise(lib().bem_msh_physical(self._h, i, ct.byref(d), ct.byref(t), name, 256),
                   "bem_msh_physical")
            out.append((d.value, t.value, name.value.decode(errors="replace")))
        return out

    def select(self, include="all", exclude="") -> dict:
        """Triangles (N x 9), quadrilaterals (M x 12) and their physical /
        geometric numbers after the include / exclude selection."""
        inc = " ".join(include) if isinstance(include, (list, tuple)) else str(include)
        exc = " ".join(exclude) if isinstance(exclude, (list, tuple)) else str(exclude)
        nt, nq = ct.c_int64(), ct.c_int64()
        _raise(lib().bem_msh_select(self._h, inc.encode(), exc.encode(), ct.byref(nt),
                                    ct.byref(nq)), "bem_msh_select")
        out = {"tri": np.zeros((nt.value, 9)), "tri_phys": np.zeros(nt.value, np.int32),
               "tri_geom": np.zeros(nt.value, np.int32), "quad": np.zeros((nq.value, 12)),
               "quad_phys": np.zeros(nq.value, np.int32),
               "quad_geom": np.zeros(nq.value, np.int32)}
        _raise(lib().bem_msh_elements(self._h, *(_ptr(out[k]) for k in (
            "tri", "tri_phys", "tri_geom", "quad", "quad_phys", "quad_geom"))), "bem_msh_elements")
        return out


def _raise(st, what):
    if st != BEM_OK:
        raise BemError(st, what)


def quads_to_triangles(quads) -> np.ndarray:
    """global::quadrilateralsToTriangles: M x 12 -> 2M x 9 (shorter diagonal)."""
    q = np.ascontiguousarray(quads, np.float64).reshape(-1, 12)
    out = np.zeros((2 * q.shape[0], 9))
    _raise(lib().bem_quads_to_triangles(_ptr(q), q.shape[0], _ptr(out)), "bem_quads_to_triangles")
    return out


def read_msh(path, include="all", exclude=""):
    """Triangles of a .msh file as the solver takes them: the selected
    triangles, then the selected quadrilaterals split in two; returns
    (tri, phys, geom)."""
    m = MshFile(path)
    sel = m.select(include, exclude)
    m.close()
    tri = np.vstack([sel["tri"], quads_to_triangles(sel["quad"])])
    phys = np.concatenate([sel["tri_phys"], np.repeat(sel["quad_phys"], 2)])
    geom = np.concatenate([sel["tri_geom"], np.repeat(sel["quad_geom"], 2)])
    return tri, phys, geom


def refine_triangles(tri, edge_length=None, mesh_frequency=None, c=343.0):
    """Longest-edge bisection of an Elements section (elementSection.cpp:
    688-800) to edge_length, or to (c / mesh_frequency) / 2 as
    solvingscriptreader.cpp:1113-1116 derives it; returns (triangles,
    parent index of each)."""
    if edge_length is None:
        if not mesh_frequency:
            raise BemError(BEM_EINVAL, "edge_length or mesh_frequency required")
        edge_length = (c / mesh_frequency) / 2
    t = np.ascontiguousarray(tri, np.float64).reshape(-1, 9)
    cnt = ct.c_int64()
    _raise(lib().bem_refine_triangles(_ptr(t), t.shape[0], float(edge_length), None, 0,
                                      ct.byref(cnt), None), "bem_refine_triangles")
    out = np.zeros((cnt.value, 9))
    parent = np.zeros(cnt.value, np.int64)
    _raise(lib().bem_refine_triangles(_ptr(t), t.shape[0], float(edge_length), _ptr(out),
                                      cnt.value, ct.byref(cnt), _ptr(parent)),
           "bem_refine_triangles")
    return out, parent


IMP_REFLECTION, IMP_DAMPING, IMP_IMPEDANCE, IMP_ADMITTANCE = 0, 1, 2, 3


def wall_beta(imp_type: int, value, normalized: bool = True, medium_impedance: float = 0.0):
    """beta of a wall section (a = i k beta, b = 1), WallImpedanceSection::setUpValues."""
    v = np.array([complex(value).real, complex(value).imag])
    b = np.zeros(2)
    _raise(lib().bem_wall_beta(imp_type, int(bool(normalized)), _ptr(v), medium_impedance,
                               _ptr(b)), "bem_wall_beta")
    return complex(b[0], b[1])


class mshReader:
    """Mirror of mshReader (mshreader.h): ``readMsh(filename, elementIndex,
    includeAll, include, exclude)`` fills ``triangles`` (N x 9),
    ``quadrilaterals`` (M x 12), ``physicalGroupsNames`` and
    ``physicalGroupsNumbers``; ``elementIndex`` is kept as the index the
    reference stamps on every element."""

    def __init__(self):
        self.triangles = np.zeros((0, 9))
        self.quadrilaterals = np.zeros((0, 12))
        self.physicalGroupsNames: list = []
        self.physicalGroupsNumbers: list = []
        self.elementIndex = 0

    def readMsh(self, filename, elementIndex=0, includeAll=True, include=(), exclude=()):
        self.elementIndex = elementIndex
        m = MshFile(filename)
        inc = list(include) + (["all"] if includeAll and not include else [])
        sel = m.select(inc, list(exclude))
        names = m.physical_names
        m.close()
        self.triangles, self.quadrilaterals = sel["tri"], sel["quad"]
        self.physicalGroupsNames = [n for _, _, n in names]
        self.physicalGroupsNumbers = [t for _, t, _ in names]
        return self


# ---------------------------------------------------------------------------
# Reference-named facade
# ---------------------------------------------------------------------------
@dataclass
class BemSolverParameters:
    """bemparameters.h:21-34 (+ the constants the reference hard-wires)."""
    hMatSolving: bool = True
    acaRelativeError: float = 0.01
    acaMaxRank: int = 0
    usePreconditioner: bool = False
    preconditionerRank: int = 2
    preconditionerRelError: float = 0.0
    coupling: int = 2  # KirkupCoupling
    leafSize: int = 32
    eta: float = 2.0
    gmresTolerance: float | None = None  # None: 1e-3 * acaRelativeError as the reference
    gmresRestart: int = 300
    gmresMaxIterations: int = 1000


@dataclass
class BoundaryElements:
    """Triangles (N x 9) and their Robin data a*phi + b*dphi/dn = g."""
    triangles: np.ndarray
    a: np.ndarray
    b: np.ndarray
    g: np.ndarray
    phiSolution: np.ndarray | None = None
    dPhiSolution: np.ndarray | None = None
    soundPressure: np.ndarray | None = None


@dataclass
class ObservationField:
    """ObservationField (ObservationScript/observationfield.h): observation
    triangles (M x 9); the field is evaluated at their midpoints."""
    triangles: np.ndarray
    phiSolution: np.ndarray | None = None
    soundPressure: np.ndarray | None = None

    def calculateTrianglesMidpoints(self) -> np.ndarray:
        """observationfield.cpp:4-11 with global::midpointOfTriangle
        (global.cpp:910-913): (node1 + node2 + node3) / 3."""
        t = np.asarray(self.triangles, np.float64).reshape(-1, 9)
        return (t[:, 0:3] + t[:, 3:6] + t[:, 6:9]) / 3.0


@dataclass
class BoundaryElementSolver:
    """Mirror of BoundaryElementSolver (boundaryelementsolver.h) for the
    H-matrix path: set ``boundaryElements``, ``frequency``, ``waveSpeed``,
    ``airDensity`` and call :meth:`calculateBoundarySolution`; then
    :meth:`calculateFieldSolution` fills ``observationFields``.
    ``pointSources``: rows (x, y, z, complex weight)."""
    boundaryElements: BoundaryElements
    frequency: float
    waveSpeed: float = 343.0
    airDensity: float = 1.2041
    bemSolverParameters: BemSolverParameters = field(default_factory=BemSolverParameters)
    observationFields: list = field(default_factory=list)
    pointSources: list = field(default_factory=list)
    info: dict | None = None
    _s: "Solver | None" = field(default=None, repr=False)

    def _solver(self) -> Solver:
        if self._s is not None:
            return self._s
        p = self.bemSolverParameters
        if not p.hMatSolving:
            raise BemError(BEM_EINVAL, "only the H-matrix path is accelerated")
        tol = p.gmresTolerance if p.gmresTolerance is not None else 1e-3 * p.acaRelativeError
        s = Solver(leaf_size=p.leafSize, eta=p.eta, aca_tol=p.acaRelativeError,
                   aca_max_rank=p.acaMaxRank, gmres_tol=tol, gmres_restart=p.gmresRestart,
                   gmres_maxit=p.gmresMaxIterations, coupling=p.coupling,
                   wave_speed=self.waveSpeed, density=self.airDensity,
                   use_preconditioner=int(p.usePreconditioner),
                   precond_rank=p.preconditionerRank, precond_tol=p.preconditionerRelError)
        s.set_mesh(self.boundaryElements.triangles)
        s.set_bc(self.boundaryElements.a, self.boundaryElements.b)
        if self.pointSources:
            s.set_point_sources(self.pointSources)
        self._s = s
        return s

    def calculateBoundarySolution(self):
        s = self._solver()
        phi, dphi, p, info = s.solve(self.frequency, self.boundaryElements.g)
        be = self.boundaryElements
        be.phiSolution, be.dPhiSolution, be.soundPressure = phi[:, 0], dphi[:, 0], p[:, 0]
        self.info = info
        return info

    hMatrixSolve = calculateBoundarySolution

    def calculateFieldSolution(self):
        """calculateFieldSolution (boundaryelementsolver.cpp:2192-2249):
        phiSolution and soundPressure of every observation field from the
        boundary solution and the point sources (bem_field)."""
        be = self.boundaryElements
        if be.phiSolution is None or be.dPhiSolution is None:
            raise BemError(BEM_EINVAL, "no boundary solution")
        s = self._solver()
        for f in self.observationFields:
            pf, pp = s.field(self.frequency, f.calculateTrianglesMidpoints(), be.phiSolution,
                             be.dPhiSolution, self.pointSources)
            f.phiSolution, f.soundPressure = pf[:, 0], pp[:, 0]

    def close(self):
        if self._s is not None:
            self._s.close()
            self._s = None


class HMatrix:
    """An assembled H-matrix living on the GPU (``which`` 0 = phi, 1 = dPhi)."""

    def __init__(self, solver: Solver, which: int):
        self.solver, self.which = solver, which


class HArithm:
    @staticmethod
    def MVM(y: np.ndarray, hmatrix: HMatrix, x: np.ndarray) -> np.ndarray:
        """y += H x (harithm.cpp:3-28); returns the updated y."""
        return hmatrix.solver.hmatvec(hmatrix.which, x, y, accumulate=True)


class GMRES:
    @staticmethod
    def gmresSolve(A: HMatrix, xGuess, b):
        """GMRES on the assembled system matrix (gmres.h:170-180); the
        tolerance and restart come from the solver configuration."""
        x, info = A.solver.gmres(b, xGuess)
        return x
