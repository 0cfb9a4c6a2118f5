"""ctypes binding of the CPU FP64 oracle (test infrastructure only).

Only the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module; the GPU library never does.  See
``bem_oracle.h`` for the reference functions each entry point restates.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libbem_oracle.so")
_lib = None

I64P = ct.POINTER(ct.c_int64)
F64P = ct.POINTER(ct.c_double)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (a few seconds; make skips an
    up-to-date library)."""
    if force:
        subprocess.run(["make", "-s", "-C", _HERE, "clean"], check=True)
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ct.CDLL(_LIB_PATH)
        vp = ct.c_void_p
        L.orc_create.restype = vp
        L.orc_create.argtypes = [F64P, ct.c_int64, ct.c_int64, ct.c_double]
        L.orc_destroy.argtypes = [vp]
        L.orc_n.restype = ct.c_int64
        L.orc_n.argtypes = [vp]
        L.orc_perm.argtypes = [vp, I64P]
        L.orc_num_clusters.restype = ct.c_int64
        L.orc_num_clusters.argtypes = [vp]
        L.orc_clusters.argtypes = [vp, I64P, F64P]
        L.orc_num_blocks.restype = ct.c_int64
        L.orc_num_blocks.argtypes = [vp]
        L.orc_blocks.argtypes = [vp, I64P]
        L.orc_geometry.argtypes = [vp, F64P, F64P, F64P, F64P]
        L.orc_operators.argtypes = [vp, ct.c_double, I64P, I64P, ct.c_int64, F64P]
        L.orc_entries.argtypes = [vp, ct.c_double, ct.c_int, F64P, F64P, I64P, I64P,
                                  ct.c_int64, F64P, F64P]
        L.orc_hassemble.restype = vp
        L.orc_hassemble.argtypes = [vp, ct.c_double, ct.c_int, F64P, F64P, ct.c_int,
                                    ct.c_double, ct.c_int64, ct.c_uint64, ct.c_int]
        L.orc_hdestroy.argtypes = [vp]
        L.orc_hmatvec.argtypes = [vp, F64P, F64P]
        L.orc_hdense.argtypes = [vp, F64P]
        L.orc_hranks.argtypes = [vp, I64P]
        L.orc_hblock.restype = ct.c_int64
        L.orc_hblock.argtypes = [vp, ct.c_int64, F64P, F64P, F64P, F64P]
        L.orc_hrecompress.argtypes = [vp, ct.c_int64, ct.c_double]
        L.orc_hassemble_points.restype = vp
        L.orc_hassemble_points.argtypes = [F64P, ct.c_int64, F64P, ct.c_int64, ct.c_double,
                                           ct.c_int64, ct.c_double, ct.c_double, ct.c_int64,
                                           ct.c_uint64, I64P, I64P]
        L.orc_gmres.restype = ct.c_int64
        L.orc_gmres.argtypes = [vp, F64P, F64P, ct.c_double, ct.c_int64, ct.c_int64, F64P]
        L.orc_lower_solve.argtypes = [ct.c_int64, ct.c_int64, I64P, F64P, F64P, F64P]
        L.orc_upper_solve.argtypes = [ct.c_int64, ct.c_int64, I64P, F64P, F64P, F64P]
        L.orc_solve.restype = ct.c_int
        L.orc_solve.argtypes = [vp, ct.c_double, ct.c_double, ct.c_double, ct.c_int, F64P, F64P,
                                F64P, ct.c_int64, ct.c_double, ct.c_int64, ct.c_double,
                                ct.c_int64, ct.c_int64, ct.c_uint64, ct.c_int, F64P, F64P,
                                F64P, F64P]
        L.orc_solve_precond.restype = ct.c_int
        L.orc_solve_precond.argtypes = [vp, ct.c_double, ct.c_double, ct.c_double, ct.c_int, F64P,
                                        F64P, F64P, ct.c_int64, ct.c_double, ct.c_int64,
                                        ct.c_double, ct.c_int64, ct.c_int64, ct.c_uint64, ct.c_int,
                                        ct.c_int64, ct.c_double, F64P, F64P, F64P, F64P]
        L.orc_hlu_factor.restype = vp
        L.orc_hlu_factor.argtypes = [vp, vp, ct.c_int64, ct.c_double]
        L.orc_hlu_sizes.argtypes = [vp, I64P]
        L.orc_hlu_get.argtypes = [vp, I64P, F64P, I64P, F64P]
        L.orc_hlu_free.argtypes = [vp]
        L.orc_dense.argtypes = [vp, ct.c_double, ct.c_int, F64P, F64P, F64P, F64P, ct.c_int]
        L.orc_triangle_rule.restype = ct.c_int64
        L.orc_triangle_rule.argtypes = [ct.c_int64, F64P]
        L.orc_line_rule.restype = ct.c_int64
        L.orc_line_rule.argtypes = [ct.c_int64, F64P]
        L.orc_field.argtypes = [F64P, ct.c_int64, ct.c_double, ct.c_double, ct.c_double,
                                F64P, ct.c_int64, F64P, F64P, ct.c_int64, F64P, ct.c_int64,
                                F64P, ct.c_int, F64P, F64P]
        L.orc_set_plane.argtypes = [vp, F64P, F64P]
        L.orc_set_sources.argtypes = [vp, F64P, ct.c_int64]
        L.orc_pivot_hash.restype = ct.c_uint64
        L.orc_pivot_hash.argtypes = [ct.c_uint64, ct.c_uint64, ct.c_uint64]
        _lib = L
    return _lib


def _f(a):
    return a.ctypes.data_as(F64P)


def _i(a):
    return a.ctypes.data_as(I64P)


def _c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


class Problem:
    """Mesh + cluster tree + partition, as ``hMatrixSolve`` builds them."""

    def __init__(self, tri: np.ndarray, leaf: int = 32, eta: float = 2.0):
        L = lib()
        self.tri = np.ascontiguousarray(tri, dtype=np.float64).reshape(-1, 9)
        self.n = self.tri.shape[0]
        self._h = L.orc_create(_f(self.tri), self.n, leaf, eta)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def set_sources(self, sources=None):
        """Point sources of the right-hand side: rows (x, y, z, complex weight)."""
        src = np.zeros((0, 5))
        if sources is not None and len(sources):
            q = np.asarray(sources, np.complex128).reshape(-1, 4)
            src = np.column_stack([q[:, :3].real, q[:, 3].real, q[:, 3].imag])
        src = np.ascontiguousarray(src, np.float64)
        lib().orc_set_sources(self._h, _f(src), src.shape[0])

    def set_plane(self, point=None, normal=None):
        """One impedance plane (None removes it)."""
        if normal is None:
            lib().orc_set_plane(self._h, None, None)
            return
        p = np.ascontiguousarray(point, np.float64)
        n = np.ascontiguousarray(normal, np.float64)
        lib().orc_set_plane(self._h, _f(p), _f(n))

    @property
    def perm(self):
        p = np.zeros(self.n, np.int64)
        lib().orc_perm(self._h, _i(p))
        return p

    def clusters(self):
        nc = lib().orc_num_clusters(self._h)
        info = np.zeros((nc, 6), np.int64)
        boxes = np.zeros((nc, 6), np.float64)
        lib().orc_clusters(self._h, _i(info), _f(boxes))
        return info, boxes

    def blocks(self):
        nb = lib().orc_num_blocks(self._h)
        info = np.zeros((nb, 5), np.int64)
        lib().orc_blocks(self._h, _i(info))
        return info

    def geometry(self):
        n = self.n
        nrm = np.zeros((n, 3))
        area = np.zeros(n)
        col = np.zeros((n, 3))
        avg = np.zeros(1)
        lib().orc_geometry(self._h, _f(nrm), _f(area), _f(col), _f(avg))
        return nrm, area, col, float(avg[0])

    def operators(self, k, rows, cols):
        rows = np.ascontiguousarray(rows, np.int64)
        cols = np.ascontiguousarray(cols, np.int64)
        out = np.zeros((rows.size, 4), np.complex128)
        lib().orc_operators(self._h, k, _i(rows), _i(cols), rows.size, _f(out))
        return out

    def entries(self, k, coupling, a, b, rows, cols):
        """a, b in cluster order."""
        rows = np.ascontiguousarray(rows, np.int64)
        cols = np.ascontiguousarray(cols, np.int64)
        a, b = _c128(a), _c128(b)
        phi = np.zeros(rows.size, np.complex128)
        dphi = np.zeros(rows.size, np.complex128)
        lib().orc_entries(self._h, k, coupling, _f(a), _f(b), _i(rows), _i(cols), rows.size,
                          _f(phi), _f(dphi))
        return phi, dphi

    def dense(self, k, coupling, a, b, nthreads=0):
        n = self.n
        a, b = _c128(a), _c128(b)
        phi = np.zeros((n, n), np.complex128, order="F")
        dphi = np.zeros((n, n), np.complex128, order="F")
        lib().orc_dense(self._h, k, coupling, _f(a), _f(b), _f(phi), _f(dphi), nthreads)
        return phi, dphi

    def hassemble(self, k, coupling, a, b, which, tol, max_rank=0, seed=1234, nthreads=0):
        a, b = _c128(a), _c128(b)
        h = lib().orc_hassemble(self._h, k, coupling, _f(a), _f(b), which, tol, max_rank,
                                seed, nthreads)
        return HMatrix(h, self.n, self.n, self.blocks())

    def solve(self, freq, c, rho, coupling, a, b, g, aca_tol, gmres_tol, max_rank=0,
              restart=300, maxit=1000, seed=1234, nthreads=0, precond_rank=0, precond_tol=0.0):
        """Whole frequency solve; a, b, g in caller order; g is N x R. With
        precond_rank >= 1 GMRES runs on the H-LU preconditioned system (the
        reference's usePreconditioner)."""
        n = self.n
        g = np.asfortranarray(np.asarray(g, np.complex128).reshape(n, -1))
        R = g.shape[1]
        a, b = _c128(a), _c128(b)
        phi = np.zeros((n, R), np.complex128, order="F")
        dphi = np.zeros((n, R), np.complex128, order="F")
        p = np.zeros((n, R), np.complex128, order="F")
        st = np.zeros(9)
        lib().orc_solve_precond(self._h, freq, c, rho, coupling, _f(a), _f(b), _f(g), R, aca_tol,
                                max_rank, gmres_tol, restart, maxit, seed, nthreads, precond_rank,
                                precond_tol, _f(phi), _f(dphi), _f(p), _f(st))
        keys = ["t_assemble_phi", "t_rhs", "t_assemble_dphi", "t_gmres", "iters",
                "rel_resid", "t_total", "max_rank", "t_factor"]
        return phi, dphi, p, dict(zip(keys, st.tolist()))

    def hlu(self, hmat, rank, tol=0.0):
        """H-LU factors of an assembled H-matrix of this problem: (L leaves,
        L data, U leaves, U data), leaves as rows r0, m, c0, n, kind, rank,
        offset (the format of bem_hlu_export)."""
        f = lib().orc_hlu_factor(self._h, hmat._h, rank, tol)
        try:
            sz = np.zeros(4, np.int64)
            lib().orc_hlu_sizes(f, _i(sz))
            Ll = np.zeros((sz[0], 7), np.int64)
            Ld = np.zeros(sz[1], np.complex128)
            Ul = np.zeros((sz[2], 7), np.int64)
            Ud = np.zeros(sz[3], np.complex128)
            lib().orc_hlu_get(f, _i(Ll), _f(Ld), _i(Ul), _f(Ud))
        finally:
            lib().orc_hlu_free(f)
        return Ll, Ld, Ul, Ud


class HMatrix:
    def __init__(self, h, nr, nc, blocks):
        self._h = h
        self.nr, self.nc = nr, nc
        self.blocks = blocks

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_hdestroy(self._h)
            self._h = None

    def matvec(self, x, y=None):
        x = _c128(x)
        y = np.zeros(self.nr, np.complex128) if y is None else _c128(y).copy()
        lib().orc_hmatvec(self._h, _f(x), _f(y))
        return y

    def dense(self):
        out = np.zeros((self.nr, self.nc), np.complex128, order="F")
        lib().orc_hdense(self._h, _f(out))
        return out

    def ranks(self):
        r = np.zeros(len(self.blocks), np.int64)
        lib().orc_hranks(self._h, _i(r))
        return r

    def block(self, i):
        r0, m, c0, n, adm = self.blocks[i]
        if adm:
            k = int(self.ranks()[i])
            U = np.zeros((k, m), np.complex128)  # columns stored contiguously
            s = np.zeros(k, np.complex128)
            V = np.zeros((k, n), np.complex128)
            lib().orc_hblock(self._h, i, _f(U), _f(s), _f(V), None)
            return U.T.copy(), s, V
        F = np.zeros((n, m), np.complex128)
        lib().orc_hblock(self._h, i, None, None, None, _f(F))
        return F.T.copy()

    def recompress(self, rank, tol):
        lib().orc_hrecompress(self._h, rank, tol)

    def gmres(self, b, x0=None, tol=1e-8, restart=300, maxit=1000):
        b = _c128(b)
        x = np.zeros(self.nr, np.complex128) if x0 is None else _c128(x0).copy()
        res = np.zeros(1)
        it = lib().orc_gmres(self._h, _f(b), _f(x), tol, restart, maxit, _f(res))
        return x, int(it), float(res[0])


def hassemble_points(rowpts, colpts, k, leaf, eta, tol, max_rank=0, seed=1234):
    rowpts = np.ascontiguousarray(rowpts, np.float64)
    colpts = np.ascontiguousarray(colpts, np.float64)
    nr, nc = rowpts.shape[0], colpts.shape[0]
    rp = np.zeros(nr, np.int64)
    cp = np.zeros(nc, np.int64)
    h = lib().orc_hassemble_points(_f(rowpts), nr, _f(colpts), nc, k, leaf, eta, tol, max_rank,
                                   seed, _i(rp), _i(cp))
    return HMatrix(h, nr, nc, None), rp, cp


def lower_solve(n, blocks, data, b):
    blocks = np.ascontiguousarray(blocks, np.int64)
    data = _c128(data)
    b = _c128(b)
    y = np.zeros(n, np.complex128)
    lib().orc_lower_solve(n, blocks.shape[0], _i(blocks), _f(data), _f(b), _f(y))
    return y


def upper_solve(n, blocks, data, y):
    blocks = np.ascontiguousarray(blocks, np.int64)
    data = _c128(data)
    y = _c128(y)
    x = np.zeros(n, np.complex128)
    lib().orc_upper_solve(n, blocks.shape[0], _i(blocks), _f(data), _f(y), _f(x))
    return x


def triangle_rule(order):
    out = np.zeros((64, 3))
    n = lib().orc_triangle_rule(order, _f(out))
    return out[:n].copy()


def line_rule(n):
    out = np.zeros((32, 2))
    k = lib().orc_line_rule(n, _f(out))
    return out[:k].copy()


def field(tri, freq, pts, phi, dphi, sources=None, c=343.0, rho=1.2041, nthreads=0,
          plane=None):
    """Velocity potential and sound pressure at observation points (npts x R
    each) from a boundary solution phi, dphi (n x R, caller order); sources:
    rows (x, y, z, complex weight)."""
    tri = np.ascontiguousarray(tri, np.float64)
    n = tri.shape[0]
    pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
    phi = np.asfortranarray(np.asarray(phi, np.complex128).reshape(n, -1))
    dphi = np.asfortranarray(np.asarray(dphi, np.complex128).reshape(n, -1))
    R = phi.shape[1]
    src = np.zeros((0, 5))
    if sources is not None and len(sources):
        s = np.asarray(sources, np.complex128).reshape(-1, 4)
        src = np.column_stack([s[:, :3].real, s[:, 3].real, s[:, 3].imag])
    src = np.ascontiguousarray(src, np.float64)
    pf = np.zeros((pts.shape[0], R), np.complex128, order="F")
    pp = np.zeros((pts.shape[0], R), np.complex128, order="F")
    # complex arrays are passed by their data pointers (interleaved re, im)
    pl = None if plane is None else np.ascontiguousarray(np.concatenate(
        [np.asarray(plane[0], np.float64).ravel(), np.asarray(plane[1], np.float64).ravel()]))
    lib().orc_field(_f(tri), n, freq, c, rho, _f(pts), pts.shape[0], _f(phi), _f(dphi), R,
                    _f(src), src.shape[0], _f(pl) if pl is not None else None, nthreads,
                    _f(pf), _f(pp))
    return pf, pp


def pivot_hash(seed, a, b):
    return int(lib().orc_pivot_hash(seed, a, b))
