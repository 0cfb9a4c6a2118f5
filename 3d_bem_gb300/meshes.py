"""Seeded synthetic surface meshes for the benchmark and test workloads.

No mesh files ship with the library; every workload is generated here from a
seed so that the GPU run and the CPU oracle see the same triangles.  Triangles
are returned as ``(N, 9)`` float64 arrays (node1 xyz, node2 xyz, node3 xyz),
counter-clockwise seen from outside the body, so the normal
``(n2 - n1) x (n3 - n1)`` points into the acoustic medium
(global.cpp:903-908 uses the same orientation rule).
"""
from __future__ import annotations

import numpy as np


def icosphere(subdivisions: int, radius: float = 1.0) -> np.ndarray:
    """Icosahedron refined ``subdivisions`` times (20 * 4**s triangles)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
             (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
             (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
             (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
             (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    V = [np.array(v, float) / np.linalg.norm(v) for v in verts]
    F = list(faces)
    for _ in range(subdivisions):
        cache = {}

        def mid(i, j):
            key = (min(i, j), max(i, j))
            if key not in cache:
                m = V[i] + V[j]
                V.append(m / np.linalg.norm(m))
                cache[key] = len(V) - 1
            return cache[key]

        F2 = []
        for (a, b, c) in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            F2 += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = F2
    V = np.array(V) * radius
    F = np.array(F)
    tri = np.concatenate([V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]], axis=1)
    # orient outward
    n = np.cross(tri[:, 3:6] - tri[:, 0:3], tri[:, 6:9] - tri[:, 0:3])
    c = (tri[:, 0:3] + tri[:, 3:6] + tri[:, 6:9]) / 3.0
    flip = (n * c).sum(1) < 0
    tri[flip] = np.concatenate([tri[flip, 0:3], tri[flip, 6:9], tri[flip, 3:6]], axis=1)
    return np.ascontiguousarray(tri)


def _grid_face(origin, e1, e2, n1, n2, rng, jitter):
    """Structured triangulation of a rectangle with jittered interior nodes."""
    xs = np.linspace(0.0, 1.0, n1 + 1)
    ys = np.linspace(0.0, 1.0, n2 + 1)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    dx, dy = 1.0 / n1, 1.0 / n2
    inner = (X > 0) & (X < 1) & (Y > 0) & (Y < 1)
    X = X + inner * rng.uniform(-jitter, jitter, X.shape) * dx
    Y = Y + inner * rng.uniform(-jitter, jitter, Y.shape) * dy
    P = origin[None, None, :] + X[..., None] * e1[None, None, :] + Y[..., None] * e2[None, None, :]
    tris = []
    for i in range(n1):
        for j in range(n2):
            a, b, c, d = P[i, j], P[i + 1, j], P[i + 1, j + 1], P[i, j + 1]
            if (i + j) % 2 == 0:
                tris += [np.r_[a, b, c], np.r_[a, c, d]]
            else:
                tris += [np.r_[a, b, d], np.r_[b, c, d]]
    return np.array(tris)


def _box_cells(L, n_target, exact):
    """Cells per axis (nx, ny, nz) of the box grids: rounded from a uniform
    spacing, or, with ``exact``, the nearby triple whose total
    4 (nx ny + ny nz + nx nz) equals ``n_target`` with the most uniform
    spacing (the rounded triple when no such triple is near)."""
    area = 2 * (L[0] * L[1] + L[1] * L[2] + L[0] * L[2])
    h = (2.0 * area / n_target) ** 0.5
    ideal = [x / h for x in L]
    base = [max(1, round(v)) for v in ideal]
    if not exact or n_target % 4:
        return base
    best, score = None, None
    rng3 = [range(max(1, b - 3), b + 4) for b in base]
    for nx in rng3[0]:
        for ny in rng3[1]:
            for nz in rng3[2]:
                if 4 * (nx * ny + ny * nz + nx * nz) != n_target:
                    continue
                sp = [L[0] / nx, L[1] / ny, L[2] / nz]
                s = max(sp) / min(sp)
                if score is None or s < score:
                    best, score = [nx, ny, nz], s
    return best if best is not None else base


def box(lx=0.3, ly=0.2, lz=0.4, n_target=5120, seed=20260103, jitter=0.25,
        exact=False) -> np.ndarray:
    """Closed box surface with seeded jittered triangulation of every face.

    The face grids are sized so the total is close to ``n_target`` triangles
    (exactly ``n_target`` with ``exact`` when a grid of near-uniform spacing
    has that count) with near-uniform element size; interior nodes are
    jittered by up to ``jitter`` of the local spacing (edge nodes stay put so
    faces conform).
    """
    rng = np.random.default_rng(seed)
    faces = []
    dims = {(0, 1): (lx, ly), (1, 2): (ly, lz), (0, 2): (lx, lz)}
    cells = _box_cells([lx, ly, lz], n_target, exact)
    counts = {(i, j): (cells[i], cells[j]) for (i, j) in dims}
    E = np.eye(3)
    L = np.array([lx, ly, lz])
    for (i, j), (n1, n2) in counts.items():
        k = 3 - i - j
        for side in (0, 1):
            origin = np.zeros(3)
            origin[k] = side * L[k]
            e1, e2 = E[i] * L[i], E[j] * L[j]
            f = _grid_face(origin, e1, e2, n1, n2, rng, jitter)
            faces.append(f)
    tri = np.concatenate(faces)
    # orient outward with respect to the box centre
    ctr = L / 2
    n = np.cross(tri[:, 3:6] - tri[:, 0:3], tri[:, 6:9] - tri[:, 0:3])
    c = (tri[:, 0:3] + tri[:, 3:6] + tri[:, 6:9]) / 3.0 - ctr
    flip = (n * c).sum(1) < 0
    tri[flip] = np.concatenate([tri[flip, 0:3], tri[flip, 6:9], tri[flip, 3:6]], axis=1)
    return np.ascontiguousarray(tri)


def pencil(radius=0.004, length=0.2, tip=0.01, n_target=81920, seed=20260105,
           jitter=0.05) -> np.ndarray:
    """Cylinder with a flat back cap and a conical tip, structured rings.

    ``n_target`` triangles are split between the cylinder, the cone and the cap
    in proportion to their areas; ring nodes are jittered by up to ``jitter`` of
    the local spacing along the axis and around the ring. The mesh has
    2 m (nz + ncone + ncap - 1) triangles for m nodes around; m is taken among
    the divisors of n_target / 2 within 25 % of the uniform spacing, so that
    the count is exactly ``n_target`` (81,920: m = 64), else rounded.
    """
    rng = np.random.default_rng(seed)
    cone_slant = (tip ** 2 + radius ** 2) ** 0.5
    a_cyl = 2 * np.pi * radius * length
    a_cone = np.pi * radius * cone_slant
    a_cap = np.pi * radius ** 2
    total = a_cyl + a_cone + a_cap
    h = (2.0 * total / n_target) ** 0.5
    m0 = 2 * np.pi * radius / h
    m = max(8, int(round(m0)))  # nodes around
    divs = [d for d in range(8, int(1.25 * m0) + 1)
            if n_target % 2 == 0 and (n_target // 2) % d == 0 and d >= 0.8 * m0]
    ncone = max(1, int(round((n_target * a_cone / total) / (2 * m))))
    ncap = max(1, int(round((n_target * a_cap / total) / (2 * m))))
    nz = max(1, int(round((n_target * a_cyl / total) / (2 * m))))
    if divs:
        m = min(divs, key=lambda d: abs(d - m0))
        rings_total = n_target // (2 * m) + 1  # nz + ncone + ncap
        ncone = max(1, int(round((n_target * a_cone / total) / (2 * m))))
        ncap = max(1, int(round((n_target * a_cap / total) / (2 * m))))
        nz = rings_total - ncone - ncap
        if nz < 1:
            raise ValueError("pencil: n_target too small for the cone and cap rings")
    ang = 2 * np.pi * np.arange(m) / m

    def ring(z, r, jit_axis, jit_ang):
        a = ang + (rng.uniform(-jit_ang, jit_ang, m) * 2 * np.pi / m if jit_ang else 0)
        zz = z + (rng.uniform(-jit_axis, jit_axis, m) if jit_axis else 0)
        return np.stack([r * np.cos(a), r * np.sin(a), np.broadcast_to(zz, (m,))], axis=1)

    rings = []
    dz = length / nz
    for i in range(nz + 1):
        edge = i == 0 or i == nz
        rings.append(ring(i * dz, radius, 0 if edge else jitter * dz, 0 if edge else jitter))
    # cone rings from z = length to the apex
    for i in range(1, ncone):
        s = i / ncone
        rings.append(ring(length + s * tip, radius * (1 - s), jitter * tip / ncone, jitter))
    tris = []
    for i in range(len(rings) - 1):
        A, B = rings[i], rings[i + 1]
        for j in range(m):
            j2 = (j + 1) % m
            tris += [np.r_[A[j], A[j2], B[j2]], np.r_[A[j], B[j2], B[j]]]
    apex = np.array([0.0, 0.0, length + tip])
    last = rings[-1]
    for j in range(m):
        tris.append(np.r_[last[j], last[(j + 1) % m], apex])
    # back cap at z = 0: concentric rings
    cap_rings = [rings[0]]
    for i in range(1, ncap):
        r = radius * (1 - i / ncap)
        cap_rings.append(ring(0.0, r, 0, jitter))
    for i in range(len(cap_rings) - 1):
        A, B = cap_rings[i], cap_rings[i + 1]
        for j in range(m):
            j2 = (j + 1) % m
            tris += [np.r_[A[j], B[j2], A[j2]], np.r_[A[j], B[j], B[j2]]]
    centre = np.zeros(3)
    lastc = cap_rings[-1]
    for j in range(m):
        tris.append(np.r_[lastc[j], centre, lastc[(j + 1) % m]])
    tri = np.array(tris)
    # orient outward: normal away from the axis (side) or along -z (cap)
    n = np.cross(tri[:, 3:6] - tri[:, 0:3], tri[:, 6:9] - tri[:, 0:3])
    c = (tri[:, 0:3] + tri[:, 3:6] + tri[:, 6:9]) / 3.0
    ref = c - np.array([0.0, 0.0, length * 0.5])
    flip = (n * ref).sum(1) < 0
    tri[flip] = np.concatenate([tri[flip, 0:3], tri[flip, 6:9], tri[flip, 3:6]], axis=1)
    return np.ascontiguousarray(tri)


def random_patches(tri: np.ndarray, count: int, frac: float, seed: int) -> np.ndarray:
    """Seeded random-velocity patches: each column drives a random ~frac of
    the elements (nearest to a random centre) with velocities in [-1, 1]."""
    rng = np.random.default_rng(seed)
    c = (tri[:, 0:3] + tri[:, 3:6] + tri[:, 6:9]) / 3.0
    n = tri.shape[0]
    out = np.zeros((n, count), np.complex128)
    k = max(1, int(round(frac * n)))
    for r in range(count):
        ctr = c[rng.integers(n)]
        idx = np.argsort(((c - ctr) ** 2).sum(1))[:k]
        out[idx, r] = rng.uniform(-1.0, 1.0, k)
    return out


def box_piston_rhs(tri: np.ndarray, lx=0.3, ly=0.2, lz=0.4, radius=0.05, patches=3,
                   seed=20260103) -> np.ndarray:
    """Driving velocities of the box sweep: column 0 is a circular piston of
    the given radius centred on the z = lz face (unit velocity), columns
    1..patches are seeded random-velocity patches on ~5 % of the elements."""
    c = (tri[:, 0:3] + tri[:, 3:6] + tri[:, 6:9]) / 3.0
    on_face = np.abs(c[:, 2] - lz) < 1e-9 * max(lx, ly, lz)
    r = np.hypot(c[:, 0] - lx / 2, c[:, 1] - ly / 2)
    g = np.zeros((tri.shape[0], 1 + patches), np.complex128)
    g[on_face & (r <= radius), 0] = 1.0
    if patches:
        g[:, 1:] = random_patches(tri, patches, 0.05, seed)
    return g


def log_frequencies(count=64, f0=50.0, f1=2000.0) -> np.ndarray:
    """count log-spaced frequencies from f0 to f1 (Hz)."""
    return np.exp(np.linspace(np.log(f0), np.log(f1), count))


def pencil_rhs(tri: np.ndarray, radius=0.004, patches=7, seed=20260105) -> np.ndarray:
    """Driving data of the pencil sweep: column 0 is g = 1 on the outer ring
    of the back cap (z = 0, r > radius / 2), columns 1..patches are seeded
    random-velocity patches on ~5 % of the elements."""
    c = (tri[:, 0:3] + tri[:, 3:6] + tri[:, 6:9]) / 3.0
    on_cap = np.abs(c[:, 2]) < 1e-12
    ring = on_cap & (np.hypot(c[:, 0], c[:, 1]) > 0.5 * radius)
    g = np.zeros((tri.shape[0], 1 + patches), np.complex128)
    g[ring, 0] = 1.0
    if patches:
        g[:, 1:] = random_patches(tri, patches, 0.05, seed)
    return g


def wall_admittance(n: int, seed=20260105, zmin=0.5, zmax=50.0) -> np.ndarray:
    """Seeded per-element admittance ratios beta = rho c / Z with the wall
    impedance Z log-uniform in [zmin, zmax] rho c (real, resistive walls)."""
    rng = np.random.default_rng(seed)
    z = np.exp(rng.uniform(np.log(zmin), np.log(zmax), n))
    return (1.0 / z).astype(np.complex128)
