"""Near-field triangle pairs for the learned quadrature-order selector.

Pairs are drawn from seeded jittered surface patches: a planar grid of
triangles, interior vertices jittered by up to 20 % of the edge length,
stretched anisotropically (aspect 1-8), optionally bent onto a cylinder, and
placed with a random rotation. From each patch the (collocation triangle P,
source triangle Q) pairs are binned by centroid distance over sqrt(area Q)
and drawn evenly over [0, 3] (two thirds of the pairs) and [3, 10] (the rest,
the distances that the inadmissible blocks of leaf-32 cluster trees reach),
each with a wavenumber k from kh log-uniform in [0.01, 1.5], h = sqrt(area Q).
"""
from __future__ import annotations

import numpy as np

SEED = 20260105


def _rotation(rng):
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def patch(rng, nv=11):
    """Triangles (T x 3 x 3) of one jittered, stretched, possibly bent patch."""
    x, y = np.meshgrid(np.arange(nv, dtype=float), np.arange(nv, dtype=float), indexing="ij")
    x = x + 0.5 * (np.arange(nv)[None, :] % 2)  # staggered rows: near-equilateral
    y = y * np.sqrt(3) / 2
    inner = (np.arange(nv)[:, None] > 0) & (np.arange(nv)[:, None] < nv - 1) \
        & (np.arange(nv)[None, :] > 0) & (np.arange(nv)[None, :] < nv - 1)
    r = rng.uniform(0, 0.2, (nv, nv)) * inner
    th = rng.uniform(0, 2 * np.pi, (nv, nv))
    x = x + r * np.cos(th)
    y = y + r * np.sin(th)
    aspect = rng.uniform(1, 8)
    phi = rng.uniform(0, np.pi)
    c, s = np.cos(phi), np.sin(phi)
    u = c * x + s * y
    v = -s * x + c * y
    u = u * aspect
    z = np.zeros_like(u)
    if rng.random() < 0.5:  # bend onto a cylinder around the v axis
        R = rng.uniform(3, 60) * aspect
        ang = u / R
        u, z = R * np.sin(ang), R * (1 - np.cos(ang))
    P = np.stack([u, v, z], -1) @ _rotation(rng).T
    idx = np.arange(nv * nv).reshape(nv, nv)
    tris = []
    for i in range(nv - 1):
        for j in range(nv - 1):
            a, b, cc, d = idx[i, j], idx[i + 1, j], idx[i, j + 1], idx[i + 1, j + 1]
            tris += [(a, b, d), (a, d, cc)]
    tris = np.array(tris)
    flat = P.reshape(-1, 3)
    return flat[tris]


def pairs(n, seed=SEED, near_frac=2 / 3, max_patches=100000):
    """n pairs: (P triangles n x 9, Q triangles n x 9, k n, d/h n).

    Each distance bin has a quota; bins that the patches rarely reach (very
    short distances need strongly stretched patches) hand their shortfall to
    the other bins of the same range once the rest is full."""
    rng = np.random.default_rng(seed)
    n_near = int(round(n * near_frac))
    edges = [np.linspace(0.0, 3.0, 13), np.linspace(3.0, 10.0, 15)]
    totals = (n_near, n - n_near)
    quota = []
    for part in (0, 1):
        nb = len(edges[part]) - 1
        q = np.full(nb, totals[part] // nb)
        q[: totals[part] - q.sum()] += 1
        quota.append(q)
    pools = [[[] for _ in q] for q in quota]
    count = [np.zeros_like(q) for q in quota]
    patches_at_full = None
    for it in range(max_patches):
        if all((c >= 2 * q).all() for c, q in zip(count, quota)):
            break
        ok = all(np.minimum(c, q).sum() + np.minimum(np.maximum(c - q, 0), q).sum() >= t
                 for c, q, t in zip(count, quota, totals))
        if ok and patches_at_full is None:
            patches_at_full = it
        if patches_at_full is not None and it >= 2 * patches_at_full + 10:
            break
        T = patch(rng)
        c = T.mean(1)
        area = 0.5 * np.linalg.norm(np.cross(T[:, 1] - T[:, 0], T[:, 2] - T[:, 0]), axis=1)
        i, j = np.divmod(rng.permutation(len(T) * len(T)), len(T))
        keep = i != j
        i, j = i[keep], j[keep]
        dh = np.linalg.norm(c[i] - c[j], axis=1) / np.sqrt(area[j])
        for part in (0, 1):
            b = np.digitize(dh, edges[part]) - 1
            valid = (b >= 0) & (b < len(quota[part]))
            order = np.argsort(b[valid], kind="stable")
            bs = b[valid][order]
            ids = np.flatnonzero(valid)[order]
            starts = np.searchsorted(bs, np.arange(len(quota[part]) + 1))
            for q in range(len(quota[part])):
                room = 2 * quota[part][q] - count[part][q]
                sel = ids[starts[q]:starts[q + 1]][: min(max(room, 0), 256)]
                if sel.size:
                    pools[part][q].append((T[i[sel]], T[j[sel]], dh[sel]))
                    count[part][q] += sel.size
    Ps, Qs, Ds = [], [], []
    for part in (0, 1):
        take = np.minimum(count[part], quota[part])
        short = totals[part] - take.sum()
        while short > 0:  # hand the shortfall to bins with surplus
            extra = count[part] - take
            live = np.flatnonzero(extra > 0)
            if live.size == 0:
                break
            add = np.minimum(extra[live], max(1, short // live.size))
            add[np.cumsum(add) > short] = 0
            if add.sum() == 0:
                add[0] = min(extra[live[0]], short)
            take[live] += add
            short -= int(add.sum())
        for q in range(len(quota[part])):
            if take[q] == 0:
                continue
            Ps.append(np.concatenate([g[0] for g in pools[part][q]])[: take[q]])
            Qs.append(np.concatenate([g[1] for g in pools[part][q]])[: take[q]])
            Ds.append(np.concatenate([g[2] for g in pools[part][q]])[: take[q]])
    Pt = np.concatenate(Ps).reshape(-1, 9)
    Qt = np.concatenate(Qs).reshape(-1, 9)
    dh = np.concatenate(Ds)
    order = rng.permutation(len(dh))
    Pt, Qt, dh = Pt[order], Qt[order], dh[order]
    hq = np.sqrt(0.5 * np.linalg.norm(np.cross(Qt[:, 3:6] - Qt[:, 0:3], Qt[:, 6:9] - Qt[:, 0:3]),
                                      axis=1))
    kh = np.exp(rng.uniform(np.log(0.01), np.log(1.5), len(dh)))
    return np.ascontiguousarray(Pt), np.ascontiguousarray(Qt), kh / hq, dh


def far_pairs(n, seed=SEED + 1, dmin=2.0, dmax=200.0):
    """n well-separated pairs for the rule table of ACA entries: a source
    triangle Q from a jittered patch and a collocation triangle P from
    another, translated so that the centroid distance over sqrt(area Q) is
    log-uniform in [dmin, dmax], in a random direction; kh log-uniform in
    [0.01, 1.5]. Returns (P n x 9, Q n x 9, k n, d/h n)."""
    rng = np.random.default_rng(seed)
    Ps, Qs = [], []
    got = 0
    while got < n:
        A, B = patch(rng), patch(rng)
        m = min(256, n - got)
        ia = rng.integers(0, len(A), m)
        ib = rng.integers(0, len(B), m)
        Ps.append(A[ia])
        Qs.append(B[ib])
        got += m
    P = np.concatenate(Ps)
    Q = np.concatenate(Qs)
    aq = 0.5 * np.linalg.norm(np.cross(Q[:, 1] - Q[:, 0], Q[:, 2] - Q[:, 0]), axis=1)
    hq = np.sqrt(aq)
    dh = np.exp(rng.uniform(np.log(dmin), np.log(dmax), n))
    u = rng.standard_normal((n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    target = Q.mean(1) + u * (dh * hq)[:, None]
    P = P + (target - P.mean(1))[:, None, :]
    kh = np.exp(rng.uniform(np.log(0.01), np.log(1.5), n))
    return (np.ascontiguousarray(P.reshape(-1, 9)), np.ascontiguousarray(Q.reshape(-1, 9)),
            kh / hq, dh)
