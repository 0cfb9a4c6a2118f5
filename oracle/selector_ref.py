"""CPU oracle of the selector's labels (test infrastructure only): the four
operators L, M, Mt, N of (collocation triangle, source triangle) pairs with a
given triangle rule, in float64 numpy, following the integrand of
boundaryelementsolver.cpp:872-887; the per-rule relative errors against the
64-point collapsed Gauss-Legendre product rule on a subdivision of the source
triangle; the cheapest passing rule."""
from __future__ import annotations

import numpy as np

CLASS_ORDERS = (1, 2, 5, 7, 10)   # 1, 3, 7, 13, 25 points
PLAIN_ORDER = 8                   # 16 points


def reference_rule():
    """64-point collapsed Gauss-Legendre product rule (x1, x2, w rows)."""
    x, w = np.polynomial.legendre.leggauss(8)
    u = 0.5 * (x + 1)
    U, V = np.meshgrid(u, u, indexing="ij")
    WU, WV = np.meshgrid(w, w, indexing="ij")
    x1 = U.ravel()
    x2 = ((1 - U) * V).ravel()
    ww = (2 * 0.25 * WU * WV * (1 - U)).ravel()
    return np.stack([x1, x2, ww], 1)


def subdivided(rule, n=4):
    """The rule replicated on the n^2 sub-triangles of an n-fold subdivision."""
    out = []
    h = 1.0 / n
    for i in range(n):
        for j in range(n - i):
            corners = [((i, j), (i + 1, j), (i, j + 1))]
            if i + j <= n - 2:
                corners.append(((i + 1, j), (i + 1, j + 1), (i, j + 1)))
            for (a, b, c) in corners:
                s1, s2 = rule[:, 0], rule[:, 1]
                s3 = 1 - s1 - s2
                x1 = h * (s1 * a[0] + s2 * b[0] + s3 * c[0])
                x2 = h * (s1 * a[1] + s2 * b[1] + s3 * c[1])
                out.append(np.stack([x1, x2, rule[:, 2] * h * h], 1))
    return np.concatenate(out)


def geometry(tri):
    t = np.asarray(tri, np.float64).reshape(-1, 3, 3)
    c = ((t[:, 0] + t[:, 1]) + t[:, 2]) / 3.0
    nv = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    area = 0.5 * np.linalg.norm(nv, axis=1)
    return t, c, nv / (2 * area)[:, None], area


def ops(ptri, qtri, k, rule):
    """(n, 4) complex: L, M, Mt, N of each pair with the rule (x1, x2, w rows)."""
    _, p, npv, _ = geometry(ptri)
    T, _, nq, area = geometry(qtri)
    x1, x2, w = rule[:, 0], rule[:, 1], rule[:, 2]
    x3 = 1 - x1 - x2
    q = (x1[None, :, None] * T[:, None, 0] + x2[None, :, None] * T[:, None, 1]
         + x3[None, :, None] * T[:, None, 2])
    rv = p[:, None, :] - q
    rr = (rv * rv).sum(-1)
    r = np.sqrt(rr)
    rnq = -(rv * nq[:, None, :]).sum(-1) / r
    rnp = (rv * npv[:, None, :]).sum(-1) / r
    upNq = (npv * nq).sum(-1)[:, None]
    kk = np.asarray(k, np.float64)[:, None]
    ikr = 1j * kk * r
    G = np.exp(ikr) / (4 * np.pi * r)
    dG = G / r * (ikr - 1)
    d2G = G / rr * (2 - 2 * ikr - kk ** 2 * rr)
    L = (w * G).sum(-1)
    M = (w * dG * rnq).sum(-1)
    Mt = (w * dG * rnp).sum(-1)
    N = (w * (dG * (-(upNq + rnp * rnq) / r) + d2G * rnp * rnq)).sum(-1)
    return np.stack([L, M, Mt, N], 1) * area[:, None]


def label_reference(ptri, qtri, k):
    """The labels' reference operators: the 64-point product rule on an 8-fold
    subdivision of the source triangle when the centroid distance is below
    3 sqrt(area), a 4-fold one beyond (pairs closer than one source size are
    labelled against the split-polar rule, which this module does not state)."""
    _, cp, _, _ = geometry(ptri)
    _, cq, _, aq = geometry(qtri)
    dh = np.linalg.norm(cp - cq, axis=1) / np.sqrt(aq)
    out = np.zeros((len(dh), 4), complex)
    for n, m in ((8, dh < 3), (4, dh >= 3)):
        if m.any():
            out[m] = ops(ptri[m], qtri[m], np.asarray(k)[m], subdivided(reference_rule(), n))
    return out


def rel_err(o, ref, floor=1e-3):
    mx = np.abs(ref).max(1, keepdims=True)
    return (np.abs(o - ref) / np.maximum(np.abs(ref), floor * mx)).max(1)


def errors_and_labels(ptri, qtri, k, rules, tol, ref=None):
    """rules: dict order -> (npts, 3) table (oracle.triangle_rule). ref: the
    reference operators (default: label_reference)."""
    if ref is None:
        ref = label_reference(ptri, qtri, k)
    err = np.stack([rel_err(ops(ptri, qtri, k, rules[o]), ref) for o in CLASS_ORDERS]
                   + [rel_err(ops(ptri, qtri, k, rules[PLAIN_ORDER]), ref)], 1)
    lab = np.full(err.shape[0], 5)
    for c in reversed(range(5)):
        lab = np.where(err[:, c] <= tol, c, lab)
    return err, lab
