"""Generate tests/golden/operators.npz: high-accuracy element integrals that pin
the oracle (and through it the GPU kernels) to the mathematics, independently
of the rule tables both of them use.

The reference ships no golden vectors and cannot be built here (it needs Qt 6
and Eigen), so these known answers are computed from the definitions:

  L  = int_T G dS_q,            G = exp(ikr) / (4 pi r),  r = |p - q|
  M  = int_T dG/dn_q dS_q,      Mt = int_T dG/dn_p dS_q,
  N  = int_T d2G/(dn_p dn_q) dS_q

(boundaryelementsolver.cpp:867-888 states the same integrands), with a
Duffy-collapsed Gauss-Legendre product rule on a recursively refined source
triangle (numpy only, nothing shared with the oracle).  For the self pairs the
k -> 0 closed form of the single layer at the centroid is stored
(int_T 1/(4 pi r) dS = sum over the three sub-triangles of
c sin B ln(tan((A+B)/2) / tan(B/2)) / (4 pi)).

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def gauss01(n):
    x, w = np.polynomial.legendre.leggauss(n)
    return 0.5 * (x + 1.0), 0.5 * w


def duffy_points(A, B, C, n):
    """Quadrature points/weights on triangle (A,B,C), collapsed at A."""
    u, wu = gauss01(n)
    v, wv = gauss01(n)
    U, V = np.meshgrid(u, v, indexing="ij")
    W = np.outer(wu, wv)
    q = A[None, None, :] + U[..., None] * (B - A)[None, None, :] + (U * V)[..., None] * (C - B)[None, None, :]
    area2 = np.linalg.norm(np.cross(B - A, C - A))
    return q.reshape(-1, 3), (W * U * area2).reshape(-1)


def refine(tri, levels):
    tris = [tri]
    for _ in range(levels):
        nxt = []
        for (a, b, c) in tris:
            ab, bc, ca = (a + b) / 2, (b + c) / 2, (c + a) / 2
            nxt += [(a, ab, ca), (ab, b, bc), (ca, bc, c), (ab, bc, ca)]
        tris = nxt
    return tris


def integrals(p, npv, tri, nqv, k, levels=3, n=20):
    qs, ws = [], []
    for (a, b, c) in refine(tri, levels):
        q, w = duffy_points(a, b, c, n)
        qs.append(q)
        ws.append(w)
    q = np.concatenate(qs)
    w = np.concatenate(ws)
    rv = p[None, :] - q
    rr = (rv ** 2).sum(1)
    r = np.sqrt(rr)
    rnq = -(rv @ nqv) / r
    rnp = (rv @ npv) / r
    ikr = 1j * k * r
    G = np.exp(ikr) / (4 * np.pi * r)
    dG = G / r * (ikr - 1.0)
    d2G = G / rr * (2.0 - 2.0 * ikr - k * k * rr)
    upnq = float(npv @ nqv)
    L = (w * G).sum()
    M = (w * dG * rnq).sum()
    Mt = (w * dG * rnp).sum()
    N = (w * (dG * (-(upnq + rnp * rnq) / r) + d2G * rnp * rnq)).sum()
    return np.array([L, M, Mt, N])


def laplace_self(tri):
    """k -> 0 single layer of a flat triangle at its centroid, closed form."""
    n1, n2, n3 = tri
    c = (n1 + n2 + n3) / 3.0
    tot = 0.0
    for a, b in ((n1, n2), (n2, n3), (n3, n1)):
        # sub-triangle (a, b, c): distances from the centroid to a and b
        da, db = np.linalg.norm(a - c), np.linalg.norm(b - c)
        ab = np.linalg.norm(b - a)
        A = np.arccos((da * da + db * db - ab * ab) / (2 * da * db))  # angle at c
        # integrate R(theta) from the ray c->a: R = da sin(Ba) / sin(theta + Ba)
        Ba = np.arccos((da * da + ab * ab - db * db) / (2 * da * ab))  # angle at a
        tot += da * np.sin(Ba) * np.log(np.tan((A + Ba) / 2) / np.tan(Ba / 2))
    return tot / (4 * np.pi)


def main():
    meshes = importlib.import_module("3d_bem_gb300.meshes")
    tri = meshes.icosphere(2, 1.0)  # 320 triangles
    rng = np.random.default_rng(20260101)
    nodes = tri.reshape(-1, 3, 3)
    nrm = np.cross(nodes[:, 1] - nodes[:, 0], nodes[:, 2] - nodes[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    cen = nodes.sum(1) / 3.0
    area = 0.5 * np.linalg.norm(np.cross(nodes[:, 0] - nodes[:, 1], nodes[:, 0] - nodes[:, 2]), axis=1)
    avgdim = np.sqrt(area).mean() / 2.0
    n = tri.shape[0]
    d = np.linalg.norm(cen[:, None, :] - cen[None, :, :], axis=2)
    far = np.argwhere(d >= 4 * avgdim)
    near = np.argwhere((d < 4 * avgdim) & (d > 0))
    pf = far[rng.choice(len(far), 48, replace=False)]
    pn = near[rng.choice(len(near), 24, replace=False)]
    pairs = np.concatenate([pf, pn])
    kinds = np.array([0] * len(pf) + [1] * len(pn))
    ks = np.array([0.5, 3.66, 12.0])
    vals = np.zeros((len(ks), len(pairs), 4), np.complex128)
    for a, k in enumerate(ks):
        for i, (r, c) in enumerate(pairs):
            lev = 2 if kinds[i] == 0 else 4
            vals[a, i] = integrals(cen[r], nrm[r], nodes[c], nrm[c], k, levels=lev, n=16)
    selfL = np.array([laplace_self(nodes[i]) for i in range(0, n, 16)])
    np.savez_compressed(os.path.join(HERE, "operators.npz"), tri=tri, pairs=pairs, kinds=kinds,
                        ks=ks, vals=vals, self_idx=np.arange(0, n, 16), self_laplace=selfL)
    print("wrote", os.path.join(HERE, "operators.npz"), vals.shape)


if __name__ == "__main__":
    main()
