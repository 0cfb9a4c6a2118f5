"""Train the learned quadrature-order selector on the GPU.

Data: seeded near-field pairs (selector_data.pairs), features and labels from
the library's label kernel (every candidate rule against the reference rule,
FP64). Training: the library's FP32 gradient and Adam kernels (bem_mlp_grad,
bem_mlp_adam) over minibatches; torch only holds the device buffers.
Evaluation on the held-out 20 %: BF16 tensor-core inference (bem_sel_infer)
with the guard band, against the plain 16-point rule.

    python 3d_bem_gb300/selector_train.py            # writes selector_weights.npz
"""
from __future__ import annotations

import argparse
import ctypes as ct
import importlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

NF, H, C, NPARAM = 24, 64, 5, 6085
WORK_PER_SAMPLE = 4 * H + 8 + 1
POINTS = np.array([1, 3, 7, 13, 25])
PLAIN_POINTS = 16


def init_params(seed):
    rng = np.random.default_rng(seed)
    parts = []
    for fan_in, shape in ((NF, (NF, H)), (None, (H,)), (H, (H, H)), (None, (H,)), (H, (H, C)),
                          (None, (C,))):
        if fan_in is None:
            parts.append(np.zeros(shape))
        else:
            parts.append(rng.standard_normal(shape).ravel() * np.sqrt(2.0 / fan_in))
    return np.concatenate([p.ravel() for p in parts]).astype(np.float32)


def softmax(z):
    e = np.exp(z - z.max(1, keepdims=True))
    return e / e.sum(1, keepdims=True)


def evaluate(pkg, params, mu, sigma, feat, lab, err, tol, guard):
    """Selector quality on held-out pairs: classes from BF16 inference with the
    guard band, the fraction of pairs whose chosen rule meets tol, points."""
    import torch
    L = pkg.lib()
    B = feat.shape[0]
    f_d = torch.from_numpy(np.ascontiguousarray(feat, np.float32)).cuda()
    logits = torch.zeros((B, 8), dtype=torch.float32, device="cuda")
    cls = torch.zeros(B, dtype=torch.uint8, device="cuda")
    prm = np.ascontiguousarray(params, np.float32)
    mu = np.ascontiguousarray(mu, np.float32)
    sigma = np.ascontiguousarray(sigma, np.float32)
    st = L.bem_sel_infer(prm.ctypes.data_as(ct.c_void_p), mu.ctypes.data_as(ct.c_void_p),
                         sigma.ctypes.data_as(ct.c_void_p), ct.c_void_p(f_d.data_ptr()), B,
                         ct.c_void_p(logits.data_ptr()), ct.c_void_p(cls.data_ptr()), None)
    if st != 0:
        raise RuntimeError(f"bem_sel_infer failed: {st}")
    z = logits.cpu().numpy()[:, :C]
    c = cls.cpu().numpy().astype(int)
    p = softmax(z).max(1)
    cg = np.where(p < guard, C - 1, c)
    ok = err[np.arange(B), cg] <= tol
    plain_ok = err[:, 5] <= tol
    lab_c = np.minimum(lab, C - 1)
    reach = lab < C
    return {
        "pairs": int(B),
        "accuracy": float(np.mean(c == lab_c)),
        "under_integrated": float(np.mean(cg < lab_c)),
        "guard_fraction": float(np.mean(p < guard)),
        "within_tol_learned": float(np.mean(ok)),
        "within_tol_plain16": float(np.mean(plain_ok)),
        "within_tol_best_possible": float(np.mean(reach)),
        # among the pairs some candidate rule can integrate to tol
        "achievable_within_tol_learned": float(np.mean(ok[reach])) if reach.any() else 1.0,
        "achievable_within_tol_plain16": float(np.mean(plain_ok[reach])) if reach.any() else 1.0,
        "mean_points_learned": float(np.mean(POINTS[cg])),
        "mean_points_plain": float(PLAIN_POINTS),
        "mean_points_oracle_labels": float(np.mean(POINTS[lab_c])),
    }


# Rule table of the ACA entries (far pairs): class as a function of
# x = log(d / e_max) and y = log(k e_max), d the centroid distance, e_max the
# source triangle's longest edge.
TAB_N = 12
TAB_AXES = (np.log(0.25), (np.log(200.0) - np.log(0.25)) / TAB_N,
            np.log(0.005), (np.log(15.0) - np.log(0.005)) / TAB_N)


def table_coords(feat):
    """Bin indices of pairs from their features (f0 = d/h, f8 = kh,
    f13 = e_max/h)."""
    x = np.log(feat[:, 0] / feat[:, 13])
    y = np.log(feat[:, 8] * feat[:, 13])
    x0, dx, y0, dy = TAB_AXES
    ix = np.clip(np.floor((x - x0) / dx).astype(int), 0, TAB_N - 1)
    iy = np.clip(np.floor((y - y0) / dy).astype(int), 0, TAB_N - 1)
    return ix, iy


def build_rule_table(feat, lab):
    """Largest class needed by any training pair of a bin (label 5, no rule
    reaches the tolerance, counts as the highest class), closed so that a bin
    never needs less than a farther bin or one with smaller k e_max; bins
    without pairs get the highest class."""
    ix, iy = table_coords(feat)
    need = np.minimum(lab, C - 1).astype(int)
    tab = np.full((TAB_N, TAB_N), -1, int)
    np.maximum.at(tab, (ix, iy), need)
    for i in range(TAB_N - 2, -1, -1):  # nearer needs at least what farther needs
        tab[i] = np.maximum(tab[i], tab[i + 1])
    for j in range(1, TAB_N):  # larger k e_max needs at least what smaller needs
        tab[:, j] = np.maximum(tab[:, j], tab[:, j - 1])
    tab[tab < 0] = C - 1
    return tab.astype(np.uint8)


def eval_rule_table(tab, feat, lab, err, tol):
    ix, iy = table_coords(feat)
    cls = tab[ix, iy].astype(int)
    ok = err[np.arange(len(cls)), cls] <= tol
    reach = lab < C
    return {"pairs": int(len(cls)),
            "within_tol_table": float(np.mean(ok)),
            "within_tol_plain16": float(np.mean(err[:, 5] <= tol)),
            "achievable_within_tol_table": float(np.mean(ok[reach])) if reach.any() else 1.0,
            "under_integrated": float(np.mean(cls < np.minimum(lab, C - 1))),
            "mean_points_table": float(np.mean(POINTS[cls])),
            "mean_points_plain": float(PLAIN_POINTS)}


def train(pkg, X, y, *, epochs, batch, lr, seed, log=print):
    """FP32 training with the library kernels; X normalised (n x 24)."""
    import torch
    L = pkg.lib()
    n = X.shape[0]
    Xd = torch.from_numpy(np.ascontiguousarray(X, np.float32)).cuda()
    yd = torch.from_numpy(np.ascontiguousarray(y, np.uint8)).cuda()
    prm = torch.from_numpy(init_params(seed)).cuda()
    m = torch.zeros_like(prm)
    v = torch.zeros_like(prm)
    g = torch.zeros_like(prm)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    work = torch.zeros(batch * WORK_PER_SAMPLE, dtype=torch.float32, device="cuda")
    stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    gen = torch.Generator().manual_seed(seed)
    steps = epochs * (n // batch)
    step = 0
    hist = []
    for ep in range(epochs):
        perm = torch.randperm(n, generator=gen).cuda()
        tot = 0.0
        for b0 in range(0, n - batch + 1, batch):
            idx = perm[b0:b0 + batch]
            xb = Xd.index_select(0, idx).contiguous()
            yb = yd.index_select(0, idx).contiguous()
            step += 1
            lr_t = 1e-5 + 0.5 * (lr - 1e-5) * (1 + np.cos(np.pi * step / steps))
            st = L.bem_mlp_grad(ct.c_void_p(prm.data_ptr()), ct.c_void_p(xb.data_ptr()),
                                ct.c_void_p(yb.data_ptr()), batch, ct.c_void_p(g.data_ptr()),
                                ct.c_void_p(loss.data_ptr()), ct.c_void_p(work.data_ptr()),
                                stream)
            st |= L.bem_mlp_adam(ct.c_void_p(prm.data_ptr()), ct.c_void_p(g.data_ptr()),
                                 ct.c_void_p(m.data_ptr()), ct.c_void_p(v.data_ptr()), step,
                                 lr_t, 0.9, 0.999, 1e-8, stream)
            if st != 0:
                raise RuntimeError("training kernels failed")
            if b0 == 0:
                tot = float(loss.item())
        hist.append(tot)
        log(f"epoch {ep}: loss {tot:.4f}")
    torch.cuda.synchronize()
    return prm.cpu().numpy(), hist


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=2_000_000)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--tol", type=float, default=1e-7)
    ap.add_argument("--guard", type=float, default=0.9)
    ap.add_argument("--seed", type=int, default=20260105)
    ap.add_argument("--aca-pairs", type=int, default=1_000_000)
    ap.add_argument("--aca-tol", type=float, default=1e-6)
    ap.add_argument("--aca-floor", type=float, default=1.0,
                    help="ACA labels: operator errors relative to the pair's largest")
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                  "selector_weights.npz"))
    args = ap.parse_args(argv)
    pkg = importlib.import_module("3d_bem_gb300")
    data = importlib.import_module("3d_bem_gb300.selector_data")
    pkg.build()
    t0 = time.time()
    P, Q, k, dh = data.pairs(args.pairs, seed=args.seed)
    t1 = time.time()
    feat, lab, err = pkg.sel_label(P, Q, k, tol=args.tol, want_err=True)
    t2 = time.time()
    ntr = int(0.8 * len(lab))
    mu = feat[:ntr].mean(0).astype(np.float32)
    sigma = np.maximum(feat[:ntr].std(0), 1e-6).astype(np.float32)
    X = (feat[:ntr] - mu) / sigma
    y = np.minimum(lab[:ntr], C - 1)
    params, hist = train(pkg, X, y, epochs=args.epochs, batch=args.batch, lr=args.lr,
                         seed=args.seed)
    t3 = time.time()
    ev = evaluate(pkg, params, mu, sigma, feat[ntr:], lab[ntr:], err[ntr:], args.tol, args.guard)
    reg = dh[ntr:] >= 2.0
    ev_reg = evaluate(pkg, params, mu, sigma, feat[ntr:][reg], lab[ntr:][reg], err[ntr:][reg],
                      args.tol, args.guard)
    # rule table of the ACA entries, from far pairs labelled at the ACA-level
    # tolerance; evaluated on far pairs of another seed
    Pf, Qf, kf, dhf = data.far_pairs(args.aca_pairs, seed=args.seed + 1)
    ff, lf, ef = pkg.sel_label(Pf, Qf, kf, tol=args.aca_tol, want_err=True,
                               floor_rel=args.aca_floor)
    table = build_rule_table(ff, lf)
    Pv, Qv, kv, dhv = data.far_pairs(200_000, seed=args.seed + 2)
    fv, lv, ev_ = pkg.sel_label(Pv, Qv, kv, tol=args.aca_tol, want_err=True,
                                floor_rel=args.aca_floor)
    tab_eval = eval_rule_table(table, fv, lv, ev_, args.aca_tol)
    report = {"pairs": int(len(lab)), "train": ntr, "test": int(len(lab) - ntr),
              "aca_table": table.tolist(), "aca_tol": args.aca_tol,
              "aca_floor": args.aca_floor,
              "aca_table_eval": tab_eval,
              "label_hist": np.bincount(lab, minlength=C + 1).tolist(), "tol": args.tol,
              "guard": args.guard, "epochs": args.epochs, "batch": args.batch,
              "loss_history": hist, "seconds": {"pairs": t1 - t0, "labels": t2 - t1,
                                                "train": t3 - t2}, "test_metrics": ev,
              "test_metrics_regular_pairs": ev_reg}
    np.savez(args.out, params=params, mu=mu, sigma=sigma, aca_table=table,
             aca_axes=np.array(TAB_AXES, np.float32), report=np.array(json.dumps(report)))
    print(json.dumps(report))


if __name__ == "__main__":
    main()
