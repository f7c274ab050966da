#!/usr/bin/env python3
"""Runs the reference's optimizers on the 1024^2 wave loss on the CPU and
writes wave1024_optimizers_reference.json beside this script.

The reference drives L-BFGS through scipy's fmin_l_bfgs_b with m = 50,
pgtol = 1e-16, factr = 0, maxls = 50 (optimizer.py:61-99), and Adam through
the explicit update of optimizer.py:271-322 (lr 1e-3).  Both run here on the
restated FP64 loss of the 1024 x 1024 wave workload (16-mode sine profile,
seed 1, c = 1; oracle/wave.py), 2000 iterations each from u = 0, exactly as
the GPU optimizers of the benchmark do, and record the loss every 100
iterations, the final loss, the error against the exact solution and the
relative error against the FP64 discrete solution.  The operator is affine,
so J is assembled once and loss_grad(u) = (mean f^2, (2/N) J^T f) with
f = f(0) + J u.  Takes ~15-25 minutes on one core.

    python tests/golden/make_optimizer_reference.py [--iters 2000] [--n 1024]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from oracle import optim as O  # noqa: E402
from oracle import wave as W  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--iters", type=int, default=2000)
    ap.add_argument("--out", default=os.path.join(
        HERE, "wave1024_optimizers_reference.json"))
    a = ap.parse_args()
    n = a.n
    s = W.make_setup(n, n, "sine", seed=1, nmodes=16, c=1.0)
    f0, J = W.linearize(s, np.zeros((n, n)))
    f0 = np.concatenate([c.ravel() for c in f0])
    JT = J.T.tocsr()
    N = f0.size
    ref = W.solve_march(s, rounds=2)
    exact = s.exact_u if hasattr(s, "exact_u") else None
    hist = {}

    def lg(x):
        f = f0 + J @ x
        return float(np.mean(f * f)), (2.0 / N) * (JT @ f)

    def record(name, x, k):
        hist.setdefault(name, []).append([k, lg(x)[0]])

    out = {"workload": "wave1d_%dx%d_sine16_seed1" % (n, n),
           "iterations": a.iters, "initial_loss": lg(np.zeros(N))[0]}
    # L-BFGS-B with the reference settings; history through the callback.
    it = [0]

    def cb(x):
        it[0] += 1
        if it[0] % 100 == 0:
            record("lbfgsb", x, it[0])

    import scipy.optimize
    t0 = time.perf_counter()
    x, fval, info = scipy.optimize.fmin_l_bfgs_b(
        func=lg, x0=np.zeros(N), maxiter=a.iters, pgtol=1e-16, m=50,
        maxls=50, factr=0, maxfun=np.inf, callback=cb)
    t = time.perf_counter() - t0
    xs = x.reshape(n, n)
    out["lbfgsb"] = {"settings": "scipy fmin_l_bfgs_b m=50 pgtol=1e-16 "
                                 "factr=0 maxls=50 (optimizer.py:86-94)",
                     "final_loss": float(fval), "nit": int(info["nit"]),
                     "funcalls": int(info["funcalls"]),
                     "warnflag": int(info["warnflag"]),
                     "task": str(info["task"]),
                     "rel_err_vs_oracle": W.rel_err(xs, ref),
                     "wall_s": t, "loss_every_100": hist.get("lbfgsb", [])}
    if exact is not None:
        out["lbfgsb"]["err_vs_exact_l2"] = W.l2_error(xs, exact)
    # Adam, the reference's explicit update (optimizer.py:301-314).
    t0 = time.perf_counter()
    xa = np.zeros(N)
    m = np.zeros(N)
    v = np.zeros(N)
    b1, b2, eps, lr = 0.9, 0.999, 1e-7, 1e-3
    for k in range(1, a.iters + 1):
        _, g = lg(xa)
        alpha = lr * np.sqrt(1 - b2**k) / (1 - b1**k)
        m += (g - m) * (1 - b1)
        v += (g * g - v) * (1 - b2)
        xa -= (m * alpha) / (np.sqrt(v) + eps)
        if k % 100 == 0:
            record("adam", xa, k)
    t = time.perf_counter() - t0
    xs = xa.reshape(n, n)
    out["adam"] = {"settings": "optimizer.py:301-314, lr 1e-3, beta 0.9/"
                               "0.999, epsilon 1e-7",
                   "final_loss": lg(xa)[0],
                   "rel_err_vs_oracle": W.rel_err(xs, ref), "wall_s": t,
                   "loss_every_100": hist.get("adam", [])}
    if exact is not None:
        out["adam"]["err_vs_exact_l2"] = W.l2_error(xs, exact)
    with open(a.out, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps({k: (v if not isinstance(v, dict) else
                          {kk: vv for kk, vv in v.items()
                           if kk != "loss_every_100"})
                      for k, v in out.items()}))


if __name__ == "__main__":
    main()
