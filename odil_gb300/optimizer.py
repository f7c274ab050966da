"""Optimizers with the reference's protocol (optimizer.py:8-338):

    x, info = make_optimizer(name).run(x0, loss_grad, epochs, callback,
                                       epoch_start=0, lr=..., **kwargs)

``loss_grad(x, epoch) -> (loss, grad, residuals)`` works on packed device
vectors.  Every vector update runs in libodil_gb300 kernels; only scalars of
the line search and the 2m x 2m compact L-BFGS algebra live on the host.

Names: "lbfgsb" (L-BFGS, m = 50, strong-Wolfe line search, maxls = 50; the
reference wraps scipy's fmin_l_bfgs_b without bounds), "lbfgs" (same
algorithm; the reference's TF-Probability variant), "adam" (Keras Adam, run
for epochs + 1 steps as Keras model.fit does in the reference), "adamn"
(AdamNativeOptimizer), "gd".
"""
import math
from argparse import Namespace

import numpy as np
import torch

from . import vec


class Optimizer:
    """optimizer.py:8-28."""

    def __init__(self, name=None, displayname=None, dtype=None):
        self.name = name
        self.displayname = displayname if displayname is not None else name
        self.dtype = dtype
        self.last_loss = None
        self.last_residual = None
        self.evals = 0

    def run(self, x0, loss_grad, epochs, callback=None, epoch_start=0,
            **kwargs):
        info = Namespace()
        info.evals = 0
        info.epochs = 0
        return x0, info


def _scalar(t):
    return float(t) if not isinstance(t, torch.Tensor) else float(t.item())


class LbfgsOptimizer(Optimizer):
    """Limited-memory BFGS in the compact representation (Byrd, Nocedal and
    Schnabel 1994; Nocedal & Wright eq. 7.24) with a strong-Wolfe line search
    (Nocedal & Wright Alg. 3.5/3.6, cubic interpolation in the zoom).

    Correction pairs live on the device as rows of one [2m, n] array
    (s0, y0, s1, y1, ...); per iteration one multi-dot pass gives S^T g, Y^T g
    and the new pair's products, and one linear-combination pass gives the
    direction.  Settings follow optimizer.py:33-99: m = 50, maxls = 50,
    pgtol = 1e-16, factr = 0 (no early stop short of a stalled line search).
    """

    def __init__(self, pgtol=1e-16, m=50, maxls=50, factr=0, dtype=None,
                 name="lbfgsb", displayname="L-BFGS-B", c1=1e-4, c2=0.9,
                 graph=False, **kwargs):
        super().__init__(name=name, displayname=displayname, dtype=dtype)
        self.pgtol = pgtol
        self.graph = bool(graph)
        self.m = int(m)
        self.maxls = int(maxls)
        self.factr = factr
        self.c1, self.c2 = c1, c2

    # -- compact two-loop replacement ---------------------------------------
    def _direction(self, g, d, H, rows, order, SY, YY, gamma, dots_g,
                   coef_dev):
        """d = -H_k g from the dots of the stored pairs with g (dots_g[row])."""
        if not order:
            vec.axpby(d, -1.0, g, 0.0, g)
            return
        a = np.array([dots_g[2 * j] for j in order])      # S^T g, oldest first
        b = np.array([dots_g[2 * j + 1] for j in order])  # Y^T g
        R = np.triu(SY)
        D = np.diag(np.diag(SY))
        t = _solve_upper(R, a)
        p = _solve_upper(R.T, (D + gamma * YY) @ t - gamma * b, lower=True)
        q = -gamma * t
        coef = np.zeros(rows + 1)
        for c, j in enumerate(order):
            coef[2 * j] = -p[c]
            coef[2 * j + 1] = -q[c]
        coef[-1] = -gamma
        coef_dev[:rows + 1].copy_(torch.as_tensor(coef))
        vec.lincomb(d, g, H, rows, coef_dev)

    def run(self, x0, loss_grad, epochs=None, callback=None, epoch_start=0,
            **kwargs):
        """The device form (`run_device`) for CUDA vectors and m <= 128;
        the host-algebra form (`run_host`) otherwise."""
        if x0.is_cuda and self.m <= 128 and x0.dtype in (torch.float32,
                                                         torch.float64):
            return self.run_device(x0, loss_grad, epochs, callback,
                                   epoch_start)
        return self.run_host(x0, loss_grad, epochs, callback, epoch_start)

    def run_device(self, x0, loss_grad, epochs=None, callback=None,
                   epoch_start=0):
        """The same iteration with the compact-form algebra, the first trial
        step, its Wolfe test and the pair/ring update on the device
        (csrc/lbfgs.cu): per iteration one direction (coefficient kernel +
        one linear combination that also gives g . d), the trial point, one
        loss+gradient there, one pass forming the new pair with its dots and
        the Wolfe test, one multi-dot of the stored rows with (g_new, s, y),
        the ring update and commit, and one host read of the 16 scalars (the
        status).  A trial that fails the Wolfe test
        (rare once pairs are held) falls back to the host line search from
        the same state.

        With ``graph=True`` (constructor) and a loss_grad that returns device
        tensors and can be captured (no host synchronisation, fixed
        buffers), the whole iteration is recorded into a CUDA graph once m
        pairs have been formed (from then on its launch shapes are fixed),
        one graph per parity of the iterate buffers, and every later
        iteration is one replay plus the status read.  The kernels after the
        Wolfe test are guarded by the status on the device, so a replayed
        iteration whose trial is rejected changes no state; the host line
        search then runs eagerly as without graphs.  Iterates are the same
        as without graphs."""
        from . import _capi
        from ._capi import call, ptr, stream_handle
        x = x0.detach().clone()
        n = x.numel()
        dev = x.device
        m = self.m
        sfx = "f32" if x.dtype == torch.float32 else "f64"
        H = torch.zeros((2 * m, n), dtype=x.dtype, device=dev)
        SYp = torch.zeros((2, n), dtype=x.dtype, device=dev)
        md = vec.MultiDot(n, 2 * m, 3, device=dev)
        md1 = vec.MultiDot(n, 1, 1, device=dev)
        lib = _capi.load()
        lc_ws = torch.zeros(int(lib.odil_lincomb_dot_workspace_bytes(n)),
                            dtype=torch.uint8, device=dev)
        pd_ws = torch.zeros(int(lib.odil_lbfgs_pair_dots_workspace_bytes(n)),
                            dtype=torch.uint8, device=dev)
        dots = torch.zeros(1, dtype=torch.float64, device=dev)
        Q = torch.zeros(4, dtype=torch.float64, device=dev)
        coef = torch.zeros(2 * m + 1, dtype=torch.float64, device=dev)
        ring = torch.tensor([0, 0, m, -1], dtype=torch.int32, device=dev)
        SY = torch.zeros((m, m), dtype=torch.float64, device=dev)
        YY = torch.zeros((m, m), dtype=torch.float64, device=dev)
        dg = torch.zeros(2 * m, dtype=torch.float64, device=dev)
        sc = torch.zeros(16, dtype=torch.float64, device=dev)
        sc_host = torch.zeros(16, dtype=torch.float64).pin_memory()
        d = torch.empty_like(x)
        xt = torch.empty_like(x)
        self.epoch = epoch_start
        loss, g, res = loss_grad(x, self.epoch)
        g = g.detach().clone()
        self.evals += 1
        eps = 1e-6 if x.dtype == torch.float32 else 1e-12
        sc[0] = loss.double() if isinstance(loss, torch.Tensor) else float(loss)
        sc[1] = 1.0
        sc[7], sc[8], sc[9] = self.c1, self.c2, eps
        self.last_loss, self.last_residual = float(sc[0]), res
        info = Namespace(epochs=0, evals=1, task="", fallbacks=0, replays=0)
        epochs = epochs if epochs is not None else 1 << 30

        def pair_dots(gt, ft_dev, mode):
            """s, y into SYp, their dots (Q), g_trial . d and (mode 0) the
            Wolfe test of the trial, in one pass."""
            call("odil_lbfgs_pair_dots_" + sfx, n, ptr(SYp), ptr(d), ptr(gt),
                 ptr(g), ptr(ft_dev), mode, ptr(sc), ptr(Q), ptr(pd_ws),
                 pd_ws.numel(), stream_handle())

        def trial(x, xt, rows):
            """Direction (with g . d), trial point, loss+gradient there, pair
            and Wolfe test."""
            st = stream_handle()
            if rows:
                call("odil_lbfgs_coef", m, rows, ptr(ring), ptr(SY), ptr(YY),
                     ptr(dg), ptr(sc), ptr(coef), st)
                call("odil_lincomb_dot_" + sfx, ptr(d), ptr(g), ptr(H), n, rows,
                     ptr(coef), n, ptr(dots), ptr(lc_ws), lc_ws.numel(), st)
                gd = dots
            else:
                vec.axpby(d, -1.0, g, 0.0, g)
                gd = md1(g, 1, [d])
            call("odil_lbfgs_trial_" + sfx, n, ptr(xt), ptr(x), ptr(d),
                 ptr(gd), ptr(ring), ptr(sc), st)
            ft, gt, res = loss_grad(xt, self.epoch)
            ft_dev = ft.reshape(1).double() if isinstance(ft, torch.Tensor) \
                else torch.tensor([float(ft)], dtype=torch.float64, device=dev)
            pair_dots(gt, ft_dev, 0)
            return gt, res

        def update(gt, rows):
            """Dots of the stored pairs with (g_trial, s, y), ring/matrix
            update, commit with g <- g_trial (guarded by the status)."""
            st = stream_handle()
            P = md(H, max(rows, 1), [gt, SYp[0], SYp[1]]) if rows else None
            call("odil_lbfgs_update", ptr(ring), ptr(SY), ptr(YY), ptr(dg),
                 ptr(sc), ptr(P), rows, ptr(Q), st)
            call("odil_lbfgs_commit_" + sfx, n, ptr(H), n, ptr(SYp), ptr(g),
                 ptr(gt), ptr(ring), ptr(sc), st)

        graphs = {}          # x.data_ptr() -> (graph, gt, res)
        use_graph = self.graph
        accepted = 0  # upper bound of the pairs held: rows the dots need
        it = 0
        while it < epochs:
            rows = 2 * min(accepted, m)
            replayed = False
            if use_graph and rows == 2 * m:
                key = x.data_ptr()
                if key not in graphs:
                    graphs[key] = self._capture(
                        lambda: trial(x, xt, rows), update, rows, sc, sc_host,
                        dev)
                    use_graph = graphs[key] is not None
                if use_graph:
                    gr, gt, res = graphs[key]
                    gr.replay()
                    replayed = True
                    info.replays += 1
            if not replayed:
                gt, res = trial(x, xt, rows)
                sc_host.copy_(sc, non_blocking=True)
            self.evals += 1
            torch.cuda.current_stream(dev).synchronize()
            status = int(sc_host[6])
            if status == 2:
                # Not a descent direction: restart from steepest descent.
                if int(ring[0].item()) == 0:
                    info.task = "CONVERGENCE: zero gradient"
                    break
                ring.copy_(torch.tensor([0, 0, m, -1], dtype=torch.int32))
                continue
            if status == 1:
                info.fallbacks += 1
                f0 = float(sc_host[0])
                dphi0 = float(sc_host[2])
                ok, alpha, fa, gt = self._line_search(
                    x, d, xt, f0, dphi0, float(sc_host[3]), loss_grad, md1)
                if not ok:
                    info.task = "ABNORMAL_TERMINATION_IN_LNSRCH"
                    break
                sc[3], sc[4], sc[6] = alpha, fa, 0.0
                pair_dots(gt, None, 1)
                update(gt, rows)
            elif not replayed:
                update(gt, rows)
            accepted += 1
            x, xt = xt, x
            self.last_loss = float(sc_host[4]) if status == 0 else float(fa)
            self.last_residual = res
            self.epoch += 1
            info.epochs += 1
            it += 1
            if callback:
                callback(x, self.epoch, opt=self)
        info.evals = self.evals
        return x, info

    @staticmethod
    def _capture(trial, update, rows, sc, sc_host, dev):
        """One iteration (trial, update, status copy into the pinned host
        buffer) recorded into a CUDA graph, or None when the loss_grad
        cannot be captured (it synchronises or returns host values)."""
        torch.cuda.synchronize(dev)
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        gr = torch.cuda.CUDAGraph()
        try:
            with torch.cuda.graph(gr, stream=side):
                gt, res = trial()
                update(gt, rows)
                sc_host.copy_(sc, non_blocking=True)
        except Exception:  # noqa: BLE001 - not capturable: run eagerly
            torch.cuda.synchronize(dev)
            return None
        torch.cuda.current_stream(dev).wait_stream(side)
        return gr, gt, res

    def run_host(self, x0, loss_grad, epochs=None, callback=None,
                 epoch_start=0, **kwargs):
        x = x0.detach().clone()
        n = x.numel()
        dev = x.device
        m = self.m
        H = torch.zeros((2 * m, n), dtype=x.dtype, device=dev)
        md = vec.MultiDot(n, 2 * m, 3, device=dev)
        md1 = vec.MultiDot(n, 1, 1, device=dev)
        coef_dev = torch.zeros(2 * m + 1, dtype=torch.float64, device=dev)
        d = torch.empty_like(x)
        xt = torch.empty_like(x)
        order = []          # ring slots holding pairs, oldest first
        nfill = 0           # slots ever written (rows 0 .. 2 nfill - 1 used)
        SY = np.zeros((0, 0))
        YY = np.zeros((0, 0))
        gamma = 1.0
        dots_g = None
        self.epoch = epoch_start
        loss, g, res = loss_grad(x, self.epoch)
        g = g.detach().clone()
        self.evals += 1
        f = _scalar(loss)
        self.last_loss, self.last_residual = f, res
        info = Namespace(epochs=0, evals=1, task="")
        epochs = epochs if epochs is not None else 1 << 30
        for it in range(epochs):
            self._direction(g, d, H, 2 * nfill, order, SY, YY, gamma, dots_g,
                            coef_dev)
            dphi0 = _scalar(vec.dot(g, d, md1))
            if not dphi0 < 0:
                # Not a descent direction: restart from steepest descent.
                vec.axpby(d, -1.0, g, 0.0, g)
                order, SY, YY = [], np.zeros((0, 0)), np.zeros((0, 0))
                dphi0 = _scalar(vec.dot(g, d, md1))
                if not dphi0 < 0:
                    info.task = "CONVERGENCE: zero gradient"
                    break
            if not order:
                gnorm = math.sqrt(max(-dphi0, 0.0))
                alpha0 = min(1.0, 1.0 / max(gnorm, 1e-300))
            else:
                alpha0 = 1.0
            ok, alpha, ft, gt = self._line_search(x, d, xt, f, dphi0, alpha0,
                                                  loss_grad, md1)
            if not ok:
                info.task = "ABNORMAL_TERMINATION_IN_LNSRCH"
                break
            # New correction pair into the oldest (or next free) slot.
            if len(order) == m:
                slot = order.pop(0)
                SY, YY = SY[1:, 1:], YY[1:, 1:]
            else:
                slot = len(order) if len(order) >= nfill else \
                    min(set(range(nfill)) - set(order))
            nfill = max(nfill, slot + 1)
            s_row, y_row = H[2 * slot], H[2 * slot + 1]
            vec.axpby(s_row, alpha, d, 0.0, d)
            vec.axpby(y_row, 1.0, gt, -1.0, g)
            # One pass: dots of every stored row with (g_new, s_new, y_new).
            P = md(H, 2 * nfill, [gt, s_row, y_row]).cpu().numpy()
            sy = P[2 * slot, 2]
            yy = P[2 * slot + 1, 2]
            if np.isfinite(sy) and sy > 1e-12 * yy:
                order.append(slot)
                k = len(order)
                SYn = np.zeros((k, k))
                YYn = np.zeros((k, k))
                SYn[:k - 1, :k - 1] = SY
                YYn[:k - 1, :k - 1] = YY
                for c, j in enumerate(order):
                    SYn[c, k - 1] = P[2 * j, 2]        # s_j . y_new
                    SYn[k - 1, c] = P[2 * j + 1, 1]    # y_j . s_new
                    YYn[c, k - 1] = P[2 * j + 1, 2]    # y_j . y_new
                    YYn[k - 1, c] = P[2 * j + 1, 2]
                SY, YY = SYn, YYn
                gamma = sy / yy
            dots_g = P[:, 0]
            x, xt = xt, x
            g.copy_(gt)
            f = ft
            self.last_loss = f
            self.epoch += 1
            info.epochs += 1
            if callback:
                callback(x, self.epoch, opt=self)
        info.evals = self.evals
        return x, info

    def _line_search(self, x, d, xt, f0, dphi0, alpha, loss_grad, md1):
        """Wolfe line search on phi(a) = f(x + a d).

        Accepts a step satisfying the Wolfe conditions
            phi(a) <= phi(0) + c1 a phi'(0),  phi'(a) >= c2 phi'(0),
        or the approximate Wolfe conditions of Hager & Zhang (2005),
            phi(a) <= phi(0) + eps |phi(0)|,
            c2 phi'(0) <= phi'(a) <= (2 c1 - 1) phi'(0),
        which stay decidable when the decrease is below the rounding level of
        an FP32 loss (eps = 1e-6 for FP32 fields, 1e-12 for FP64).  The
        bracket is driven by the sign of phi' (secant steps, bisection
        safeguard), which is accurate where differences of phi are not."""
        c1, c2 = self.c1, self.c2
        eps = (1e-6 if x.dtype == torch.float32 else 1e-12) * abs(f0)

        def phi(a):
            vec.axpby(xt, 1.0, x, a, d)
            loss, gt, res = loss_grad(xt, self.epoch)
            self.evals += 1
            fa = _scalar(loss)
            dpa = _scalar(vec.dot(gt, d, md1))
            self.last_loss, self.last_residual = fa, res
            return fa, dpa, gt

        def accept(a, fa, dpa):
            if not np.isfinite(fa) or not np.isfinite(dpa):
                return False
            if dpa < c2 * dphi0:
                return False
            if fa <= f0 + c1 * a * dphi0:
                return True
            return fa <= f0 + eps and dpa <= (2 * c1 - 1) * dphi0

        lo = (0.0, f0, dphi0)  # phi' < 0 end of the bracket
        hi = None
        a = alpha
        evals = 0
        best = None
        while evals < self.maxls:
            fa, dpa, gt = phi(a)
            evals += 1
            if accept(a, fa, dpa):
                return True, a, fa, gt.detach().clone()
            if np.isfinite(fa) and fa < f0 and (best is None or fa < best[1]):
                best = (a, fa)
            bad = not np.isfinite(fa) or fa > f0 + eps
            if hi is None:
                if bad or dpa >= 0:
                    hi = (a, fa, dpa)
                else:
                    lo = (a, fa, dpa)
                    a = 2.0 * a
                    continue
            else:
                if bad or dpa >= 0:
                    hi = (a, fa, dpa)
                else:
                    lo = (a, fa, dpa)
            al, ah = lo[0], hi[0]
            if abs(ah - al) <= 1e-14 * max(abs(al), abs(ah), 1e-300):
                break
            # Secant on phi' when the upper end has a usable derivative.
            cand = None
            if np.isfinite(hi[2]) and hi[2] >= 0 and hi[2] != lo[2]:
                cand = al - lo[2] * (ah - al) / (hi[2] - lo[2])
            lo_b, hi_b = min(al, ah), max(al, ah)
            if cand is None or not np.isfinite(cand) or not (
                    lo_b + 0.05 * (hi_b - lo_b) <= cand <= hi_b - 0.05 * (hi_b - lo_b)):
                cand = 0.5 * (al + ah)
            a = cand
        if best is not None:
            fa, dpa, gt = phi(best[0])
            if np.isfinite(fa) and fa < f0:
                return True, best[0], fa, gt.detach().clone()
        return False, 0.0, f0, None


def _cubic_min(a, fa, da, b, fb, db):
    """Minimizer of the cubic interpolating (a, fa, da), (b, fb, db),
    safeguarded to the inner 80% of the interval (bisection fallback)."""
    lo, hi = min(a, b), max(a, b)
    try:
        d1 = da + db - 3 * (fa - fb) / (a - b)
        s = d1 * d1 - da * db
        if s >= 0 and np.isfinite(s):
            d2 = math.copysign(math.sqrt(s), b - a)
            t = b - (b - a) * (db + d2 - d1) / (db - da + 2 * d2)
            if np.isfinite(t) and lo + 0.1 * (hi - lo) <= t <= hi - 0.1 * (hi - lo):
                return t
    except (ZeroDivisionError, ValueError):
        pass
    return 0.5 * (a + b)


def _solve_upper(R, b, lower=False):
    import scipy.linalg
    if len(b) == 0:
        return b
    return scipy.linalg.solve_triangular(R, b, lower=lower)


class AdamNativeOptimizer(Optimizer):
    """optimizer.py:271-322, the update in one fused kernel per step."""

    def __init__(self, dtype=None, name="adamn", displayname="AdamNative",
                 **kwargs):
        super().__init__(name=name, displayname=displayname, dtype=dtype)

    def _steps(self, epoch_start, epochs):
        return range(epoch_start + 1, epoch_start + epochs + 1)

    def run(self, x0, loss_grad, epochs=None, callback=None, lr=1e-3,
            epoch_start=0, beta_1=0.9, beta_2=0.999, epsilon=1e-7, **kwargs):
        x = x0.detach().clone()
        m = torch.zeros_like(x)
        v = torch.zeros_like(x)
        t = 0
        for epoch in self._steps(epoch_start, epochs):
            loss, grad, res = loss_grad(x, epoch)
            self.evals += 1
            self.last_loss, self.last_residual = loss, res
            t += 1
            alpha = lr * math.sqrt(1 - beta_2**t) / (1 - beta_1**t)
            vec.adam_step(x, grad, m, v, alpha, beta_1, beta_2, epsilon)
            if epoch > 0 and callback is not None:
                callback(x, epoch=epoch, opt=self)
        info = Namespace(epochs=epochs, evals=self.evals)
        return x, info


class AdamOptimizer(AdamNativeOptimizer):
    """optimizer.py:183-238: Keras Adam run by model.fit for epochs + 1
    steps; the same update equations as AdamNative."""

    def __init__(self, dtype=None, **kwargs):
        super().__init__(dtype=dtype, name="adam", displayname="Adam")

    def _steps(self, epoch_start, epochs):
        return range(epoch_start, epoch_start + epochs + 1)


class GdOptimizer(Optimizer):
    """optimizer.py:241-268: x -= lr * grad."""

    def __init__(self, dtype=None, **kwargs):
        super().__init__(name="gd", displayname="GD", dtype=dtype)

    def run(self, x0, loss_grad, epochs=None, callback=None, lr=1e-3,
            epoch_start=0, **kwargs):
        x = x0.detach().clone()
        for epoch in range(epoch_start + 1, epoch_start + epochs + 1):
            loss, grad, res = loss_grad(x, epoch)
            vec.axpby(x, 1.0, x, -lr, grad)
            self.evals += 1
            self.last_loss, self.last_residual = loss, res
            if epoch > 0 and callback is not None:
                callback(x, epoch=epoch, opt=self)
        return x, Namespace(epochs=epochs, evals=self.evals)


def make_optimizer(name, dtype=None, **kwargs):
    """optimizer.py:325-338."""
    if name == "lbfgsb":
        return LbfgsOptimizer(dtype=dtype, **kwargs)
    if name == "lbfgs":
        return LbfgsOptimizer(dtype=dtype, name="lbfgs",
                              displayname="L-BFGS", **kwargs)
    if name == "adam":
        return AdamOptimizer(dtype=dtype, **kwargs)
    if name == "adamn":
        return AdamNativeOptimizer(dtype=dtype, **kwargs)
    if name == "gd":
        return GdOptimizer(dtype=dtype, **kwargs)
    raise ValueError("Unknown optimizer '{}'".format(name))
