"""2D advection operator family: the registered, fused-kernel form of
advection_2d.py:103-223 (direct problem, periodic, first-order upwind) for a
constant velocity, and its Newton solver with a matrix-free FP32 multigrid
preconditioner.

Newton (util.py:242-268, advection_2d.py:527-604) in mixed precision: every
epoch computes the FP64 residual r = F(p) on all SMs, solves J d = -r in FP32
by BiCGStab (van der Vorst 1992) right-preconditioned with one geometric
multigrid V-cycle (multigrid.py:567-602: 2 damped-Jacobi pre- and
post-smoothing sweeps, full-weighting restriction, trilinear prolongation,
dense FP64 direct solve on the coarsest level), and applies p += d in FP64.
Coarse operators rediscretise the upwind operator with doubled steps (the
Galerkin product R J P loses the diagonal dominance damped Jacobi needs).
"""
import math
import ctypes

import numpy as np
import torch

from . import _capi, vec
from ._capi import call, ptr, stream_handle


class AdvectionOperator:
    """Registered operator family "advect": fp of advection_2d.py:217-220
    with the frozen velocity (ax, ay) constant; ``p_init`` [nx, ny] is the
    previous-time value of row 0 (the reference's exact_pp at row 0)."""
    family = "advect"

    def __init__(self, ax, ay, p_init):
        self.ax, self.ay = float(ax), float(ay)
        self.p_init = np.asarray(p_init, np.float64)

    def bind(self, domain):
        assert domain.ndim == 3 and len(domain.fieldnames) == 1, \
            "the advection family has one field p on a (t, x, y) grid"
        nt, nx, ny = domain.shape
        return AdvectKernels(nt, nx, ny, domain.step(0), domain.step(1),
                             domain.step(2), self.ax, self.ay, self.p_init,
                             device=domain.device)

    def __call__(self, mod, ctx):
        """Op-by-op form (generic path) of advection_2d.py:179-220."""
        key = ctx.domain.fieldnames[0]
        dt, dx, dy = ctx.step(0), ctx.step(1), ctx.step(2)
        it = ctx.cell_index(0)
        p = ctx.field(key)
        ptm = ctx.field(key, -1, 0, 0)
        ptm = mod.where(it == 0, mod.constant(self.p_init)[None], ptm)
        pxm, pxp = ctx.field(key, 0, -1, 0), ctx.field(key, 0, 1, 0)
        pym, pyp = ctx.field(key, 0, 0, -1), ctx.field(key, 0, 0, 1)
        p_x = (p - pxm) / dx if self.ax > 0 else (pxp - p) / dx
        p_y = (p - pym) / dy if self.ay > 0 else (pyp - p) / dy
        p_t = (p - ptm) / dt
        return [p_t + self.ax * p_x + self.ay * p_y]


class _Level:
    pass


class AdvectKernels:
    """Device-side state of one advection instance."""

    def __init__(self, nt, nx, ny, dt, dx, dy, ax, ay, p_init, device="cuda"):
        _capi.load()
        self.nt, self.nx, self.ny = int(nt), int(nx), int(ny)
        self.shape = (self.nt, self.nx, self.ny)
        self.n = self.nt * self.nx * self.ny
        self.dt, self.dx, self.dy = float(dt), float(dx), float(dy)
        self.ax, self.ay = float(ax), float(ay)
        self.device = torch.device(device)
        p_init = np.asarray(p_init, np.float64).reshape(self.nx, self.ny)
        self.init64 = torch.as_tensor(p_init, device=self.device)
        self.init32 = self.init64.float()
        self.p64 = self._params(self.shape, (self.dt, self.dx, self.dy),
                                self.init64)
        self.p32 = self._params(self.shape, (self.dt, self.dx, self.dy),
                                self.init32)
        nb = _capi.load().odil_advect_workspace_bytes(ctypes.byref(self.p64))
        self.workspace = torch.zeros(int(nb), dtype=torch.uint8,
                                     device=self.device)
        self.loss_buf = torch.zeros(1, dtype=torch.float64, device=self.device)
        self._mg = None
        self._scratch = {}

    def _params(self, shape, steps, init=None):
        p = _capi.OdilAdvectParams()
        p.nt, p.nx, p.ny = shape
        p.dt, p.dx, p.dy = steps
        p.ax, p.ay = self.ax, self.ay
        p.p_init = None if init is None else init.data_ptr()
        return p

    def _pp(self, t):
        if t.dtype == torch.float64:
            return ctypes.byref(self.p64), "f64"
        if t.dtype == torch.float32:
            return ctypes.byref(self.p32), "f32"
        raise TypeError("advection kernels take float32 or float64")

    def _check(self, t):
        if t.numel() != self.n:
            raise ValueError("field has %d cells, expected %d" %
                             (t.numel(), self.n))
        if not t.is_cuda:
            raise ValueError("field on %s: CUDA tensors only" % t.device)

    def residual(self, u, out=None):
        self._check(u)
        p, sfx = self._pp(u)
        out = torch.empty_like(u) if out is None else out
        call("odil_advect_residual_" + sfx, p, ptr(u), ptr(out), stream_handle())
        return out

    def jv(self, v, out=None):
        self._check(v)
        p, sfx = self._pp(v)
        out = torch.empty_like(v) if out is None else out
        call("odil_advect_jv_" + sfx, p, ptr(v), ptr(out), stream_handle())
        return out

    def jtv(self, w, out=None):
        self._check(w)
        p, sfx = self._pp(w)
        out = torch.empty_like(w) if out is None else out
        call("odil_advect_jtv_" + sfx, p, ptr(w), ptr(out), stream_handle())
        return out

    def loss_grad(self, u, grad=None, loss=None):
        self._check(u)
        p, sfx = self._pp(u)
        grad = torch.empty_like(u) if grad is None else grad
        loss = self.loss_buf if loss is None else loss
        call("odil_advect_loss_grad_" + sfx, p, ptr(u), ptr(grad), ptr(loss),
             ptr(self.workspace), self.workspace.numel(), stream_handle())
        return loss, grad

    def update_residual_mixed(self, u, d, u_out, rhs, rnorm2=None):
        self._check(u)
        ws = self.workspace if rnorm2 is not None else None
        call("odil_advect_update_residual_mixed", ctypes.byref(self.p64),
             ptr(u), ptr(d), ptr(u_out if d is not None else None), ptr(rhs),
             ptr(rnorm2), ptr(ws), 0 if ws is None else ws.numel(),
             stream_handle())
        return rhs

    # -- multigrid ----------------------------------------------------------
    def multigrid(self, omega=0.8, pre=2, post=2, nmin=4):
        """Builds (once) the level hierarchy: halve every axis while all sizes
        stay even and >= 2 nmin."""
        if self._mg is not None:
            return self._mg
        levels = []
        shape = self.shape
        steps = (self.dt, self.dx, self.dy)
        while True:
            L = _Level()
            L.shape = shape
            L.n = int(np.prod(shape))
            L.params = self._params(shape, steps)
            kw = dict(dtype=torch.float32, device=self.device)
            L.x = torch.empty(shape, **kw)
            L.x2 = torch.empty(shape, **kw)
            L.b = torch.empty(shape, **kw)
            L.r = torch.empty(shape, **kw)
            L.e = torch.empty(shape, **kw)  # this level's correction (output)
            levels.append(L)
            if min(shape) < 2 * nmin or any(s % 2 for s in shape) or \
                    L.n <= 64:
                break
            shape = tuple(s // 2 for s in shape)
            steps = tuple(2 * h for h in steps)
        last = levels[-1]
        if last.n > 1024:
            raise ValueError("coarsest multigrid level has %d cells (> 1024);"
                             " the grid sizes need more factors of 2" % last.n)
        A = torch.empty((last.n, last.n), dtype=torch.float64,
                        device=self.device)
        call("odil_advect_dense", ctypes.byref(last.params), ptr(A),
             stream_handle())
        # The coarsest operator is tiny (<= 1024 cells): invert it once here,
        # on the device (cuSOLVER LU in libodil_gb300).
        lib = _capi.load()
        nb = lib.odil_dense_inverse_workspace_bytes(last.n)
        ws = torch.empty(max(nb, 256), dtype=torch.uint8, device=self.device)
        last.Ainv = torch.empty_like(A)
        call("odil_dense_inverse_f64", last.n, ptr(A), ptr(last.Ainv), ptr(ws),
             ws.numel(), stream_handle())
        self._mg = dict(levels=levels, omega=omega, pre=pre, post=post)
        return self._mg

    def vcycle(self, b, out, lvl=0):
        """out = V(b): one V-cycle from a zero initial guess (FP32)."""
        mg = self.multigrid()
        levels = mg["levels"]
        L = levels[lvl]
        st = stream_handle()
        if lvl == len(levels) - 1:
            call("odil_dense_apply_f64", L.n, ptr(L.Ainv), ptr(b), ptr(out), st)
            return out
        om = ctypes.c_float(mg["omega"])
        P = ctypes.byref(L.params)
        # Pre-smoothing from x = 0 (the first sweep needs no stencil).
        cur, nxt = L.x, L.x2
        call("odil_advect_mg_jacobi", P, None, ptr(b), ptr(cur), om, None, st)
        for _ in range(mg["pre"] - 1):
            call("odil_advect_mg_jacobi", P, ptr(cur), ptr(b), ptr(nxt), om,
                 None, st)
            cur, nxt = nxt, cur
        call("odil_advect_mg_jacobi", P, ptr(cur), ptr(b), None, om, ptr(L.r),
             st)
        C = levels[lvl + 1]
        call("odil_advect_mg_restrict", *L.shape, ptr(L.r), ptr(C.b), st)
        self.vcycle(C.b, C.e, lvl + 1)
        call("odil_advect_mg_prolong_add", *L.shape, ptr(C.e), ptr(cur), st)
        for k in range(mg["post"]):
            dst = out if k == mg["post"] - 1 else nxt
            call("odil_advect_mg_jacobi", P, ptr(cur), ptr(b), ptr(dst), om,
                 None, st)
            cur, nxt = dst, cur
        if mg["post"] == 0:
            out.copy_(cur)
        return out

    def _buf(self, name, dtype=torch.float32):
        t = self._scratch.get(name)
        if t is None:
            t = self._scratch[name] = torch.empty(self.shape, dtype=dtype,
                                                  device=self.device)
        return t

    def _vcycle_graphs(self, p, ph, s, sh):
        """The two V-cycles of a BiCGStab iteration (p -> ph, s -> sh) as
        CUDA graphs, captured once: a V-cycle is ~40 launches, most of them
        on small coarse levels, so replaying them saves the per-launch host
        cost."""
        g = self._scratch.get("vc_graphs")
        if g is not None:
            return g
        self.vcycle(p, ph)  # builds the hierarchy, warms up
        torch.cuda.synchronize(self.device)
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        g = []
        for src, dst in ((p, ph), (s, sh)):
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph, stream=side):
                self.vcycle(src, dst)
            g.append(graph)
        torch.cuda.current_stream(self.device).wait_stream(side)
        self._scratch["vc_graphs"] = g
        return g

    def bicgstab(self, b, x, tol=1e-6, maxit=100):
        """Right-preconditioned BiCGStab on J x = b in FP32 (x overwritten,
        zero initial guess); returns the iteration count.  The step scalars
        stay on the device (odil_bicgstab_*); the host reads the two residual
        norms it tests per iteration.

        Breakdown (<r^, r> = 0, <r^, v> = 0 or <t, t> = 0) makes the norm of
        s non-finite before x is touched in that iteration: the solve stops
        there with x at the last valid iterate and records the iteration in
        ``self.breakdowns``.  A non-finite right-hand side raises
        FloatingPointError."""
        md = self._scratch.get("md")
        if md is None:
            md = self._scratch["md"] = vec.MultiDot(self.n, 2, 2,
                                                    device=self.device)
        r, rh, p, v, ph, s, sh, t = [self._buf(k) for k in
                                     ("r", "rh", "p", "v", "ph", "s", "sh",
                                      "t")]
        vc = self._vcycle_graphs(p, ph, s, sh)
        fl = lambda a: a.reshape(-1)
        if self.n % 4:
            return self._bicgstab_host(b, x, tol, maxit, md, vc)
        sc = self._scratch.get("bicg_sc")
        if sc is None:
            sc = self._scratch["bicg_sc"] = torch.empty(4, dtype=torch.float64,
                                                        device=self.device)
        st = stream_handle()
        n = self.n
        x.zero_()
        r.copy_(b)
        rh.copy_(b)
        p.zero_()
        v.zero_()
        sc.fill_(1.0)  # rho, alpha, omega = 1; beta (sc[3]) is set before use
        nb = self._rhs_norm(md, b)
        if nb == 0:
            return 0
        for it in range(maxit):
            dots = md(fl(rh), 1, [fl(r)])
            call("odil_bicgstab_scalars", ptr(dots), ptr(sc), 0, st)
            call("odil_bicgstab_update_p", ptr(p), ptr(r), ptr(v), ptr(sc), n, st)
            vc[0].replay()  # ph = V(p)
            self.jv(ph, out=v)
            dots = md(fl(rh), 1, [fl(v)])
            call("odil_bicgstab_scalars", ptr(dots), ptr(sc), 1, st)
            call("odil_bicgstab_update_s", ptr(s), ptr(r), ptr(v), ptr(sc), n, st)
            ns = md(fl(s), 1, [fl(s)])[0, 0].item()**0.5
            if not math.isfinite(ns):
                return self._breakdown(it)
            if ns <= tol * nb:
                call("odil_bicgstab_update_xr", ptr(x), None, ptr(ph), None, None,
                     None, ptr(sc), n, 0, st)
                return it + 1
            vc[1].replay()  # sh = V(s)
            self.jv(sh, out=t)
            dots = md(fl(t), 1, [fl(t), fl(s)])
            call("odil_bicgstab_scalars", ptr(dots), ptr(sc), 2, st)
            call("odil_bicgstab_update_xr", ptr(x), ptr(r), ptr(ph), ptr(sh), ptr(s),
                 ptr(t), ptr(sc), n, 1, st)
            nr = md(fl(r), 1, [fl(r)])[0, 0].item()**0.5
            if not math.isfinite(nr):
                raise FloatingPointError(
                    "BiCGStab: non-finite residual norm in iteration %d" % it)
            if nr <= tol * nb:
                return it + 1
        return maxit

    def _rhs_norm(self, md, b):
        nb = md(b.reshape(-1), 1, [b.reshape(-1)])[0, 0].item()**0.5
        if not math.isfinite(nb):
            raise FloatingPointError("BiCGStab: non-finite right-hand side")
        return nb

    def _breakdown(self, it):
        """Records a breakdown in iteration `it` (x holds the last valid
        iterate) and returns the number of completed iterations."""
        self.breakdowns = getattr(self, "breakdowns", [])
        self.breakdowns.append(it)
        return it

    def _bicgstab_host(self, b, x, tol, maxit, md, vc):
        """The same iteration with host scalars (cell counts not divisible
        by 4)."""
        r, rh, p, v, ph, s, sh, t = [self._buf(k) for k in
                                     ("r", "rh", "p", "v", "ph", "s", "sh",
                                      "t")]
        fl = lambda a: a.reshape(-1)
        x.zero_()
        r.copy_(b)
        rh.copy_(b)
        p.zero_()
        v.zero_()
        nb = self._rhs_norm(md, b)
        if nb == 0:
            return 0
        rho = alpha = w = 1.0
        for it in range(maxit):
            rho1 = md(fl(rh), 1, [fl(r)])[0, 0].item()
            if rho1 == 0.0 or not math.isfinite(rho1) or w == 0.0:
                return self._breakdown(it)
            beta = (rho1 / rho) * (alpha / w)
            rho = rho1
            vec.axpby(p, 1.0, p, -w, v)
            vec.axpby(p, 1.0, r, beta, p)
            vc[0].replay()
            self.jv(ph, out=v)
            rv = md(fl(rh), 1, [fl(v)])[0, 0].item()
            if rv == 0.0 or not math.isfinite(rv):
                return self._breakdown(it)
            alpha = rho / rv
            vec.axpby(s, 1.0, r, -alpha, v)
            ns = md(fl(s), 1, [fl(s)])[0, 0].item()**0.5
            if not math.isfinite(ns):
                return self._breakdown(it)
            if ns <= tol * nb:
                vec.axpby(x, 1.0, x, alpha, ph)
                return it + 1
            vc[1].replay()
            self.jv(sh, out=t)
            tt = md(fl(t), 1, [fl(t), fl(s)])
            tt_ts = tt[0].cpu().numpy()
            w = tt_ts[1] / tt_ts[0] if tt_ts[0] > 0 else 0.0
            if not math.isfinite(w):
                w = 0.0
            vec.axpby(x, 1.0, x, alpha, ph)
            vec.axpby(x, 1.0, x, w, sh)
            vec.axpby(r, 1.0, s, -w, t)
            nr = md(fl(r), 1, [fl(r)])[0, 0].item()**0.5
            if not math.isfinite(nr):
                raise FloatingPointError(
                    "BiCGStab: non-finite residual norm in iteration %d" % it)
            if nr <= tol * nb:
                return it + 1
        return maxit

    def solve_mixed(self, u, epochs=3, tol=1e-5, rnorm2=None):
        """Mixed-precision Newton on the FP64 field u (in place); returns the
        inner iteration counts."""
        rhs = self._buf("rhs")
        d = self._buf("d")
        ub = self._buf("u64", torch.float64)
        ua = u
        self.update_residual_mixed(ua, None, None, rhs)
        its = []
        for e in range(epochs):
            its.append(self.bicgstab(rhs, d, tol=tol))
            self.update_residual_mixed(ua, d, ub, rhs,
                                       rnorm2 if e == epochs - 1 else None)
            ua, ub = ub, ua
        if ua is not u:
            u.copy_(ua)
        return its
