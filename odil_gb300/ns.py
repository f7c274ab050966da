"""Steady Navier-Stokes lid-driven cavity: the registered, kernel form of
ns_steady.py:142-433 (operator) with its defaults, forward and inverse
(imposed points, Laplacian penalty) problems.

Fields (u, v, p) on an (n, n) grid of [0, 1]^2.  The Jacobian at the state is
computed by a kernel as per-shift coefficient fields (the reference's
split-shift linearize, util_op.py:585-614) and applied as stencil operators:
J v and J^T w run through libodil_gb300's stencil kernels.
"""
import ctypes
import math

import numpy as np
import torch

from . import _capi
from ._capi import call, ptr, stream_handle
from .stencil import StencilOp

SHIFTS = ((0, 0), (-1, 0), (1, 0), (0, -1), (0, 1))
FIELDS = ("u", "v", "p")


class NsCavityOperator:
    """Registered operator family "ns_cavity".

    Re: Reynolds number (mu = 1/Re, ns_steady.py:867); mask/u_imp/v_imp:
    imposed points (ns_steady.py:396-404) with weight alpha; kreg: Laplacian
    penalty (406-411); pin: (ix, iy) of a cell whose pressure is pinned to 0
    with weight pin_weight (removes the constant-pressure null space)."""
    family = "ns_cavity"

    def __init__(self, Re, mask=None, u_imp=None, v_imp=None, alpha=1.0,
                 kreg=0.0, pin=None, pin_weight=1.0):
        self.Re = float(Re)
        self.mask = None if mask is None else np.asarray(mask, np.float64)
        self.u_imp = None if u_imp is None else np.asarray(u_imp, np.float64)
        self.v_imp = None if v_imp is None else np.asarray(v_imp, np.float64)
        self.alpha = float(alpha)
        self.kreg = float(kreg)
        self.pin = pin
        self.pin_weight = float(pin_weight)

    def __call__(self, mod, ctx):
        """Op-by-op form of ns_steady.py:142-433 (no-slip walls with the lid
        u = 1 at y = 1 by quadratic extrapolation to the face, Rhie-Chow
        continuity, deferred-correction upwinding): the generic path, which
        the stencil compiler traces.  Terms: fu, fv, fp, then the imposed
        points, the Laplacian penalty and the pressure pin when set."""
        from .problem import extrap_linear, extrap_quadh
        dx, dy = ctx.step(0), ctx.step(1)
        ix, iy = ctx.cell_index(0), ctx.cell_index(1)
        nx, ny = ctx.size(0), ctx.size(1)
        mu = 1.0 / self.Re
        zeros = ctx.field("zeros")
        last_x, last_y = ix == nx - 1, iy == ny - 1
        first_x, first_y = ix == 0, iy == 0

        def var(key, freeze=False):
            """q, qxm, qxp, qym, qyp"""
            return [ctx.field(key, *sh, freeze=freeze) for sh in SHIFTS]

        def walls(st, lid):
            # halo values from the wall values (0, or `lid` at y = 1)
            st[1] = mod.where(first_x, extrap_quadh(st[2], st[0], 0), st[1])
            st[2] = mod.where(last_x, extrap_quadh(st[1], st[0], 0), st[2])
            st[3] = mod.where(first_y, extrap_quadh(st[4], st[0], 0), st[3])
            st[4] = mod.where(last_y, extrap_quadh(st[3], st[0], lid), st[4])
            return st

        def linear(st):
            st[1] = mod.where(first_x, extrap_linear(st[2], st[0]), st[1])
            st[2] = mod.where(last_x, extrap_linear(st[1], st[0]), st[2])
            st[3] = mod.where(first_y, extrap_linear(st[4], st[0]), st[3])
            st[4] = mod.where(last_y, extrap_linear(st[3], st[0]), st[4])
            return st

        def outer(st):
            """qxmm, qxpp, qymm, qypp: second neighbours, the first ones
            repeated at the walls."""
            far = [mod.roll(st[1], shift=1, axis=0),
                   mod.roll(st[2], shift=-1, axis=0),
                   mod.roll(st[3], shift=1, axis=1),
                   mod.roll(st[4], shift=-1, axis=1)]
            edge = (first_x, last_x, first_y, last_y)
            return [mod.where(e, st[q + 1], f)
                    for q, (e, f) in enumerate(zip(edge, far))]

        def upwind2(st, st5, a, b):
            q, qxm, qxp, qym, qyp = st
            qxmm, qxpp, qymm, qypp = st5
            dxm = mod.where(first_x, (q - qxm) / dx,
                            (qxmm - 4 * qxm + 3 * q) / (2 * dx))
            dxp = mod.where(last_x, (qxp - q) / dx,
                            (-3 * q + 4 * qxp - qxpp) / (2 * dx))
            dym = mod.where(first_y, (q - qym) / dy,
                            (qymm - 4 * qym + 3 * q) / (2 * dy))
            dyp = mod.where(last_y, (qyp - q) / dy,
                            (-3 * q + 4 * qyp - qypp) / (2 * dy))
            return mod.where(a > 0, dxm, dxp), mod.where(b > 0, dym, dyp)

        def upwind1(st, a, b):
            q, qxm, qxp, qym, qyp = st
            return (mod.where(a > 0, (q - qxm) / dx, (qxp - q) / dx),
                    mod.where(b > 0, (q - qym) / dy, (qyp - q) / dy))

        def second(st):
            q, qxm, qxp, qym, qyp = st
            return (qxp - 2 * q + qxm) / dx**2, (qyp - 2 * q + qym) / dy**2

        u_st, uf_st = walls(var("u"), 1), walls(var("u", True), 1)
        v_st, vf_st = walls(var("v"), 0), walls(var("v", True), 0)
        p_st, pf_st = linear(var("p")), linear(var("p", True))
        uf, vf = uf_st[0], vf_st[0]

        def deferred(live, frozen):
            # high order on the frozen field + (low order: live - frozen)
            hx, hy = upwind2(frozen, outer(frozen), uf, vf)
            lx, ly = upwind1(live, uf, vf)
            fx, fy = upwind1(frozen, uf, vf)
            return hx + lx - fx, hy + ly - fy

        u_x, u_y = deferred(u_st, uf_st)
        v_x, v_y = deferred(v_st, vf_st)
        u_xx, u_yy = second(u_st)
        v_xx, v_yy = second(v_st)
        p, pxm, pxp, pym, pyp = p_st
        fu = uf * u_x + vf * u_y - mu * (u_xx + u_yy) + (pxp - pxm) / (2 * dx)
        fv = uf * v_x + vf * v_y - mu * (v_xx + v_yy) + (pyp - pym) / (2 * dy)

        # Rhie-Chow face velocities (ns_steady.py:339-386) with the diagonal
        # g of the frozen momentum operator.
        g = mod.abs(uf) / dx + mod.abs(vf) / dy + mu * (2 / dx**2 + 2 / dy**2)
        gxm, gxp = mod.roll(g, shift=1, axis=0), mod.roll(g, shift=-1, axis=0)
        gym, gyp = mod.roll(g, shift=1, axis=1), mod.roll(g, shift=-1, axis=1)
        pf, pfxm, pfxp, pfym, pfyp = pf_st
        pfxmm, pfxpp, pfymm, pfypp = outer(pf_st)
        u, uxm, uxp = u_st[0], u_st[1], u_st[2]
        v, vym, vyp = v_st[0], v_st[3], v_st[4]
        qxm = (u + uxm) * 0.5 + (1 / gxm * (pf - pfxmm) / (2 * dx)) * 0.5 + \
            (1 / g * (pfxp - pfxm) / (2 * dx)) * 0.5 - \
            (1 / gxm + 1 / g) * 0.5 * (p - pxm) / dx
        qxp = (u + uxp) * 0.5 + (1 / gxp * (pfxpp - pf) / (2 * dx)) * 0.5 + \
            (1 / g * (pfxp - pfxm) / (2 * dx)) * 0.5 - \
            (1 / gxp + 1 / g) * 0.5 * (pxp - p) / dx
        qym = (v + vym) * 0.5 + (1 / gym * (pf - pfymm) / (2 * dy)) * 0.5 + \
            (1 / g * (pfyp - pfym) / (2 * dy)) * 0.5 - \
            (1 / gym + 1 / g) * 0.5 * (p - pym) / dy
        qyp = (v + vyp) * 0.5 + (1 / gyp * (pfypp - pf) / (2 * dy)) * 0.5 + \
            (1 / g * (pfyp - pfym) / (2 * dy)) * 0.5 - \
            (1 / gyp + 1 / g) * 0.5 * (pyp - p) / dy
        qxm = mod.where(first_x, zeros, qxm)
        qxp = mod.where(last_x, zeros, qxp)
        qym = mod.where(first_y, zeros, qym)
        qyp = mod.where(last_y, zeros, qyp)
        fp = (qxp - qxm) / dx + (qyp - qym) / dy
        res = [fu, fv, fp]
        if self.mask is not None:
            coeff = self.alpha * nx * ny / float(np.sum(self.mask))
            m = mod.constant(self.mask)
            res += [m * (u - mod.constant(self.u_imp)) * coeff,
                    m * (v - mod.constant(self.v_imp)) * coeff]
        if self.kreg:
            k = self.kreg
            res += [u_xx * k, u_yy * k, v_xx * k, v_yy * k]
        if self.pin is not None:
            pin = np.zeros((nx, ny))
            pin[tuple(self.pin)] = 1.0
            res += [mod.constant(pin) * p * self.pin_weight]
        return res

    def bind(self, domain):
        assert domain.ndim == 2 and tuple(domain.fieldnames[:3]) == FIELDS
        n = domain.shape[0]
        assert domain.shape == (n, n)
        return NsKernels(n, self, device=domain.device)


class NsKernels:
    """Device state of one cavity problem."""

    def __init__(self, n, op, device="cuda"):
        _capi.load()
        self.n = int(n)
        self.shape = (self.n, self.n)
        self.N = self.n * self.n
        self.op = op
        self.device = torch.device(device)
        dev = self.device
        self._arr = {}
        for dt in (torch.float32, torch.float64):
            self._arr[dt] = [None if a is None else
                             torch.as_tensor(a, dtype=dt, device=dev)
                             for a in (op.mask, op.u_imp, op.v_imp)]
        self.params = {dt: self._params(dt) for dt in self._arr}
        self.neq = _capi.load().odil_ns_num_equations(
            ctypes.byref(self.params[torch.float64]))
        if self.neq < 0:
            raise ValueError("invalid cavity parameters")
        self.loss_buf = torch.zeros(1, dtype=torch.float64, device=dev)

    def _params(self, dt):
        q = _capi.OdilNsParams()
        q.n = self.n
        q.re = self.op.Re
        q.kreg = self.op.kreg
        mask, ui, vi = self._arr[dt]
        q.mask = None if mask is None else mask.data_ptr()
        q.u_imp = None if ui is None else ui.data_ptr()
        q.v_imp = None if vi is None else vi.data_ptr()
        nimp = 0 if self.op.mask is None else float(np.sum(self.op.mask))
        q.imp_coeff = self.op.alpha * self.N / nimp if nimp else 0.0
        q.pin = -1 if self.op.pin is None else \
            int(self.op.pin[0]) * self.n + int(self.op.pin[1])
        q.pin_weight = self.op.pin_weight
        return q

    def _sfx(self, t):
        if t.dtype not in self.params:
            raise TypeError("cavity kernels take float32 or float64")
        return ctypes.byref(self.params[t.dtype]), \
            "f64" if t.dtype == torch.float64 else "f32"

    def residual(self, u, v, p, out=None):
        """[neq, n, n] residual terms."""
        q, sfx = self._sfx(u)
        out = torch.empty((self.neq, ) + self.shape, dtype=u.dtype,
                          device=u.device) if out is None else out
        call("odil_ns_residual_" + sfx, q, ptr(u), ptr(v), ptr(p), ptr(out),
             stream_handle())
        return out

    def jacobian(self, u, v, p):
        """J[e][field]: StencilOp of d f_e / d field at the state."""
        q, sfx = self._sfx(u)
        coef = torch.empty((self.neq, 15) + self.shape, dtype=u.dtype,
                           device=u.device)
        call("odil_ns_jacobian_" + sfx, q, ptr(u), ptr(v), ptr(p), ptr(coef),
             stream_handle())
        return [[StencilOp(SHIFTS, coef[e, 5 * j:5 * j + 5].contiguous(),
                           self.shape) for j in range(3)]
                for e in range(self.neq)]

    @staticmethod
    def jv(J, w):
        """J w for w = (wu, wv, wp): list of neq fields."""
        out = []
        for row in J:
            acc = None
            for j, A in enumerate(row):
                if acc is None:
                    acc = A.mul_field(w[j])
                else:
                    A.mul_field(w[j], out=acc, beta=1.0)
            out.append(acc)
        return out

    @staticmethod
    def jtv(J, r, scale=1.0):
        """J^T r for r = list of neq fields: (gu, gv, gp)."""
        out = []
        for j in range(3):
            acc = None
            for e, row in enumerate(J):
                if acc is None:
                    acc = row[j].mul_transpose_field(r[e], alpha=scale)
                else:
                    row[j].mul_transpose_field(r[e], out=acc, alpha=scale,
                                               beta=1.0)
            out.append(acc)
        return out

    def loss_grad(self, u, v, p):
        """loss = sum_e mean(f_e^2), grads = (2/N) J^T f (the reference's
        tape gradient through the live fields, util_op.py:627-654)."""
        f = self.residual(u, v, p)
        J = self.jacobian(u, v, p)
        g = self.jtv(J, list(f), scale=2.0 / self.N)
        loss = (f.double()**2).mean(dim=(1, 2)).sum()
        return loss, g


class NsDirectNewton:
    """Newton for the forward cavity problem with a direct GPU solve.

    The reference solves each Newton step's normal equations with SuperLU
    (util.py:242-268, linsolver.py:28-45).  Here the square Jacobian, with the
    continuity row of the pinned cell replaced by p[pin] = 0, is factored in
    FP32 as a block-tridiagonal LU (odil_ns_direct_factor), and each step
    J d = -F is solved by iterative refinement: the FP32 factors give a
    correction, the FP64 stencil J d (current Jacobian) the new residual of
    the linear system.  The factors are reused across epochs while the
    refinement still contracts fast (the Jacobian changes slowly near the
    solution); a step that needs more than `max_refine` // 2 corrections
    triggers a new factorisation for the next one.  Each linear system is
    solved to `rtol` of its right-hand side: the outer iteration converges
    linearly anyway (the Jacobian leaves out the frozen second-order upwind
    part, as the reference's does), so an inexact step costs no epochs.  The
    pressure is fixed at the pinned cell; the reference leaves the constant
    free, so compare pressures up to a constant.  Forward problem only."""

    def __init__(self, kernels, pin=(0, 0)):
        if kernels.neq != 3:
            raise ValueError("direct Newton needs the forward problem "
                             "(no imposed points, penalty or pin term)")
        self.k = kernels
        self.n = kernels.n
        self.pin = int(pin[0]) * self.n + int(pin[1])
        lib = _capi.load()
        nb = lib.odil_ns_direct_workspace_bytes(self.n)
        if nb <= 0:
            raise ValueError("cavity side %d outside the direct solver's range"
                             % self.n)
        dev = kernels.device
        self.ws = torch.empty(nb, dtype=torch.uint8, device=dev)
        shape = (3, 15, self.n, self.n)
        self.coef = torch.empty(shape, dtype=torch.float64, device=dev)
        self.coef_fac = torch.empty(shape, dtype=torch.float64, device=dev)
        self.b32 = torch.empty((3, self.n, self.n), dtype=torch.float32,
                               device=dev)
        self.x32 = torch.empty_like(self.b32)
        self.factored = False
        self.stats = []

    def _pinned(self, r, p_field):
        i, j = divmod(self.pin, self.n)
        r[2, i, j] = p_field[i, j]
        return r

    def jacobian(self, u, v, p):
        q = ctypes.byref(self.k.params[torch.float64])
        call("odil_ns_jacobian_f64", q, ptr(u), ptr(v), ptr(p), ptr(self.coef),
             stream_handle())

    def factor(self):
        """Factors the current Jacobian (call jacobian() first)."""
        self.coef_fac.copy_(self.coef)
        call("odil_ns_direct_factor", self.n, ptr(self.coef_fac), self.pin,
             ptr(self.ws), self.ws.numel(), stream_handle())
        self.factored = True

    def solve32(self, b):
        self.b32.copy_(b)
        call("odil_ns_direct_solve", self.n, ptr(self.coef_fac), self.pin,
             ptr(self.ws), self.ws.numel(), ptr(self.b32), ptr(self.x32),
             stream_handle())
        return self.x32

    def apply(self, d):
        """J' d in FP64 with the current Jacobian (pinned row = d_p[pin])."""
        J = [[StencilOp(SHIFTS, self.coef[e, 5 * f:5 * f + 5], self.k.shape)
              for f in range(3)] for e in range(3)]
        out = torch.stack(self.k.jv(J, [d[0], d[1], d[2]]))
        return self._pinned(out, d[2])

    def _refine(self, r, max_refine, rtol):
        """d with J' d ~= -r by refinement on the current factors; stops at
        `rtol`, after `max_refine` corrections, or when a correction fails to
        halve the residual (stale factors)."""
        d = torch.zeros_like(r)
        res = -r
        rn0 = float(torch.linalg.vector_norm(res))
        rn, it, ok = rn0, 0, True
        for it in range(1, max_refine + 1):
            d_new = d + self.solve32(res).double()
            res_new = -r - self.apply(d_new)
            rn_new = float(torch.linalg.vector_norm(res_new))
            if not rn_new < 0.5 * rn:  # no contraction (or NaN): keep d
                ok = False
                break
            d, res, rn = d_new, res_new, rn_new
            if rn <= rtol * rn0:
                break
        return d, rn, rn0, it, ok and rn <= rtol * rn0

    def step(self, u, v, p, refactor=None, max_refine=8, rtol=1e-13):
        """One Newton step in place; returns the FP64 residual rms before it.
        refactor: True / False, or None to factor when the factors are stale
        (and again within the step if refinement on the old ones stalls)."""
        f = self.k.residual(u, v, p)
        rms = float(torch.sqrt((f**2).mean()))
        r = self._pinned(f.clone(), p)
        self.jacobian(u, v, p)
        st = torch.cuda.current_stream(self.k.device)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        did = False
        e0.record(st)
        if refactor or not self.factored or (
                refactor is None and getattr(self, "_stale", True)):
            self.factor()
            did = True
        e1.record(st)
        d, rn, rn0, it, ok = self._refine(r, max_refine, rtol)
        if not ok and not did and refactor is None:
            self.factor()
            did = True
            d, rn, rn0, it, ok = self._refine(r, max_refine, rtol)
        self._stale = not ok or it > max_refine // 2
        self.stats.append({"rms": rms, "refine": it, "factored": did,
                           "lin_rel": rn / max(rn0, 1e-300),
                           "factor_ms": e0.elapsed_time(e1)})
        u += d[0]
        v += d[1]
        p += d[2]
        return rms

    def solve(self, u, v, p, epochs=60, tol=1e-10, rtol=1e-4, callback=None):
        """Inexact Newton epochs (each linear system to `rtol`) until the
        residual rms is below `tol`; returns the final rms."""
        self._stale = True
        for ep in range(epochs):
            rms = self.step(u, v, p, rtol=rtol)
            if callback is not None:
                callback(ep, rms)
            if rms <= tol:
                break
        f = self.k.residual(u, v, p)
        return float(torch.sqrt((f**2).mean()))


class NsGaussNewton:
    """Gauss-Newton for the cavity with imposed points and/or the Laplacian
    penalty (the inverse problem, ns_steady.py:396-411), whose Jacobian J
    stacks more residual terms than unknowns.  The reference solves each
    step's normal equations J^T J d = -J^T f with SuperLU (linsolver.py:
    35-45).  Here they are solved by preconditioned CG in FP64 (J^T J v by
    stencil products), with the preconditioner (J3'^T J3')^-1 applied by the
    FP32 block-tridiagonal factors of the forward Jacobian J3' (the three
    flow equations, continuity row of the pinned cell replaced): one
    transposed and one forward block solve per iteration.  The pressure
    constant is the null space of J^T J; CG stays in its complement since
    J^T f is orthogonal to it.  Each system is solved to `rtol`."""

    def __init__(self, kernels, pin=(0, 0)):
        if kernels.neq <= 3:
            raise ValueError("use NsDirectNewton for the forward problem")
        self.k = kernels
        self.n = kernels.n
        self.pin = int(pin[0]) * self.n + int(pin[1])
        lib = _capi.load()
        nb = lib.odil_ns_direct_workspace_bytes(self.n)
        if nb <= 0:
            raise ValueError("cavity side %d outside the direct solver's range"
                             % self.n)
        dev = kernels.device
        self.ws = torch.empty(nb, dtype=torch.uint8, device=dev)
        self.coef = torch.empty((kernels.neq, 15, self.n, self.n),
                                dtype=torch.float64, device=dev)
        self.b32 = torch.empty((3, self.n, self.n), dtype=torch.float32,
                               device=dev)
        self.x32 = torch.empty_like(self.b32)
        self.y32 = torch.empty_like(self.b32)
        self.stats = []

    def _J(self):
        return [[StencilOp(SHIFTS, self.coef[e, 5 * f:5 * f + 5], self.k.shape)
                 for f in range(3)] for e in range(self.k.neq)]

    def _prec(self, r):
        """(J3'^T J3')^-1 r in FP32 by the block factors."""
        self.b32.copy_(r)
        args = (self.n, ptr(self.coef), self.pin, ptr(self.ws), self.ws.numel())
        call("odil_ns_direct_solve_t", *args, ptr(self.b32), ptr(self.y32),
             stream_handle())
        call("odil_ns_direct_solve", *args, ptr(self.y32), ptr(self.x32),
             stream_handle())
        return self.x32.double()

    def step(self, u, v, p, rtol=1e-3, maxit=2000):
        """One Gauss-Newton step in place; returns the loss sum_e mean f_e^2
        before it and records the CG iterations."""
        k = self.k
        f = k.residual(u, v, p)
        loss = float((f**2).mean(dim=(1, 2)).sum())
        q = ctypes.byref(k.params[torch.float64])
        call("odil_ns_jacobian_f64", q, ptr(u), ptr(v), ptr(p), ptr(self.coef),
             stream_handle())
        call("odil_ns_direct_factor", self.n, ptr(self.coef), self.pin,
             ptr(self.ws), self.ws.numel(), stream_handle())
        J = self._J()

        def normal(w):
            return torch.stack(k.jtv(J, k.jv(J, [w[0], w[1], w[2]])))

        b = -torch.stack(k.jtv(J, list(f)))
        x = torch.zeros_like(b)
        r = b.clone()
        z = self._prec(r)
        pdir = z.clone()
        rz = float((r * z).sum())
        nb = float(torch.linalg.vector_norm(b))
        it = 0
        for it in range(1, maxit + 1):
            ap = normal(pdir)
            alpha = rz / float((pdir * ap).sum())
            x += alpha * pdir
            r -= alpha * ap
            if float(torch.linalg.vector_norm(r)) <= rtol * nb:
                break
            z = self._prec(r)
            rz_new = float((r * z).sum())
            pdir = z + (rz_new / rz) * pdir
            rz = rz_new
        self.stats.append({"loss": loss, "cg": it,
                           "lin_rel": float(torch.linalg.vector_norm(r)) /
                           max(nb, 1e-300)})
        u += x[0]
        v += x[1]
        p += x[2]
        return loss

    def solve(self, u, v, p, epochs=30, rtol=1e-3, callback=None):
        for ep in range(epochs):
            loss = self.step(u, v, p, rtol=rtol)
            if callback is not None:
                callback(ep, loss)
        f = self.k.residual(u, v, p)
        return float((f**2).mean(dim=(1, 2)).sum())


class _MgLevel:
    pass


class NsMultigridNewton:
    """Newton (forward problem) and Gauss-Newton (imposed points, penalty)
    for the cavity with the normal equations J^T J d = -J^T f solved by
    preconditioned conjugate gradients in FP32, preconditioned by one V-cycle
    of a cell-centred geometric multigrid on J^T J -- the method of the
    reference's util.optimize_multigridop_base (util.py:509-604, V-cycles of
    multigrid.py:543-602 on the normal equations of linsolver.py:35-45),
    here as hand-written kernels (csrc/ns_mg.cu):

      * fine level: J^T J applied matrix-free from the FP32 Jacobian
        coefficients (w = J x, y = J^T w), damped 3 x 3 block Jacobi;
      * coarse levels (n/2, n/4, ... while even and >= `nmin`): Galerkin
        R A P of the explicit 25-point J^T J with bilinear cell-centred
        transfers (the reference's node-based transfer needs odd sizes, the
        configuration's grid is even), same smoother;
      * coarsest level: FP64 dense inverse (Gauss-Jordan on the device);
      * each Newton step: FP64 residual f and right-hand side -J^T f, FP32
        PCG to `rtol` (device-side step scalars; one host read of |r| per
        `check` iterations), FP64 update of the fields.

    The operator must carry the pressure pin term (NsCavityOperator(...,
    pin=(i, j))): it removes the constant-pressure null space, so J^T J is
    definite on every level.  Forward solutions equal those with the pinned
    continuity row (p[pin] = 0); compare pressures up to a constant with the
    reference, which leaves the constant free."""

    def __init__(self, kernels, omega=0.5, pre=3, post=3, nmin=4, check=2):
        if kernels.op.pin is None:
            raise ValueError("NsMultigridNewton needs the pressure pin term: "
                             "NsCavityOperator(..., pin=(i, j))")
        self.k = kernels
        self.n = n = kernels.n
        self.neq = kernels.neq
        self.omega, self.pre, self.post = float(omega), int(pre), int(post)
        self.check = max(1, int(check))
        dev = kernels.device
        f32 = dict(dtype=torch.float32, device=dev)
        self.coef64 = torch.empty((self.neq, 15, n, n), dtype=torch.float64,
                                  device=dev)
        self.coef32 = torch.empty((self.neq, 15, n, n), **f32)
        self.w32 = torch.empty((self.neq, n, n), **f32)
        self.s32 = torch.empty((3, n, n), **f32)
        self.fw32 = torch.empty((self.neq, n, n), **f32)
        self.w64 = torch.empty((self.neq, n, n), dtype=torch.float64,
                               device=dev)
        self.b64 = torch.empty((3, n, n), dtype=torch.float64, device=dev)
        sizes = [n]
        while sizes[-1] % 2 == 0 and sizes[-1] // 2 >= nmin:
            sizes.append(sizes[-1] // 2)
        if 3 * sizes[-1]**2 > 1024:
            raise ValueError("cavity side %d: the coarsest multigrid level "
                             "(%d) is too large for the dense solve; use a "
                             "side of the form m 2^k with m <= 18" %
                             (n, sizes[-1]))
        self.levels = []
        for m in sizes:
            L = _MgLevel()
            L.n = m
            L.A = torch.empty((9, 25, m, m), **f32)
            L.dinv = torch.empty((9, m, m), **f32)
            for name in ("x", "x2", "b", "r", "e"):
                setattr(L, name, torch.empty((3, m, m), **f32))
            self.levels.append(L)
        last = self.levels[-1]
        K = 3 * last.n**2
        last.minv = torch.empty((K, K), dtype=torch.float64, device=dev)
        # PCG vectors and device scalars.
        from . import vec
        self.md = vec.MultiDot(3 * n * n, 1, 2, device=dev)
        self.x, self.r, self.z, self.p, self.q = [
            torch.empty((3, n, n), **f32) for _ in range(5)]
        self.sc = torch.zeros(4, dtype=torch.float64, device=dev)
        self._graph = None
        self.stats = []

    # -- operators ---------------------------------------------------------
    def _fine_apply(self, x, out, b=None, mode=0, xin=None):
        st = stream_handle()
        call("odil_nsmg_jx_f32", self.n, self.neq, ptr(self.coef32), ptr(x),
             ptr(self.w32), st)
        call("odil_nsmg_jtw_f32", self.n, self.neq, ptr(self.coef32),
             ptr(self.w32), ptr(b), ptr(xin), ptr(self.levels[0].dinv),
             ptr(out), self.omega, mode, st)
        return out

    def setup(self):
        """Hierarchy from the FP32 coefficients of the last linearisation:
        explicit fine J^T J, Galerkin levels, coarsest inverse."""
        st = stream_handle()
        L0 = self.levels[0]
        call("odil_nsmg_fine_ata", self.n, self.neq, ptr(self.coef32),
             ptr(L0.A), ptr(L0.dinv), st)
        for L, C in zip(self.levels[:-1], self.levels[1:]):
            call("odil_nsmg_galerkin", L.n, ptr(L.A), ptr(C.A), ptr(C.dinv), st)
        last = self.levels[-1]
        call("odil_nsmg_coarse_inverse", last.n, ptr(last.A), ptr(last.minv),
             st)

    def _smooth(self, lvl, x, b, out, mode):
        L = self.levels[lvl]
        if lvl == 0:
            return self._fine_apply(x, out, b=b, mode=mode, xin=x)
        call("odil_nsmg_smooth", L.n, ptr(L.A), ptr(L.dinv), ptr(x), ptr(b),
             ptr(out), self.omega, mode, stream_handle())
        return out

    def vcycle(self, b, out, lvl=0):
        """out = V(b): one V-cycle from zero on level `lvl` (FP32)."""
        L = self.levels[lvl]
        st = stream_handle()
        if lvl == len(self.levels) - 1:
            call("odil_nsmg_coarse_apply", L.n, ptr(L.minv), ptr(b), ptr(out),
                 st)
            return out
        cur, nxt = L.x, L.x2
        call("odil_nsmg_jacobi0", L.n, ptr(L.dinv), ptr(b), ptr(cur),
             self.omega, st)
        for _ in range(self.pre - 1):
            self._smooth(lvl, cur, b, nxt, 2)
            cur, nxt = nxt, cur
        self._smooth(lvl, cur, b, L.r, 1)
        C = self.levels[lvl + 1]
        call("odil_nsmg_restrict", L.n, ptr(L.r), ptr(C.b), st)
        self.vcycle(C.b, C.e, lvl + 1)
        call("odil_nsmg_prolong_add", L.n, ptr(C.e), ptr(cur), st)
        for k in range(self.post):
            dst = out if k == self.post - 1 else nxt
            self._smooth(lvl, cur, b, dst, 2)
            cur, nxt = dst, cur
        if self.post == 0:
            out.copy_(cur)
        return out

    def apply_normal(self, x, out):
        """out = J^T J x in FP32 (matrix-free)."""
        return self._fine_apply(x, out, mode=0)

    # -- PCG ---------------------------------------------------------------
    def _iteration(self):
        """One PCG iteration on the device (q = A p, alpha, x, r, z = V(r),
        beta, p); returns nothing, dots of r kept in self.md.out."""
        st = stream_handle()
        N = 3 * self.n * self.n
        fl = lambda a: a.reshape(-1)
        self.apply_normal(self.p, self.q)
        d = self.md(fl(self.p), 1, [fl(self.q)])
        call("odil_pcg_scalars", ptr(d), ptr(self.sc), 0, st)
        call("odil_pcg_update_xr", N, ptr(self.x), ptr(self.r), ptr(self.p),
             ptr(self.q), ptr(self.sc), st)
        self.vcycle(self.r, self.z)
        d = self.md(fl(self.r), 1, [fl(self.z), fl(self.r)])
        self.rr.copy_(d[0, 1:2])
        call("odil_pcg_scalars", ptr(d), ptr(self.sc), 1, st)
        call("odil_pcg_update_p", N, ptr(self.p), ptr(self.z), ptr(self.sc),
             st)

    def _graphs(self):
        if self._graph is not None:
            return self._graph
        dev = self.k.device
        self.rr = torch.zeros(1, dtype=torch.float64, device=dev)
        self._iteration()  # warm-up outside capture
        torch.cuda.synchronize(dev)
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side):
            for _ in range(self.check):
                self._iteration()
        torch.cuda.current_stream(dev).wait_stream(side)
        self._graph = g
        return g

    def pcg(self, b32, rtol=1e-2, maxit=500):
        """x ~= (J^T J)^-1 b32 by PCG from zero to |r| <= rtol |b|; returns
        the iteration count.  Uses the hierarchy of the last setup()."""
        st = stream_handle()
        fl = lambda a: a.reshape(-1)
        self.x.zero_()
        self.r.copy_(b32)
        nb = float(self.md(fl(b32), 1, [fl(b32)])[0, 0])**0.5
        if not math.isfinite(nb):
            raise FloatingPointError("PCG: non-finite right-hand side")
        if nb == 0.0:
            return 0
        self.vcycle(self.r, self.z)
        d = self.md(fl(self.r), 1, [fl(self.z)])
        call("odil_pcg_scalars", ptr(d), ptr(self.sc), 2, st)
        self.p.copy_(self.z)
        first = self._graph is None
        g = self._graphs()  # its first build runs one iteration eagerly
        it = 1 if first else 0
        while it < maxit:
            g.replay()
            it += self.check
            rn = float(self.rr.item())**0.5
            if not math.isfinite(rn):
                raise FloatingPointError("PCG: non-finite residual")
            if rn <= rtol * nb:
                break
        return it

    # -- Newton ------------------------------------------------------------
    def linearize(self, u, v, p):
        """FP64 Jacobian coefficients at the state (coef64) and their FP32
        copy (coef32)."""
        q = ctypes.byref(self.k.params[torch.float64])
        call("odil_ns_jacobian_f64", q, ptr(u), ptr(v), ptr(p),
             ptr(self.coef64), stream_handle())
        self.coef32.copy_(self.coef64)

    def _linearize32(self, u, v, p):
        """FP32 Jacobian coefficients at the state rounded to FP32 (the
        preconditioned FP32 solve needs no more; GB300's FP64 pipe makes the
        FP64 coefficient kernel ~15x slower)."""
        s = self.s32
        s[0].copy_(u)
        s[1].copy_(v)
        s[2].copy_(p)
        q = ctypes.byref(self.k.params[torch.float32])
        call("odil_ns_jacobian_f32", q, ptr(s[0]), ptr(s[1]), ptr(s[2]),
             ptr(self.coef32), stream_handle())

    def step(self, u, v, p, rtol=1e-2, maxit=500, f=None):
        """One (Gauss-)Newton step in place; returns the loss
        sum_e mean(f_e^2) of the state before the step (FP64).  `f`: the
        FP64 residual at the state, if already computed."""
        f = self.k.residual(u, v, p) if f is None else f
        loss = float((f**2).mean(dim=(1, 2)).sum())
        rms = float(torch.sqrt((f[:3]**2).mean()))
        self._linearize32(u, v, p)
        # b = -J^T f in FP32 (the FP64 residual rounded; the FP32 PCG solves
        # to rtol >= 1e-6 of it, and the FP64 residual drives convergence).
        self.fw32.copy_(f)
        b32 = self.levels[0].b
        call("odil_nsmg_jtw_f32", self.n, self.neq, ptr(self.coef32),
             ptr(self.fw32), None, None, None, ptr(b32), 1.0, 0,
             stream_handle())
        b32.neg_()
        self.setup()
        its = self.pcg(b32, rtol=rtol, maxit=maxit)
        self.stats.append({"loss": loss, "rms": rms, "pcg": its})
        u += self.x[0]
        v += self.x[1]
        p += self.x[2]
        return loss

    def solve(self, u, v, p, epochs=100, tol=1e-10, rtol=1e-2, callback=None):
        """(Gauss-)Newton epochs until the rms of the three flow terms is at
        most `tol` (checked before each step) or `epochs` steps are done;
        returns the final loss."""
        for ep in range(epochs):
            f = self.k.residual(u, v, p)
            if float(torch.sqrt((f[:3]**2).mean())) <= tol:
                break
            self.step(u, v, p, rtol=rtol, f=f)
            if callback is not None:
                callback(ep, self.stats[-1])
        f = self.k.residual(u, v, p)
        self.final_rms = float(torch.sqrt((f[:3]**2).mean()))
        return float((f**2).mean(dim=(1, 2)).sum())
