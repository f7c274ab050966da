"""1D wave operator family: the registered, fused-kernel form of
wave.py:67-122 (operator_fd) of the reference.

``WaveOperator`` is a drop-in ``operator(mod, ctx)``: called with the torch
``mod`` it evaluates the residual op by op (generic path, used to validate the
fused path), and ``Problem`` binds it to ``WaveKernels``, which run the
hand-written kernels of libodil_gb300 on the GPU.
"""
import ctypes

import numpy as np
import torch

from . import _capi
from ._capi import call, ptr, stream_handle


from .problem import extrap_quadh  # noqa: E402  (util_op.py:1017-1023)


class WaveOperator:
    """Registered operator family "wave".

    Boundary data as wave.py:457-464 builds them: ``init_u``, ``init_ut``
    ([nx], at t=0 and x cell centres), ``left_u``/``right_u`` ([nt], at
    x = lower/upper and t cell centres).  ``c`` is the wave speed (the
    reference has c = 1).
    """
    family = "wave"

    def __init__(self, init_u, init_ut, left_u, right_u, c=1.0):
        self.init_u = np.asarray(init_u, np.float64)
        self.init_ut = np.asarray(init_ut, np.float64)
        self.left_u = np.asarray(left_u, np.float64)
        self.right_u = np.asarray(right_u, np.float64)
        self.c = float(c)

    def bind(self, domain):
        assert domain.ndim == 2 and len(domain.fieldnames) == 1, \
            "the wave family has one field on a (t, x) grid"
        nt, nx = domain.shape
        return WaveKernels(nt, nx, domain.step(0), domain.step(1), self.c,
                           self.init_u, self.init_ut, self.left_u,
                           self.right_u, device=domain.device)

    def __call__(self, mod, ctx):
        """Op-by-op form of wave.py:67-122 (generic path)."""
        dt = ctx.step(0)
        dx = ctx.step(1)
        it = ctx.cell_index(0)
        ix = ctx.cell_index(1)
        nx = ctx.size(1)
        key = ctx.domain.fieldnames[0]
        st = [
            ctx.field(key),
            ctx.field(key, -1, 0),
            ctx.field(key, -2, 0),
            ctx.field(key, -1, -1),
            ctx.field(key, -1, 1)
        ]
        left_utm = mod.roll(self.left_u, 1, axis=0)
        right_utm = mod.roll(self.right_u, 1, axis=0)
        st[3] = mod.where(ix == 0, extrap_quadh(st[4], st[1], left_utm[:, None]),
                          st[3])
        st[4] = mod.where(ix == nx - 1,
                          extrap_quadh(st[3], st[1], right_utm[:, None]),
                          st[4])
        u, utm, utmm, uxm, uxp = st
        init_ut = mod.constant(self.init_ut)
        u_t_tm = (u - utm) / dt
        u_t_tmm = (utm - utmm) / dt
        u_t_tmm = mod.where(it == 1, init_ut[None, :], u_t_tmm)
        u_tt = (u_t_tm - u_t_tmm) / dt
        u_xx = (uxm - 2 * utm + uxp) / (dx**2)
        fu = u_tt - self.c**2 * u_xx
        u0 = mod.constant(self.init_u + 0.5 * dt * self.init_ut)
        fu = mod.where(it == 0, u - u0[None, :], fu)
        return [fu]


class WaveKernels:
    """Device-side state of one wave instance and its fused kernels.

    Holds the boundary data in FP64 and FP32 copies, the C-ABI parameter
    structs and the loss workspace.  One instance per CUDA stream: the
    workspace is reused by every loss call.
    """

    def __init__(self, nt, nx, dt, dx, c, init_u, init_ut, left_u, right_u,
                 device="cuda"):
        _capi.load()
        self.nt, self.nx = int(nt), int(nx)
        self.shape = (self.nt, self.nx)
        self.n = self.nt * self.nx
        self.dt, self.dx, self.c = float(dt), float(dx), float(c)
        self.device = torch.device(device)
        bc = [init_u, init_ut, left_u, right_u]
        sizes = [self.nx, self.nx, self.nt, self.nt]
        for a, s in zip(bc, sizes):
            if np.asarray(a).shape != (s, ):
                raise ValueError("boundary array has shape %s, expected (%d,)"
                                 % (np.asarray(a).shape, s))
        # The four FP64 arrays are views of one buffer (each segment starts
        # on a 16-byte boundary), so new boundary data arrive in one copy.
        offs, o = [], 0
        for s in sizes:
            offs.append(o)
            o += (s + 1) // 2 * 2
        self.bc64_all = torch.zeros(o, dtype=torch.float64, device=self.device)
        self.bc64 = [self.bc64_all[q:q + s] for q, s in zip(offs, sizes)]
        for d, a in zip(self.bc64, bc):
            d.copy_(torch.as_tensor(np.asarray(a, np.float64)))
        self.bc32 = [a.float() for a in self.bc64]
        self.p64 = self._params(self.bc64)
        self.p32 = self._params(self.bc32)
        nbytes = _capi.load().odil_wave_workspace_bytes(ctypes.byref(self.p64))
        self.workspace = torch.zeros(int(nbytes), dtype=torch.uint8,
                                     device=self.device)
        self.loss_buf = torch.zeros(1, dtype=torch.float64, device=self.device)
        self.ur_workspace = None

    def _params(self, bc):
        p = _capi.OdilWaveParams()
        p.nt, p.nx, p.dt, p.dx, p.c = self.nt, self.nx, self.dt, self.dx, self.c
        p.init_u, p.init_ut, p.left_u, p.right_u = [t.data_ptr() for t in bc]
        return p

    def _pp(self, t):
        if t.dtype == torch.float64:
            return ctypes.byref(self.p64), "f64"
        if t.dtype == torch.float32:
            return ctypes.byref(self.p32), "f32"
        raise TypeError("wave kernels take float32 or float64, got %s" % t.dtype)

    def _check(self, t):
        if tuple(t.shape) != self.shape and t.numel() != self.n:
            raise ValueError("field has shape %s, expected %s" %
                             (tuple(t.shape), self.shape))
        if t.device != self.device and not (t.is_cuda and
                                            self.device.type == "cuda"):
            raise ValueError("field on %s, kernels on %s" %
                             (t.device, self.device))

    def residual(self, u, out=None):
        self._check(u)
        p, sfx = self._pp(u)
        out = torch.empty_like(u) if out is None else out
        call("odil_wave_residual_" + sfx, p, ptr(u), ptr(out), stream_handle())
        return out

    def jv(self, v, out=None):
        self._check(v)
        p, sfx = self._pp(v)
        out = torch.empty_like(v) if out is None else out
        call("odil_wave_jv_" + sfx, p, ptr(v), ptr(out), stream_handle())
        return out

    def jtv(self, w, out=None):
        self._check(w)
        p, sfx = self._pp(w)
        out = torch.empty_like(w) if out is None else out
        call("odil_wave_jtv_" + sfx, p, ptr(w), ptr(out), stream_handle())
        return out

    def jtj_v(self, v, out=None):
        """J^T J v in one pass (the normal-equation matrix of
        linsolver.py:35-41, never formed)."""
        self._check(v)
        p, sfx = self._pp(v)
        out = torch.empty_like(v) if out is None else out
        ws = getattr(self, "_jtj_ws", None)
        if ws is None:
            nb = _capi.load().odil_wave_jtj_workspace_bytes(p)
            ws = self._jtj_ws = torch.zeros(nb, dtype=torch.uint8,
                                            device=self.device)
        call("odil_wave_jtj_v_" + sfx, p, ptr(v), ptr(out), ptr(ws),
             ws.numel(), stream_handle())
        return out

    def jtj_diag(self, dtype=torch.float64):
        """diag(J^T J) as a field."""
        out = torch.empty(self.shape, dtype=dtype, device=self.device)
        p, sfx = self._pp(out)
        call("odil_wave_jtj_diag_" + sfx, p, ptr(out), stream_handle())
        return out

    def loss_grad(self, u, grad=None, loss=None):
        """Fused loss+adjoint: returns (loss [1] float64 tensor, grad)."""
        self._check(u)
        p, sfx = self._pp(u)
        grad = torch.empty_like(u) if grad is None else grad
        loss = self.loss_buf if loss is None else loss
        call("odil_wave_loss_grad_" + sfx, p, ptr(u), ptr(grad), ptr(loss),
             ptr(self.workspace), self.workspace.numel(), stream_handle())
        return loss, grad

    def march(self, b, out=None):
        """Direct solve of J x = b by forward substitution."""
        self._check(b)
        p, sfx = self._pp(b)
        out = torch.empty_like(b) if out is None else out
        call("odil_wave_march_" + sfx, p, ptr(b), ptr(out), stream_handle())
        return out

    def march_shape(self, b, out, cpt, pf=None):
        """Forward substitution with an explicit launch shape: `cpt` is a
        shape dict or, with `pf`, the block shape's column count.  Shapes:
        {"kind": "block", "cpt", "pf"}: one thread block (FP32 only);
        {"kind": "tiled", "cpt", "halo", "pf", "warps", "exchange"}: column
        tiles over a thread-block cluster; {"kind": "default"}: the plain
        entry point's own choice."""
        cfg = cpt if isinstance(cpt, dict) else {"kind": "block", "cpt": cpt,
                                                 "pf": pf}
        kind = cfg.get("kind", "block")
        p, sfx = self._pp(b)
        if kind == "tiled":
            call("odil_wave_march_tiled_" + sfx, p, ptr(b), ptr(out),
                 int(cfg["cpt"]), int(cfg["halo"]), int(cfg["pf"]),
                 int(cfg["warps"]), int(cfg.get("exchange", 0)),
                 stream_handle())
        elif kind == "default":
            call("odil_wave_march_" + sfx, p, ptr(b), ptr(out),
                 stream_handle())
        else:
            if sfx != "f32":
                raise ValueError("explicit block shapes are FP32 only")
            call("odil_wave_march_shape_f32", p, ptr(b), ptr(out),
                 int(cfg["cpt"]), int(cfg["pf"]), stream_handle())
        return out

    def march_tuned(self, b, out):
        """Forward substitution with the autotuned launch shape for b's
        precision (FP32 or FP64)."""
        tuned = self.__dict__.setdefault("_march_cfgs", {})
        if b.dtype not in tuned:
            from . import autotune
            tuned[b.dtype] = autotune.tune_march(self, dtype=b.dtype)
        return self.march_shape(b, out, tuned[b.dtype])

    def initial_rhs(self, rhs):
        """rhs = float32(-F(0)) (boundary cells only do FP64 work)."""
        call("odil_wave_initial_rhs_mixed", ctypes.byref(self.p64), ptr(rhs),
             stream_handle())
        return rhs

    def initial_table(self, tbl):
        """tbl[:n] = float32(-F(0)) at the n boundary cells (rows 0 and 1,
        then columns 0 and nx-1 of each further row), FP64 work only."""
        call("odil_wave_initial_table_mixed", ctypes.byref(self.p64), ptr(tbl),
             stream_handle())
        return tbl

    def march_table(self, tbl, out):
        """out = J^-1 b for b = 0 except the boundary table ``tbl`` (see
        initial_table), with the tuned cluster-tiled FP32 shape."""
        cfg = self.__dict__.get("_march_cfgs", {}).get(torch.float32)
        if not cfg or cfg.get("kind") != "tiled":
            raise ValueError("the table march needs a tuned cluster-tiled shape")
        call("odil_wave_march_tiled_table_f32", ctypes.byref(self.p32),
             ptr(tbl), ptr(out), int(cfg["cpt"]), int(cfg["halo"]),
             int(cfg["pf"]), int(cfg["warps"]), int(cfg.get("exchange", 0)),
             stream_handle())
        return out

    def march_from_zero(self, out, rhs):
        """out = J^-1 float32(-F(0)), the first correction of a mixed solve
        from u = 0, with the tuned FP32 march shape.  A cluster-tiled shape
        reads only the boundary table of -F(0) (written at the start of
        ``rhs``; the zero interior is neither stored nor loaded); the
        single-block march gets the full right-hand side in ``rhs``.  The
        result is bitwise the same either way."""
        tuned = self.__dict__.setdefault("_march_cfgs", {})
        if torch.float32 not in tuned:
            from . import autotune
            tuned[torch.float32] = autotune.tune_march(self, dtype=torch.float32)
        cfg = tuned[torch.float32]
        if cfg.get("kind") == "tiled" and self.nx > cfg["cpt"]:
            self.initial_table(rhs)
            return self.march_table(rhs, out)
        self.initial_rhs(rhs)
        return self.march_shape(rhs, out, cfg)

    # Shifts (t, x) of the Jacobian's five slots (see wave.cu).
    SLOT_SHIFTS = ((0, 0), (-1, 0), (-2, 0), (-1, -1), (-1, 1))

    def coefficients(self, dtype=torch.float64):
        """[5, nt, nx] per-slot coefficient fields of J (the reference's
        split-shift Jacobian, util_op.py:585-614), from the column-class
        factors the kernels use (computed in FP64)."""
        nt, nx = self.nt, self.nx
        kw = dict(device=self.device, dtype=torch.float64)
        A = 1.0 / self.dt**2
        B = self.c**2 / self.dx**2
        ktm = torch.full((nx, ), 2.0, **kw)
        kxm = torch.ones(nx, **kw)
        kxp = torch.ones(nx, **kw)
        if nx == 1:
            ktm[0], kxm[0], kxp[0] = 20.0 / 3.0, 0.0, 4.0 / 9.0
        else:
            ktm[0] = ktm[-1] = 4.0
            kxm[0], kxm[-1] = 0.0, 4.0 / 3.0
            kxp[0], kxp[-1] = 4.0 / 3.0, 0.0
        cu = torch.full((nt, nx), A, **kw)
        ctm = (-2.0 * A + B * ktm)[None, :].repeat(nt, 1)
        ctmm = torch.full((nt, nx), A, **kw)
        cxm = (-B * kxm)[None, :].repeat(nt, 1)
        cxp = (-B * kxp)[None, :].repeat(nt, 1)
        cu[0] = 1.0
        for c in (ctm, ctmm, cxm, cxp):
            c[0] = 0.0
        ctmm[:2] = 0.0
        if nt > 1:
            ctm[1] = -A + B * ktm
        return torch.stack([cu, ctm, ctmm, cxm, cxp]).to(dtype)

    def pair_residual(self, hi, lo, rhs):
        """rhs = float32(-F(hi + lo)) for FP32 arrays hi, lo (lo may be None)."""
        call("odil_wave_pair_residual_mixed", ctypes.byref(self.p64), ptr(hi),
             ptr(lo), ptr(rhs), stream_handle())
        return rhs

    def update_residual_mixed(self, u, d, u_out, rhs, rnorm2=None):
        """u_out = u + d (d FP32 or None), rhs = float32(-F(u_out)) with the
        residual in FP64; optionally rnorm2[0] = sum(F^2)."""
        self._check(u)
        if u.dtype != torch.float64 or rhs.dtype != torch.float32:
            raise TypeError("FP64 field and FP32 right-hand side expected")
        if d is not None and (d.dtype != torch.float32 or u_out is None):
            raise TypeError("FP32 correction and an FP64 output expected")
        if rnorm2 is not None and self.ur_workspace is None:
            nb = _capi.load().odil_wave_update_residual_workspace_bytes(
                ctypes.byref(self.p64))
            self.ur_workspace = torch.zeros(int(nb), dtype=torch.uint8,
                                            device=self.device)
        ws = self.ur_workspace if rnorm2 is not None else None
        call("odil_wave_update_residual_mixed", ctypes.byref(self.p64), ptr(u),
             ptr(d), ptr(u_out if d is not None else None), ptr(rhs),
             ptr(rnorm2), ptr(ws), 0 if ws is None else ws.numel(),
             stream_handle())
        return rhs
