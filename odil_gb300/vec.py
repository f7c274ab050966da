"""Vector operations on device tensors through libodil_gb300 (no torch math on
the hot path): Adam step, axpby, deterministic dot / multi-dot, linear
combination."""
import ctypes

import torch

from . import _capi
from ._capi import call, ptr, stream_handle


def _sfx(t):
    if t.dtype == torch.float32:
        return "f32"
    if t.dtype == torch.float64:
        return "f64"
    raise TypeError("expected float32 or float64, got %s" % t.dtype)


def adam_step(x, g, m, v, alpha, beta1, beta2, eps):
    call("odil_adam_step_" + _sfx(x), ptr(x), ptr(g), ptr(m), ptr(v),
         x.numel(), float(alpha), float(beta1), float(beta2), float(eps),
         stream_handle())


def axpby(z, a, x, b, y):
    """z = a x + b y."""
    call("odil_axpby_" + _sfx(z), ptr(z), ptr(x), ptr(y), z.numel(), float(a),
         float(b), stream_handle())
    return z


class MultiDot:
    """out[i, j] = <M[i], q[j]> with a reusable workspace and output buffer."""

    def __init__(self, n, kmax, rmax=3, device="cuda"):
        self.n = int(n)
        lib = _capi.load()
        nb = lib.odil_multidot_workspace_bytes(self.n, int(kmax), int(rmax))
        self.ws = torch.zeros(int(nb), dtype=torch.uint8, device=device)
        self.out = torch.zeros(int(kmax) * int(rmax), dtype=torch.float64,
                               device=device)
        self.kmax, self.rmax = int(kmax), int(rmax)

    def __call__(self, M, k, qs, ld=None):
        r = len(qs)
        assert 1 <= k <= self.kmax and 1 <= r <= self.rmax
        arr = (ctypes.c_void_p * r)(*[q.data_ptr() for q in qs])
        ld = self.n if ld is None else ld
        call("odil_multidot_" + _sfx(M), ptr(M), ld, int(k), arr, r, self.n,
             ptr(self.out), ptr(self.ws), self.ws.numel(), stream_handle())
        return self.out[:k * r].view(k, r)


def dot(x, y, md):
    """<x, y> in FP64 (deterministic); md: a MultiDot sized for x."""
    return md(x, 1, [y])[0, 0]


def lincomb(out, x, M, k, coef, ld=None):
    """out = coef[k] x + sum_{i<k} coef[i] M[i]; coef: device float64 [k+1]."""
    n = out.numel()
    ld = n if ld is None else ld
    call("odil_lincomb_" + _sfx(out), ptr(out), ptr(x), ptr(M), ld, int(k),
         ptr(coef), n, stream_handle())
    return out
