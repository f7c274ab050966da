"""Operators in stencil form on the GPU (the reference's SparseOperator,
multigrid.py:877-1214) and the geometric multigrid built on them
(MultigridOp, multigrid.py:342-602).

A ``StencilOp`` holds shifts and a device tensor of coefficient fields
[nshift, *nwh]; every product runs in libodil_gb300 (stencil.cu).
"""
import ctypes
import itertools

import numpy as np
import torch

from . import _capi
from ._capi import call, ptr, stream_handle

_pair_ws = {}


def _pair_workspace(device):
    key = str(device)
    if key not in _pair_ws:
        nb = _capi.load().odil_stencil_pair_workspace_bytes()
        _pair_ws[key] = torch.zeros(int(nb), dtype=torch.uint8, device=device)
    return _pair_ws[key]


def _sfx(t):
    return "f64" if t.dtype == torch.float64 else "f32"


class StencilOp:
    """(A u)[c] = sum_s coef[s][c] u[stride c + s]."""

    def __init__(self, shifts, coef, nw, stride=1, periodic=None):
        self.nw = tuple(int(n) for n in nw)
        self.dim = len(self.nw)
        self.stride = int(stride)
        self.periodic = tuple(bool(p) for p in (periodic or (False, ) * self.dim))
        self.nwh = tuple((n // 2) if (p and stride == 2) else (n - 1) // stride + 1
                         for n, p in zip(self.nw, self.periodic))
        self.shifts = [tuple(int(v) for v in s) for s in shifts]
        if len(self.shifts) > _capi.STENCIL_MAXS:
            raise ValueError("too many shifts (%d)" % len(self.shifts))
        self.coef = coef.reshape((len(self.shifts), ) + self.nwh).contiguous()
        self._s = self._struct()

    @property
    def dtype(self):
        return self.coef.dtype

    @property
    def device(self):
        return self.coef.device

    def _struct(self):
        st = _capi.OdilStencil()
        st.dim = self.dim
        st.stride = self.stride
        for a in range(3):
            st.periodic[a] = int(self.periodic[a]) if a < self.dim else 0
            st.nw[a] = self.nw[a] if a < self.dim else 1
        st.nshift = len(self.shifts)
        for i, s in enumerate(self.shifts):
            for a in range(3):
                st.shifts[i][a] = s[a] if a < self.dim else 0
        st.coef = self.coef.data_ptr()
        return st

    def ref(self):
        return ctypes.byref(self._s)

    def to_csr(self):
        """The operator as a device CSR matrix (torch.sparse_csr_tensor) in
        the reference's column convention (util_op.py:877-896): entry
        (c, c + shift) with the neighbour index wrapped periodically on every
        axis, zero coefficients dropped.  Stride 1 only."""
        if self.stride != 1:
            raise ValueError("to_csr supports stride 1")
        dev = self.coef.device
        n = 1
        for v in self.nw:
            n *= v
        idx = torch.arange(n, device=dev).reshape(self.nw)
        rows, cols, vals = [], [], []
        for k, sh in enumerate(self.shifts):
            col = torch.roll(idx, tuple(-v for v in sh), tuple(range(self.dim)))
            c = self.coef[k].reshape(-1)
            keep = c != 0
            rows.append(idx.reshape(-1)[keep])
            cols.append(col.reshape(-1)[keep])
            vals.append(c[keep])
        r = torch.cat(rows)
        c = torch.cat(cols)
        v = torch.cat(vals)
        order = torch.argsort(r * n + c)
        coo = torch.sparse_coo_tensor(torch.stack([r[order], c[order]]), v[order],
                                      (n, n)).coalesce()
        return coo.to_sparse_csr()

    def mul_field(self, u, out=None, alpha=1.0, beta=0.0):
        out = torch.empty(self.nwh, dtype=u.dtype, device=u.device) \
            if out is None else out
        call("odil_stencil_apply_" + _sfx(u), self.ref(), ptr(u), ptr(out),
             float(alpha), float(beta), stream_handle())
        return out

    def mul_transpose_field(self, uh, out=None, alpha=1.0, beta=0.0):
        out = torch.empty(self.nw, dtype=uh.dtype, device=uh.device) \
            if out is None else out
        call("odil_stencil_apply_t_" + _sfx(uh), self.ref(), ptr(uh), ptr(out),
             float(alpha), float(beta), stream_handle())
        return out

    def mul_transpose_op(self, other):
        """A^T B as a stencil (multigrid.py:1035-1071)."""
        shifts = sorted({tuple(np.array(b) - np.array(a)) for a in self.shifts
                         for b in other.shifts})
        coef = torch.empty((len(shifts), ) + self.nw, dtype=self.dtype,
                           device=self.device)
        C = StencilOp(shifts, coef, self.nw, 1, self.periodic)
        ws = _pair_workspace(self.device)
        call("odil_stencil_mul_transpose_op_" + _sfx(self.coef), self.ref(),
             other.ref(), C.ref(), ptr(ws), ws.numel(), stream_handle())
        return C

    def diag(self):
        z = tuple([0] * self.dim)
        if z in self.shifts:
            return self.coef[self.shifts.index(z)]
        return torch.zeros(self.nwh, dtype=self.dtype, device=self.device)

    def to(self, dtype):
        return StencilOp(self.shifts, self.coef.to(dtype), self.nw,
                         self.stride, self.periodic)

    # -- constructors and coefficient-field algebra (multigrid.py:923-1216);
    # torch ops on the coefficient fields, on the fields' device.
    @staticmethod
    def eye(nw, stride=1, periodic=None, dtype=torch.float64, device="cuda"):
        """Identity (multigrid.py:923-927), restricted by `stride`."""
        nw = tuple(int(n) for n in nw)
        per = tuple(bool(p) for p in (periodic or (False, ) * len(nw)))
        nwh = tuple((n // 2) if (p and stride == 2) else (n - 1) // stride + 1
                    for n, p in zip(nw, per))
        return StencilOp([(0, ) * len(nw)],
                         torch.ones((1, ) + nwh, dtype=dtype, device=device),
                         nw, stride, per)

    @staticmethod
    def from_diag(c, nw, stride=1, periodic=None):
        """diag(c) (the reference's static `SparseOperator.diag`,
        multigrid.py:929-933); `c` has the output grid's shape."""
        nw = tuple(int(n) for n in nw)
        return StencilOp([(0, ) * len(nw)], c.reshape((1, ) + tuple(c.shape)),
                         nw, stride, periodic)

    @staticmethod
    def apply_stride(u, stride):
        """u[::stride, ...] (multigrid.py:935-940)."""
        return u[(slice(None, None, int(stride)), ) * u.dim()]

    @staticmethod
    def apply_shift(u, dw, periodic=None):
        """The field u[i + dw] (multigrid.py:942-947): zero where i + dw is
        outside the grid, wrapped on periodic axes."""
        dw = tuple(int(v) for v in dw)
        periodic = periodic or (False, ) * u.dim()
        res = u
        for ax, (s, p) in enumerate(zip(dw, periodic)):
            if s == 0:
                continue
            if p:
                res = torch.roll(res, -s, ax)
                continue
            out = torch.zeros_like(res)
            n = res.shape[ax]
            if abs(s) < n:
                src = [slice(None)] * res.dim()
                dst = [slice(None)] * res.dim()
                if s > 0:
                    src[ax], dst[ax] = slice(s, n), slice(0, n - s)
                else:
                    src[ax], dst[ax] = slice(0, n + s), slice(-s, n)
                out[tuple(dst)] = res[tuple(src)]
            res = out
        return res

    def _with(self, shifts, coef):
        return StencilOp(shifts, coef, self.nw, self.stride, self.periodic)

    def eliminate_zeros(self):
        """Drops the shifts whose coefficients are all zero, in place
        (multigrid.py:949-956)."""
        keep = [i for i in range(len(self.shifts))
                if bool(torch.any(self.coef[i] != 0))]
        self.shifts = [self.shifts[i] for i in keep]
        self.coef = self.coef[keep].contiguous() if keep else \
            self.coef[:0].contiguous()
        self._s = self._struct()
        return self

    def mul_self_transpose(self):
        """A^T A (multigrid.py:1073-1074)."""
        return self.mul_transpose_op(self)

    def mul_op(self, other):
        """A B: not provided by the reference either (multigrid.py:1076-1093
        raises before its body)."""
        raise NotImplementedError

    def mul_elementwise(self, other):
        """Hadamard product on the common shifts (multigrid.py:1095-1136)."""
        if self.nw != other.nw or self.stride != other.stride:
            raise ValueError("grid sizes or strides differ")
        common = [s for s in self.shifts if s in other.shifts]
        common = sorted(common, key=_serialize)
        coef = torch.stack([self.coef[self.shifts.index(s)] *
                            other.coef[other.shifts.index(s)]
                            for s in common]) if common else \
            self.coef[:0].clone()
        return self._with(common, coef)

    def add_elementwise(self, other):
        """A + B (multigrid.py:1138-1184)."""
        if self.nw != other.nw or self.stride != other.stride:
            raise ValueError("grid sizes or strides differ")
        return self.add(other)

    def shift_left(self, shift):
        """The operator whose output is shifted: (A' u)[i] = (A u)[i + shift]
        (multigrid.py:1186-1201)."""
        shift = tuple(int(v) for v in shift)
        shifts = [tuple(a + self.stride * b for a, b in zip(dw, shift))
                  for dw in self.shifts]
        coef = torch.stack([self.apply_shift(c, shift, self.periodic)
                            for c in self.coef]) if self.shifts else self.coef
        return self._with(shifts, coef)

    def shift_right(self, shift):
        """The operator applied to a shifted input: (A' u)[i] = sum_dw
        c_dw[i] u[stride i + dw + shift] (multigrid.py:1203-1215)."""
        shift = tuple(int(v) for v in shift)
        shifts = [tuple(a + b for a, b in zip(dw, shift)) for dw in self.shifts]
        return self._with(shifts, self.coef.clone())

    def add(self, other):
        """Elementwise sum (multigrid.py:1153-1196)."""
        shifts = sorted(set(self.shifts) | set(other.shifts))
        coef = torch.zeros((len(shifts), ) + self.nwh, dtype=self.dtype,
                           device=self.device)
        for s, c in zip(self.shifts, self.coef):
            coef[shifts.index(s)] += c
        for s, c in zip(other.shifts, other.coef):
            coef[shifts.index(s)] += c
        return StencilOp(shifts, coef, self.nw, self.stride, self.periodic)


def _serialize(dw, bits=3):
    """Sort key of a shift, the reference's StencilDict.serialize
    (multigrid.py:684-687)."""
    return sum((i + 2**bits) << ((1 + bits) * n) for n, i in enumerate(dw))


def _shifts(dim, r):
    return [tuple(s) for s in itertools.product(range(-r, r + 1), repeat=dim)]


def get_R(nw, restriction="full", periodic=None, dtype=torch.float64,
          device="cuda"):
    """multigrid.py:496-534: full weighting 0.5^(|s|+dim) on inner coarse
    nodes, injection on the boundary ones (non-periodic axes)."""
    nw = tuple(nw)
    dim = len(nw)
    per = tuple(bool(p) for p in (periodic or (False, ) * dim))
    nwh = tuple((n // 2) if p else (n - 1) // 2 + 1 for n, p in zip(nw, per))
    if restriction == "full":
        shifts = _shifts(dim, 1)
        coeff = lambda s: 0.5**(sum(abs(v) for v in s) + dim)
    elif restriction == "half":
        shifts = [(0, ) * dim]
        for i in range(dim):
            shifts.append(tuple(1 if j == i else 0 for j in range(dim)))
            shifts.append(tuple(-1 if j == i else 0 for j in range(dim)))
        coeff = lambda s: 0.5 if not any(s) else 0.25 / dim
    elif restriction == "injection":
        shifts = [(0, ) * dim]
        coeff = lambda s: 1.0
    else:
        raise ValueError("Unknown restriction=" + restriction)
    grids = np.meshgrid(*[np.arange(n) for n in nwh], indexing="ij")
    inner = np.ones(nwh, bool)
    for ax in range(dim):
        if not per[ax]:
            inner &= (grids[ax] > 0) & (grids[ax] + 1 < nwh[ax])
    coefs = np.stack([np.where(inner, coeff(s), 1.0 if not any(s) else 0.0)
                      for s in shifts])
    return StencilOp(shifts, torch.as_tensor(coefs, dtype=dtype, device=device),
                     nw, 2, per)


def get_TT(nw, periodic=None, dtype=torch.float64, device="cuda"):
    """multigrid.py:471-494: transpose of multilinear interpolation."""
    nw = tuple(nw)
    dim = len(nw)
    per = tuple(bool(p) for p in (periodic or (False, ) * dim))
    nwh = tuple((n // 2) if p else (n - 1) // 2 + 1 for n, p in zip(nw, per))
    shifts = _shifts(dim, 1)
    coefs = np.stack([np.full(nwh, 0.5**sum(abs(v) for v in s))
                      for s in shifts])
    return StencilOp(shifts, torch.as_tensor(coefs, dtype=dtype, device=device),
                     nw, 2, per)


def galerkin(A, R, TT):
    """Coarse operator R A T in stencil form (multigrid.py:125-131)."""
    dim = A.dim
    span = max(max(abs(v) for v in s) for s in A.shifts)
    rc = (span + 2) // 2
    shifts = _shifts(dim, rc)
    coef = torch.empty((len(shifts), ) + R.nwh, dtype=A.dtype,
                       device=A.device)
    Ac = StencilOp(shifts, coef, R.nwh, 1, A.periodic)
    ws = _pair_workspace(A.device)
    call("odil_stencil_galerkin_" + _sfx(A.coef), R.ref(), A.ref(), TT.ref(),
         Ac.ref(), ptr(ws), ws.numel(), stream_handle())
    # Drop all-zero shift fields (multigrid.py:418-421).
    keep = [i for i in range(len(shifts)) if bool(coef[i].abs().max() > 0)]
    return StencilOp([shifts[i] for i in keep], coef[keep].contiguous(),
                     R.nwh, 1, A.periodic)


def block_row(ops, us, f, u_i=None, diag=None, u_out=None, r_out=None,
              omega=1.0):
    """r = f - sum_j A_j u_j; u_out = u_i + omega r / diag."""
    n = len(ops)
    arr_ops = (ctypes.c_void_p * n)(*[ctypes.addressof(o._s) for o in ops])
    arr_us = (ctypes.c_void_p * n)(*[u.data_ptr() for u in us])
    t = us[0]
    call("odil_stencil_block_row_" + _sfx(t), n, arr_ops, arr_us, ptr(f),
         ptr(u_i), ptr(diag), ptr(u_out), ptr(r_out), float(omega),
         stream_handle())


class MultigridOp:
    """multigrid.py:342-602 on the GPU: nvar coupled fields, Galerkin
    coarsening, damped Jacobi on the diagonal blocks, V-cycle; the coarsest
    level is solved directly in FP64 (explicit inverse of the assembled
    matrix, formed once per update_A)."""

    def __init__(self, nw, nvar=1, nlevels=None, restriction="full",
                 periodic=None, dtype=torch.float64, device="cuda"):
        nw = np.array(nw)
        self.dim = len(nw)
        per = tuple(bool(p) for p in (periodic or (False, ) * self.dim))
        max_nlevels = 0
        while 2**(max_nlevels + 1) < min(nw):
            max_nlevels += 1
        nlevels = max_nlevels if nlevels is None else min(nlevels, max_nlevels)
        nnw = [tuple(int(n) for n in nw)]
        for _ in range(1, nlevels):
            nnw.append(tuple((n // 2) if p else (n - 1) // 2 + 1
                             for n, p in zip(nnw[-1], per)))
        self.nnw = nnw
        self.nlevels = nlevels
        self.nvar = nvar
        self.periodic = per
        self.dtype = dtype
        self.device = device
        self.RR = [get_R(n, restriction, per, dtype, device) for n in nnw]
        self.TT = [get_TT(n, per, dtype, device) for n in nnw]

    def update_A(self, A0):
        """A0: nvar x nvar list of StencilOp (None for empty blocks)."""
        nvar = self.nvar
        AA = [A0]
        for lvl in range(1, self.nlevels):
            AA.append([[None if A is None else
                        galerkin(A, self.RR[lvl - 1], self.TT[lvl - 1])
                        for A in row] for row in AA[-1]])
        self.AA = AA
        self.DD = [[A[i][i].diag().contiguous() for i in range(nvar)]
                   for A in AA]
        self._coarse_inv = {}

    def residual(self, A, u, f, out=None):
        r = [torch.empty_like(x) for x in f] if out is None else out
        for i in range(self.nvar):
            ops = [A[i][j] for j in range(self.nvar) if A[i][j] is not None]
            us = [u[j] for j in range(self.nvar) if A[i][j] is not None]
            block_row(ops, us, f[i], r_out=r[i])
        return r

    def smoother_jacobi(self, level, u, f, omega=1.0):
        A = self.AA[level]
        out = []
        for i in range(self.nvar):
            ops = [A[i][j] for j in range(self.nvar) if A[i][j] is not None]
            us = [u[j] for j in range(self.nvar) if A[i][j] is not None]
            ui = torch.empty_like(u[i])
            block_row(ops, us, f[i], u_i=u[i], diag=self.DD[level][i],
                      u_out=ui, omega=omega)
            out.append(ui)
        return out

    def _dense(self, level):
        """Dense matrix of level `level` (small), FP64, built by applying the
        operator to unit vectors column by column in one batched pass."""
        if level in self._coarse_inv:
            return self._coarse_inv[level]
        A = self.AA[level]
        nw = self.nnw[level]
        n = int(np.prod(nw))
        N = n * self.nvar
        M = torch.zeros((N, N), dtype=torch.float64, device=self.device)
        for j in range(self.nvar):
            for k in range(n):
                e = torch.zeros(n, dtype=self.dtype, device=self.device)
                e[k] = 1
                for i in range(self.nvar):
                    if A[i][j] is not None:
                        col = A[i][j].mul_field(e.reshape(nw)).reshape(-1)
                        M[i * n:(i + 1) * n, j * n + k] = col.double()
        # Pseudo-inverse on the device (the coarsest matrix may be singular,
        # as the reference's spsolve tolerates).
        inv = torch.linalg.pinv(M)
        self._coarse_inv[level] = inv
        return inv

    def smoother_direct(self, level, u, f):
        inv = self._dense(level)
        b = torch.cat([x.reshape(-1).double() for x in f])
        x = inv @ b  # FP64 direct solve with the precomputed inverse
        n = int(np.prod(self.nnw[level]))
        return [x[i * n:(i + 1) * n].reshape(self.nnw[level]).to(f[0].dtype)
                for i in range(self.nvar)]

    def step(self, u, f, smoother, level=0, ndirect=5, pre=2, post=2):
        """multigrid.py:567-602."""
        if level + 1 >= self.nlevels or min(self.nnw[level]) <= ndirect:
            return self.smoother_direct(level, u, f)
        for _ in range(pre):
            u = smoother(level, u, f)
        A = self.AA[level]
        R = self.RR[level]
        T = self.TT[level]
        r = [R.mul_field(x) for x in self.residual(A, u, f)]
        du = self.step([torch.zeros_like(x) for x in r], r, smoother,
                       level + 1, ndirect, pre, post)
        u = [T.mul_transpose_field(d, out=x.clone(), beta=1.0)
             for d, x in zip(du, u)]
        for _ in range(post):
            u = smoother(level, u, f)
        return u
