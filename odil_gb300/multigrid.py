"""Geometric multigrid on assembled matrices (multigrid.py:70-339), with the
reference's module layout.

``Multigrid`` keeps the interface of the reference's CSR class: node-based
coarsening nnw[l+1] = (nnw[l] - 1) // 2 + 1 while 2^(L+1) < min(nw),
full-weighting (or half / injection) restriction with injection at the
coarse boundary nodes, multilinear interpolation, Galerkin coarse matrices
A_{l+1} = R A_l T (block-diagonal R and T for `nvar` fields), damped Jacobi
on the diagonal blocks (or on the per-cell nvar x nvar blocks with
``full=True``), a direct solve on the coarsest level, and the recursive
V-cycle ``step``.  Matrices are torch sparse CSR tensors on whatever device
the operator lives on (cuSPARSE products on the GPU); the transfer
operators are built once on the host.  The stencil-form classes are
re-exported under the reference's names: ``MultigridOp`` and
``SparseOperator`` (``odil_gb300.stencil.StencilOp``).

Two deliberate differences: the reference sizes its transfer operators with
n // 2 + 1 while its levels use (n - 1) // 2 + 1, which fails for even
sizes; here both use (n - 1) // 2 + 1.  Its recursive call does not pass
`pre` and `post` down (multigrid.py:327-329), which is kept.  The
smoothers return a new vector rather than updating `u` in place.
"""
import ctypes
import math
import itertools

import numpy as np
import torch

from ._capi import call, ptr, stream_handle
from .stencil import MultigridOp, StencilOp, _sfx

SparseOperator = StencilOp

__all__ = ["Multigrid", "MultigridDecomp", "MultigridOp", "SparseOperator"]


def _flat(idx, nw):
    """Flat C-order index of multi-indices idx [m, dim] on a grid nw."""
    return np.ravel_multi_index(tuple(idx.T), tuple(nw))


def _csr(rows, cols, vals, shape, dtype, device):
    m = torch.sparse_coo_tensor(
        torch.as_tensor(np.stack([rows, cols])),
        torch.as_tensor(np.asarray(vals, np.float64), dtype=dtype), shape,
        check_invariants=False)
    return m.coalesce().to_sparse_csr().to(device)


def _block_diag(m, nvar):
    if nvar == 1:
        return m
    coo = m.to_sparse_coo().coalesce()
    r, c = coo.indices()
    n0, n1 = m.shape
    rows = torch.cat([r + k * n0 for k in range(nvar)])
    cols = torch.cat([c + k * n1 for k in range(nvar)])
    vals = torch.cat([coo.values()] * nvar)
    return torch.sparse_coo_tensor(torch.stack([rows, cols]), vals,
                                   (n0 * nvar, n1 * nvar),
                                   check_invariants=False).coalesce() \
        .to_sparse_csr()


class Multigrid:
    """multigrid.py:70-339 on torch sparse CSR matrices."""

    def __init__(self, nw, nvar=1, nlevels=None, restriction="full",
                 dtype=torch.float64, device="cuda"):
        nw = np.array(nw)
        max_nlevels = 0
        while 2**(max_nlevels + 1) < min(nw):
            max_nlevels += 1
        nlevels = max_nlevels if nlevels is None else min(nlevels, max_nlevels)
        nnw = [nw]
        for _ in range(1, nlevels):
            nnw.append((nnw[-1] - 1) // 2 + 1)
        self.dim = len(nw)
        self.nvar = nvar
        self.nlevels = nlevels
        self.nnw = [tuple(int(v) for v in n) for n in nnw]
        self.restriction = restriction
        self.dtype = dtype
        self.device = device
        self.RRsingle = [self.get_R(n, restriction, dtype, device)
                         for n in self.nnw]
        self.RR = [_block_diag(R, nvar) for R in self.RRsingle]
        self.TT = [_block_diag(self.get_T(n, dtype, device), nvar)
                   for n in self.nnw]

    @staticmethod
    def get_T(nw, dtype=torch.float64, device="cuda"):
        """multigrid.py:194-227: interpolation [prod(nw), prod(nwh)]; fine
        node iw takes coarse nodes iw // 2 + dw, dw in {0, 1}^dim with
        dw <= iw % 2, weight 0.5^sum(iw % 2)."""
        nw = np.array(nw)
        dim = len(nw)
        nwh = (nw - 1) // 2 + 1
        iw = np.array(list(itertools.product(*[range(n) for n in nw])))
        rw = iw % 2
        rows, cols, vals = [], [], []
        for dw in itertools.product([0, 1], repeat=dim):
            dw = np.array(dw)
            ok = np.all(dw <= rw, axis=1)
            rows.append(_flat(iw[ok], nw))
            cols.append(_flat(iw[ok] // 2 + dw, nwh))
            vals.append(0.5**rw[ok].sum(1))
        return _csr(np.concatenate(rows), np.concatenate(cols),
                    np.concatenate(vals), (int(nw.prod()), int(nwh.prod())),
                    dtype, device)

    @staticmethod
    def get_R(nw, restriction="full", dtype=torch.float64, device="cuda"):
        """multigrid.py:229-281: restriction [prod(nwh), prod(nw)]; inner
        coarse nodes average the 3^dim fine nodes around 2 iwh with the
        normalised weights of `restriction`, boundary coarse nodes inject."""
        nw = np.array(nw)
        dim = len(nw)
        nwh = (nw - 1) // 2 + 1
        if restriction == "full":
            coeff = lambda dw: 0.5**np.abs(dw).sum()  # noqa: E731
        elif restriction == "half":
            coeff = lambda dw: (2 * dim if np.abs(dw).sum() == 0 else  # noqa
                                1 if np.abs(dw).sum() == 1 else 0)
        elif restriction == "injection":
            coeff = lambda dw: 1 if np.abs(dw).sum() == 0 else 0  # noqa
        else:
            raise ValueError("Unknown restriction=" + restriction)
        ddw = [np.array(d) for d in itertools.product([-1, 0, 1], repeat=dim)]
        csum = sum(coeff(d) for d in ddw)
        iwh = np.array(list(itertools.product(*[range(n) for n in nwh])))
        inner = np.all(iwh > 0, axis=1) & np.all(iwh + 1 < nwh, axis=1)
        rows, cols, vals = [], [], []
        for d in ddw:
            c = coeff(d) / csum
            if c == 0:
                continue
            rows.append(_flat(iwh[inner], nwh))
            cols.append(_flat(iwh[inner] * 2 + d, nw))
            vals.append(np.full(int(inner.sum()), c))
        b = ~inner
        rows.append(_flat(iwh[b], nwh))
        cols.append(_flat(iwh[b] * 2, nw))
        vals.append(np.ones(int(b.sum())))
        return _csr(np.concatenate(rows), np.concatenate(cols),
                    np.concatenate(vals), (int(nwh.prod()), int(nw.prod())),
                    dtype, device)

    def update_A(self, A0, DD=None, compute_lower=False):
        """multigrid.py:116-156: the matrices of every level (A0 a sparse
        matrix of the finest level, or a list of one per level) and the
        diagonals of their nvar x nvar blocks."""
        if isinstance(A0, list):
            assert len(A0) == self.nlevels
            AA = [a.to_sparse_csr() for a in A0]
        else:
            AA = [A0.to_sparse_csr()]
            for level in range(1, self.nlevels):
                AA.append(self.RR[level - 1] @ AA[-1] @ self.TT[level - 1])
        nvar = self.nvar
        DD = []
        for A in AA:
            coo = A.to_sparse_coo().coalesce()
            r, c = coo.indices()
            ns = A.shape[0] // nvar
            d = torch.zeros((nvar, nvar, ns), dtype=A.dtype, device=A.device)
            same = (r % ns) == (c % ns)
            d.index_put_(((r[same] // ns), (c[same] // ns), (r[same] % ns)),
                         coo.values()[same], accumulate=True)
            DD.append(d)
        self.AA = AA
        self.DD = DD
        # Lower triangles with the diagonal for Gauss-Seidel (the reference's
        # compute_lower path raises NameError at multigrid.py:149).
        self.LL = [self._tril(A) for A in AA] if compute_lower \
            else [None] * self.nlevels
        self._inv = {}

    @staticmethod
    def _tril(A):
        coo = A.to_sparse_coo().coalesce()
        r, c = coo.indices()
        keep = c <= r
        return torch.sparse_coo_tensor(coo.indices()[:, keep],
                                       coo.values()[keep], A.shape,
                                       check_invariants=False) \
            .coalesce().to_sparse_csr()

    def smoother_jacobi(self, level, u, f, omega=1.0, full=False):
        """multigrid.py:283-299: u += omega D^-1 (f - A u), with D the
        diagonal blocks (full=False) or the per-cell nvar x nvar blocks."""
        A, D = self.AA[level], self.DD[level]
        r = f - A @ u
        if full:
            ns = A.shape[0] // self.nvar
            d = D.permute(2, 0, 1)  # [ns, nvar, nvar]
            du = torch.linalg.solve(d, r.reshape(self.nvar, ns).T.unsqueeze(-1))
            du = du.squeeze(-1).T.reshape(-1)
        else:
            du = r / torch.cat([D[i, i] for i in range(self.nvar)])
        return u + du * omega

    def smoother_gauss_seidel(self, level, u, f, omega=1.0):
        """multigrid.py:301-305: u += omega (L^-1 (f - (A - L) u) - u), L
        the lower triangle of A with its diagonal (update_A with
        compute_lower=True)."""
        A, L = self.AA[level], self.LL[level]
        b = (f - (A @ u - L @ u)).reshape(-1, 1)
        x = torch.triangular_solve(b, L, upper=False).solution.reshape(-1)
        return u + (x - u) * omega

    DIRECT_MAX = 16384  # unknowns of a level the direct solve accepts

    def smoother_direct(self, level, u, f):
        """multigrid.py:307-310: the direct solve of the level (a dense LU
        of the assembled matrix, formed once per update_A).  The reference's
        spsolve has no size limit; a dense factor here is kept to at most
        DIRECT_MAX unknowns (2 GiB in FP64).  Larger levels are solved by
        BiCGStab on the sparse matrix to a relative residual of 1e-12
        (`_solve_iterative`), which stands in for the exact solve."""
        lu = self._inv.get(level)
        if lu is None:
            n = self.AA[level].shape[0]
            if n > self.DIRECT_MAX:
                return self._solve_iterative(self.AA[level], f.reshape(-1))
            lu = self._inv[level] = torch.linalg.lu_factor(
                self.AA[level].to_dense())
        return torch.linalg.lu_solve(*lu, f.reshape(-1, 1)).reshape(-1)

    @staticmethod
    def _solve_iterative(A, f, rtol=1e-12, maxiter=None):
        """BiCGStab (van der Vorst) on the sparse matrix A from zero, until
        |f - A x| <= rtol |f|, at most `maxiter` (default 4 sqrt(n) + 100)
        iterations; stops early at a breakdown (a zero inner product).
        Raises FloatingPointError if the iterate becomes non-finite."""
        n = f.numel()
        maxiter = maxiter or int(4 * n**0.5) + 100
        x = torch.zeros_like(f)
        r = f.clone()
        nf = torch.linalg.vector_norm(f).item()
        if nf == 0.0:
            return x
        rt = r.clone()
        p = torch.zeros_like(f)
        v = torch.zeros_like(f)
        rho = alpha = omega = 1.0
        for _ in range(maxiter):
            rho1 = torch.dot(rt, r).item()
            if rho1 == 0.0 or omega == 0.0:
                break
            p = r + (rho1 / rho) * (alpha / omega) * (p - omega * v)
            rho = rho1
            v = A @ p
            rv = torch.dot(rt, v).item()
            if rv == 0.0:
                break
            alpha = rho / rv
            s = r - alpha * v
            if torch.linalg.vector_norm(s).item() <= rtol * nf:
                x = x + alpha * p
                break
            t = A @ s
            tt = torch.dot(t, t).item()
            omega = torch.dot(t, s).item() / tt if tt > 0 else 0.0
            x = x + alpha * p + omega * s
            r = s - omega * t
            nr = torch.linalg.vector_norm(r).item()
            if not math.isfinite(nr):
                raise FloatingPointError("coarse-level BiCGStab diverged")
            if nr <= rtol * nf:
                break
        return x

    def step(self, u, f, smoother, level=0, ndirect=5, pre=2, post=2):
        """multigrid.py:312-339: one V-cycle from `u`."""
        if level + 1 >= self.nlevels or min(self.nnw[level]) <= ndirect:
            return self.smoother_direct(level, u, f)
        for _ in range(pre):
            u = smoother(level, u, f)
        A, R, T = self.AA[level], self.RR[level], self.TT[level]
        r = R @ (f - A @ u)
        u = u + T @ self.step(torch.zeros_like(r), r, smoother,
                              level=level + 1, ndirect=ndirect)
        for _ in range(post):
            u = smoother(level, u, f)
        return u


# -- multigrid decomposition of a field (multigrid.py:1217-1426) -------------


def _sizes(shape):
    arr = (ctypes.c_int64 * len(shape))(*[int(v) for v in shape])
    return arr


def _fine(shape, cell):
    return tuple(2 * n if cell else 2 * n - 1 for n in shape)


def _check(u, cell):
    if not u.is_cuda:
        raise ValueError("MultigridDecomp runs on CUDA tensors (libodil_gb300); "
                         "got device %s" % u.device)
    if u.dtype not in (torch.float32, torch.float64):
        raise ValueError("MultigridDecomp supports float32 and float64")
    if not 1 <= u.dim() <= 3:
        raise NotImplementedError("MultigridDecomp supports 1 to 3 axes, got %d"
                                  % u.dim())
    if cell and min(u.shape) < 2:
        raise ValueError("cell refinement needs at least 2 cells per axis")


def _refine(u, cell, alpha=1.0, add=None, beta=0.0):
    """alpha * (one level of refinement of u) + beta * add, on the device."""
    u = u.contiguous()
    out = torch.empty(_fine(u.shape, cell), dtype=u.dtype, device=u.device)
    n = _sizes(u.shape)
    call("odil_mgdecomp_refine_" + _sfx(u), u.dim(), n, int(cell), ptr(u),
         ptr(out), float(alpha), ptr(None if add is None else add.contiguous()),
         float(beta), stream_handle(u.device))
    return out


def _refine_t(g, coarse, cell, want_gc=True, wc_alpha=None, wf_beta=None):
    """Adjoint of one refinement level: (refine^T g, wc_alpha * refine^T g,
    wf_beta * g), each None when not asked for."""
    g = g.contiguous()
    mk = lambda shape: torch.empty(shape, dtype=g.dtype, device=g.device)  # noqa
    gc = mk(coarse) if want_gc else None
    wc = mk(coarse) if wc_alpha is not None else None
    wf = mk(g.shape) if wf_beta is not None else None
    call("odil_mgdecomp_refine_t_" + _sfx(g), len(coarse), _sizes(coarse),
         int(cell), ptr(g), ptr(gc), ptr(wc),
         float(wc_alpha if wc_alpha is not None else 0.0), ptr(wf),
         float(wf_beta if wf_beta is not None else 0.0),
         stream_handle(g.device))
    return gc, wc, wf


class _Refine(torch.autograd.Function):

    @staticmethod
    def forward(ctx, u, cell):
        ctx.cell = cell
        ctx.coarse = tuple(u.shape)
        return _refine(u, cell)

    @staticmethod
    def backward(ctx, g):
        gc, _, _ = _refine_t(g, ctx.coarse, ctx.cell)
        return gc, None


class _WeightsToField(torch.autograd.Function):
    """weights_to_field as one autograd node: L refinement launches forward
    (each fused with the scale and add of its level), L adjoint launches
    backward (each fused with the scaled copies into the weights' gradient)."""

    @staticmethod
    def forward(ctx, uw, nnw, factors, cell):
        ctx.nnw, ctx.factors, ctx.cell = nnw, factors, cell
        levels = _split(uw, nnw)
        L = len(nnw)
        if L == 1:
            return levels[0] * factors[0]
        res = levels[L - 1]
        alpha = factors[L - 1]
        for lv in range(L - 2, -1, -1):
            res = _refine(res, cell, alpha, levels[lv], factors[lv])
            alpha = 1.0
        return res

    @staticmethod
    def backward(ctx, g):
        nnw, factors, cell = ctx.nnw, ctx.factors, ctx.cell
        L = len(nnw)
        if L == 1:
            return (g * factors[0]).reshape(-1), None, None, None
        parts = [None] * L
        for lv in range(L - 1):
            last = lv + 1 == L - 1
            gc, wc, wf = _refine_t(g, nnw[lv + 1], cell, want_gc=not last,
                                   wc_alpha=factors[L - 1] if last else None,
                                   wf_beta=factors[lv])
            parts[lv] = wf
            if last:
                parts[L - 1] = wc
            g = gc
        return torch.cat([p.reshape(-1) for p in parts]), None, None, None


def _split(uw, nnw):
    out, s = [], 0
    for nw in nnw:
        n = int(np.prod(nw))
        out.append(uw[s:s + n].reshape(nw))
        s += n
    if s != uw.numel():
        raise ValueError("weights have %d entries, levels %s need %d"
                         % (uw.numel(), nnw, s))
    return out


def _method(method, dim, cell):
    if method is None:
        return
    if method == "conv":
        assert dim <= 3, "method={} requires dim=1,2,3".format(method)
    elif method == "manual":
        if dim > (2 if cell else 3):
            raise NotImplementedError(
                "Expected dim=1,2{}, got {:}".format("" if cell else ",3", dim))
    elif method != "roll":
        raise NotImplementedError("Unknown method=" + method)


class MultigridDecomp:
    """multigrid.py:1217-1426: a field as the sum of weights on levels
    (finest first) refined to the finest grid.  Node levels refine
    n -> 2n - 1 (multilinear), cell levels n -> 2n (weights 3/4, 1/4 with
    linearly extrapolated halo cells).  Every refinement runs in
    libodil_gb300 (mgdecomp.cu) on CUDA tensors and is differentiable
    (the adjoint runs there too).  The reference's interpolation methods
    ('conv', 'roll', 'manual') give one result; `method` is validated as
    the reference does and otherwise ignored.  `mod` is accepted for
    signature compatibility.  Up to 3 axes."""

    @staticmethod
    def interp_node_field(u, depth=1, mod=None, method=None):
        return MultigridDecomp.interp_field(u, depth, mod, method, cell=False)

    @staticmethod
    def interp_cell_field(u, depth=1, mod=None, method=None):
        return MultigridDecomp.interp_field(u, depth, mod, method, cell=True)

    @staticmethod
    def interp_field(u, depth=1, mod=None, method=None, cell=False):
        if depth == 0:
            return u
        _method(method, u.dim(), cell)
        _check(u, cell)
        for _ in range(depth):
            u = _Refine.apply(u, bool(cell))
        return u

    @staticmethod
    def weights_to_fields(uw, nnw, mod=None, method=None, factors=None,
                          cell=False):
        nnw = _check_levels(nnw, cell)
        factors = [1.0] * len(nnw) if factors is None else factors
        return [MultigridDecomp.interp_field(u * float(f), i, mod, method,
                                             cell)
                for i, (u, f) in enumerate(zip(_split(uw, nnw), factors))]

    @staticmethod
    def get_weights_coarse_ones(nnw, dtype, mod=None, device="cuda"):
        return torch.cat([torch.full((int(np.prod(nw)), ),
                                     float(i == len(nnw) - 1), dtype=dtype,
                                     device=device)
                          for i, nw in enumerate(nnw)])

    @staticmethod
    def weights_to_field(uw, nnw, mod=None, method=None, factors=None,
                         cell=False):
        nnw = _check_levels(nnw, cell)
        factors = [float(f) for f in
                   ([1.0] * len(nnw) if factors is None else factors)]
        if len(factors) != len(nnw):
            raise ValueError("%d factors for %d levels" % (len(factors),
                                                           len(nnw)))
        _method(method, len(nnw[0]), cell)
        _check(uw, False)
        if uw.dim() != 1:
            raise ValueError("weights must be a flat vector")
        return _WeightsToField.apply(uw, nnw, factors, bool(cell))


def _check_levels(nnw, cell):
    """Level sizes, finest first; each level must refine onto the next
    finer one exactly (the sum of weights_to_field is taken point by point)."""
    nnw = [tuple(int(v) for v in nw) for nw in nnw]
    if not nnw or any(len(nw) != len(nnw[0]) for nw in nnw):
        raise ValueError("levels must be non-empty and of one rank: %s" % nnw)
    if not 1 <= len(nnw[0]) <= 3:
        raise NotImplementedError("MultigridDecomp supports 1 to 3 axes")
    for lv in range(len(nnw) - 1):
        if min(nnw[lv + 1]) < (2 if cell else 1) or \
                _fine(nnw[lv + 1], cell) != nnw[lv]:
            raise ValueError("level %d %s does not refine onto level %d %s"
                             % (lv + 1, nnw[lv + 1], lv, nnw[lv]))
    return nnw
