"""Oracle: geometric multigrid in stencil form, restated in NumPy.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).

Follows multigrid.py of the reference:
  * SparseOperator (multigrid.py:877-1214): an operator is a list of shifts s
    with coefficient fields C_s on the output grid (stride 1 or 2):
        (A u)[c] = sum_s C_s[c] * u[stride * c + s]   (zero outside the grid),
    mul_field 958-969, mul_transpose_field_np 1006-1027, mul_transpose_op
    1035-1071 (A^T B as a stencil);
  * MultigridOp.get_R 496-534 (full weighting 0.5^(|s|+dim) on inner coarse
    nodes, injection on boundary coarse nodes), get_TT 471-494 (transpose of
    multilinear interpolation), coarsen_sparse_operator 390-427 (Galerkin
    R A T), smoother_jacobi 543-552, step 567-602 (V-cycle), the level rule
    n -> (n - 1) // 2 + 1 while 2^(L+1) < min(n) (342-369).

Extension used by the advection workload: axes can be periodic (indices wrap
instead of dropping); with every axis non-periodic this is exactly the
reference's semantics, which tests/test_multigrid_oracle.py pins against the
reference's own outputs.
"""
import itertools

import numpy as np
import scipy.sparse
import scipy.sparse.linalg


class Stencil:
    """Stencil operator: shifts [S, dim] and coefficients [S, *nwh]."""

    def __init__(self, shifts, coefs, nw, stride=1, periodic=None):
        self.nw = np.array(nw, dtype=int)
        self.dim = len(self.nw)
        self.stride = int(stride)
        self.periodic = np.zeros(self.dim, bool) if periodic is None else \
            np.array(periodic, bool)
        self.nwh = np.array([(n // stride) if p and stride > 1 else
                             (n - 1) // stride + 1
                             for n, p in zip(self.nw, self.periodic)])
        self.shifts = np.array(shifts, dtype=int).reshape(-1, self.dim)
        self.coefs = np.asarray(coefs, np.float64).reshape(
            (len(self.shifts), ) + tuple(self.nwh))

    def _src(self, s):
        """Fine index stride*c + s per axis for every output cell, and a
        validity mask (zero padding on non-periodic axes)."""
        grids = np.meshgrid(*[np.arange(n) for n in self.nwh], indexing='ij')
        idx = []
        ok = np.ones(tuple(self.nwh), bool)
        for ax in range(self.dim):
            e = self.stride * grids[ax] + s[ax]
            if self.periodic[ax]:
                e = e % self.nw[ax]
            else:
                ok &= (e >= 0) & (e < self.nw[ax])
                e = np.clip(e, 0, self.nw[ax] - 1)
            idx.append(e)
        return tuple(idx), ok

    def mul_field(self, u):
        """multigrid.py:958-969."""
        u = np.asarray(u, np.float64).reshape(tuple(self.nw))
        out = np.zeros(tuple(self.nwh))
        for s, c in zip(self.shifts, self.coefs):
            idx, ok = self._src(s)
            out += np.where(ok, c * u[idx], 0.0)
        return out

    def mul_transpose_field(self, uh):
        """multigrid.py:1006-1027: A^T uh (scatter of the same entries)."""
        uh = np.asarray(uh, np.float64).reshape(tuple(self.nwh))
        out = np.zeros(tuple(self.nw))
        for s, c in zip(self.shifts, self.coefs):
            idx, ok = self._src(s)
            np.add.at(out, tuple(i[ok] for i in idx), (c * uh)[ok])
        return out

    def tocsr(self):
        n = int(np.prod(self.nw))
        nh = int(np.prod(self.nwh))
        rows, cols, vals = [], [], []
        out_idx = np.arange(nh).reshape(tuple(self.nwh))
        for s, c in zip(self.shifts, self.coefs):
            idx, ok = self._src(s)
            col = np.ravel_multi_index(idx, tuple(self.nw))
            rows.append(out_idx[ok])
            cols.append(col[ok])
            vals.append(c[ok])
        return scipy.sparse.csr_matrix(
            (np.concatenate(vals), (np.concatenate(rows),
                                    np.concatenate(cols))), shape=(nh, n))

    def diag(self):
        assert self.stride == 1
        for s, c in zip(self.shifts, self.coefs):
            if not np.any(s):
                return c
        return np.zeros(tuple(self.nwh))


def all_shifts(dim, r):
    return [tuple(s) for s in itertools.product(range(-r, r + 1), repeat=dim)]


def get_R(nw, restriction='full', periodic=None):
    """multigrid.py:496-534 (MultigridOp.get_R)."""
    nw = np.array(nw)
    dim = len(nw)
    per = np.zeros(dim, bool) if periodic is None else np.array(periodic, bool)
    nwh = np.array([(n // 2) if p else (n - 1) // 2 + 1
                    for n, p in zip(nw, per)])
    if restriction == 'full':
        shifts = all_shifts(dim, 1)
        coeff = lambda s: 0.5**(sum(abs(np.array(s))) + dim)
    elif restriction == 'half':
        shifts = [(0, ) * dim]
        for i in range(dim):
            shifts.append(tuple(1 if j == i else 0 for j in range(dim)))
            shifts.append(tuple(-1 if j == i else 0 for j in range(dim)))
        coeff = lambda s: (0.5 if sum(abs(np.array(s))) == 0 else 0.25 / dim)
    elif restriction == 'injection':
        shifts = [(0, ) * dim]
        coeff = lambda s: 1.0
    else:
        raise ValueError("Unknown restriction=" + restriction)
    grids = np.meshgrid(*[np.arange(n) for n in nwh], indexing='ij')
    inner = np.ones(tuple(nwh), bool)
    for ax in range(dim):
        if not per[ax]:
            inner &= (grids[ax] > 0) & (grids[ax] + 1 < nwh[ax])
    coefs = []
    for s in shifts:
        val = 1.0 if not any(s) else 0.0
        coefs.append(np.where(inner, coeff(s), val))
    return Stencil(shifts, coefs, nw, stride=2, periodic=per)


def get_TT(nw, periodic=None):
    """multigrid.py:471-494: transpose of multilinear interpolation, stored
    as a stride-2 stencil on the coarse grid (weights 0.5^|s|)."""
    nw = np.array(nw)
    dim = len(nw)
    per = np.zeros(dim, bool) if periodic is None else np.array(periodic, bool)
    nwh = np.array([(n // 2) if p else (n - 1) // 2 + 1
                    for n, p in zip(nw, per)])
    shifts = all_shifts(dim, 1)
    coefs = []
    for s in shifts:
        c = np.full(tuple(nwh), 0.5**sum(abs(np.array(s))))
        # The reference builds the field on nw//2+1 - |s| nodes and pads with
        # zeros on the side the shift points to: entries whose fine target
        # falls outside the grid carry no weight.
        coefs.append(c)
    return Stencil(shifts, coefs, nw, stride=2, periodic=per)


def mul_transpose_op(A, B):
    """multigrid.py:1035-1071: A^T B as a stride-1 stencil."""
    assert A.stride == 1 and B.stride == 1
    dim = A.dim
    res = {}
    for sa, ca in zip(A.shifts, A.coefs):
        for sb, cb in zip(B.shifts, B.coefs):
            d = tuple(sb - sa)
            prod = ca * cb
            # res[e] += prod[e - sa] (zero-padded / periodic), exactly the
            # reference's noncircular shift of ca * cb by sa.
            src = []
            ok = np.ones(tuple(A.nw), bool)
            grids = np.meshgrid(*[np.arange(n) for n in A.nw], indexing='ij')
            for ax in range(dim):
                k = grids[ax] - sa[ax]
                if A.periodic[ax]:
                    k = k % A.nw[ax]
                else:
                    ok &= (k >= 0) & (k < A.nw[ax])
                    k = np.clip(k, 0, A.nw[ax] - 1)
                src.append(k)
            shifted = np.where(ok, prod[tuple(src)], 0.0)
            res[d] = res.get(d, 0.0) + shifted
    shifts = sorted(res)
    return Stencil(shifts, [res[s] for s in shifts], A.nw, 1, A.periodic)


def galerkin(A, R, TT):
    """multigrid.py:390-427: coarse operator R A T in stencil form, here by
    the direct formula
        Ac_d[C] = sum_{r, a} R_r[C] A_a[2C + r] TT_t[C + d],  t = r + a - 2d,
    with every index checked against the grid (zero padding) or wrapped
    (periodic axes).  Shifts d with an all-zero field are dropped."""
    dim = A.dim
    nwh = R.nwh
    per = A.periodic
    res = {}
    Rs = {tuple(s): c for s, c in zip(R.shifts, R.coefs)}
    Ts = {tuple(s): c for s, c in zip(TT.shifts, TT.coefs)}
    grids = np.meshgrid(*[np.arange(n) for n in nwh], indexing='ij')
    for r, cr in Rs.items():
        for a, ca in zip(A.shifts, A.coefs):
            for t in Ts:
                twod = np.array(r) + a - np.array(t)
                if np.any(twod % 2):
                    continue
                d = tuple(twod // 2)
                ok = np.ones(tuple(nwh), bool)
                fine, fine2, coarse2 = [], [], []
                for ax in range(dim):
                    e = 2 * grids[ax] + r[ax]
                    e2 = e + a[ax]
                    c2 = grids[ax] + d[ax]
                    if per[ax]:
                        e, e2, c2 = e % A.nw[ax], e2 % A.nw[ax], c2 % nwh[ax]
                    else:
                        ok &= (e >= 0) & (e < A.nw[ax]) & (e2 >= 0) & \
                            (e2 < A.nw[ax]) & (c2 >= 0) & (c2 < nwh[ax])
                        e = np.clip(e, 0, A.nw[ax] - 1)
                        c2 = np.clip(c2, 0, nwh[ax] - 1)
                    fine.append(e)
                    coarse2.append(c2)
                val = np.where(ok, cr * ca[tuple(fine)] * Ts[t][tuple(coarse2)],
                               0.0)
                res[d] = res.get(d, 0.0) + val
    shifts = [d for d in sorted(res) if np.any(res[d] != 0)]
    return Stencil(shifts, [res[d] for d in shifts], nwh, 1, per)


def level_sizes(nw, nlevels=None, periodic=None):
    """multigrid.py:359-369."""
    nw = np.array(nw)
    per = np.zeros(len(nw), bool) if periodic is None else np.array(periodic)
    max_nlevels = 0
    while 2**(max_nlevels + 1) < min(nw):
        max_nlevels += 1
    nlevels = max_nlevels if nlevels is None else min(nlevels, max_nlevels)
    nnw = [nw]
    for _ in range(1, nlevels):
        nnw.append(np.array([(n // 2) if p else (n - 1) // 2 + 1
                             for n, p in zip(nnw[-1], per)]))
    return nnw


class MultigridOp:
    """multigrid.py:342-602 for one unknown field (nvar = 1)."""

    def __init__(self, nw, nlevels=None, restriction='full', periodic=None):
        self.nnw = level_sizes(nw, nlevels, periodic)
        self.nlevels = len(self.nnw)
        self.periodic = periodic
        self.RR = [get_R(n, restriction, periodic) for n in self.nnw]
        self.TT = [get_TT(n, periodic) for n in self.nnw]

    def update_A(self, A0):
        self.AA = [A0]
        for lvl in range(1, self.nlevels):
            self.AA.append(galerkin(self.AA[-1], self.RR[lvl - 1],
                                    self.TT[lvl - 1]))
        self.DD = [A.diag() for A in self.AA]

    def smoother_jacobi(self, level, u, f, omega=1.0):
        A = self.AA[level]
        r = f - A.mul_field(u)
        return u + r / self.DD[level] * omega

    def smoother_direct(self, level, u, f):
        A = self.AA[level].tocsr().tocsc()
        return scipy.sparse.linalg.spsolve(A, f.ravel()).reshape(f.shape)

    def step(self, u, f, smoother, level=0, ndirect=5, pre=2, post=2):
        if level + 1 >= self.nlevels or min(self.nnw[level]) <= ndirect:
            return self.smoother_direct(level, u, f)
        for _ in range(pre):
            u = smoother(level, u, f)
        A = self.AA[level]
        r = self.RR[level].mul_field(f - A.mul_field(u))
        du = self.step(np.zeros_like(r), r, smoother, level + 1, ndirect, pre,
                       post)
        u = u + self.TT[level].mul_transpose_field(du)
        for _ in range(post):
            u = smoother(level, u, f)
        return u


# -- multigrid decomposition of a field (multigrid.py:1217-1426) -------------
#
# A field on the finest grid is the sum over levels l of the level-l weights
# interpolated l times.  Node grids refine n -> 2n - 1 by multilinear
# interpolation; cell grids refine n -> 2n with weights 3/4 and 1/4 per axis
# after a halo of linearly extrapolated cells, ghost = 2 u[edge] - u[next],
# taken on all axes at once (multigrid.py:1298-1302: 2 * symmetric pad -
# reflect pad; a corner ghost is 2 u[0, 0] - u[1, 1]).


def interp_node(u):
    """One level of interp_node_field (multigrid.py:1220-1289): fine node 2i
    takes u[i], fine node 2i + 1 the mean of u[i] and u[i + 1], per axis."""
    u = np.asarray(u, np.float64)
    for ax in range(u.ndim):
        n = u.shape[ax]
        shape = list(u.shape)
        shape[ax] = 2 * n - 1
        out = np.zeros(shape)
        ev = [slice(None)] * u.ndim
        od = [slice(None)] * u.ndim
        ev[ax] = slice(0, None, 2)
        od[ax] = slice(1, None, 2)
        lo = [slice(None)] * u.ndim
        hi = [slice(None)] * u.ndim
        lo[ax] = slice(0, n - 1)
        hi[ax] = slice(1, n)
        out[tuple(ev)] = u
        out[tuple(od)] = 0.5 * (u[tuple(lo)] + u[tuple(hi)])
        u = out
    return u


def pad_extrap(u):
    """The halo of interp_cell_field (multigrid.py:1298-1302): one ghost
    cell per side on every axis, 2 * (symmetric pad) - (reflect pad)."""
    u = np.asarray(u, np.float64)
    return 2 * np.pad(u, 1, mode="symmetric") - np.pad(u, 1, mode="reflect")


def interp_cell(u):
    """One level of interp_cell_field (multigrid.py:1291-1362): fine cell 2k
    takes 3/4 u[k] + 1/4 u[k - 1], fine cell 2k + 1 takes 3/4 u[k] + 1/4
    u[k + 1], per axis, over the extrapolated halo."""
    up = pad_extrap(u)
    dim = up.ndim
    n = [s - 2 for s in up.shape]
    out = np.zeros([2 * v for v in n])
    for par in itertools.product((0, 1), repeat=dim):
        acc = 0.0
        for nb in itertools.product((0, 1), repeat=dim):
            w = 1.0
            sel = []
            for d in range(dim):
                # neighbour offset -1 (par 0) or +1 (par 1) when nb[d] = 1
                off = 0 if nb[d] == 0 else (-1 if par[d] == 0 else 1)
                w *= 0.25 if nb[d] else 0.75
                sel.append(slice(1 + off, 1 + off + n[d]))
            acc = acc + w * up[tuple(sel)]
        out[tuple(slice(p, None, 2) for p in par)] = acc
    return out


def interp_field(u, depth=1, cell=False):
    """multigrid.py:1364-1375: `depth` levels of refinement."""
    for _ in range(depth):
        u = interp_cell(u) if cell else interp_node(u)
    return np.asarray(u, np.float64)


def _levels(uw, nnw, factors):
    factors = [1.0] * len(nnw) if factors is None else factors
    out, s = [], 0
    for nw, f in zip(nnw, factors):
        n = int(np.prod(nw))
        out.append(np.asarray(uw[s:s + n], np.float64).reshape(nw) * f)
        s += n
    return out


def weights_to_fields(uw, nnw, factors=None, cell=False):
    """multigrid.py:1377-1394: level l interpolated l times, per level."""
    return [interp_field(u, i, cell) for i, u in enumerate(
        _levels(uw, nnw, factors))]


def weights_to_field(uw, nnw, factors=None, cell=False):
    """multigrid.py:1409-1426: from the coarsest level, refine and add."""
    res = None
    for u in reversed(_levels(uw, nnw, factors)):
        res = u if res is None else interp_field(res, 1, cell) + u
    return res


def weights_coarse_ones(nnw):
    """multigrid.py:1396-1407: zero weights except ones on the coarsest
    level."""
    return np.concatenate([np.full(int(np.prod(nw)), float(i == len(nnw) - 1))
                           for i, nw in enumerate(nnw)])
