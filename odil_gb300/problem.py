"""ODIL problem: operator evaluation, loss and gradient, linearization.

Same API as util_op.py:432-973 (``Context``, ``Problem``): a user operator
``operator(mod, ctx)`` returns a list of residual arrays, the loss is the sum
of their mean squares (``Problem.Raw`` terms are averaged as given), and the
gradient is the adjoint of that sum.

Two routes:
  * registered operator families (objects with ``bind(domain)``, e.g.
    ``WaveOperator``) run the fused CUDA kernels of libodil_gb300;
  * any other operator runs op by op as torch CUDA tensors with autograd
    (``mod`` is the tf-style namespace of ``odil_gb300.mod``).
Both run on the GPU; CPU tensors are rejected.
"""
import os

import numpy as np
import torch

from .domain import State
from .mod import TorchMod


def extrap_quadh(u0, u1, u1p):
    """util_op.py:1017-1023: quadratic extrapolation from points 0, 1 and
    1.5 to point 2 (the face value u1p sits half a cell out)."""
    return (u0 - 6 * u1 + 8 * u1p) / 3


def extrap_quad(u0, u1, u2):
    """util_op.py:1026-1029: quadratic extrapolation from 0, 1, 2 to 3."""
    return u0 - 3 * u1 + 3 * u2


def extrap_linear(u0, u1):
    """util_op.py:1032-1035: linear extrapolation from 0, 1 to 2."""
    return 2 * u1 - u0


def latin_hypercube(ndim, size, rng=None):
    """util_op.py:1082-1098: `size` points of the unit cube [size, ndim],
    one in each of the `size` equal strata of every axis, the strata matched
    across axes by independent random permutations.  Draws from numpy's
    global generator (as the reference does) unless `rng` (a numpy
    Generator) is given."""
    rand = np.random.rand if rng is None else (lambda *s: rng.random(s))
    perm = np.random.permutation if rng is None else rng.permutation
    pts = (np.arange(size)[:, None] + rand(size, ndim)) / size
    for j in range(ndim):
        pts[:, j] = pts[perm(size), j]
    return pts


def operator_laplace(mod, ctx):
    """util_op.py:1038-1079: the reference's sample operator, Laplacians of
    fields u and v on an (x, y) grid with linear extrapolation to the halo
    cells, and a zero third term."""
    dx, dy = ctx.step("x"), ctx.step("y")
    ix, iy = ctx.cell_index("x"), ctx.cell_index("y")
    nx, ny = ctx.size("x"), ctx.size("y")

    def stencil_var(key):
        return [ctx.field(key), ctx.field(key, -1, 0), ctx.field(key, 1, 0),
                ctx.field(key, 0, -1), ctx.field(key, 0, 1)]

    def apply_bc_extrap(st):
        st[1] = mod.where(ix == 0, extrap_linear(st[2], st[0]), st[1])
        st[2] = mod.where(ix == nx - 1, extrap_linear(st[1], st[0]), st[2])
        st[3] = mod.where(iy == 0, extrap_linear(st[4], st[0]), st[3])
        st[4] = mod.where(iy == ny - 1, extrap_linear(st[3], st[0]), st[4])
        return st

    def laplace(st):
        q, qxm, qxp, qym, qyp = st
        return (qxp - 2 * q + qxm) / dx**2 + (qyp - 2 * q + qym) / dy**2

    u_st = apply_bc_extrap(stencil_var("u"))
    v_st = apply_bc_extrap(stencil_var("v"))
    return [laplace(u_st), laplace(v_st), ctx.field("zeros")]


def _torch_dtype(np_dtype):
    return torch.float32 if np.dtype(np_dtype) == np.float32 else torch.float64


class Context:
    """util_op.py:432-563 over torch tensors.

    ``field(name, *shift)`` returns the field rolled by ``-shift``
    (``field('u', -1, 0)[i, j] == u[i-1, j]``, periodic), ``freeze=True``
    detaches it.
    """

    def __init__(self, domain, state_fields, epoch=0, extra=None, mod=None):
        self.domain = domain
        self.state_fields = state_fields
        self.epoch = epoch
        self.extra = extra
        self.dtype = _torch_dtype(domain.dtype)
        self.mod = mod

    def cast(self, value, dtype=None):
        return self.mod.cast(value, dtype or self.dtype)

    def size(self, i):
        return self.domain.size(i)

    def step(self, i):
        return self.domain.step(i)

    def cell_index(self, i):
        return self.domain.cell_index(i)

    def node_index(self, i):
        return self.domain.node_index(i)

    def cell_center(self, i):
        return self.domain.cell_center(i)

    def neural_net(self, name, *inputs, **kw):
        raise KeyError("Weights with name '{:}' not found in domain.neuralnets"
                       .format(name))

    def field(self, name, *shift, freeze=False):
        domain = self.domain
        assert len(shift) <= domain.ndim, "Shift is too long {:}".format(shift)
        shift = tuple(shift) + (0, ) * (domain.ndim - len(shift))
        if name == "zeros":
            return self.mod.zeros(domain.shape)
        if name == "ones":
            return self.mod.ones(domain.shape)
        if name not in domain.fieldnames:
            raise ValueError("Unknown field name '" + name + "'")
        u = self.state_fields[name]
        if freeze:
            u = u.detach()
        if any(shift):
            u = torch.roll(u, tuple(-s for s in shift), tuple(range(domain.ndim)))
        return u


class FusedLoss(torch.autograd.Function):
    """loss = sum_k mean(f_k^2) of a registered family, with the gradient from
    the fused adjoint kernel (residuals recomputed in-tile, never stored)."""

    @staticmethod
    def forward(ctx, u, kernels):
        loss, grad = kernels.loss_grad(u.detach())
        ctx.save_for_backward(grad)
        return loss.reshape(()).clone()

    @staticmethod
    def backward(ctx, gout):
        grad, = ctx.saved_tensors
        return grad * gout.to(grad.dtype), None


class JitLoss(torch.autograd.Function):
    """loss = sum_k mean(f_k^2) of a compiled generic operator on the packed
    state, with the gradient from its fused adjoint kernel."""

    @staticmethod
    def forward(ctx, u, problem):
        fields = {k: v.contiguous() for k, v in
                  problem.unpack_fields(u.detach()).items()}
        loss, grads, _ = problem.jit.loss_grad(fields)
        ctx.save_for_backward(problem.pack_fields(grads))
        return loss.to(u.dtype).reshape(()).clone()

    @staticmethod
    def backward(ctx, gout):
        grad, = ctx.saved_tensors
        return grad * gout.to(grad.dtype), None


class Jacobian:
    """Matrix-free Jacobian of a registered family (the stencil form of the
    CSR matrix util_op.py:859-937 assembles).  ``matvec``/``rmatvec`` act on
    packed vectors; ``solve`` is the direct Newton solve."""

    def __init__(self, kernels, shape):
        self.kernels = kernels
        self.shape = shape

    def matvec(self, v):
        return self.kernels.jv(v.reshape(self.kernels.shape)).reshape(-1)

    def rmatvec(self, w):
        return self.kernels.jtv(w.reshape(self.kernels.shape)).reshape(-1)

    def jtj_v(self, v):
        """J^T J v (one fused pass where the family provides it)."""
        if hasattr(self.kernels, "jtj_v"):
            return self.kernels.jtj_v(
                v.reshape(self.kernels.shape).contiguous()).reshape(-1)
        return self.rmatvec(self.matvec(v))

    def jtj_diag(self):
        """diag(J^T J), packed (families that provide it)."""
        return self.kernels.jtj_diag().reshape(-1)

    def stencil_blocks(self):
        """{(0, 0): StencilOp} from the family's per-slot coefficient fields
        (families that expose them)."""
        if not hasattr(self.kernels, "coefficients"):
            raise NotImplementedError("this family has no coefficient fields")
        from .stencil import StencilOp
        return {(0, 0): StencilOp(self.kernels.SLOT_SHIFTS,
                                  self.kernels.coefficients(),
                                  self.kernels.shape)}

    def solve(self, rhs):
        return self.kernels.march(rhs.reshape(self.kernels.shape)).reshape(-1)

    def to_csr(self):
        """J as a device CSR matrix in the reference's layout (what
        util_op.py:859-937 assembles), for callers that want the explicit
        matrix; the registered family must expose per-slot coefficients."""
        if not hasattr(self.kernels, "coefficients"):
            raise NotImplementedError("this family has no coefficient fields")
        from .stencil import StencilOp
        coef = self.kernels.coefficients()
        return StencilOp(self.kernels.SLOT_SHIFTS, coef,
                         self.kernels.shape).to_csr()


class StencilJacobian:
    """Jacobian of a compiled generic operator: one stencil per (term,
    field) with the coefficient fields df_k(c)/du_j(c + s) (util_op.py:
    585-614).  Rows are the terms stacked (term k: rows k N .. k N + N - 1),
    columns the fields (field j: j N ..), as util_op.py:859-937 lays out
    the CSR matrix; shifts wrap periodically."""

    DENSE_MAX = 16384  # unknowns up to which `solve` is a dense direct solve

    def __init__(self, coef, blocks, nterms, nfields, shape):
        from .stencil import StencilOp
        self.grid = tuple(shape)
        self.n = int(np.prod(shape))
        per = (True, ) * len(self.grid)
        self.ops = {kj: StencilOp([sh for _, sh in lst],
                                  coef[[q for q, _ in lst]], self.grid, 1, per)
                    for kj, lst in blocks.items()}
        self.nterms, self.nfields = nterms, nfields
        self.shape = (nterms * self.n, nfields * self.n)
        self.dtype, self.device = coef.dtype, coef.device

    def stencil_blocks(self):
        """{(term, field): StencilOp} of the Jacobian."""
        return dict(self.ops)

    def matvec(self, v):
        n = self.n
        out = torch.zeros(self.shape[0], dtype=v.dtype, device=v.device)
        for (k, j), op in self.ops.items():
            op.mul_field(v[j * n:(j + 1) * n].reshape(self.grid).contiguous(),
                         out=out[k * n:(k + 1) * n].view(self.grid), beta=1.0)
        return out

    def rmatvec(self, w):
        n = self.n
        out = torch.zeros(self.shape[1], dtype=w.dtype, device=w.device)
        for (k, j), op in self.ops.items():
            op.mul_transpose_field(
                w[k * n:(k + 1) * n].reshape(self.grid).contiguous(),
                out=out[j * n:(j + 1) * n].view(self.grid), beta=1.0)
        return out

    def to_csr(self):
        """The matrix as a device CSR tensor (reference layout)."""
        n = self.n
        rows, cols, vals = [], [], []
        for (k, j), op in self.ops.items():
            b = op.to_csr().to_sparse_coo().coalesce()
            i = b.indices()
            rows.append(i[0] + k * n)
            cols.append(i[1] + j * n)
            vals.append(b.values())
        coo = torch.sparse_coo_tensor(
            torch.stack([torch.cat(rows), torch.cat(cols)]), torch.cat(vals),
            self.shape).coalesce()
        return coo.to_sparse_csr()

    def solve(self, rhs, tol=1e-12, maxiter=None):
        """d minimising |J d - rhs| (the normal equations of
        linsolver.py:28-45): a dense direct solve up to DENSE_MAX unknowns,
        else conjugate gradients on the normal equations, matrix-free."""
        rhs = rhs.to(self.dtype)
        if self.shape[1] <= self.DENSE_MAX:
            J = self.to_csr().to_dense()
            if self.shape[0] == self.shape[1]:
                return torch.linalg.solve(J, rhs)
            return torch.linalg.solve(J.T @ J, J.T @ rhs)
        x = torch.zeros(self.shape[1], dtype=self.dtype, device=self.device)
        r = rhs.clone()
        z = self.rmatvec(r)
        p = z.clone()
        zz = torch.dot(z, z)
        z0 = zz.sqrt().item()
        maxiter = maxiter or 10 * self.shape[1]
        for _ in range(maxiter):
            if zz.sqrt().item() <= tol * max(z0, 1e-300):
                break
            w = self.matvec(p)
            alpha = zz / torch.dot(w, w)
            x += alpha * p
            r -= alpha * w
            z = self.rmatvec(r)
            zn = torch.dot(z, z)
            p = z + (zn / zz) * p
            zz = zn
        return x


class Problem:
    """util_op.py:566-973."""

    class Raw:
        """A pre-reduced loss term: averaged as given, not squared."""

        def __init__(self, value):
            self.value = value

    def __init__(self, operator, domain, extra=None, jit=None):
        """jit: compile an unregistered operator to CUDA kernels (the stencil
        compiler of ``odil_gb300.jit``).  None means yes unless the
        environment sets ODIL_GB300_JIT=0; operators it cannot trace run op
        by op on CUDA tensors."""
        self.domain = domain
        self.operator = operator
        self.extra = extra
        self.kernels = operator.bind(domain) if hasattr(operator, "bind") \
            else None
        self.mod = TorchMod(device=domain.device,
                            dtype=_torch_dtype(domain.dtype))
        self.jit = None
        if jit is None:
            jit = os.environ.get("ODIL_GB300_JIT", "1") != "0"
        if self.kernels is None and jit:
            from .jit import JitOperator, JitUnsupported
            try:
                self.jit = JitOperator(operator, domain, extra)
            except JitUnsupported:
                self.jit = None
            except Exception as e:  # an operator the tracer did not foresee
                import warnings
                warnings.warn("stencil compiler: %s: %s; the operator runs "
                              "op by op" % (type(e).__name__, e))
                self.jit = None

    def _jit_ready(self):
        """True when the compiled operator can run; a failed build (no nvcc,
        or a compiler error) drops to the op-by-op path with a warning."""
        if self.jit is None:
            return False
        try:
            self.jit.lib()
            return True
        except (RuntimeError, OSError) as e:
            import warnings
            warnings.warn("stencil compiler: build failed (%s); the operator "
                          "runs op by op" % str(e).splitlines()[0])
            self.jit = None
            return False

    # -- state handling (util_op.py:733-857) --------------------------------
    @property
    def tdtype(self):
        return _torch_dtype(self.domain.dtype)

    def init_missing(self, state):
        for name in self.domain.fieldnames:
            if name not in state.fields:
                state.fields[name] = torch.zeros(self.domain.shape,
                                                 dtype=self.tdtype,
                                                 device=self.domain.device)
            elif not isinstance(state.fields[name], torch.Tensor):
                state.fields[name] = torch.as_tensor(
                    np.asarray(state.fields[name]), dtype=self.tdtype,
                    device=self.domain.device)

    def pack_fields(self, fields):
        return torch.cat([fields[n].reshape(-1)
                          for n in self.domain.fieldnames])

    def unpack_fields(self, packed):
        n = self.domain.cells()
        return {name: packed[i * n:(i + 1) * n].reshape(self.domain.shape)
                for i, name in enumerate(self.domain.fieldnames)}

    def pack_state(self, state, with_frozen=False):
        return self.pack_fields(state.fields)

    def unpack_state(self, packed, with_frozen=False):
        return State(fields=self.unpack_fields(packed))

    # -- evaluation ---------------------------------------------------------
    def _check_device(self, state):
        for name in self.domain.fieldnames:
            if not state.fields[name].is_cuda:
                raise RuntimeError(
                    "field '%s' is on %s: the ODIL engine runs on CUDA only" %
                    (name, state.fields[name].device))

    def _generic(self, fields, epoch):
        ctx = Context(self.domain, fields, epoch=epoch, extra=self.extra,
                      mod=self.mod)
        ff = self.operator(self.mod, ctx)
        if not isinstance(ff, (list, tuple)):
            ff = [ff]
        return list(ff)

    def eval_operator(self, state, epoch=0):
        """util_op.py:968-973: list of residual fields."""
        self.init_missing(state)
        self._check_device(state)
        if self.kernels is not None:
            u = state.fields[self.domain.fieldnames[0]]
            return [self.kernels.residual(u)]
        if self._jit_ready():
            return self.jit.residual(state.fields, epoch)
        with torch.no_grad():
            ff = self._generic(state.fields, epoch)
        return [f.value if isinstance(f, Problem.Raw) else f for f in ff]

    def eval_loss_grad(self, state, epoch=0):
        """util_op.py:939-966: (loss, grads, wgrads, loss_split)."""
        self.init_missing(state)
        self._check_device(state)
        names = self.domain.fieldnames
        if self.kernels is not None:
            u = state.fields[names[0]]
            loss, grad = self.kernels.loss_grad(u)
            loss = loss.reshape(()).clone()
            return loss, {names[0]: grad}, {}, [loss]
        if self._jit_ready():
            loss, grads, split = self.jit.loss_grad(state.fields, epoch)
            return loss, grads, {}, split
        fields = {k: v.detach().requires_grad_(True)
                  for k, v in state.fields.items()}
        ff = self._generic(fields, epoch)
        loss_split = [
            torch.mean(f.value) if isinstance(f, Problem.Raw) else
            torch.mean(torch.square(f)) for f in ff
        ]
        loss = sum(loss_split)
        gg = torch.autograd.grad(loss, [fields[n] for n in names],
                                 allow_unused=True)
        grads = {n: (g if g is not None else torch.zeros_like(fields[n]))
                 for n, g in zip(names, gg)}
        return loss.detach(), grads, {}, [l.detach() for l in loss_split]

    def eval_diag(self, state, epoch=0, nsmp=10, generator=None):
        """util_op.py:675-731: stochastic estimate of the diagonal of
        sum_k J_k^T J_k / N_k as the mean over `nsmp` samples of g^2, with
        g = sum_k J_k^T z_k / sqrt(N_k) and z_k ~ N(0, 1) per residual cell.
        Registered families form J^T z with their adjoint kernel, compiled
        generic operators with their Jacobian stencils, others by autograd.
        Returns the packed diagonal."""
        self.init_missing(state)
        self._check_device(state)
        names = self.domain.fieldnames
        acc = None
        jac = None
        if self.kernels is None and self._jit_ready():
            const = self.jit.residual(state.fields, epoch)
            coef, blocks = self.jit.jacobian(state.fields, epoch)
            jac = StencilJacobian(coef, blocks, len(const), len(names),
                                  self.domain.shape)
        for _ in range(nsmp):
            if jac is not None:
                # one z_k per residual term, J^T z through the compiled
                # Jacobian's stencils
                z = torch.randn(jac.shape[0], dtype=jac.dtype,
                                device=jac.device, generator=generator)
                z /= float(jac.n)**0.5
                g = jac.rmatvec(z)
            elif self.kernels is not None:
                k = self.kernels
                u = state.fields[names[0]]
                z = torch.randn(k.shape, dtype=u.dtype, device=u.device,
                                generator=generator)
                z /= float(z.numel())**0.5
                g = k.jtv(z).reshape(-1)
            else:
                fields = {n: v.detach().requires_grad_(True)
                          for n, v in state.fields.items()}
                ff = self._generic(fields, epoch)
                lossn = 0
                for f in ff:
                    if isinstance(f, Problem.Raw):
                        lossn = lossn + f.value
                    else:
                        z = torch.randn(f.shape, dtype=f.dtype,
                                        device=f.device, generator=generator)
                        lossn = lossn + (f * z).sum() / float(f.numel())**0.5
                gg = torch.autograd.grad(lossn, [fields[n] for n in names],
                                         allow_unused=True)
                g = torch.cat([(x if x is not None else
                                torch.zeros_like(fields[n])).reshape(-1)
                               for n, x in zip(names, gg)])
            acc = g * g if acc is None else acc + g * g
        return acc / nsmp

    def loss(self, u):
        """Differentiable loss of the packed state (torch.autograd.Function
        over the fused adjoint for registered families)."""
        if self.kernels is not None:
            return FusedLoss.apply(u.reshape(self.kernels.shape), self.kernels)
        if self._jit_ready():
            return JitLoss.apply(u, self)
        fields = self.unpack_fields(u)
        ff = self._generic(fields, 0)
        return sum(torch.mean(f.value) if isinstance(f, Problem.Raw) else
                   torch.mean(torch.square(f)) for f in ff)

    def linearize(self, state, epoch=0):
        """util_op.py:859-937: (const, J) with J matrix-free on the GPU."""
        self.init_missing(state)
        self._check_device(state)
        if self.kernels is None and self._jit_ready():
            const = self.jit.residual(state.fields, epoch)
            coef, blocks = self.jit.jacobian(state.fields, epoch)
            return const, StencilJacobian(coef, blocks, len(const),
                                          len(self.domain.fieldnames),
                                          self.domain.shape)
        if self.kernels is None:
            raise NotImplementedError(
                "linearize needs a registered operator family or an operator "
                "the stencil compiler traces; others use eval_loss_grad")
        const = self.eval_operator(state, epoch)
        n = self.domain.cells()
        return const, Jacobian(self.kernels, (len(const) * n, n))
