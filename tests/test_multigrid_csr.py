"""The CSR multigrid (odil_gb300.multigrid.Multigrid) against the outputs
of the reference's Multigrid class (multigrid.py:70-339) in
tests/golden/multigrid_csr_ref.npz (tests/golden/make_golden.py,
make_multigrid_csr): coarse matrices R A T of every level, block
diagonals, V-cycle iterates with damped Jacobi, one Gauss-Seidel sweep.
The class is device-agnostic torch sparse code; these tests run it on CPU
tensors."""
import os
from functools import partial

import numpy as np
import pytest
import torch

from odil_gb300.multigrid import Multigrid

G = np.load(os.path.join(os.path.dirname(__file__), "golden",
                         "multigrid_csr_ref.npz"))

CASES = {
    # name: nvar, restriction, ndirect, pre, post, cycles
    "p17": (1, "full", 5, 2, 2, 3),
    "h17": (1, "half", 5, 2, 2, 3),
    "i33": (1, "injection", 5, 2, 2, 3),
    "v9": (2, "full", 3, 2, 2, 2),
    "d3": (1, "full", 2, 1, 3, 2),
}


def _run(name, device, gauss_seidel=True):
    nvar, restr, ndirect, pre, post, cycles = CASES[name]
    nnw = G[name + "_nnw"]
    A0 = torch.as_tensor(G[name + "_A0"], device=device).to_sparse_csr()
    f = torch.as_tensor(G[name + "_f"], device=device)
    m = Multigrid(tuple(nnw[0]), nvar=nvar, restriction=restr,
                  dtype=torch.float64, device=device)
    assert [list(v) for v in m.nnw] == [list(v) for v in nnw]
    m.update_A(A0, compute_lower=(nvar == 1 and gauss_seidel))
    for level in range(1, m.nlevels):
        np.testing.assert_allclose(m.AA[level].to_dense().cpu().numpy(),
                                   G["%s_A%d" % (name, level)], rtol=1e-12,
                                   atol=1e-12)
    for level in range(m.nlevels):
        np.testing.assert_allclose(m.DD[level].cpu().numpy(),
                                   G["%s_D%d" % (name, level)], rtol=1e-12,
                                   atol=1e-12)
    u = torch.zeros_like(f)
    for it in range(cycles):
        u = m.step(u, f, ndirect=ndirect, pre=pre, post=post,
                   smoother=partial(m.smoother_jacobi, omega=0.7))
        ref = G["%s_u%d" % (name, it)]
        np.testing.assert_allclose(u.cpu().numpy(), ref, rtol=1e-9,
                                   atol=1e-10 * np.abs(ref).max())
    if nvar == 1 and gauss_seidel:
        v = m.smoother_gauss_seidel(0, f * 0.1, f, omega=0.9)
        np.testing.assert_allclose(v.cpu().numpy(), G[name + "_gs"],
                                   rtol=1e-10, atol=1e-12)
    return m, A0, f


@pytest.mark.parametrize("name", list(CASES))
def test_multigrid_csr_matches_reference(name):
    _run(name, "cpu")


def test_multigrid_csr_converges():
    """10 more V-cycles drive the residual of the 17^2 system down by
    orders of magnitude (test_multigrid.py:340-364 asks 1e-6 of its
    Laplacian)."""
    m, A0, f = _run("p17", "cpu")
    u = torch.zeros_like(f)
    for _ in range(12):
        u = m.step(u, f, smoother=partial(m.smoother_jacobi, omega=0.7))
    assert float(torch.linalg.norm(f - A0 @ u)) < 1e-6 * float(
        torch.linalg.norm(f))


def test_multigrid_csr_full_block_jacobi():
    """smoother_jacobi(full=True): the per-cell nvar x nvar blocks of the
    diagonal blocks are inverted together (multigrid.py:288-295)."""
    m, A0, f = _run("v9", "cpu")
    u = torch.zeros_like(f)
    v = m.smoother_jacobi(0, u, f, omega=0.5, full=True)
    D = G["v9_D0"]  # [nvar, nvar, ns]
    r = (f - A0 @ u).numpy().reshape(2, -1)
    du = np.linalg.solve(np.moveaxis(D, 2, 0), r.T[:, :, None])[:, :, 0]
    np.testing.assert_allclose(v.numpy(), 0.5 * du.T.reshape(-1),
                               rtol=1e-12, atol=1e-14)


def test_multigrid_csr_transfer_operators():
    """get_R / get_T on 9 x 5 nodes: full weighting normalised to one per
    inner coarse row, injection on boundary rows, interpolation reproduces
    linear functions."""
    R = Multigrid.get_R((9, 5), device="cpu").to_dense().numpy()
    T = Multigrid.get_T((9, 5), device="cpu").to_dense().numpy()
    assert R.shape == (15, 45) and T.shape == (45, 15)
    np.testing.assert_allclose(R.sum(1), 1.0)
    x, y = np.meshgrid(np.arange(9), np.arange(5), indexing="ij")
    xc, yc = np.meshgrid(np.arange(5) * 2, np.arange(3) * 2, indexing="ij")
    lin = (3 * x + 2 * y + 1).reshape(-1)
    linc = (3 * xc + 2 * yc + 1).reshape(-1)
    np.testing.assert_allclose(T @ linc, lin)
    np.testing.assert_allclose(R @ lin, linc)


def test_transfer_operators_match_reference_test_variant():
    """The reference's own multigrid tests switch g_reuse_multigridop off
    (test_multigrid.py:4), which builds R and T from node multi-indices
    flattened with the first axis fastest (multigrid.py:160-190); on odd
    grids they are these operators with rows and columns reordered."""
    nw = (9, 5)
    nwh = (5, 3)

    def perm(shape):
        return np.arange(int(np.prod(shape))).reshape(shape).reshape(
            -1, order="F")

    pf, pc = perm(nw), perm(nwh)
    R = Multigrid.get_R(nw, device="cpu").to_dense().numpy()
    T = Multigrid.get_T(nw, device="cpu").to_dense().numpy()
    np.testing.assert_array_equal(R[np.ix_(pc, pf)], G["fortran_R_9x5"])
    np.testing.assert_array_equal(T[np.ix_(pf, pc)], G["fortran_T_9x5"])


class _CpuProblem:
    """A Problem whose linearize assembles the Jacobian on the CPU with
    autograd (the generated Jacobian kernels need a GPU)."""

    def __init__(self, op, dom):
        from odil_gb300.problem import Problem
        self.p = Problem(op, dom, jit=False)
        self.domain = dom

    def __getattr__(self, k):
        return getattr(self.p, k)

    def linearize(self, state, epoch=0):
        p = self.p
        packed = p.pack_state(state)

        def res(x):
            return torch.cat([r.reshape(-1) for r in
                              p._generic(p.unpack_fields(x), epoch)])

        const = p._generic(p.unpack_fields(packed), epoch)
        J = torch.autograd.functional.jacobian(res, packed)

        class _J:
            def to_csr(self):
                return J.to_sparse_csr()

        return [c.detach() for c in const], _J()


def test_optimize_multigrid_reaches_newton_solution():
    """util.optimize_multigrid (util.py:382-495): Newton epochs with CSR
    V-cycles on J^T J reach the direct Newton solution of a nonlinear
    screened-Poisson problem on 17 x 17 nodes (periodic stencil, non-periodic
    transfer operators, as in the reference)."""
    import argparse
    from odil_gb300 import util
    from odil_gb300.domain import Domain, State
    dom = Domain(ndim=2, shape=(17, 17), lower=(0, 0), upper=(1, 1),
                 varnames=("x", "y"), fieldnames=["u"], device="cpu")

    def op(mod, ctx):
        u = ctx.field("u")
        lap = (ctx.field("u", 1, 0) + ctx.field("u", -1, 0) +
               ctx.field("u", 0, 1) + ctx.field("u", 0, -1) - 4 * u)
        return [3 * u - 0.5 * lap - mod.sin(ctx.cell_center(0)) + 0.1 * u * u]

    pj = _CpuProblem(op, dom)
    ref = torch.zeros(dom.shape, dtype=torch.float64)
    st = State(fields={"u": ref})
    for _ in range(6):
        const, J = pj.linearize(st)
        Jd = J.to_csr().to_dense()
        ref += torch.linalg.solve(Jd, -const[0].reshape(-1)).reshape(dom.shape)
    args = argparse.Namespace(epochs=6, epoch_start=0, nlvl=None,
                              restriction="full", omega=0.6,
                              linsolver_maxiter=30, ndirect=3, smooth_pre=2,
                              smooth_post=2)
    u = torch.zeros(dom.shape, dtype=torch.float64)
    seen = []
    util.optimize_multigrid(args, pj, State(fields={"u": u}),
                            callback=lambda packed, epoch, **kw:
                            seen.append(epoch))
    assert seen == list(range(7))
    assert float((u - ref).abs().max() / ref.abs().max()) < 1e-8


def test_optimize_multigrid_with_per_level_problems():
    """util.optimize_multigrid with `datalevels` (util.py:414-441): the
    coarse matrices come from the same operator on the coarse grids,
    linearised at the restricted fields; the fine-level smoothing and
    residuals keep the iteration on the fine problem, which reaches its
    Newton solution."""
    import argparse
    from types import SimpleNamespace
    from odil_gb300 import util
    from odil_gb300.domain import Domain, State

    def op(mod, ctx):
        u = ctx.field("u")
        lap = (ctx.field("u", 1, 0) + ctx.field("u", -1, 0) +
               ctx.field("u", 0, 1) + ctx.field("u", 0, -1) - 4 * u)
        return [3 * u - 0.5 * lap - mod.sin(ctx.cell_center(0)) + 0.1 * u * u]

    def make(n):
        return Domain(ndim=2, shape=(n, n), lower=(0, 0), upper=(1, 1),
                      varnames=("x", "y"), fieldnames=["u"], device="cpu")

    dom = make(17)
    pj = _CpuProblem(op, dom)
    ref = torch.zeros(dom.shape, dtype=torch.float64)
    st = State(fields={"u": ref})
    for _ in range(6):
        const, J = pj.linearize(st)
        ref += torch.linalg.solve(J.to_csr().to_dense(),
                                  -const[0].reshape(-1)).reshape(dom.shape)
    u = torch.zeros(dom.shape, dtype=torch.float64)
    state = State(fields={"u": u})
    levels = [SimpleNamespace(problem=pj, state=state)]
    for n in (9, 5, 3):
        d = make(n)
        levels.append(SimpleNamespace(
            problem=_CpuProblem(op, d),
            state=State(fields={"u": torch.zeros(d.shape,
                                                 dtype=torch.float64)})))
    args = argparse.Namespace(epochs=6, epoch_start=0, nlvl=None,
                              restriction="full", omega=0.6,
                              linsolver_maxiter=40, ndirect=3, smooth_pre=2,
                              smooth_post=2)
    seen_A, seen_u = [], []
    orig = Multigrid.update_A

    def spy(self, A, *a, **kw):
        seen_A.append(list(A) if isinstance(A, (list, tuple)) else [A])
        return orig(self, A, *a, **kw)

    def cb(packed, epoch, **kw):
        seen_u.append(packed.clone())

    Multigrid.update_A = spy
    try:
        util.optimize_multigrid(args, pj, state, callback=cb,
                                datalevels=levels)
    finally:
        Multigrid.update_A = orig
    assert float((u - ref).abs().max() / ref.abs().max()) < 1e-7
    # The level matrices of epoch 1 (a nonzero fine state, where the
    # nonlinear term makes J depend on the state): level l's matrix is
    # J_l^T J_l of the level-l problem linearised at the fine field
    # restricted l times by the single-field full-weighting restriction.
    mg = Multigrid((17, 17), nvar=1, restriction="full", dtype=torch.float64,
                   device="cpu")
    f = seen_u[1].reshape(17, 17)
    for level in range(1, mg.nlevels):
        f = (mg.RRsingle[level - 1] @ f.reshape(-1)).reshape(
            tuple(levels[level].problem.domain.shape))
        _, Jl = levels[level].problem.linearize(State(fields={"u": f}))
        Jm = Jl.to_csr().to_dense()
        np.testing.assert_allclose(seen_A[1][level].to_dense().numpy(),
                                   (Jm.T @ Jm).numpy(), rtol=1e-12,
                                   atol=1e-12)
    # the coarse states hold the restricted fine fields of the last epoch
    assert levels[1].state.fields["u"].shape == (9, 9)
    assert float(levels[1].state.fields["u"].abs().max()) > 0


def test_direct_solve_above_dense_limit_is_iterative(monkeypatch):
    """Above DIRECT_MAX unknowns the coarsest-level solve of
    Multigrid.smoother_direct is BiCGStab on the sparse matrix to 1e-12
    relative residual (the reference's spsolve has no size limit); it
    agrees with the dense solve."""
    m, A0, f = _run("p17", "cpu")
    exact = m.smoother_direct(0, torch.zeros_like(f), f)
    m._inv.clear()
    monkeypatch.setattr(Multigrid, "DIRECT_MAX", 16)
    it = m.smoother_direct(0, torch.zeros_like(f), f)
    assert 0 not in m._inv
    np.testing.assert_allclose(it.numpy(), exact.numpy(), rtol=1e-9,
                               atol=1e-10 * float(exact.abs().max()))
