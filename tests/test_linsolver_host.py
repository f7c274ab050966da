"""CPU tests of the iterative linear solvers of odil_gb300.linsolver
(linsolver.py:28-107 of the reference): BiCGStab and LSQR against scipy's
bicgstab and lsqr (the reference's own solver calls) on the same systems,
and the multigrid-preconditioned CG against a direct solve.  The solvers
only use the Jacobian's matvec / rmatvec / to_csr, so a dense matrix on CPU
tensors stands in for the device Jacobian."""
import argparse

import numpy as np
import pytest
import scipy.sparse
import scipy.sparse.linalg
import torch

from odil_gb300 import linsolver


class DenseJacobian:

    def __init__(self, M, grid=None, nfields=1):
        self.M = torch.as_tensor(M, dtype=torch.float64)
        self.shape = tuple(self.M.shape)
        if grid is not None:
            self.grid, self.nfields = grid, nfields

    def matvec(self, v):
        return self.M @ v

    def rmatvec(self, w):
        return self.M.T @ w

    def to_csr(self):
        return self.M.to_sparse_csr()


def _screened(n, rng):
    """J of a variable-coefficient screened Poisson operator on n x n
    cells (periodic), well conditioned."""
    N = n * n
    idx = np.arange(N).reshape(n, n)
    J = np.zeros((N, N))
    c = 3 + rng.uniform(0, 1, (n, n))
    for s in ((1, 0), (-1, 0), (0, 1), (0, -1)):
        nb = np.roll(idx, (-s[0], -s[1]), (0, 1))
        J[idx.ravel(), nb.ravel()] -= 0.5
    J[idx.ravel(), idx.ravel()] += c.ravel() + 2
    return J


@pytest.mark.parametrize("beta,betadiag", [(0.0, 0.0), (0.3, 0.0),
                                           (0.0, 0.2), (0.1, 0.5)])
def test_bicgstab_matches_scipy(beta, betadiag):
    rng = np.random.default_rng(0)
    J = _screened(6, rng) + 0.3 * rng.standard_normal((36, 36))
    rhs = rng.standard_normal(36)
    A = J.T @ J + beta**2 * np.eye(36)
    A = A + betadiag**2 * np.diag(np.diag(A))
    b = J.T @ rhs
    calls = []
    x_ref, info = scipy.sparse.linalg.bicgstab(
        scipy.sparse.csr_matrix(A), b, rtol=0, atol=1e-8, maxiter=15,
        callback=lambda x: calls.append(x))
    dh = {}
    x = linsolver.bicgstab(DenseJacobian(J), torch.as_tensor(rhs), 1e-8, 15,
                           beta, betadiag, dh)
    np.testing.assert_allclose(x.numpy(), x_ref, rtol=1e-9, atol=1e-11)
    assert dh["linsolver_niter"] == len(calls)
    np.testing.assert_allclose(dh["linsolver_residual"],
                               np.mean((A @ x_ref - b)**2)**0.5, rtol=1e-6)


@pytest.mark.parametrize("damp", [0.0, 0.4])
@pytest.mark.parametrize("shape,iters", [((40, 30), 1000), ((40, 30), 7),
                                         ((25, 25), 1000)])
def test_lsqr_matches_scipy(damp, shape, iters):
    rng = np.random.default_rng(1)
    J = rng.standard_normal(shape)
    if shape[0] == shape[1]:  # a well-conditioned square system
        J = 3 * np.eye(shape[0]) + 0.3 * J
    rhs = rng.standard_normal(shape[0])
    ref = scipy.sparse.linalg.lsqr(J, rhs, damp=damp, atol=1e-10, btol=1e-10,
                                   iter_lim=iters)
    dh = {}
    x = linsolver.lsqr(DenseJacobian(J), torch.as_tensor(rhs), damp, 1e-10,
                       1e-10, iter_lim=iters, dhistory=dh)
    # same iterates up to rounding, amplified by cond(J) near convergence
    np.testing.assert_allclose(x.numpy(), ref[0], rtol=1e-6,
                               atol=1e-8 * np.abs(ref[0]).max())
    # a stopping test met within rounding may fire one iteration apart
    assert abs(dh["linsolver_niter"] - ref[2]) <= (0 if iters < 10 else 1)
    if iters < 10:
        # early iterations: the scalar recurrences agree to rounding
        np.testing.assert_allclose(dh["linsolver_anorm"], ref[5], rtol=1e-10)
        np.testing.assert_allclose(dh["linsolver_acond"], ref[6], rtol=1e-9)
        np.testing.assert_allclose(dh["linsolver_residual"], ref[7],
                                   rtol=1e-8)
    else:
        # run to convergence: the Lanczos vectors lose orthogonality in the
        # last iterations, so the |A| and cond(A) estimates (sums over all
        # iterations) pick up rounding at ~1e-5; |A^T r| is negligible in
        # both
        np.testing.assert_allclose(dh["linsolver_anorm"], ref[5], rtol=1e-4)
        np.testing.assert_allclose(dh["linsolver_acond"], ref[6], rtol=1e-4)
        thr = 1e-8 * ref[5] * np.linalg.norm(rhs)
        assert ref[7] <= thr and dh["linsolver_residual"] <= thr


def test_lsqr_zero_rhs():
    x = linsolver.lsqr(DenseJacobian(np.eye(4)), torch.zeros(4))
    assert torch.all(x == 0)


def test_multigrid_cg_reaches_direct_solution():
    rng = np.random.default_rng(2)
    n = 17
    J = _screened(n, rng)
    rhs = rng.standard_normal(n * n)
    args = argparse.Namespace(linsolver_tol=1e-10, linsolver_maxiter=60,
                              nlvl=None, restriction="full", omega=0.6,
                              ndirect=3, smooth_pre=2, smooth_post=2,
                              beta=0.0, betadiag=0.0)
    dh = {}
    x = linsolver.solve(DenseJacobian(J, (n, n)), torch.as_tensor(rhs), args,
                        dh, "multigrid")
    ref = np.linalg.solve(J, rhs)
    np.testing.assert_allclose(x.numpy(), ref, rtol=1e-8, atol=1e-9)
    assert dh["linsolver_residual"] < 1e-10 * np.linalg.norm(J.T @ rhs)
    assert 2 <= dh["linsolver_niter"] < 30


def test_solve_dispatch():
    """lsqr and bicgstab are their own solvers; the GPU-less choices of the
    reference map to the direct solve; unknown names raise ValueError
    (linsolver.py:104-105)."""
    assert "lsqr" not in linsolver.ALIASES
    assert "bicgstab" not in linsolver.ALIASES
    assert linsolver.ALIASES["direct_cu"] == "direct"
    with pytest.raises(ValueError, match="Unknown linsolver"):
        linsolver.solve(DenseJacobian(np.eye(2)), torch.ones(2),
                        argparse.Namespace(), {}, "cholesky")
