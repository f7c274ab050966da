"""CPU tests: the multigrid oracle reproduces the reference's multigrid.py
outputs (fixtures from tests/golden/make_golden.py), and behaves as the
reference's own unit tests require (test_multigrid.py:251-368)."""
import os

import numpy as np
import pytest

from oracle import multigrid as M

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden",
                            "multigrid_ref.npz"))
SIZES = [(9, ), (17, ), (9, 9), (5, 9), (17, 17), (5, 5, 9)]


def _field(nw, seed):
    n = int(np.prod(nw))
    return np.sin(seed * 0.123 + np.linspace(0, 3, n)).reshape(nw)


def _key(nw):
    return "x".join(map(str, nw))


@pytest.mark.parametrize("nw", SIZES)
def test_restriction_interpolation(nw):
    R = M.get_R(nw)
    TT = M.get_TT(nw)
    u = _field(nw, 1)
    uh = _field(tuple(R.nwh), 2)
    assert np.allclose(R.mul_field(u).ravel(), GOLD["R_" + _key(nw)],
                       rtol=0, atol=1e-14)
    assert np.allclose(TT.mul_transpose_field(uh).ravel(),
                       GOLD["T_" + _key(nw)], rtol=0, atol=1e-14)
    Rcsr = GOLD["Rcsr_" + _key(nw)]
    if Rcsr.ndim == 2:
        assert np.allclose(R.tocsr().toarray(), Rcsr, atol=1e-15)


@pytest.mark.parametrize("nw", SIZES)
def test_stencil_products_and_galerkin(nw):
    k = _key(nw)
    A = M.Stencil(GOLD["A_shifts_" + k], GOLD["A_coefs_" + k], nw)
    u = _field(nw, 1)
    assert np.allclose(A.mul_field(u).ravel(), GOLD["Au_" + k], atol=1e-13)
    assert np.allclose(A.mul_transpose_field(u).ravel(), GOLD["ATu_" + k],
                       atol=1e-13)
    AtA = M.mul_transpose_op(A, A)
    ref = dict(zip(map(tuple, GOLD["AtA_shifts_" + k]), GOLD["AtA_coefs_" + k]))
    got = dict(zip(map(tuple, AtA.shifts), AtA.coefs))
    assert set(ref) == set(got)
    for s in ref:
        assert np.allclose(got[s], ref[s], atol=1e-13), s
    # Galerkin coarsening equals the reference's CSR Galerkin product
    # (multigrid.py:125-131) for this variable, nonsymmetric operator.
    Ah = M.galerkin(A, M.get_R(nw), M.get_TT(nw))
    assert np.allclose(Ah.tocsr().toarray(), GOLD["AhCSR_" + k], atol=1e-13)


def test_galerkin_on_reference_laplacian():
    """test_multigrid.py:197-249: the reference's stencil coarsening of the
    padded 11x11 Laplacian (where it is exact)."""
    nw = (11, 11)
    pad = lambda: np.pad(np.ones((9, 9)), 1)
    A = M.Stencil([(0, 0), (-1, 0), (1, 0), (0, -1), (0, 1)],
                  [4 * np.ones(nw), -pad(), -pad(), -pad(), -pad()], nw)
    Ah = M.galerkin(A, M.get_R(nw), M.get_TT(nw))
    assert np.allclose(Ah.tocsr().toarray(), GOLD["lap11_Ah"], atol=1e-14)


def test_multigrid_poisson_converges():
    """test_multigrid.py:251-368: 10 V-cycles (Jacobi omega 0.7) on the 17^2
    Laplacian bring the residual below 1e-6."""
    nw = (17, 17)
    h = 1.0 / 16
    shifts = [(0, 0), (1, 0), (-1, 0), (0, 1), (0, -1)]
    coefs = [np.full(nw, -4 / h**2)] + [np.full(nw, 1 / h**2)] * 4
    A = M.Stencil(shifts, coefs, nw)
    mg = M.MultigridOp(nw)
    mg.update_A(A)
    x, y = np.meshgrid(np.linspace(0, 1, 17), np.linspace(0, 1, 17),
                       indexing='ij')
    f = np.sin(np.pi * x) * np.sin(2 * np.pi * y)
    u = np.zeros(nw)
    sm = lambda lvl, u, f: mg.smoother_jacobi(lvl, u, f, omega=0.7)
    for _ in range(10):
        u = mg.step(u, f, sm, ndirect=3)
    r = f - A.mul_field(u)
    assert np.mean(r**2)**0.5 < 1e-6


def test_periodic_galerkin_matches_csr():
    """Periodic axes (the advection extension): R A T from the stencil
    formula equals the CSR triple product."""
    nw = (8, 6)
    per = (True, False)
    rng = np.random.default_rng(0)
    shifts = M.all_shifts(2, 1)
    A = M.Stencil(shifts, rng.standard_normal((9, ) + nw), nw, periodic=per)
    R = M.get_R(nw, periodic=per)
    TT = M.get_TT(nw, periodic=per)
    Ah = M.galerkin(A, R, TT)
    dense = (R.tocsr() @ A.tocsr() @ TT.tocsr().T).toarray()
    assert np.allclose(Ah.tocsr().toarray(), dense, atol=1e-12)
