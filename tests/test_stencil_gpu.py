"""GPU stencil operators and multigrid against the reference's multigrid.py
outputs (tests/golden/multigrid_ref.npz, from tests/golden/make_golden.py)
and the behaviour its unit tests require (test_multigrid.py)."""
import os

import numpy as np
import pytest
import torch

from oracle import multigrid as M

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden",
                            "multigrid_ref.npz"))
SIZES = [(9, ), (17, ), (9, 9), (5, 9), (17, 17), (5, 5, 9)]


def _field(nw, seed):
    n = int(np.prod(nw))
    return np.sin(seed * 0.123 + np.linspace(0, 3, n)).reshape(nw)


def _key(nw):
    return "x".join(map(str, nw))


def _dense(op, nw, dev):
    """Dense matrix of a GPU StencilOp (columns by unit vectors)."""
    n = int(np.prod(nw))
    cols = []
    for k in range(n):
        e = torch.zeros(n, dtype=torch.float64, device=dev)
        e[k] = 1
        cols.append(op.mul_field(e.reshape(nw)).reshape(-1).cpu().numpy())
    return np.stack(cols, 1)


@pytest.mark.parametrize("nw", SIZES)
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_products_match_reference(cuda, nw, dtype):
    from odil_gb300 import stencil as S
    k = _key(nw)
    tol = 1e-12 if dtype == torch.float64 else 2e-5
    R = S.get_R(nw, dtype=dtype, device=cuda)
    TT = S.get_TT(nw, dtype=dtype, device=cuda)
    u = torch.as_tensor(_field(nw, 1), dtype=dtype, device=cuda)
    uh = torch.as_tensor(_field(R.nwh, 2), dtype=dtype, device=cuda)
    assert np.allclose(R.mul_field(u).cpu().numpy().ravel(), GOLD["R_" + k],
                       atol=tol)
    assert np.allclose(TT.mul_transpose_field(uh).cpu().numpy().ravel(),
                       GOLD["T_" + k], atol=tol)
    A = S.StencilOp([tuple(s) for s in GOLD["A_shifts_" + k]],
                    torch.as_tensor(GOLD["A_coefs_" + k], dtype=dtype,
                                    device=cuda), nw)
    assert np.allclose(A.mul_field(u).cpu().numpy().ravel(), GOLD["Au_" + k],
                       atol=tol * 10)
    assert np.allclose(A.mul_transpose_field(u).cpu().numpy().ravel(),
                       GOLD["ATu_" + k], atol=tol * 10)
    AtA = A.mul_transpose_op(A)
    ref = dict(zip(map(tuple, GOLD["AtA_shifts_" + k]), GOLD["AtA_coefs_" + k]))
    assert set(ref) == set(AtA.shifts)
    for s, c in zip(AtA.shifts, AtA.coef):
        assert np.allclose(c.cpu().numpy(), ref[s], atol=tol * 10), s


@pytest.mark.parametrize("nw", SIZES)
def test_galerkin_matches_reference_csr(cuda, nw):
    from odil_gb300 import stencil as S
    k = _key(nw)
    A = S.StencilOp([tuple(s) for s in GOLD["A_shifts_" + k]],
                    torch.as_tensor(GOLD["A_coefs_" + k], device=cuda), nw)
    Ah = S.galerkin(A, S.get_R(nw, device=cuda), S.get_TT(nw, device=cuda))
    dense = _dense(Ah, Ah.nw, cuda)
    assert np.allclose(dense, GOLD["AhCSR_" + k], atol=1e-12)


def test_galerkin_reference_laplacian(cuda):
    from odil_gb300 import stencil as S
    nw = (11, 11)
    pad = np.pad(np.ones((9, 9)), 1)
    coef = np.stack([4 * np.ones(nw), -pad, -pad, -pad, -pad])
    A = S.StencilOp([(0, 0), (-1, 0), (1, 0), (0, -1), (0, 1)],
                    torch.as_tensor(coef, device=cuda), nw)
    Ah = S.galerkin(A, S.get_R(nw, device=cuda), S.get_TT(nw, device=cuda))
    assert np.allclose(_dense(Ah, Ah.nw, cuda), GOLD["lap11_Ah"], atol=1e-13)


def test_periodic_matches_oracle(cuda):
    from odil_gb300 import stencil as S
    nw = (8, 6)
    per = (True, False)
    rng = np.random.default_rng(0)
    shifts = M.all_shifts(2, 1)
    coefs = rng.standard_normal((9, ) + nw)
    Ao = M.Stencil(shifts, coefs, nw, periodic=per)
    A = S.StencilOp(shifts, torch.as_tensor(coefs, device=cuda), nw,
                    periodic=per)
    u = rng.standard_normal(nw)
    ut = torch.as_tensor(u, device=cuda)
    assert np.allclose(A.mul_field(ut).cpu().numpy(), Ao.mul_field(u))
    assert np.allclose(A.mul_transpose_field(ut).cpu().numpy(),
                       Ao.mul_transpose_field(u))
    Ah = S.galerkin(A, S.get_R(nw, periodic=per, device=cuda),
                    S.get_TT(nw, periodic=per, device=cuda))
    Aho = M.galerkin(Ao, M.get_R(nw, periodic=per), M.get_TT(nw, periodic=per))
    assert np.allclose(_dense(Ah, Ah.nw, cuda), Aho.tocsr().toarray(),
                       atol=1e-12)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_multigrid_poisson(cuda, dtype):
    """test_multigrid.py:251-368: 10 V-cycles (Jacobi omega 0.7) on the 17^2
    Laplacian reach a residual below 1e-6 (FP64; FP32 to its precision)."""
    from odil_gb300 import stencil as S
    nw = (17, 17)
    h = 1.0 / 16
    shifts = [(0, 0), (1, 0), (-1, 0), (0, 1), (0, -1)]
    coef = np.stack([np.full(nw, -4 / h**2)] + [np.full(nw, 1 / h**2)] * 4)
    A = S.StencilOp(shifts, torch.as_tensor(coef, dtype=dtype, device=cuda),
                    nw)
    mg = S.MultigridOp(nw, dtype=dtype, device=cuda)
    mg.update_A([[A]])
    x, y = np.meshgrid(np.linspace(0, 1, 17), np.linspace(0, 1, 17),
                       indexing='ij')
    f = torch.as_tensor(np.sin(np.pi * x) * np.sin(2 * np.pi * y),
                        dtype=dtype, device=cuda)
    u = [torch.zeros(nw, dtype=dtype, device=cuda)]
    sm = lambda lvl, u, f: mg.smoother_jacobi(lvl, u, f, omega=0.7)
    for _ in range(10):
        u = mg.step(u, [f], sm, ndirect=3)
    r = mg.residual(mg.AA[0], u, [f])[0]
    rms = float(torch.sqrt(torch.mean(r.double()**2)))
    assert rms < (1e-6 if dtype == torch.float64 else 1e-3)
    # Same iterates as the NumPy restatement of the reference V-cycle.
    Ao = M.Stencil(shifts, coef, nw)
    mgo = M.MultigridOp(nw)
    mgo.update_A(Ao)
    uo = np.zeros(nw)
    smo = lambda lvl, u, f: mgo.smoother_jacobi(lvl, u, f, omega=0.7)
    for _ in range(10):
        uo = mgo.step(uo, f.double().cpu().numpy(), smo, ndirect=3)
    if dtype == torch.float64:
        assert np.allclose(u[0].cpu().numpy(), uo, atol=1e-10)


def test_coefficient_algebra_applies_on_device(cuda):
    """Operators built by the coefficient algebra (shift_left/right,
    mul_elementwise, add_elementwise, eye, from_diag, mul_self_transpose)
    applied by the device kernel equal the products they stand for."""
    from odil_gb300.stencil import StencilOp
    rng = np.random.default_rng(3)
    nw = (7, 6)
    n = int(np.prod(nw))
    sh = [(0, 0), (-1, 0), (1, 0), (0, 1), (1, -1)]
    A = StencilOp(sh, torch.as_tensor(rng.standard_normal((5, ) + nw),
                                      device=cuda), nw)
    B = StencilOp([(0, 0), (0, 1)], torch.as_tensor(
        rng.standard_normal((2, ) + nw), device=cuda), nw)
    dA, dB = _dense(A, nw, cuda), _dense(B, nw, cuda)
    u = torch.as_tensor(rng.standard_normal(nw), device=cuda)
    un = u.cpu().numpy().ravel()
    for s in [(1, 0), (-1, 2)]:
        Au = torch.as_tensor((dA @ un).reshape(nw))
        ref = StencilOp.apply_shift(Au, s).numpy()
        got = A.shift_left(s).mul_field(u).cpu().numpy()
        assert np.allclose(got, ref, atol=1e-13), s
        got = A.shift_right(s).mul_field(u).cpu().numpy()
        ref = sum(A.coef[k].cpu().numpy() * StencilOp.apply_shift(
            u, tuple(a + b for a, b in zip(dw, s))).cpu().numpy()
            for k, dw in enumerate(sh))
        assert np.allclose(got, ref, atol=1e-13), s
    assert np.allclose(_dense(A.add_elementwise(B), nw, cuda), dA + dB)
    assert np.allclose(_dense(A.mul_elementwise(B), nw, cuda), dA * dB)
    assert np.allclose(_dense(StencilOp.eye(nw, dtype=torch.float64,
                                            device=cuda), nw, cuda), np.eye(n))
    c = torch.as_tensor(rng.standard_normal(nw), device=cuda)
    assert np.allclose(_dense(StencilOp.from_diag(c, nw), nw, cuda),
                       np.diag(c.cpu().numpy().ravel()))
    assert np.allclose(_dense(A.mul_self_transpose(), nw, cuda), dA.T @ dA,
                       atol=1e-12)
