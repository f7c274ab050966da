"""GPU tests of the cavity multigrid on the normal equations (csrc/ns_mg.cu,
ns.NsMultigridNewton): each kernel against a NumPy/SciPy statement of the
same operation built from the oracle's CSR Jacobian (util_op.py:859-937
restated), the V-cycle against the same V-cycle in NumPy FP64, and the
Newton / Gauss-Newton solves against the oracle operator and the
reference's own cavity solution."""
import os

import numpy as np
import pytest
import scipy.sparse as sp
import torch

from oracle import ns as NS

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden",
                            "cavity_N128.npz"))


def _p1(n):
    """1D cell-centred prolongation, fine n -> coarse n/2: weights 3/4 (own
    parent), 1/4 (the neighbour parent toward the cell's side), the 1/4 kept
    on the own parent at a wall."""
    m = n // 2
    P = np.zeros((n, m))
    for i in range(n):
        c = i // 2
        P[i, c] += 0.75
        nb = c - 1 if i % 2 == 0 else c + 1
        if 0 <= nb < m:
            P[i, nb] += 0.25
        else:
            P[i, c] += 0.25
    return P


def _P(n):
    p = _p1(n)
    return sp.block_diag([sp.csr_matrix(np.kron(p, p))] * 3).tocsr()


def _st25_to_csr(A):
    """[9, 25, n, n] 25-point operator -> CSR (3 n^2 square)."""
    A = np.asarray(A, np.float64)
    n = A.shape[-1]
    N = n * n
    rows, cols, vals = [], [], []
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    for fg in range(9):
        f, g = divmod(fg, 3)
        for d in range(25):
            dx, dy = d // 5 - 2, d % 5 - 2
            ti, tj = ii + dx, jj + dy
            ok = (ti >= 0) & (ti < n) & (tj >= 0) & (tj < n) & (A[fg, d] != 0)
            rows.append(f * N + (ii * n + jj)[ok])
            cols.append(g * N + (ti * n + tj)[ok])
            vals.append(A[fg, d][ok])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows),
                                                 np.concatenate(cols))),
                         shape=(3 * N, 3 * N))


def _problem(n, variant, seed, cuda, Re=400.0):
    from odil_gb300.ns import NsCavityOperator, NsKernels
    rng = np.random.default_rng(seed)
    kw = dict(pin=(n // 3, n // 2), pin_weight=1.0)
    if variant == "inverse":
        mask = np.zeros((n, n))
        mask.ravel()[rng.choice(n * n, max(2, n * n // 8), replace=False)] = 1
        kw.update(mask=mask, u_imp=rng.standard_normal((n, n)),
                  v_imp=rng.standard_normal((n, n)), kreg=1e-4)
    op = NsCavityOperator(Re, **kw)
    k = NsKernels(n, op, device=cuda)
    s = NS.NsSetup(n, Re, **kw)
    st = {c: 0.3 * rng.standard_normal((n, n)) for c in "uvp"}
    return k, s, st, rng


def _solver(k, **kw):
    from odil_gb300.ns import NsMultigridNewton
    return NsMultigridNewton(k, **kw)


def _rel(a, b):
    return np.abs(np.asarray(a) - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("variant", ["forward", "inverse"])
def test_jx_jtw_and_normal_matrix(cuda, variant):
    n = 10
    k, s, st, rng = _problem(n, variant, 1, cuda)
    mg = _solver(k, nmin=2)
    t = [torch.as_tensor(st[c], device=cuda) for c in "uvp"]
    mg.linearize(*t)
    mg.setup()
    _, J = NS.linearize(s, st)
    x = rng.standard_normal(3 * n * n)
    w = rng.standard_normal(J.shape[0])
    x64 = torch.as_tensor(x, device=cuda).reshape(3, n, n)
    w64 = torch.as_tensor(w, device=cuda).reshape(-1, n, n)
    from odil_gb300._capi import call, ptr, stream_handle
    out = torch.empty((mg.neq, n, n), dtype=torch.float64, device=cuda)
    call("odil_nsmg_jx_f64", n, mg.neq, ptr(mg.coef64), ptr(x64), ptr(out),
         stream_handle())
    assert _rel(out.cpu().numpy().ravel(), J @ x) < 1e-12
    y = torch.empty((3, n, n), dtype=torch.float64, device=cuda)
    call("odil_nsmg_jtw_f64", n, mg.neq, ptr(mg.coef64), ptr(w64), ptr(y),
         stream_handle())
    assert _rel(y.cpu().numpy().ravel(), J.T @ w) < 1e-12
    # FP32 J^T J x, and the explicit 25-point J^T J
    AtA = (J.T @ J).tocsr()
    y32 = mg.apply_normal(x64.float(), torch.empty_like(x64, dtype=torch.float32))
    assert _rel(y32.cpu().numpy().ravel(), AtA @ x) < 1e-5
    A0 = _st25_to_csr(mg.levels[0].A.cpu().numpy())
    assert _rel(A0.toarray(), AtA.toarray()) < 1e-5
    # block-diagonal inverses
    N = n * n
    D = mg.levels[0].dinv.cpu().numpy().reshape(3, 3, N)
    Ad = AtA.toarray()
    for c in (0, 17, N - 1):
        blk = Ad[np.ix_([c, N + c, 2 * N + c], [c, N + c, 2 * N + c])]
        assert _rel(D[:, :, c], np.linalg.inv(blk)) < 1e-4


def test_galerkin_transfers_and_coarse_inverse(cuda):
    n = 16
    k, s, st, rng = _problem(n, "forward", 2, cuda)
    mg = _solver(k, nmin=2)
    t = [torch.as_tensor(st[c], device=cuda) for c in "uvp"]
    mg.linearize(*t)
    mg.setup()
    A = _st25_to_csr(mg.levels[0].A.cpu().numpy())
    for L, C in zip(mg.levels[:-1], mg.levels[1:]):
        P = _P(L.n)
        Ac = (P.T @ A @ P) * 0.25
        got = _st25_to_csr(C.A.cpu().numpy())
        assert _rel(got.toarray(), Ac.toarray()) < 1e-5, (L.n, C.n)
        A = got
    # restriction and prolongation
    from odil_gb300._capi import call, ptr, stream_handle
    L, C = mg.levels[0], mg.levels[1]
    r = rng.standard_normal((3, n, n))
    rt = torch.as_tensor(r, dtype=torch.float32, device=cuda)
    rc = torch.empty((3, n // 2, n // 2), dtype=torch.float32, device=cuda)
    call("odil_nsmg_restrict", n, ptr(rt), ptr(rc), stream_handle())
    P = _P(n)
    assert _rel(rc.cpu().numpy().ravel(), 0.25 * (P.T @ r.ravel())) < 1e-6
    e = rng.standard_normal((3, n // 2, n // 2))
    x = rng.standard_normal((3, n, n))
    xt = torch.as_tensor(x, dtype=torch.float32, device=cuda)
    call("odil_nsmg_prolong_add", n, ptr(torch.as_tensor(
        e, dtype=torch.float32, device=cuda)), ptr(xt), stream_handle())
    assert _rel(xt.cpu().numpy().ravel(), x.ravel() + P @ e.ravel()) < 1e-6
    # coarsest dense inverse (FP64 of the FP32 stencil values)
    last = mg.levels[-1]
    M = _st25_to_csr(last.A.cpu().numpy()).toarray()
    assert _rel(last.minv.cpu().numpy(), np.linalg.inv(M)) < 1e-9


def _vcycle_np(mg, levels_A, levels_D, b, lvl=0):
    """The V-cycle of NsMultigridNewton in NumPy FP64 from the same level
    matrices (CSR) and block inverses."""
    A, D = levels_A[lvl], levels_D[lvl]
    if lvl == len(levels_A) - 1:
        return np.linalg.solve(A.toarray(), b)
    om = mg.omega
    x = om * (D @ b)
    for _ in range(mg.pre - 1):
        x = x + om * (D @ (b - A @ x))
    r = b - A @ x
    n = mg.levels[lvl].n
    P = _P(n)
    e = _vcycle_np(mg, levels_A, levels_D, 0.25 * (P.T @ r), lvl + 1)
    x = x + P @ e
    for _ in range(mg.post):
        x = x + om * (D @ (b - A @ x))
    return x


def _dinv_csr(Dinv):
    D = np.asarray(Dinv, np.float64)
    N = D.shape[-1] * D.shape[-2]
    D = D.reshape(3, 3, N)
    rows, cols, vals = [], [], []
    for f in range(3):
        for g in range(3):
            rows.append(f * N + np.arange(N))
            cols.append(g * N + np.arange(N))
            vals.append(D[f, g])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows),
                                                 np.concatenate(cols))),
                         shape=(3 * N, 3 * N))


def test_vcycle_matches_numpy(cuda):
    n = 32
    k, s, st, rng = _problem(n, "inverse", 3, cuda)
    mg = _solver(k)
    t = [torch.as_tensor(st[c], device=cuda) for c in "uvp"]
    mg.linearize(*t)
    mg.setup()
    As = [_st25_to_csr(L.A.cpu().numpy()) for L in mg.levels]
    Ds = [_dinv_csr(L.dinv.cpu().numpy()) for L in mg.levels]
    b = rng.standard_normal((3, n, n))
    out = torch.empty((3, n, n), dtype=torch.float32, device=cuda)
    mg.vcycle(torch.as_tensor(b, dtype=torch.float32, device=cuda), out)
    ref = _vcycle_np(mg, As, Ds, b.ravel())
    assert _rel(out.cpu().numpy().ravel(), ref) < 2e-4


def test_pcg_solves_normal_equations(cuda):
    n = 64
    k, s, _, rng = _problem(n, "forward", 4, cuda)
    x1 = (np.arange(n) + 0.5) / n
    xx, yy = np.meshgrid(x1, x1, indexing="ij")
    st = {"u": 0.5 * np.sin(np.pi * xx) * np.sin(2 * np.pi * yy),
          "v": -0.5 * np.sin(2 * np.pi * xx) * np.sin(np.pi * yy),
          "p": 0.1 * np.cos(np.pi * xx)}
    mg = _solver(k)
    t = [torch.as_tensor(st[c], device=cuda) for c in "uvp"]
    mg.linearize(*t)
    mg.setup()
    const, J = NS.linearize(s, st)
    AtA = (J.T @ J).tocsr()
    # The right-hand side of a Newton step, -J^T f (a random one would load
    # the near-null pressure-constant mode that the pin term barely fixes,
    # where FP32 cannot resolve the residual).
    f = np.concatenate([c.ravel() for c in const])
    b = -(J.T @ f)
    its = mg.pcg(torch.as_tensor(b, dtype=torch.float32,
                                 device=cuda).reshape(3, n, n), rtol=1e-4)
    x = mg.x.cpu().numpy().ravel().astype(np.float64)
    assert np.linalg.norm(AtA @ x - b) <= 2e-3 * np.linalg.norm(b)
    # the step reduces the linearised residual
    assert np.linalg.norm(J @ x + f) <= 0.5 * np.linalg.norm(f)
    assert its <= 80, its


def test_newton_reaches_reference_cavity(cuda):
    """Forward cavity at 128^2, Re 400, from rest with the multigrid
    normal-equation Newton: the reference's own FP64 solution
    (cavity_N128_Re400) to 1e-5 in u, v and in p up to its constant, and
    the oracle operator's residual rms <= 1e-9 at the result."""
    from odil_gb300.ns import NsCavityOperator, NsKernels
    n = 128
    k = NsKernels(n, NsCavityOperator(400.0, pin=(0, 0)), device=cuda)
    mg = _solver(k)
    t = [torch.zeros((n, n), dtype=torch.float64, device=cuda)
         for _ in range(3)]
    mg.solve(*t, epochs=120, tol=1e-10)
    assert mg.final_rms <= 1e-10, mg.stats[-3:]
    for c, x in zip("uv", t[:2]):
        ref = GOLD["Re400_" + c]
        assert np.abs(x.cpu().numpy() - ref).max() <= 1e-5 * np.abs(ref).max()
    dp = t[2].cpu().numpy() - GOLD["Re400_p"]
    assert np.abs(dp - dp.mean()).max() <= 1e-5 * np.abs(GOLD["Re400_p"]).max()
    rms, _, _ = NS.loss_grad_live(NS.NsSetup(n, 400.0, pin=(0, 0),
                                              pin_weight=1.0),
                                  {c: x.cpu().numpy() for c, x in
                                   zip("uvp", t)})
    assert max(rms[:3]) <= 1e-9, rms


def test_gauss_newton_inverse_is_stationary(cuda):
    """Inverse cavity (48^2, 64 noisy points, penalty 1e-4, pin): after
    Gauss-Newton with the multigrid PCG the oracle loss gradient is below
    1e-6 of its value at the start."""
    from odil_gb300.ns import (NsCavityOperator, NsKernels,
                               NsMultigridNewton)
    n = 48
    fk = NsKernels(n, NsCavityOperator(400.0, pin=(0, 0)), device=cuda)
    fw = [torch.zeros((n, n), dtype=torch.float64, device=cuda)
          for _ in range(3)]
    NsMultigridNewton(fk).solve(*fw, epochs=120, tol=1e-11)
    rng = np.random.default_rng(1)
    mask = np.zeros((n, n))
    mask.ravel()[rng.choice(n * n, 64, replace=False)] = 1.0
    kw = dict(mask=mask, kreg=1e-4, pin=(0, 0), pin_weight=1.0,
              u_imp=fw[0].cpu().numpy() + 0.01 * rng.standard_normal((n, n)),
              v_imp=fw[1].cpu().numpy() + 0.01 * rng.standard_normal((n, n)))
    k = NsKernels(n, NsCavityOperator(400.0, **kw), device=cuda)
    t = [torch.zeros((n, n), dtype=torch.float64, device=cuda)
         for _ in range(3)]
    mg = NsMultigridNewton(k)
    gnorm = lambda: float(torch.sqrt(sum((x**2).sum() for x in
                                         k.loss_grad(*t)[1])))
    g_start = gnorm()
    for _ in range(80):
        mg.step(*t, rtol=1e-4)
        if gnorm() <= 1e-7 * g_start:
            break
    s = NS.NsSetup(n, 400.0, **kw)
    _, l0, g0 = NS.loss_grad_live(s, {c: np.zeros((n, n)) for c in "uvp"})
    _, l1, g1 = NS.loss_grad_live(s, {c: x.cpu().numpy() for c, x in
                                      zip("uvp", t)})
    norm = lambda g: np.sqrt(sum(np.sum(x**2) for x in g.values()))
    assert norm(g1) <= 1e-6 * norm(g0), (norm(g1), norm(g0))
    assert l1 < 1e-3 * l0
