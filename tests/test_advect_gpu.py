"""GPU parity tests of the advection family against the CPU oracle."""
import numpy as np
import pytest
import torch

from oracle import advection as A

pytestmark = pytest.mark.gpu


def _kernels(s, dev):
    from odil_gb300.advection import AdvectKernels
    return AdvectKernels(s.nt, s.nx, s.ny, s.dt, s.dx, s.dy, s.ax, s.ay,
                         s.p_init, device=dev)


def _rel(a, b):
    return np.abs(np.asarray(a) - b).max() / max(np.abs(b).max(), 1e-300)


SHAPES = [(1, 3, 5), (4, 1, 6), (6, 8, 8), (16, 12, 20), (32, 32, 32)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("seed", [0, 1, 2, 5])
def test_residual_jv_jtv_loss(cuda, shape, seed):
    rng = np.random.default_rng(seed)
    a = rng.uniform(-1, 1, 2)
    s = A.AdvectSetup(*shape, a[0], a[1], rng.standard_normal(shape[1:]))
    k = _kernels(s, cuda)
    p = rng.standard_normal(shape)
    w = rng.standard_normal(shape)
    pt = torch.as_tensor(p, device=cuda)
    assert _rel(k.residual(pt).cpu().numpy(), A.residual_p(s, p)) < 1e-13
    assert _rel(k.jv(pt).cpu().numpy(), A.jv(s, p)) < 1e-13
    assert _rel(k.jtv(torch.as_tensor(w, device=cuda)).cpu().numpy(),
                A.jtv(s, w)) < 1e-13
    l, g = k.loss_grad(pt)
    lo, go = A.loss_grad(s, p)
    assert abs(l.item() - lo) <= 1e-12 * lo
    assert _rel(g.cpu().numpy(), go) < 1e-12
    p32 = pt.float()
    assert _rel(k.residual(p32).cpu().numpy(), A.residual_p(
        s, p.astype(np.float32).astype(np.float64))) < 1e-5
    l32, g32 = k.loss_grad(p32)
    assert abs(l32.item() - lo) <= 1e-4 * lo
    assert _rel(g32.cpu().numpy(), go) < 1e-4


def test_multigrid_pieces_match_oracle(cuda):
    from odil_gb300 import _capi
    from odil_gb300._capi import call, ptr, stream_handle
    import ctypes
    s = A.make_setup(16, seed=3)
    k = _kernels(s, cuda)
    rng = np.random.default_rng(0)
    b = rng.standard_normal(s.shape)
    x = rng.standard_normal(s.shape)
    bt = torch.as_tensor(b, dtype=torch.float32, device=cuda)
    xt = torch.as_tensor(x, dtype=torch.float32, device=cuda)
    out = torch.empty_like(bt)
    r = torch.empty_like(bt)
    mg = k.multigrid()
    P = ctypes.byref(mg["levels"][0].params)
    om = 0.8
    call("odil_advect_mg_jacobi", P, ptr(xt), ptr(bt), ptr(out),
         ctypes.c_float(om), ptr(r), stream_handle())
    D = A.diag(s)
    ref = x + om * (b - A.jv(s, x)) / D
    assert _rel(out.cpu().numpy(), ref) < 1e-5
    assert _rel(r.cpu().numpy(), b - A.jv(s, x)) < 1e-5
    rc = torch.empty((8, 8, 8), dtype=torch.float32, device=cuda)
    call("odil_advect_mg_restrict", 16, 16, 16, ptr(bt), ptr(rc),
         stream_handle())
    assert _rel(rc.cpu().numpy(), A.restrict(b)) < 1e-6
    e = rng.standard_normal((8, 8, 8))
    xp = xt.clone()
    call("odil_advect_mg_prolong_add", 16, 16, 16,
         ptr(torch.as_tensor(e, dtype=torch.float32, device=cuda)), ptr(xp),
         stream_handle())
    assert _rel(xp.cpu().numpy(), x + A.prolong(e)) < 1e-6
    # Whole V-cycle against the oracle's.
    levels = A.level_setup(s)
    assert [L.shape for L in levels] == [L.shape for L in mg["levels"]]
    v = k.vcycle(bt, torch.empty_like(bt)).cpu().numpy()
    assert _rel(v, A.vcycle(levels, b)) < 1e-4


@pytest.mark.parametrize("n,seed", [(32, 0), (32, 4), (64, 1), (128, 1)])
def test_mixed_newton_mg_reaches_oracle(cuda, n, seed):
    """FP64 Newton with the FP32 BiCGStab + V-cycle inner solve reaches
    rel err <= 1e-5 against the FP64 direct solution."""
    from odil_gb300 import newton
    from odil_gb300.domain import State
    from odil_gb300.problem import Problem
    from odil_gb300.workloads import AdvectInstance
    s = A.make_setup(n, seed=seed)
    ref = A.solve(s)
    inst = AdvectInstance(n, seed=seed, device=cuda)
    assert np.allclose(inst.operator.p_init, s.p_init)
    prob = Problem(inst.operator, inst.domain)
    u = torch.zeros(s.shape, dtype=torch.float64, device=cuda)
    rn = torch.zeros(1, dtype=torch.float64, device=cuda)
    newton.solve(prob, State(fields={"p": u}), "mixed", rnorm2=rn)
    err = A.rel_err(u.cpu().numpy(), ref)
    assert err <= 1e-5, err
    r = A.residual_p(s, u.cpu().numpy())
    assert abs(rn.item() - np.sum(r**2)) <= 1e-6 * np.sum(r**2) + 1e-18


def test_generic_operator_matches_fused(cuda):
    from odil_gb300.domain import State
    from odil_gb300.problem import Problem
    from odil_gb300.workloads import AdvectInstance
    inst = AdvectInstance(12, seed=2, device=cuda)
    fused = Problem(inst.operator, inst.domain)
    generic = Problem(lambda mod, ctx: inst.operator(mod, ctx), inst.domain)
    rng = np.random.default_rng(0)
    st = State(fields={"p": torch.as_tensor(rng.standard_normal((12, 12, 12)),
                                            device=cuda)})
    f1 = fused.eval_operator(st)[0].cpu().numpy()
    f2 = generic.eval_operator(st)[0].cpu().numpy()
    assert _rel(f1, f2) < 1e-12
    l1, g1, _, _ = fused.eval_loss_grad(st)
    l2, g2, _, _ = generic.eval_loss_grad(st)
    assert abs(l1.item() - l2.item()) <= 1e-12 * l2.item()
    assert _rel(g1["p"].cpu().numpy(), g2["p"].cpu().numpy()) < 1e-12


def _misaligned(t):
    """A copy of `t` whose data pointer is 4 bytes past a 16-byte boundary
    (forces the one-cell-per-thread kernels)."""
    buf = torch.empty(t.numel() + 1, dtype=t.dtype, device=t.device)
    v = buf[1:].view(t.shape)
    v.copy_(t)
    return v


@pytest.mark.parametrize("shape", [(3, 5, 4), (6, 8, 8), (5, 7, 36),
                                   (4, 3, 132), (2, 2, 1028)])
@pytest.mark.parametrize("signs", [(1, 1), (1, -1), (-1, 1), (-1, -1)])
def test_vec4_kernels_match_scalar(cuda, shape, signs):
    """The 4-cells-per-thread FP32 residual, J v and Jacobi sweep give the
    same bits as the one-cell kernels (same formula, same rounding)."""
    import ctypes
    from odil_gb300._capi import call, ptr, stream_handle
    rng = np.random.default_rng(sum(shape))
    a = rng.uniform(0.2, 1, 2) * np.array(signs)
    s = A.AdvectSetup(*shape, a[0], a[1], rng.standard_normal(shape[1:]))
    k = _kernels(s, cuda)
    p = torch.as_tensor(rng.standard_normal(shape), dtype=torch.float32,
                        device=cuda)
    pm = _misaligned(p)
    assert pm.data_ptr() % 16 == 4 and p.data_ptr() % 16 == 0
    for fn in (k.residual, k.jv):
        ref = fn(pm, out=_misaligned(torch.zeros_like(p)))
        got = fn(p)
        assert torch.equal(got, ref)
    ref = A.residual_p(s, p.double().cpu().numpy())
    assert _rel(k.residual(p).cpu().numpy(), ref) < 1e-5
    b = torch.as_tensor(rng.standard_normal(shape), dtype=torch.float32,
                        device=cuda)
    lin = k._params(k.shape, (k.dt, k.dx, k.dy))  # J without p_init
    P = ctypes.byref(lin)
    om = ctypes.c_float(0.8)
    outs = []
    for xx, bb in ((p, b), (pm, _misaligned(b))):
        xo = _misaligned(torch.zeros_like(p)) if xx is pm else \
            torch.zeros_like(p)
        ro = _misaligned(torch.zeros_like(p)) if xx is pm else \
            torch.zeros_like(p)
        call("odil_advect_mg_jacobi", P, ptr(xx), ptr(bb), ptr(xo), om,
             ptr(ro), stream_handle())
        x0 = torch.zeros_like(xo)
        call("odil_advect_mg_jacobi", P, None, ptr(bb), ptr(x0), om, None,
             stream_handle())
        outs.append((xo.clone(), ro.clone(), x0.clone()))
    for u, v in zip(*outs):
        assert torch.equal(u, v)
