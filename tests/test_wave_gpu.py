"""GPU parity tests of the wave kernels against the CPU oracle.

Tolerances: FP64 kernels agree with the FP64 oracle to 1e-10 relative to the
field's max (different but equivalent operation order); FP32 kernels to
2e-5 relative on the residual/J v/J^T w (cancellation of O(1/dt^2) terms),
and FP32 gradients to 1e-4 relative.
"""
import numpy as np
import pytest
import torch

from oracle import wave as W
from oracle import autodiff as AD

pytestmark = pytest.mark.gpu

SHAPES = [(1, 5), (2, 3), (3, 1), (4, 2), (17, 33), (64, 64), (70, 130),
          (129, 257), (256, 96)]


def _setup(nt, nx, seed=0, c=1.3):
    rng = np.random.default_rng(seed)
    return W.WaveSetup(nt, nx, rng.standard_normal(nx), rng.standard_normal(nx),
                       rng.standard_normal(nt), rng.standard_normal(nt), c=c)


def _kernels(s, dev):
    from odil_gb300.wave import WaveKernels
    return WaveKernels(s.nt, s.nx, s.dt, s.dx, s.c, s.init_u, s.init_ut,
                       s.left_u, s.right_u, device=dev)


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(
        np.abs(np.asarray(b)).max(), 1e-300)


@pytest.mark.parametrize("shape", SHAPES)
def test_residual_f64_f32(cuda, shape):
    s = _setup(*shape)
    k = _kernels(s, cuda)
    u = np.random.default_rng(1).standard_normal(shape)
    fo = W.residual(s, u)
    f64 = k.residual(torch.as_tensor(u, device=cuda)).cpu().numpy()
    assert _rel(f64, fo) < 1e-12
    f32 = k.residual(torch.as_tensor(u, dtype=torch.float32,
                                     device=cuda)).cpu().numpy()
    fo32 = W.residual(s, u.astype(np.float32).astype(np.float64))
    assert _rel(f32, fo32) < 2e-5


@pytest.mark.parametrize("shape", SHAPES)
def test_jv_jtv_against_csr(cuda, shape):
    s = _setup(*shape, seed=2)
    k = _kernels(s, cuda)
    rng = np.random.default_rng(3)
    v = rng.standard_normal(shape)
    w = rng.standard_normal(shape)
    _, J = W.linearize(s, np.zeros(shape))
    jv_o = J.dot(v.ravel()).reshape(shape)
    jtw_o = J.T.dot(w.ravel()).reshape(shape)
    jv = k.jv(torch.as_tensor(v, device=cuda)).cpu().numpy()
    jtw = k.jtv(torch.as_tensor(w, device=cuda)).cpu().numpy()
    assert _rel(jv, jv_o) < 1e-12
    assert _rel(jtw, jtw_o) < 1e-12
    # Adjoint identity <J v, w> = <v, J^T w> in FP64.
    a = float(np.sum(jv * w))
    b = float(np.sum(v * jtw))
    assert abs(a - b) <= 1e-12 * (abs(a) + np.abs(jv).max() * np.abs(w).sum())
    jv32 = k.jv(torch.as_tensor(v, dtype=torch.float32, device=cuda)).cpu()
    jtw32 = k.jtv(torch.as_tensor(w, dtype=torch.float32, device=cuda)).cpu()
    assert _rel(jv32.numpy(), jv_o) < 2e-5
    assert _rel(jtw32.numpy(), jtw_o) < 2e-5


# Besides SHAPES: rows and columns wide enough for interior tiles of the
# vectorised kernel (16-, 32- and 64-row tiles), and a width just past the
# first interior column strip.
@pytest.mark.parametrize("shape", SHAPES + [(300, 1000), (1030, 248),
                                            (2100, 2052), (4100, 4100)])
def test_loss_grad_fused(cuda, shape):
    s = _setup(*shape, seed=4)
    k = _kernels(s, cuda)
    u = np.random.default_rng(5).standard_normal(shape)
    lo, go = W.loss_grad(s, u)
    loss, grad = k.loss_grad(torch.as_tensor(u, device=cuda))
    assert abs(loss.item() - lo) <= 1e-12 * lo
    assert _rel(grad.cpu().numpy(), go) < 1e-12
    loss32, grad32 = k.loss_grad(torch.as_tensor(u, dtype=torch.float32,
                                                 device=cuda))
    u32 = u.astype(np.float32).astype(np.float64)
    lo32, go32 = W.loss_grad(s, u32)
    assert abs(loss32.item() - lo32) <= 1e-5 * lo32
    assert _rel(grad32.cpu().numpy(), go32) < 1e-4


def test_loss_grad_unaligned_rows_use_scalar_kernel(cuda):
    """Arrays that are not 16-byte aligned take the one-column-per-lane
    kernel; it agrees with the vectorised one within FP32 tolerance."""
    s = _setup(300, 1000, seed=4)
    k = _kernels(s, cuda)
    u = np.random.default_rng(5).standard_normal((300, 1000))
    store = torch.zeros(300 * 1000 + 1, dtype=torch.float32, device=cuda)
    uu = store[1:].view(300, 1000)
    uu.copy_(torch.as_tensor(u, dtype=torch.float32))
    gstore = torch.zeros_like(store)
    gu = gstore[1:].view(300, 1000)
    assert uu.data_ptr() % 16 != 0
    l1, g1 = k.loss_grad(uu, grad=gu)
    l1 = l1.item()  # the loss buffer is reused by the next call
    l2, g2 = k.loss_grad(uu.clone())
    assert abs(l1 - l2.item()) <= 1e-5 * l2.item()
    assert _rel(g1.cpu().numpy(), g2.cpu().numpy()) < 1e-4


def test_loss_grad_deterministic_and_workspace_reset(cuda):
    s = _setup(300, 200, seed=6)
    k = _kernels(s, cuda)
    u = torch.as_tensor(np.random.default_rng(7).standard_normal((300, 200)),
                        device=cuda)
    vals = []
    for _ in range(5):
        loss, grad = k.loss_grad(u)
        vals.append((loss.item(), grad.sum().item()))
    assert all(v == vals[0] for v in vals)
    # The reduction counter is back to zero after every call.
    assert int(k.workspace[:4].view(torch.int32).item()) == 0


@pytest.mark.parametrize("n", [96, 1024])
def test_gradient_against_autodiff_and_fd(cuda, n):
    """Fused FP32 adjoint gradient vs (a) the FP64 autodiff gradient of the
    op-by-op operator and (b) central finite differences (step 1e-3, FP64) on
    64 seeded coordinates; n = 1024 is the 1024^2 wave configuration itself
    (16-mode profile, seed 1)."""
    nt = nx = n
    s = W.make_setup(nt, nx, "sine", seed=1, nmodes=16)
    k = _kernels(s, cuda)
    rng = np.random.default_rng(11)
    u = W.solve_march(s) + 0.05 * rng.standard_normal((nt, nx))
    u32 = u.astype(np.float32).astype(np.float64)
    _, g_ad = AD.wave_loss_grad_autodiff(s, u32)
    _, g = k.loss_grad(torch.as_tensor(u32, dtype=torch.float32, device=cuda))
    g = g.cpu().numpy().astype(np.float64)
    assert _rel(g, g_ad) < 1e-4
    idx = rng.choice(nt * nx, 64, replace=False)
    h = 1e-3
    for q in idx:
        e = np.zeros(nt * nx)
        e[q] = h
        e = e.reshape(nt, nx)
        fd = (np.mean(W.residual(s, u32 + e)**2) -
              np.mean(W.residual(s, u32 - e)**2)) / (2 * h)
        assert abs(g.ravel()[q] - fd) <= 1e-3 * np.abs(g).max() + 1e-4 * abs(fd)


# Shapes with c dt / dx < 1 (leapfrog-stable), so the solution stays bounded
# and the FP32 solve is comparable; (nt, 2048) exercises two columns/thread.
@pytest.mark.parametrize("shape", [(1, 4), (2, 1), (3, 2), (64, 64), (100, 37),
                                   (1024, 257), (1100, 2048)])
def test_march_direct_solve(cuda, shape):
    s = _setup(*shape, seed=8, c=0.9)
    assert shape[0] <= 3 or s.c * s.dt / s.dx < 1
    k = _kernels(s, cuda)
    b = np.random.default_rng(9).standard_normal(shape)
    xo = W.march(s, b)
    x = k.march(torch.as_tensor(b, device=cuda)).cpu().numpy()
    assert _rel(x, xo) < 1e-10
    x32 = k.march(torch.as_tensor(b, dtype=torch.float32, device=cuda))
    assert _rel(x32.cpu().numpy(), xo) < 1e-3


@pytest.mark.parametrize("shape", [(5, 1), (40, 33), (300, 257), (1100, 1024)])
def test_march_shapes_agree(cuda, shape):
    """Every explicit FP32 launch shape (single block or cluster-tiled)
    gives the same forward substitution (same formula per cell; 1e-5
    relative allows for a different FMA contraction between template
    instances) and is as accurate as the single-block march against the
    FP64 solve."""
    from odil_gb300 import autotune
    s = _setup(*shape, seed=8, c=0.9)
    assert shape[0] <= 5 or s.c * s.dt / s.dx < 1  # stable march, finite x
    k = _kernels(s, cuda)
    b = torch.as_tensor(np.random.default_rng(9).standard_normal(shape),
                        dtype=torch.float32, device=cuda)
    ref = k.march(b)
    assert torch.isfinite(ref).all()
    cands = autotune.candidates_march(shape[1])
    assert cands
    if shape[1] >= 2:
        assert any(c["kind"] == "tiled" for c in cands)
    exact = k.march(b.double()).cpu().numpy()
    ref_err = _rel(ref.cpu().numpy(), exact)
    for cfg in cands:
        x = torch.full_like(b, float("nan"))
        k.march_shape(b, x, cfg)
        assert _rel(x.cpu().numpy(), ref.cpu().numpy()) < 1e-5, cfg
        err = _rel(x.cpu().numpy(), exact)
        assert err <= max(1.5 * ref_err, 1e-6), (cfg, err, ref_err)
    # FP64: the cluster-tiled shapes against the single-block march.
    b64 = b.double()
    ref64 = k.march(b64).cpu().numpy()
    for cfg in autotune.candidates_march(shape[1], torch.float64):
        x = torch.full_like(b64, float("nan"))
        k.march_shape(b64, x, cfg)
        assert _rel(x.cpu().numpy(), ref64) < 1e-12, cfg


@pytest.mark.parametrize("shape", [(3, 2), (40, 70), (130, 96), (2000, 3000)])
def test_march_tiled_matches_oracle(cuda, shape):
    """Cluster-tiled forward substitution against the FP64 oracle, including
    rows that are not a multiple of the halo depth, a window wider than the
    row, and a row too wide for the single-block march."""
    from odil_gb300 import autotune
    s = _setup(*shape, seed=4, c=0.9)
    assert shape[0] <= 3 or s.c * s.dt / s.dx < 1
    k = _kernels(s, cuda)
    b = np.random.default_rng(5).standard_normal(shape)
    xo = W.march(s, b)
    for dtype, tol in ((torch.float64, 1e-10), (torch.float32, 1e-3)):
        bt = torch.as_tensor(b, dtype=dtype, device=cuda)
        cands = [c for c in autotune.candidates_march(shape[1], dtype)
                 if c["kind"] == "tiled"]
        assert cands
        for cfg in cands:
            x = torch.full_like(bt, float("nan"))
            k.march_shape(bt, x, cfg)
            assert _rel(x.cpu().numpy(), xo) < tol, (dtype, cfg)
        x = torch.full_like(bt, float("nan"))
        k.march_tuned(bt, x)
        assert _rel(x.cpu().numpy(), xo) < tol


def test_initial_rhs_and_f32_update(cuda):
    """rhs of u = 0 from the boundary-only kernel equals the general
    update/residual kernel's; the FP32->FP64 update is exact."""
    s = _setup(129, 257, seed=2, c=0.9)
    k = _kernels(s, cuda)
    z = torch.zeros((129, 257), dtype=torch.float64, device=cuda)
    r1 = torch.empty((129, 257), dtype=torch.float32, device=cuda)
    r2 = torch.full_like(r1, float("nan"))
    k.update_residual_mixed(z, None, None, r1)
    k.initial_rhs(r2)
    assert torch.equal(r1, r2)
    from odil_gb300._capi import call, ptr, stream_handle
    u = torch.randn(1000, dtype=torch.float64, device=cuda)
    d = torch.randn(1000, dtype=torch.float32, device=cuda)
    out = torch.empty_like(u)
    call("odil_add_f32_to_f64", ptr(u), ptr(d), ptr(out), 1000, stream_handle())
    assert torch.equal(out, u + d.double())


def test_mixed_newton_from_zero(cuda):
    """The from-zero sequence keeps the iterate as FP32 corrections hi + lo
    (float-pair residuals, one final FP64 write) and reaches the FP64
    discrete solution as closely as the FP64-state sequence: 1e-3 after one
    epoch, 1e-8 after two, 1e-10 after three; the residual norm it reports is
    the FP64 one of the final field."""
    from odil_gb300 import newton
    from odil_gb300.domain import State
    from odil_gb300.problem import Problem
    from odil_gb300.workloads import WaveInstance
    n = 256
    s = W.make_setup(n, n, "sine", seed=1, nmodes=16)
    ref = W.solve_march(s)
    inst = WaveInstance(n, n, profile="sine", seed=1, nmodes=16, device=cuda)
    prob = Problem(inst.operator, inst.domain)
    for ep, tol in ((1, 1e-3), (2, 1e-8), (3, 1e-10)):
        x = torch.randn((n, n), dtype=torch.float64, device=cuda)
        rn = torch.zeros(1, dtype=torch.float64, device=cuda)
        newton.solve(prob, State(fields={"u": x}), "mixed", epochs=ep,
                     rnorm2=rn, from_zero=True)
        xh = x.cpu().numpy()
        assert W.rel_err(xh, ref) <= tol, (ep, W.rel_err(xh, ref))
        ro = np.sum(W.residual(s, xh)**2)
        assert abs(rn.item() - ro) <= 1e-6 * ro + 1e-20
        y = torch.zeros((n, n), dtype=torch.float64, device=cuda)
        newton.solve(prob, State(fields={"u": y}), "mixed", epochs=ep)
        assert W.rel_err(xh, y.cpu().numpy()) <= tol


def test_captured_solve_replays_with_new_inputs(cuda):
    """newton.CapturedSolve: a replay equals the eager solve, and refilling
    the captured input buffers (new boundary data) changes the result as an
    eager solve with that data would."""
    from odil_gb300 import newton
    from odil_gb300.domain import State
    from odil_gb300.problem import Problem
    from odil_gb300.workloads import WaveInstance
    n = 128
    inst = WaveInstance(n, n, profile="sine", seed=1, nmodes=8, device=cuda)
    prob = Problem(inst.operator, inst.domain)
    k = prob.kernels
    u = torch.zeros((n, n), dtype=torch.float64, device=cuda)
    st = State(fields={"u": u})
    host = [k.bc64[i].cpu().pin_memory() for i in range(4)]
    out = torch.empty((n, n), dtype=torch.float64).pin_memory()
    cap = newton.CapturedSolve(prob, st, "mixed", 2,
                               inputs=list(zip(host, k.bc64)),
                               outputs=[(u, out)])
    for scale in (1.0, -0.5):
        for h in host:
            h.mul_(scale)
        cap()
        torch.cuda.synchronize()
        got = out.clone()
        ref = torch.zeros_like(u)
        for h, d in zip(host, k.bc64):
            d.copy_(h)
        newton.solve(prob, State(fields={"u": ref}), "mixed", 2,
                     from_zero=True)
        assert torch.equal(got, ref.cpu())


def test_pair_to_f64_exact(cuda):
    """u = hi + lo is written exactly (equal to the FP64 sum of the two
    floats), over wide exponent gaps, cancellations, zeros and both signs."""
    from odil_gb300._capi import call, ptr, stream_handle
    g = torch.Generator().manual_seed(5)
    n = 1 << 20
    h = torch.randn(n, generator=g, dtype=torch.float64) * \
        10.0**torch.randint(-6, 6, (n, ), generator=g)
    l = h * torch.randn(n, generator=g, dtype=torch.float64) * \
        10.0**(-torch.randint(0, 14, (n, ), generator=g).double())
    l[::7] = -h[::7] * (1 + 1e-7 * torch.randn(len(h[::7]), generator=g,
                                                   dtype=torch.float64))
    l[::11] = 0.0
    h32, l32 = h.float().to(cuda), l.float().to(cuda)
    out = torch.empty(n, dtype=torch.float64, device=cuda)
    for lo in (l32, None):
        call("odil_pair_to_f64", ptr(h32), ptr(lo), ptr(out), n, stream_handle())
        ref = h32.double() + (lo.double() if lo is not None else 0.0)
        assert torch.equal(out, ref)


def test_pair_residual_accuracy(cuda):
    """float(-F(hi + lo)) from FP32 arrays agrees with the FP64 residual of
    hi + lo to ~2^-46 of the largest stencil term, also where F cancels to
    ~1e-9 of its terms (hi + lo = the discrete solution)."""
    from odil_gb300._capi import call, ptr, stream_handle
    n = 512
    s = W.make_setup(n, n, "sine", seed=1, nmodes=16)
    k = _kernels(s, cuda)
    ref = W.solve_march(s)
    hi = ref.astype(np.float32)
    lo = (ref - hi.astype(np.float64)).astype(np.float32)
    full = hi.astype(np.float64) + lo.astype(np.float64)
    scale = 4.0 / s.dt**2 * np.abs(full).max()  # largest stencil term
    rhs = torch.empty((n, n), dtype=torch.float32, device=cuda)
    th, tl = (torch.as_tensor(a, device=cuda) for a in (hi, lo))
    k.pair_residual(th, tl, rhs)
    fo = W.residual(s, full)
    assert np.abs(rhs.cpu().numpy() + fo).max() <= 2.0**-46 * scale + \
        1e-7 * np.abs(fo).max()
    # hi alone (the iterate after the first FP32 epoch).
    k.pair_residual(th, None, rhs)
    fo = W.residual(s, hi.astype(np.float64))
    err = np.abs(rhs.cpu().numpy() + fo).max()
    assert err <= 2.0**-46 * scale + 1e-6 * np.abs(fo).max()
    # u = hi + lo written in FP64 exactly.
    out = torch.empty((n, n), dtype=torch.float64, device=cuda)
    call("odil_pair_to_f64", ptr(th), ptr(tl), ptr(out), n * n, stream_handle())
    assert np.array_equal(out.cpu().numpy(), full)


def test_mixed_newton_reaches_oracle(cuda):
    """Mixed precision (FP64 residual, FP32 solve) converges to the FP64
    discrete solution of the 1024^2 benchmark wave to <= 1e-5 (here 1e-9)."""
    n = 1024
    s = W.make_setup(n, n, "sine", seed=1, nmodes=16)
    ref = W.solve_march(s)
    from odil_gb300 import newton
    from odil_gb300.domain import State
    from odil_gb300.problem import Problem
    from odil_gb300.workloads import WaveInstance
    inst = WaveInstance(n, n, profile="sine", seed=1, nmodes=16, device=cuda)
    prob = Problem(inst.operator, inst.domain)
    errs = []
    for ep in (1, 2, 3):
        x = torch.zeros((n, n), dtype=torch.float64, device=cuda)
        rn = torch.zeros(1, dtype=torch.float64, device=cuda)
        newton.solve(prob, State(fields={"u": x}), "mixed", epochs=ep,
                     rnorm2=rn)
        errs.append(W.rel_err(x.cpu().numpy(), ref))
        # The fused FP64 residual norm equals the oracle's.
        ro = np.sum(W.residual(s, x.cpu().numpy())**2)
        assert abs(rn.item() - ro) <= 1e-6 * ro + 1e-20
    assert errs[0] <= 1e-3, errs
    assert errs[1] <= 1e-8, errs
    assert errs[2] <= 1e-11, errs
    x = torch.zeros((n, n), dtype=torch.float64, device=cuda)
    newton.solve(prob, State(fields={"u": x}), "fp64")
    assert W.rel_err(x.cpu().numpy(), ref) <= 1e-12


def test_generic_operator_matches_fused(cuda):
    """The op-by-op torch path of WaveOperator equals the fused kernels."""
    from odil_gb300.workloads import WaveInstance
    from odil_gb300.problem import Problem
    inst = WaveInstance(40, 30, profile="sine", seed=3, nmodes=5, c=1.1,
                        device=cuda)
    fused = Problem(inst.operator, inst.domain)

    def op(mod, ctx):
        return inst.operator(mod, ctx)

    generic = Problem(op, inst.domain)
    from odil_gb300.domain import State
    rng = np.random.default_rng(0)
    st = State(fields={"u": torch.as_tensor(rng.standard_normal((40, 30)),
                                            device=cuda)})
    f1 = fused.eval_operator(st)[0]
    f2 = generic.eval_operator(st)[0]
    assert _rel(f1.cpu().numpy(), f2.cpu().numpy()) < 1e-12
    l1, g1, _, _ = fused.eval_loss_grad(st)
    l2, g2, _, _ = generic.eval_loss_grad(st)
    assert abs(l1.item() - l2.item()) <= 1e-12 * l2.item()
    assert _rel(g1["u"].cpu().numpy(), g2["u"].cpu().numpy()) < 1e-12


@pytest.mark.parametrize("shape", [(1, 4), (3, 1), (12, 9), (7, 2)])
def test_jacobian_csr_matches_reference_layout(cuda, shape):
    """Jacobian.to_csr() equals the CSR matrix the reference assembles
    (util_op.py:859-937, restated by the oracle), entry by entry."""
    from odil_gb300.problem import Jacobian
    s = _setup(*shape, seed=3)
    k = _kernels(s, cuda)
    J = Jacobian(k, k.shape).to_csr().to_dense().cpu().numpy()
    _, Jo = W.linearize(s, np.zeros(shape))
    Jo = Jo.toarray()
    assert np.abs(J - Jo).max() <= 1e-12 * np.abs(Jo).max()


def test_autograd_function_backward(cuda):
    from odil_gb300.workloads import WaveInstance
    from odil_gb300.problem import Problem
    inst = WaveInstance(32, 32, profile="cos", device=cuda)
    prob = Problem(inst.operator, inst.domain)
    u = torch.randn(32 * 32, dtype=torch.float64, device=cuda,
                    requires_grad=True)
    loss = prob.loss(u)
    loss.backward()
    _, g = prob.kernels.loss_grad(u.detach().reshape(32, 32))
    assert torch.equal(u.grad.reshape(32, 32), g)


def test_errors_are_loud(cuda):
    from odil_gb300._capi import OdilError
    s = _setup(8, 8)
    k = _kernels(s, cuda)
    with pytest.raises(ValueError):
        k.residual(torch.zeros((8, 8)))  # CPU tensor
    with pytest.raises(TypeError):
        k.residual(torch.zeros((8, 8), dtype=torch.float16, device=cuda))
    s2 = _setup(4, 4096)
    k2 = _kernels(s2, cuda)
    with pytest.raises(OdilError):
        k2.march(torch.zeros((4, 4096), dtype=torch.float64, device=cuda))


def test_march_tiled_wait_gives_up(cuda):
    """The bounded halo wait of the shared-memory exchange: a planted wait
    for bytes that never arrive gives up (about a second), the warps write
    NaN instead of hanging, the failure is counted, and the next regular
    launch on the same context is correct again."""
    import ctypes
    from odil_gb300._capi import call, ptr, stream_handle
    s = _setup(256, 256, seed=4, c=0.9)
    assert s.c * s.dt / s.dx < 1
    k = _kernels(s, cuda)
    b = torch.as_tensor(np.random.default_rng(5).standard_normal(s.shape),
                        dtype=torch.float32, device=cuda)
    n = ctypes.c_int64(0)
    call("odil_wave_march_tiled_wait_failures", ctypes.byref(n), 1)
    x = torch.zeros_like(b)
    call("odil_wave_march_tiled_planted_wait_f32", ctypes.byref(k.p32),
         ptr(b), ptr(x), 4, 16, 16, 1, 16, stream_handle())
    torch.cuda.synchronize(cuda)
    call("odil_wave_march_tiled_wait_failures", ctypes.byref(n), 1)
    assert n.value >= 1
    assert torch.isnan(x[16:]).any()
    cfg = {"kind": "tiled", "cpt": 4, "halo": 16, "pf": 16, "warps": 1,
           "exchange": 1}
    y = torch.full_like(b, float("nan"))
    k.march_shape(b, y, cfg)
    ref = k.march(b)
    assert torch.isfinite(ref).all()
    assert _rel(y.cpu().numpy(), ref.cpu().numpy()) < 1e-4
    call("odil_wave_march_tiled_wait_failures", ctypes.byref(n), 0)
    assert n.value == 0


def test_solve_host_out(cuda):
    """host_out receives the FP64 solution (a copy into pinned host memory)
    equal to the device state bit for bit, also when replayed from a
    graph; a host tensor that is not pinned is rejected."""
    from odil_gb300 import newton
    from odil_gb300.domain import State
    from odil_gb300.problem import Problem
    from odil_gb300.workloads import WaveInstance
    inst = WaveInstance(256, 256, profile="sine", seed=2, nmodes=5,
                        device=cuda)
    prob = Problem(inst.operator, inst.domain)
    u = torch.zeros((256, 256), dtype=torch.float64, device=cuda)
    st = State(fields={"u": u})
    host = torch.full((256, 256), float("nan"), dtype=torch.float64).pin_memory()
    for prec, ep in (("mixed", 1), ("mixed", 2), ("fp64", 1)):
        host.fill_(float("nan"))
        newton.solve(prob, st, prec, ep, from_zero=True, host_out=host)
        torch.cuda.synchronize(cuda)
        assert torch.equal(host, u.cpu()), (prec, ep)
    host.fill_(float("nan"))
    cap = newton.CapturedSolve(prob, st, "mixed", 1, host_out=host)
    host.fill_(float("nan"))
    cap()
    torch.cuda.synchronize(cuda)
    assert torch.equal(host, u.cpu())
    with pytest.raises(ValueError):
        newton.solve(prob, st, "mixed", 1, from_zero=True,
                     host_out=torch.zeros((256, 256), dtype=torch.float64))


@pytest.mark.parametrize("beta,betadiag", [(0.3, 0.0), (0.0, 0.5), (0.2, 0.4),
                                           (30.0, 0.5)])
def test_relaxed_normal_equations(cuda, beta, betadiag, monkeypatch):
    """--beta / --betadiag: the relaxed normal equations of
    linsolver.py:35-41, against the oracle's CSR Jacobian solved densely in
    numpy; the matrix-free conjugate-gradient path agrees where the relaxed
    system is well conditioned (large beta)."""
    import argparse
    from odil_gb300 import linsolver
    from odil_gb300.problem import Jacobian
    s = _setup(24, 20, seed=5, c=0.9)
    k = _kernels(s, cuda)
    J = Jacobian(k, (k.n, k.n))
    rng = np.random.default_rng(6)
    rhs = rng.standard_normal(k.n)
    _, Jo = W.linearize(s, np.zeros(s.shape))
    Jd = Jo.toarray()
    A = Jd.T @ Jd + beta**2 * np.eye(k.n)
    A += betadiag**2 * np.diag(np.diag(A))
    ref = np.linalg.solve(A, Jd.T @ rhs)
    args = argparse.Namespace(beta=beta, betadiag=betadiag)
    rt = torch.as_tensor(rhs, device=cuda)
    d = linsolver.solve(J, rt, args, None, "direct").cpu().numpy()
    assert _rel(d, ref) < 1e-9
    if beta >= 1:
        monkeypatch.setattr(linsolver, "DENSE_MAX", 0)
        d2 = linsolver.solve(J, rt, args, None, "direct").cpu().numpy()
        assert _rel(d2, ref) < 1e-8


@pytest.mark.parametrize("shape", [(1, 5), (2, 3), (3, 1), (17, 13), (40, 64),
                                   (129, 256)])
def test_jtj_v_and_diag(cuda, shape):
    """J^T J v (one fused pass, boundary data ignored) and diag(J^T J)
    against the oracle's CSR Jacobian (util_op.py:859-937 restated)."""
    s = _setup(*shape, seed=7, c=0.9)
    k = _kernels(s, cuda)
    _, Jo = W.linearize(s, np.zeros(shape))
    Jd = Jo.toarray()
    v = np.random.default_rng(8).standard_normal(shape)
    ref = (Jd.T @ (Jd @ v.ravel())).reshape(shape)
    out = k.jtj_v(torch.as_tensor(v, device=cuda)).cpu().numpy()
    assert _rel(out, ref) < 1e-12
    out32 = k.jtj_v(torch.as_tensor(v, dtype=torch.float32,
                                    device=cuda)).cpu().numpy()
    assert _rel(out32, ref) < 1e-5
    dref = (Jd**2).sum(0).reshape(shape)
    assert _rel(k.jtj_diag().cpu().numpy(), dref) < 1e-14
    assert _rel(k.jtj_diag(torch.float32).cpu().numpy(), dref) < 1e-6


@pytest.mark.parametrize("nt,nx", [(1024, 1024), (800, 1000), (700, 777),
                                   (2, 64), (97, 130), (12, 6)])
def test_table_march_from_zero_equals_full_rhs(cuda, nt, nx):
    """The first correction from u = 0 marched from the boundary table of
    -F(0) (the zero interior neither stored nor loaded) is bitwise the march
    of the full right-hand side, for every cluster-tiled launch shape; the
    table holds the full right-hand side's boundary cells in order.  Shapes
    keep the Courant number c nx / (2 nt) below the march's stability limit
    (~0.93), so the solutions are finite."""
    import ctypes
    from odil_gb300 import autotune, _capi
    from odil_gb300._capi import call, ptr, stream_handle
    s = _setup(nt, nx, seed=4)
    k = _kernels(s, cuda)
    rhs = torch.empty((nt, nx), dtype=torch.float32, device=cuda)
    k.initial_rhs(rhs)
    nb = _capi.load().odil_wave_boundary_cells(ctypes.byref(k.p64))
    rows = [(i, j) for i in range(min(nt, 2)) for j in range(nx)]
    rows += [(i, j) for i in range(2, nt) for j in (0, nx - 1)]
    assert nb == len(rows)
    tbl = torch.full((nt * nx, ), float("nan"), dtype=torch.float32,
                     device=cuda)
    call("odil_wave_initial_table_mixed", ctypes.byref(k.p64), ptr(tbl),
         stream_handle())
    ii, jj = (torch.as_tensor(v, device=cuda) for v in zip(*rows))
    assert torch.equal(tbl[:nb], rhs[ii, jj])
    tried = 0
    for cfg in autotune.candidates_march(nx, torch.float32):
        if cfg["kind"] != "tiled":
            continue
        x1 = torch.full_like(rhs, float("nan"))
        x2 = torch.full_like(rhs, float("nan"))
        try:
            k.march_shape(rhs, x1, cfg)
        except _capi.OdilError:
            continue  # the cluster does not fit
        try:
            call("odil_wave_march_tiled_table_f32", ctypes.byref(k.p32),
                 ptr(tbl), ptr(x2), cfg["cpt"], cfg["halo"], cfg["pf"],
                 cfg["warps"], cfg["exchange"], stream_handle())
        except _capi.OdilError:
            # A lane would hold both edge columns: refused, and the solve
            # from zero takes the full right-hand side instead.
            assert nx <= cfg["cpt"], cfg
            k._march_cfgs = {torch.float32: cfg}
            x3 = k.march_from_zero(torch.empty_like(rhs), torch.empty_like(rhs))
            assert torch.equal(x1, x3), cfg
            continue
        assert torch.equal(x1, x2), cfg
        tried += 1
    assert tried > 0
    assert torch.isfinite(x1).all()
    # The tuned entry point, whichever kind of march it picked.
    k._march_cfgs = {}
    x3 = torch.empty_like(rhs)
    k.march_from_zero(x3, torch.empty_like(rhs))
    assert torch.equal(x3, k.march_tuned(rhs, torch.empty_like(rhs)))


def test_captured_table_solve_follows_new_inputs_1024(cuda):
    """The headline solve (1024^2, one mixed epoch: boundary table, table
    march, FP64 write, each kernel released by the one before it) replayed
    from a CUDA graph with new boundary data every replay equals the eager
    solve of that data bitwise: no kernel reads its predecessor's output
    from the previous replay."""
    from odil_gb300 import newton
    from odil_gb300.domain import State
    from odil_gb300.problem import Problem
    from odil_gb300.workloads import WaveInstance
    n = 1024
    inst = WaveInstance(n, n, profile="sine", seed=1, nmodes=16, device=cuda)
    prob = Problem(inst.operator, inst.domain)
    k = prob.kernels
    u = torch.zeros((n, n), dtype=torch.float64, device=cuda)
    host = [k.bc64[i].cpu().pin_memory() for i in range(4)]
    out = torch.empty((n, n), dtype=torch.float64).pin_memory()
    cap = newton.CapturedSolve(prob, State(fields={"u": u}), "mixed", 1,
                               inputs=list(zip(host, k.bc64)),
                               outputs=[(u, out)])
    for scale in (1.0, -0.5, 2.0, -1.0):
        for h in host:
            h.mul_(scale)
        cap()
        torch.cuda.synchronize()
        got = out.clone()
        ref = torch.zeros_like(u)
        for h, d in zip(host, k.bc64):
            d.copy_(h)
        newton.solve(prob, State(fields={"u": ref}), "mixed", 1,
                     from_zero=True)
        assert torch.equal(got, ref.cpu()), scale
