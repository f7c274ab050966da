"""The stencil compiler for generic operators (odil_gb300.jit).

CPU: tracing, symbolic derivatives (checked against finite differences by a
numpy evaluator of the traced graph), code generation and the nvcc build.
GPU: the compiled residual and fused loss + gradient against the op-by-op
torch path of the same operator (util_op.py:627-654, 939-966)."""
import numpy as np
import pytest
import torch


def _wave(device):
    from odil_gb300.workloads import WaveInstance
    inst = WaveInstance(40, 30, profile="sine", seed=3, nmodes=5, c=1.1,
                        device=device)

    def op(mod, ctx):
        return inst.operator(mod, ctx)

    return inst.domain, op


def _nonlinear_domain(device, dtype=np.float64):
    from odil_gb300.domain import Domain
    return Domain(ndim=2, shape=(24, 20), lower=(0, 0), upper=(1, 1),
                  varnames=("t", "x"), fieldnames=["u", "v"], dtype=dtype,
                  device=device)


def _nonlinear(mod, ctx):
    """Two fields, periodic shifts, index masks, coordinates, a frozen read
    and the elementary functions the tracer differentiates."""
    u = ctx.field("u")
    v = ctx.field("v")
    dt, dx = ctx.step(0), ctx.step(1)
    nx = ctx.size(1)
    it, ix = ctx.cell_index(0), ctx.cell_index(1)
    x = ctx.cell_center(1)
    ux = (ctx.field("u", 0, 1) - ctx.field("u", 0, -1)) / (2 * dx)
    vt = (v - ctx.field("v", -1, 0)) / dt
    frozen = ctx.field("u", -1, 0, freeze=True)
    f1 = mod.where(it == 0, u - mod.sin(np.pi * x),
                   vt + u * ux - 0.1 * mod.tanh(v) + mod.exp(-u * u) * frozen)
    edge = (ix == 0) | (ix == nx - 1)
    f2 = mod.where(edge, v,
                   v * v / (1.0 + u * u) - mod.sqrt(1.0 + v * v) + 0.5 * u
                   + mod.maximum(u, 0.2 * v)**3)
    return [f1, f2]


def _eval_np(g, node, fields, memo):
    """Value of a traced node on the whole grid (numpy, FP64)."""
    if node.id in memo:
        return memo[node.id]
    op, a = node.op, node.args
    shape = g.shape

    def ev(n):
        return _eval_np(g, n, fields, memo)

    if op == "const":
        r = np.full(shape, a[0])
    elif op in ("field", "ffield"):
        r = np.roll(fields[a[0]], tuple(-s for s in a[1]), tuple(range(len(shape))))
    elif op in ("idx", "idxs"):
        r = np.broadcast_to(np.arange(shape[a[0]]).reshape(
            [-1 if d == a[0] else 1 for d in range(len(shape))]), shape)
        if op == "idxs":
            r = (r - a[1]) % shape[a[0]]
    elif op in ("ext", "exts"):
        arr, kind = g.ext[a[0]]
        r = np.broadcast_to(arr, shape)
        if op == "exts":
            r = np.roll(r, a[1], tuple(range(len(shape))))
        if kind == "b":
            r = r != 0
    elif op in ("add", "sub", "mul", "div", "eq", "ne", "lt", "le", "gt",
                "ge", "and", "or"):
        x, y = ev(a[0]), ev(a[1])
        r = {"add": np.add, "sub": np.subtract, "mul": np.multiply,
             "div": np.divide, "eq": np.equal, "ne": np.not_equal,
             "lt": np.less, "le": np.less_equal, "gt": np.greater,
             "ge": np.greater_equal, "and": np.logical_and,
             "or": np.logical_or}[op](x, y)
    elif op == "not":
        r = ~ev(a[0])
    elif op == "pow":
        r = ev(a[0])**a[1]
    elif op == "fn":
        r = {"sqrt": np.sqrt, "exp": np.exp, "log": np.log, "sin": np.sin,
             "cos": np.cos, "tanh": np.tanh, "abs": np.abs}[a[0]](ev(a[1]))
    elif op in ("max", "min"):
        r = (np.maximum if op == "max" else np.minimum)(ev(a[0]), ev(a[1]))
    elif op == "where":
        r = np.where(ev(a[0]), ev(a[1]), ev(a[2]))
    else:
        raise AssertionError(op)
    memo[node.id] = r
    return r


def test_trace_and_derivatives_match_finite_differences():
    from odil_gb300 import jit
    dom = _nonlinear_domain("cpu")
    g, terms = jit.trace(_nonlinear, dom)
    assert len(terms) == 2
    rng = np.random.default_rng(0)
    fields = {"u": rng.uniform(-1, 1, dom.shape),
              "v": rng.uniform(-1, 1, dom.shape)}
    for t in terms:
        rd = jit.reads(t)
        assert ("u", (-1, 0)) not in rd  # the frozen read has no derivative
        for wrt in rd:
            d = _eval_np(g, g.diff(t, wrt, {}), fields, {})
            h = 1e-6
            name, sh = wrt
            fp = {k: v.copy() for k, v in fields.items()}
            fm = {k: v.copy() for k, v in fields.items()}
            # perturb u[c + sh] for every c at once: the read at offset sh of
            # cell c sees the whole shifted field, so perturb all cells
            fp[name] = fp[name] + h
            fm[name] = fm[name] - h
            # other reads of the same field also move: isolate this read by
            # evaluating the term with only this leaf perturbed
            leaf = g.field(name, sh)
            vp = _eval_np(g, t, fields, {leaf.id: _eval_np(g, leaf, fp, {})})
            vm = _eval_np(g, t, fields, {leaf.id: _eval_np(g, leaf, fm, {})})
            fd = (vp - vm) / (2 * h)
            assert np.allclose(d, fd, rtol=1e-6, atol=1e-7), wrt


def test_unsupported_constructs_fall_back():
    from odil_gb300 import jit
    from odil_gb300.problem import Problem
    dom = _nonlinear_domain("cpu")

    def raw(mod, ctx):
        return [Problem.Raw(ctx.field("u"))]

    def net(mod, ctx):
        return [ctx.neural_net("n", ctx.field("u"))]

    def reduce(mod, ctx):
        return [mod.reduce_mean(ctx.field("u"))]

    for op in (raw, net, reduce):
        with pytest.raises(jit.JitUnsupported):
            jit.trace(op, dom)
        assert Problem(op, dom).jit is None


def test_generated_source_compiles():
    """nvcc builds the generated kernels for sm_103a (no GPU needed)."""
    import ctypes
    from odil_gb300 import jit
    dom, op = _wave("cpu")
    J = jit.JitOperator(op, dom)
    so = jit.compile_source(J.code)
    lib = ctypes.CDLL(so)
    assert hasattr(lib, "odil_jit_residual") and \
        hasattr(lib, "odil_jit_loss_grad")
    # FP32 and a two-field operator build too.
    J2 = jit.JitOperator(_nonlinear, _nonlinear_domain("cpu", np.float32))
    assert "typedef float T;" in J2.code
    jit.compile_source(J2.code)


def _rel(a, b):
    a = a.detach().double().cpu().numpy()
    b = b.detach().double().cpu().numpy()
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["wave", "nonlinear"])
def test_compiled_operator_matches_torch_path(cuda, case):
    from odil_gb300.domain import State
    from odil_gb300.problem import Problem
    if case == "wave":
        dom, op = _wave(cuda)
    else:
        dom, op = _nonlinear_domain(cuda), _nonlinear
    pj = Problem(op, dom)
    pt = Problem(op, dom, jit=False)
    assert pj.jit is not None and pt.jit is None
    rng = np.random.default_rng(1)
    st = State(fields={n: torch.as_tensor(rng.uniform(-1, 1, dom.shape),
                                          device=cuda)
                       for n in dom.fieldnames})
    fj = pj.eval_operator(st)
    ft = pt.eval_operator(st)
    for a, b in zip(fj, ft):
        assert _rel(a, b) < 1e-12
    lj, gj, _, sj = pj.eval_loss_grad(st)
    lt, gt, _, stt = pt.eval_loss_grad(st)
    assert abs(lj.item() - lt.item()) <= 1e-12 * lt.item()
    for a, b in zip(sj, stt):
        assert abs(a.item() - b.item()) <= 1e-12 * abs(b.item()) + 1e-300
    for n in dom.fieldnames:
        assert _rel(gj[n], gt[n]) < 1e-11, n
    # Deterministic, and the autograd Function on the packed state.
    lj2, gj2, _, _ = pj.eval_loss_grad(st)
    assert lj2.item() == lj.item()
    assert all(torch.equal(gj[n], gj2[n]) for n in dom.fieldnames)
    u = pj.pack_fields(st.fields).clone().requires_grad_(True)
    loss = pj.loss(u)
    loss.backward()
    assert torch.equal(u.grad, pj.pack_fields(gj))


@pytest.mark.gpu
def test_compiled_operator_fp32(cuda):
    from odil_gb300.domain import State
    from odil_gb300.problem import Problem
    dom = _nonlinear_domain(cuda, np.float32)
    pj = Problem(_nonlinear, dom)
    pt = Problem(_nonlinear, dom, jit=False)
    rng = np.random.default_rng(2)
    st = State(fields={n: torch.as_tensor(rng.uniform(-1, 1, dom.shape),
                                          dtype=torch.float32, device=cuda)
                       for n in dom.fieldnames})
    lj, gj, _, _ = pj.eval_loss_grad(st)
    lt, gt, _, _ = pt.eval_loss_grad(st)
    assert abs(lj.item() - lt.item()) <= 1e-5 * lt.item()
    for n in dom.fieldnames:
        assert gj[n].dtype == torch.float32
        assert _rel(gj[n], gt[n]) < 1e-4, n


@pytest.mark.gpu
def test_compiled_wave_matches_fused_kernels(cuda):
    """The wave operator compiled from its generic form equals the
    hand-written fused kernels of the registered family."""
    from odil_gb300.domain import State
    from odil_gb300.problem import Problem
    from odil_gb300.workloads import WaveInstance
    inst = WaveInstance(40, 30, profile="sine", seed=3, nmodes=5, c=1.1,
                        device=cuda)
    fused = Problem(inst.operator, inst.domain)

    def op(mod, ctx):
        return inst.operator(mod, ctx)

    pj = Problem(op, inst.domain)
    assert pj.jit is not None
    st = State(fields={"u": torch.as_tensor(
        np.random.default_rng(0).standard_normal((40, 30)), device=cuda)})
    assert _rel(pj.eval_operator(st)[0], fused.eval_operator(st)[0]) < 1e-12
    l1, g1, _, _ = fused.eval_loss_grad(st)
    l2, g2, _, _ = pj.eval_loss_grad(st)
    assert abs(l1.item() - l2.item()) <= 1e-12 * l1.item()
    assert _rel(g2["u"], g1["u"]) < 1e-12


@pytest.mark.gpu
def test_compiled_jacobian_matches_autograd(cuda):
    """linearize() of a compiled generic operator: the per-shift coefficient
    fields assembled in the reference's CSR layout (util_op.py:859-937)
    equal the autograd Jacobian of the op-by-op residual; matvec, rmatvec
    and both solve paths agree with the dense matrix."""
    from odil_gb300.domain import State
    from odil_gb300.problem import Problem
    dom = _nonlinear_domain(cuda)
    pj = Problem(_nonlinear, dom)
    pt = Problem(_nonlinear, dom, jit=False)
    rng = np.random.default_rng(4)
    st = State(fields={n: torch.as_tensor(rng.uniform(-1, 1, dom.shape),
                                          device=cuda)
                       for n in dom.fieldnames})
    const, J = pj.linearize(st)
    packed = pj.pack_fields(st.fields)

    def res(x):
        f = pt._generic(pt.unpack_fields(x), 0)
        return torch.cat([t.reshape(-1) for t in f])

    ref = torch.autograd.functional.jacobian(res, packed)
    # the frozen read (u at t-1 in term 1) is a constant for the tape too
    D = J.to_csr().to_dense()
    assert D.shape == ref.shape
    assert (D - ref).abs().max().item() <= 1e-12 * ref.abs().max().item()
    v = torch.as_tensor(rng.standard_normal(J.shape[1]), device=cuda)
    w = torch.as_tensor(rng.standard_normal(J.shape[0]), device=cuda)
    assert _rel(J.matvec(v), D @ v) < 1e-13
    assert _rel(J.rmatvec(w), D.T @ w) < 1e-13
    rhs = torch.as_tensor(rng.standard_normal(J.shape[0]), device=cuda)
    d1 = J.solve(rhs)
    assert _rel(D @ d1, rhs) < 1e-9


@pytest.mark.gpu
def test_compiled_jacobian_matrix_free_solve(cuda):
    """The matrix-free solve (conjugate gradients on the normal equations,
    used above the dense-solve size) agrees with the dense direct solve on a
    well-conditioned screened-Poisson operator."""
    from odil_gb300.domain import Domain, State
    from odil_gb300.problem import Problem
    dom = Domain(ndim=2, shape=(16, 12), lower=(0, 0), upper=(1, 1),
                 varnames=("x", "y"), fieldnames=["u"], device=cuda)

    def op(mod, ctx):
        u = ctx.field("u")
        lap = (ctx.field("u", 1, 0) + ctx.field("u", -1, 0) +
               ctx.field("u", 0, 1) + ctx.field("u", 0, -1) - 4 * u)
        return [3 * u - 0.5 * lap - mod.sin(ctx.cell_center(0))]

    pj = Problem(op, dom)
    st = State(fields={"u": torch.zeros(dom.shape, dtype=torch.float64,
                                        device=cuda)})
    _, J = pj.linearize(st)
    rhs = torch.as_tensor(np.random.default_rng(5).standard_normal(
        J.shape[0]), device=cuda)
    d1 = J.solve(rhs)
    J.DENSE_MAX = 0
    d2 = J.solve(rhs, tol=1e-13)
    assert _rel(d2, d1) < 1e-10


@pytest.mark.gpu
def test_compiled_newton_matches_fused(cuda):
    """Newton on the generic form of the wave operator (compiled Jacobian,
    direct solve) reaches the fused family's Newton solution."""
    from odil_gb300 import newton
    from odil_gb300.domain import State
    from odil_gb300.problem import Problem
    from odil_gb300.workloads import WaveInstance
    inst = WaveInstance(40, 30, profile="sine", seed=3, nmodes=5, c=0.9,
                        device=cuda)

    def op(mod, ctx):
        return inst.operator(mod, ctx)

    pj = Problem(op, inst.domain)
    u = torch.zeros((40, 30), dtype=torch.float64, device=cuda)
    st = State(fields={"u": u})
    for _ in range(2):
        const, J = pj.linearize(st)
        d = J.solve(-torch.cat([c.reshape(-1) for c in const]))
        u += d.reshape(u.shape)
    fused = Problem(inst.operator, inst.domain)
    uf = torch.zeros_like(u)
    newton.solve(fused, State(fields={"u": uf}), "fp64", 2)
    assert _rel(u, uf) < 1e-11


def _op1d(mod, ctx):
    """1D: Burgers-like residual with a where on the boundary cell."""
    u = ctx.field("u")
    dx = ctx.step(0)
    ix = ctx.cell_index(0)
    um, up = ctx.field("u", -1), ctx.field("u", 1)
    f = u * (up - um) / (2 * dx) - 0.05 * (up - 2 * u + um) / dx**2 + \
        mod.cos(ctx.cell_center(0))
    return [mod.where(ix == 0, u - 1.0, f)]


def _op3d(mod, ctx):
    """3D: upwind advection in t with a nonlinear source (periodic x, y)."""
    p = ctx.field("p")
    pt = ctx.field("p", -1, 0, 0)
    px = ctx.field("p", 0, -1, 0)
    py = ctx.field("p", 0, 0, -1)
    dt, dx, dy = ctx.step(0), ctx.step(1), ctx.step(2)
    it = ctx.cell_index(0)
    f = (p - pt) / dt + 0.7 * (p - px) / dx - 0.4 * (p - py) / dy + \
        0.1 * p * p
    return [mod.where(it == 0, p - mod.sin(2 * np.pi * ctx.cell_center(1)), f)]


def _dom(shape, names, device, fields):
    from odil_gb300.domain import Domain
    return Domain(ndim=len(shape), shape=shape, lower=(0, ) * len(shape),
                  upper=(1, ) * len(shape), varnames=names, fieldnames=fields,
                  device=device)


def test_rank1_and_rank3_operators_compile():
    from odil_gb300 import jit
    for op, dom in ((_op1d, _dom((33, ), ("x", ), "cpu", ["u"])),
                    (_op3d, _dom((6, 8, 10), ("t", "x", "y"), "cpu", ["p"]))):
        J = jit.JitOperator(op, dom)
        jit.compile_source(J.code)
        assert J.ncontrib == len(jit.reads(J.terms[0]))


@pytest.mark.gpu
@pytest.mark.parametrize("rank", [1, 3])
def test_rank1_and_rank3_match_torch_path(cuda, rank):
    from odil_gb300.domain import State
    from odil_gb300.problem import Problem
    if rank == 1:
        op, dom = _op1d, _dom((33, ), ("x", ), cuda, ["u"])
    else:
        op, dom = _op3d, _dom((6, 8, 10), ("t", "x", "y"), cuda, ["p"])
    pj, pt = Problem(op, dom), Problem(op, dom, jit=False)
    assert pj.jit is not None
    rng = np.random.default_rng(9)
    name = dom.fieldnames[0]
    st = State(fields={name: torch.as_tensor(rng.uniform(-1, 1, dom.shape),
                                             device=cuda)})
    assert _rel(pj.eval_operator(st)[0], pt.eval_operator(st)[0]) < 1e-12
    lj, gj, _, _ = pj.eval_loss_grad(st)
    lt, gt, _, _ = pt.eval_loss_grad(st)
    assert abs(lj.item() - lt.item()) <= 1e-12 * lt.item()
    assert _rel(gj[name], gt[name]) < 1e-11
    _, J = pj.linearize(st)
    packed = pj.pack_fields(st.fields)

    def res(x):
        return torch.cat([t.reshape(-1) for t in pt._generic(
            pt.unpack_fields(x), 0)])

    ref = torch.autograd.functional.jacobian(res, packed)
    D = J.to_csr().to_dense()
    assert (D - ref).abs().max().item() <= 1e-12 * ref.abs().max().item()


@pytest.mark.gpu
def test_eval_diag_compiled_matches_torch_path(cuda):
    """The stochastic diag(J^T J) estimate (util_op.py:675-731) through the
    compiled Jacobian equals the autograd estimate for the same samples."""
    from odil_gb300.domain import State
    from odil_gb300.problem import Problem
    dom = _dom((6, 8, 10), ("t", "x", "y"), cuda, ["p"])
    pj, pt = Problem(_op3d, dom), Problem(_op3d, dom, jit=False)
    st = State(fields={"p": torch.as_tensor(np.random.default_rng(3).uniform(
        -1, 1, dom.shape), device=cuda)})
    dj = pj.eval_diag(st, nsmp=4, generator=torch.Generator(cuda).manual_seed(5))
    dt = pt.eval_diag(st, nsmp=4, generator=torch.Generator(cuda).manual_seed(5))
    assert _rel(dj, dt) < 1e-12


def _op_epoch(mod, ctx):
    u = ctx.field("u")
    return [u - ctx.field("u", -1) * 0.5 - 0.1 * ctx.epoch]


def _op_branch(mod, ctx):
    u = ctx.field("u")
    return [u * 2 if ctx.epoch > 3 else u]


def test_epoch_is_a_kernel_argument():
    """ctx.epoch becomes a per-launch scalar; a Python branch on it is not
    traced (the operator then runs op by op)."""
    from odil_gb300 import jit
    from odil_gb300.problem import Problem
    dom = _dom((16, ), ("x", ), "cpu", ["u"])
    g, terms = jit.trace(_op_epoch, dom)
    assert any(n.op == "param" for n in g.nodes)
    assert "a.epoch" in jit.JitOperator(_op_epoch, dom).code
    with pytest.raises(jit.JitUnsupported):
        jit.trace(_op_branch, dom)
    assert Problem(_op_branch, dom).jit is None


@pytest.mark.gpu
def test_epoch_follows_the_evaluation(cuda):
    from odil_gb300.domain import State
    from odil_gb300.problem import Problem
    dom = _dom((16, ), ("x", ), cuda, ["u"])
    pj, pt = Problem(_op_epoch, dom), Problem(_op_epoch, dom, jit=False)
    st = State(fields={"u": torch.linspace(0, 1, 16, dtype=torch.float64,
                                           device=cuda)})
    for ep in (0, 3, 7):
        assert _rel(pj.eval_operator(st, ep)[0],
                    pt.eval_operator(st, ep)[0]) < 1e-14
        lj = pj.eval_loss_grad(st, ep)[0]
        lt = pt.eval_loss_grad(st, ep)[0]
        assert abs(lj.item() - lt.item()) <= 1e-13 * lt.item()


@pytest.mark.gpu
def test_optimize_multigrid_on_compiled_operator(cuda):
    """util.optimize_multigridop (util.py:509-617): Newton with V-cycles on the
    Galerkin J^T J stencils reaches the direct Newton solution of a
    screened-Poisson operator."""
    import argparse
    from odil_gb300 import util
    from odil_gb300.domain import Domain, State
    from odil_gb300.problem import Problem
    dom = Domain(ndim=2, shape=(16, 16), lower=(0, 0), upper=(1, 1),
                 varnames=("x", "y"), fieldnames=["u"], device=cuda)

    def op(mod, ctx):
        u = ctx.field("u")
        lap = (ctx.field("u", 1, 0) + ctx.field("u", -1, 0) +
               ctx.field("u", 0, 1) + ctx.field("u", 0, -1) - 4 * u)
        return [3 * u - 0.5 * lap - mod.sin(ctx.cell_center(0)) + 0.1 * u * u]

    pj = Problem(op, dom)
    ref = torch.zeros(dom.shape, dtype=torch.float64, device=cuda)
    st = State(fields={"u": ref})
    for _ in range(6):
        const, J = pj.linearize(st)
        ref += J.solve(-const[0].reshape(-1)).reshape(dom.shape)
    args = argparse.Namespace(epochs=6, epoch_start=0, nlvl=3,
                              restriction="full", omega=0.6,
                              linsolver_maxiter=30, ndirect=3, smooth_pre=2,
                              smooth_post=2)
    u = torch.zeros(dom.shape, dtype=torch.float64, device=cuda)
    util.optimize_multigridop(args, pj, State(fields={"u": u}))
    assert _rel(u, ref) < 1e-8


@pytest.mark.parametrize("case", ["wave", "advection", "nonlinear", "laplace",
                                  "rank1"])
def test_trace_matches_op_by_op_on_cpu(case):
    """The traced graph, evaluated with numpy, equals the op-by-op torch
    residual of the same operator on CPU tensors (the tracer's semantics:
    shifts, masks, broadcast arrays, coordinates, constants)."""
    from odil_gb300 import jit
    from odil_gb300.domain import Domain
    from odil_gb300.problem import Problem, operator_laplace
    if case == "wave":
        dom, op = _wave("cpu")
    elif case == "advection":
        from odil_gb300.advection import AdvectionOperator
        dom = Domain(ndim=3, shape=(5, 6, 7), lower=(0, 0, 0),
                     upper=(1, 1, 1), varnames=("t", "x", "y"),
                     fieldnames=["p"], device="cpu")
        A = AdvectionOperator(0.7, -0.3, np.random.default_rng(2)
                              .standard_normal((6, 7)))
        op = A.__call__
    elif case == "nonlinear":
        dom, op = _nonlinear_domain("cpu"), _nonlinear
    elif case == "laplace":
        dom = Domain(ndim=2, shape=(9, 11), lower=(0, 0), upper=(1, 2),
                     varnames=("x", "y"), fieldnames=["u", "v"],
                     device="cpu")
        op = operator_laplace
    else:
        dom, op = _dom((33, ), ("x", ), "cpu", ["u"]), _op1d
    g, terms = jit.trace(op, dom)
    rng = np.random.default_rng(7)
    fields = {n: rng.uniform(-1, 1, dom.shape) for n in dom.fieldnames}
    pt = Problem(op, dom, jit=False)
    ref = pt._generic({n: torch.as_tensor(v) for n, v in fields.items()}, 0)
    assert len(ref) == len(terms)
    for t, r in zip(terms, ref):
        got = np.broadcast_to(_eval_np(g, t, fields, {}), dom.shape)
        r = np.broadcast_to(torch.as_tensor(r).numpy(), dom.shape)
        assert np.allclose(got, r, rtol=1e-13, atol=1e-13)


def _op_roll(mod, ctx):
    """The reference's NS pattern (ns_steady.py:264-285): stencils modified
    at the boundary by where, then rolled again (second neighbours), plus a
    rolled coordinate array and a rolled index."""
    dx, dy = ctx.step(0), ctx.step(1)
    ix, iy = ctx.cell_index(0), ctx.cell_index(1)
    nx, ny = ctx.size(0), ctx.size(1)
    u = ctx.field("u")
    st = [u, ctx.field("u", -1, 0), ctx.field("u", 1, 0),
          ctx.field("u", 0, -1), ctx.field("u", 0, 1)]
    st[1] = mod.where(ix == 0, 2 * st[0] - st[2], st[1])
    st[2] = mod.where(ix == nx - 1, 2 * st[0] - st[1], st[2])
    xmm = mod.roll(st[1], shift=1, axis=0)
    xpp = mod.roll(st[2], shift=-1, axis=0)
    xmm = mod.where(ix == 0, st[1], xmm)
    xpp = mod.where(ix == nx - 1, st[2], xpp)
    q_xm = (xmm - 4 * st[1] + 3 * u) / (2 * dx)
    q_xp = (-3 * u + 4 * st[2] - xpp) / (2 * dx)
    q_x = mod.where(u > 0, q_xm, q_xp)
    yr = mod.roll(ctx.cell_center(1), shift=2, axis=1)
    irr = mod.roll(iy, shift=-1, axis=1)
    q_y = (st[4] - st[3]) / (2 * dy)
    return [u * q_x + q_y - yr * mod.where(irr == 0, 1.0, 0.5)]


def test_roll_of_traced_expressions():
    """mod.roll of traced values: the numpy evaluation of the traced graph
    equals the op-by-op torch residual, its derivatives match finite
    differences, and the generated source compiles."""
    from odil_gb300 import jit
    from odil_gb300.problem import Problem
    dom = _dom((9, 7), ("x", "y"), "cpu", ["u"])
    g, terms = jit.trace(_op_roll, dom)
    rng = np.random.default_rng(3)
    fields = {"u": rng.uniform(-1, 1, dom.shape)}
    pt = Problem(_op_roll, dom, jit=False)
    ref = pt._generic({"u": torch.as_tensor(fields["u"])}, 0)[0].numpy()
    got = _eval_np(g, terms[0], fields, {})
    assert np.allclose(got, ref, rtol=1e-13, atol=1e-13)
    assert ("u", (-2, 0)) in jit.reads(terms[0])  # a rolled first neighbour
    for wrt in jit.reads(terms[0]):
        d = _eval_np(g, g.diff(terms[0], wrt, {}), fields, {})
        leaf = g.field(*wrt)
        h = 1e-6
        vp = _eval_np(g, terms[0], fields,
                      {leaf.id: _eval_np(g, leaf, fields, {}) + h})
        vm = _eval_np(g, terms[0], fields,
                      {leaf.id: _eval_np(g, leaf, fields, {}) - h})
        assert np.allclose(d, (vp - vm) / (2 * h), rtol=1e-6, atol=1e-6), wrt
    J = jit.JitOperator(_op_roll, dom)
    assert "wrap(i0 - (" in J.code or "wrap(i1 - (" in J.code
    jit.compile_source(J.code)


@pytest.mark.parametrize("extras", [False, True])
def test_ns_generic_form_matches_oracle(extras):
    """NsCavityOperator's op-by-op form (ns_steady.py:142-433) equals the
    oracle's restatement term by term on CPU tensors, and its traced graph
    (which rolls traced stencils) evaluates to the same values."""
    from odil_gb300 import jit
    from odil_gb300.domain import Domain
    from odil_gb300.ns import NsCavityOperator
    from odil_gb300.problem import Problem
    from oracle import ns as NS
    n = 12
    rng = np.random.default_rng(5)
    kw = {}
    if extras:
        mask = (rng.random((n, n)) < 0.2).astype(np.float64)
        kw = dict(mask=mask, u_imp=rng.standard_normal((n, n)),
                  v_imp=rng.standard_normal((n, n)), alpha=0.7, kreg=1e-3,
                  pin=(2, 3), pin_weight=2.0)
    op = NsCavityOperator(400.0, **kw)
    dom = Domain(ndim=2, shape=(n, n), lower=(0, 0), upper=(1, 1),
                 varnames=("x", "y"), fieldnames=["u", "v", "p"],
                 device="cpu")
    state = {k: rng.uniform(-1, 1, (n, n)) for k in ("u", "v", "p")}
    setup = NS.NsSetup(n, 400.0, **kw)
    ref = NS.residual(setup, state)
    pt = Problem(lambda mod, ctx: op(mod, ctx), dom, jit=False)
    assert pt.kernels is None
    got = pt._generic({k: torch.as_tensor(v) for k, v in state.items()}, 0)
    assert len(got) == len(ref)
    for a, b in zip(got, ref):
        assert np.allclose(torch.as_tensor(a).numpy(), b, rtol=1e-12,
                           atol=1e-12 * np.abs(b).max())
    g, terms = jit.trace(op, dom)
    for t, b in zip(terms, ref):
        ev = np.broadcast_to(_eval_np(g, t, state, {}), (n, n))
        assert np.allclose(ev, b, rtol=1e-12, atol=1e-12 * np.abs(b).max())
    if not extras:
        jit.compile_source(jit.JitOperator(op, dom).code)


def test_unforeseen_tracing_error_falls_back():
    """An operator that fails under tracing in a way the tracer does not
    model (here: asking a traced field for its numpy array) still gets a
    Problem, on the op-by-op path, with a warning."""
    import warnings
    from odil_gb300.problem import Problem
    dom = _dom((8, ), ("x", ), "cpu", ["u"])

    def odd(mod, ctx):
        u = ctx.field("u")
        _ = u.numpy()
        return [u]

    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        p = Problem(odd, dom)
    assert p.jit is None
    assert any("op by op" in str(x.message) for x in w)


def test_failed_build_falls_back(monkeypatch):
    """A build failure at first use drops the operator to the op-by-op path
    with a warning instead of failing the evaluation."""
    import warnings
    from odil_gb300 import jit
    from odil_gb300.problem import Problem
    dom = _dom((8, ), ("x", ), "cpu", ["u"])
    p = Problem(_op1d, dom)
    assert p.jit is not None

    def broken(code):
        raise RuntimeError("nvcc failed on the generated operator:\\nboom")

    monkeypatch.setattr(jit, "compile_source", broken)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        assert p._jit_ready() is False
    assert p.jit is None
    assert any("build failed" in str(x.message) for x in w)
