"""GPU runs of code whose arithmetic is also checked on the CPU.

* the multigrid decomposition kernels (mgdecomp.cu) through
  odil_gb300.multigrid.MultigridDecomp: refinement of node and cell grids,
  weights to field(s), against the reference's MultigridDecomp outputs
  (tests/golden/mgdecomp_ref.npz), the adjoint kernels against finite
  differences (torch.autograd.gradcheck), guard bands (CPU check: a host
  build of mgdecomp.cuh);
* the CSR multigrid and the iterative linear solvers on CUDA tensors (CPU
  check: the same torch code on CPU tensors);
* compiled generic operators that roll traced expressions, and the NS
  cavity's generic form compiled (CPU check: the generated kernels built
  with g++, test_jit_cpu_emulation.py).

Collected last on purpose: a stop at the first failure here has already run
every other GPU test."""
import os
import sys

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.dirname(__file__))
from test_jit import _dom, _op_roll, _rel  # noqa: E402

G = np.load(os.path.join(os.path.dirname(__file__), "golden",
                         "mgdecomp_ref.npz"))
KEYS = ["node_5", "node_9", "node_5x9", "node_3x5x5", "cell_4", "cell_6",
        "cell_3x5", "cell_2x3x4"]


@pytest.mark.parametrize("key", KEYS)
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_interp_matches_reference(cuda, key, dtype):
    from odil_gb300.multigrid import MultigridDecomp as D
    cell = key.startswith("cell")
    u = torch.as_tensor(G[key + "_u"], dtype=dtype, device=cuda)
    tol = 1e-13 if dtype == torch.float64 else 3e-6
    for depth in (1, 2):
        r = D.interp_field(u, depth, cell=cell)
        np.testing.assert_allclose(r.double().cpu().numpy(),
                                   G["%s_d%d" % (key, depth)], rtol=tol,
                                   atol=tol)
    fn = D.interp_cell_field if cell else D.interp_node_field
    np.testing.assert_allclose(fn(u, 1, method="roll").double().cpu().numpy(),
                               G[key + "_d1"], rtol=tol, atol=tol)


@pytest.mark.parametrize("kind", ["node", "cell"])
def test_weights_to_field_matches_reference(cuda, kind):
    from odil_gb300.multigrid import MultigridDecomp as D
    cell = kind == "cell"
    uw = torch.as_tensor(G["w2f_%s_uw" % kind], device=cuda)
    nnw = [tuple(v) for v in G["w2f_%s_nnw" % kind]]
    factors = [1.0, 0.5, 2.0]
    f = D.weights_to_field(uw, nnw, factors=factors, cell=cell)
    np.testing.assert_allclose(f.cpu().numpy(), G["w2f_%s_field" % kind],
                               rtol=1e-13, atol=1e-13)
    for i, fi in enumerate(D.weights_to_fields(uw, nnw, factors=factors,
                                               cell=cell)):
        np.testing.assert_allclose(fi.cpu().numpy(),
                                   G["w2f_%s_fields%d" % (kind, i)],
                                   rtol=1e-13, atol=1e-13)
    ones = D.get_weights_coarse_ones(nnw, torch.float64, device=cuda)
    np.testing.assert_array_equal(ones.cpu().numpy(), G["w2f_%s_ones" % kind])


@pytest.mark.parametrize("shape,cell", [((5, ), False), ((3, 4), True),
                                        ((2, 3, 2), True), ((3, 2, 3), False)])
def test_interp_gradient(cuda, shape, cell):
    from odil_gb300.multigrid import MultigridDecomp as D
    u = torch.randn(shape, dtype=torch.float64, device=cuda,
                    generator=torch.Generator(cuda).manual_seed(1),
                    requires_grad=True)
    assert torch.autograd.gradcheck(
        lambda x: D.interp_field(x, 2, cell=cell), (u, ))


@pytest.mark.parametrize("cell", [False, True])
def test_weights_to_field_gradient(cuda, cell):
    from odil_gb300.multigrid import MultigridDecomp as D
    nnw = [(8, 4), (4, 2)] if cell else [(9, 5), (5, 3), (3, 2)]
    n = sum(int(np.prod(v)) for v in nnw)
    uw = torch.randn(n, dtype=torch.float64, device=cuda,
                     generator=torch.Generator(cuda).manual_seed(2),
                     requires_grad=True)
    factors = [1.5, -0.5, 2.0][:len(nnw)]
    assert torch.autograd.gradcheck(
        lambda x: D.weights_to_field(x, nnw, factors=factors, cell=cell),
        (uw, ))


@pytest.mark.parametrize("shape,cell", [((7, ), False), ((3, 5), True),
                                        ((2, 3, 4), True), ((3, 3, 2), False)])
def test_guard_bands_untouched(cuda, shape, cell):
    """Canary bands of 4096 sentinels before and after every output of both
    entry points (called through the C ABI on views into larger buffers)
    stay intact, and every output element is written."""
    import ctypes
    from odil_gb300 import _capi
    lib = _capi.load()
    G, sentinel = 4096, -12345.5
    fine = tuple(2 * v if cell else 2 * v - 1 for v in shape)
    nc, nf = int(np.prod(shape)), int(np.prod(fine))
    n = (ctypes.c_int64 * len(shape))(*shape)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    u = torch.randn(nc, dtype=torch.float64, device=cuda)
    g = torch.randn(nf, dtype=torch.float64, device=cuda)
    bufs = [torch.full((nf + 2 * G, ), sentinel, dtype=torch.float64,
                       device=cuda) for _ in range(2)] + \
        [torch.full((nc + 2 * G, ), sentinel, dtype=torch.float64,
                    device=cuda) for _ in range(2)]
    out, wf, gc, wc = [b[G:-G] for b in bufs]
    assert lib.odil_mgdecomp_refine_f64(len(shape), n, int(cell),
                                        u.data_ptr(), out.data_ptr(), 1.0,
                                        None, 0.0, st) == 0
    assert lib.odil_mgdecomp_refine_t_f64(len(shape), n, int(cell),
                                          g.data_ptr(), gc.data_ptr(),
                                          wc.data_ptr(), 2.0, wf.data_ptr(),
                                          3.0, st) == 0
    torch.cuda.synchronize()
    for b in bufs:
        assert bool(torch.all(b[:G] == sentinel))
        assert bool(torch.all(b[-G:] == sentinel))
        assert not bool(torch.any(b[G:-G] == sentinel))
    torch.testing.assert_close(wf, 3.0 * g, rtol=0, atol=0)
    torch.testing.assert_close(wc, 2.0 * gc, rtol=1e-15, atol=0)


@pytest.mark.parametrize("name", ["p17", "v9", "d3"])
def test_multigrid_csr_on_cuda(cuda, name):
    """The CSR multigrid on cuSPARSE matches the reference's outputs
    (tests/golden/multigrid_csr_ref.npz) as on the CPU."""
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    import test_multigrid_csr as T
    T._run(name, cuda, gauss_seidel=False)


def test_iterative_solvers_on_cuda(cuda):
    """bicgstab and lsqr on CUDA tensors equal their CPU runs (which match
    scipy), and the multigrid-preconditioned CG reaches the direct
    solution."""
    import argparse
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    import test_linsolver_host as L
    from odil_gb300 import linsolver
    rng = np.random.default_rng(0)
    J = L._screened(6, rng) + 0.3 * rng.standard_normal((36, 36))
    rhs = rng.standard_normal(36)

    class CudaJ(L.DenseJacobian):
        def __init__(self, M, grid=None):
            super().__init__(M, grid)
            self.M = self.M.to(cuda)

    xs = []
    for dev, Jw in (("cpu", L.DenseJacobian(J)), (cuda, CudaJ(J))):
        r = torch.as_tensor(rhs, device=dev)
        xs.append((linsolver.bicgstab(Jw, r, 1e-8, 15, 0.1, 0.2).cpu(),
                   linsolver.lsqr(Jw, r, 0.3, 1e-10, 1e-10, iter_lim=8).cpu()))
    torch.testing.assert_close(xs[0][0], xs[1][0], rtol=1e-9, atol=1e-11)
    torch.testing.assert_close(xs[0][1], xs[1][1], rtol=1e-9, atol=1e-11)
    n = 17
    Jp = L._screened(n, np.random.default_rng(2))
    b = np.random.default_rng(3).standard_normal(n * n)
    args = argparse.Namespace(linsolver_tol=1e-10, linsolver_maxiter=60,
                              nlvl=None, restriction="full", omega=0.6,
                              ndirect=3, smooth_pre=2, smooth_post=2,
                              beta=0.0, betadiag=0.0)
    x = linsolver.solve(CudaJ(Jp, (n, n)), torch.as_tensor(b, device=cuda),
                        args, {}, "multigrid")
    np.testing.assert_allclose(x.cpu().numpy(), np.linalg.solve(Jp, b),
                               rtol=1e-8, atol=1e-9)


@pytest.mark.gpu
def test_roll_compiled_matches_torch_path(cuda):
    """The compiled form of an operator that rolls traced expressions (the
    wrapped index and array reads of the generated code) against the
    op-by-op torch path."""
    from odil_gb300.domain import State
    from odil_gb300.problem import Problem
    dom = _dom((9, 7), ("x", "y"), cuda, ["u"])
    pj, pt = Problem(_op_roll, dom), Problem(_op_roll, dom, jit=False)
    assert pj.jit is not None
    st = State(fields={"u": torch.as_tensor(np.random.default_rng(4).uniform(
        -1, 1, dom.shape), device=cuda)})
    assert _rel(pj.eval_operator(st)[0], pt.eval_operator(st)[0]) < 1e-12
    lj, gj, _, _ = pj.eval_loss_grad(st)
    lt, gt, _, _ = pt.eval_loss_grad(st)
    assert abs(lj.item() - lt.item()) <= 1e-12 * lt.item()
    assert _rel(gj["u"], gt["u"]) < 1e-11


@pytest.mark.gpu
def test_ns_compiled_matches_torch_path(cuda):
    """The NS cavity operator's generic form, compiled, against its
    op-by-op torch path: residual, loss and gradient of all three fields."""
    from odil_gb300.domain import Domain, State
    from odil_gb300.ns import NsCavityOperator
    from odil_gb300.problem import Problem
    n = 16
    op = NsCavityOperator(400.0, kreg=1e-3)
    dom = Domain(ndim=2, shape=(n, n), lower=(0, 0), upper=(1, 1),
                 varnames=("x", "y"), fieldnames=["u", "v", "p"],
                 device=cuda)
    generic = lambda mod, ctx: op(mod, ctx)  # noqa: E731
    pj, pt = Problem(generic, dom), Problem(generic, dom, jit=False)
    assert pj.jit is not None
    rng = np.random.default_rng(6)
    st = State(fields={k: torch.as_tensor(rng.uniform(-1, 1, (n, n)),
                                          device=cuda) for k in "uvp"})
    for a, b in zip(pj.eval_operator(st), pt.eval_operator(st)):
        assert _rel(a, b) < 1e-11
    lj, gj, _, _ = pj.eval_loss_grad(st)
    lt, gt, _, _ = pt.eval_loss_grad(st)
    assert abs(lj.item() - lt.item()) <= 1e-11 * lt.item()
    for k in "uvp":
        assert _rel(gj[k], gt[k]) < 1e-10, k
