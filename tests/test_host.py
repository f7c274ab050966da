"""CPU tests of host-side logic: geometry, packing, checkpoints, argument
parsing, and loud failure without a GPU."""
import os
import pickle

import numpy as np
import pytest
import torch

from odil_gb300.domain import Domain, State
from oracle import wave as W


def test_domain_geometry_matches_reference_rules():
    d = Domain(ndim=2, shape=(8, 5), lower=(0, -1), upper=(1, 1),
               varnames=('t', 'x'), fieldnames=('u', ), device="cpu")
    assert d.step('t') == 1 / 8 and d.step('x') == 2 / 5
    assert np.allclose(d.cell_center_1d(1), W.cell_center_1d(-1, 1, 5))
    assert d.cell_center('x').shape == (8, 5)
    assert np.array_equal(d.cell_index('t')[:, 0], np.arange(8))
    assert d.size('x') == 5 and d.fields_size() == 40
    with pytest.raises(NotImplementedError):
        Domain(ndim=1, shape=(4, ), multigrid=True)


def test_pack_unpack_roundtrip():
    from odil_gb300.problem import Problem
    d = Domain(ndim=2, shape=(3, 4), varnames=('x', 'y'),
               fieldnames=('u', 'v'), device="cpu")

    class Op:
        def __call__(self, mod, ctx):
            return []

    p = Problem(Op(), d)
    st = State(fields={"u": torch.arange(12.).reshape(3, 4),
                       "v": -torch.arange(12.).reshape(3, 4)})
    packed = p.pack_state(st)
    assert packed.shape == (24, )
    back = p.unpack_state(packed)
    assert torch.equal(back.fields["v"], st.fields["v"])


def test_eval_refuses_cpu_tensors():
    from odil_gb300.problem import Problem
    d = Domain(ndim=1, shape=(4, ), varnames=('x', ), fieldnames=('u', ),
               device="cpu")
    p = Problem(lambda mod, ctx: [ctx.field('u')], d)
    with pytest.raises(RuntimeError, match="CUDA only"):
        p.eval_loss_grad(State(fields={"u": torch.zeros(4)}))


def test_checkpoint_layout_roundtrip(tmp_path):
    from odil_gb300.checkpoint import checkpoint_save, checkpoint_load
    st = State(fields={"u": torch.ones(2, 3), "p": torch.zeros(2, 3)})
    path = str(tmp_path / "state.pickle")
    checkpoint_save(st, path)
    with open(path, "rb") as f:
        raw = pickle.load(f)
    assert set(raw) == {"fields", "weights"}
    assert isinstance(raw["fields"]["u"], np.ndarray)
    st2 = State()
    checkpoint_load(st2, path, fields_to_load=["u"])
    assert list(st2.fields) == ["u"] and st2.fields["u"].sum() == 6
    with pytest.raises(RuntimeError):
        checkpoint_load(State(), path, fields_to_load=["w"],
                        skip_missing=False)


def test_corrupt_checkpoint_is_reported(tmp_path):
    """Failure injection on the host: a truncated checkpoint, a file that is
    not a pickle, and a pickle of the wrong layout raise ValueError naming
    the file; the state is left untouched."""
    from odil_gb300.checkpoint import checkpoint_save, checkpoint_load
    path = str(tmp_path / "state.pickle")
    checkpoint_save(State(fields={"u": torch.ones(64, 64)}), path)
    data = open(path, "rb").read()
    bad = []
    for i, blob in enumerate([data[:len(data) // 2], b"not a pickle",
                              pickle.dumps([1, 2, 3])]):
        q = str(tmp_path / ("bad%d.pickle" % i))
        with open(q, "wb") as f:
            f.write(blob)
        bad.append(q)
    for q in bad:
        st = State(fields={"u": torch.zeros(2)})
        with pytest.raises(ValueError, match="checkpoint"):
            checkpoint_load(st, q)
        assert list(st.fields) == ["u"] and float(st.fields["u"].sum()) == 0


def test_reference_cavity_pickle_loads(tmp_path):
    """The reference's checkpoint layout (fields u, v, p, psi) loads as a
    state; here from the committed fixture rewritten in that layout."""
    from odil_gb300.checkpoint import checkpoint_load
    g = np.load(os.path.join(os.path.dirname(__file__), "golden",
                             "cavity_N128.npz"))
    path = str(tmp_path / "cavity.pickle")
    with open(path, "wb") as f:
        pickle.dump({"fields": {k: g["Re400_" + k] for k in "uvp"},
                     "weights": {}}, f)
    st = State()
    checkpoint_load(st, path)
    assert st.fields["u"].shape == (128, 128)


def test_argparse_flags_match_reference_names():
    import argparse
    from odil_gb300 import util, linsolver
    ap = argparse.ArgumentParser()
    util.add_arguments(ap)
    linsolver.add_arguments(ap)
    a = ap.parse_args(["--optimizer", "lbfgsb", "--linsolver", "direct",
                       "--nlvl", "4", "--omega", "0.7", "--bfgs_m", "20",
                       "--precision", "mixed", "--epochs", "3"])
    assert a.optimizer == "lbfgsb" and a.nlvl == 4 and a.bfgs_m == 20
    assert a.smooth_pre == 2 and a.ndirect == 3 and a.restriction == "full"
    # the driver flags of util.py:109-239 parse with the reference defaults
    b = ap.parse_args(["--frames", "3", "--checkpoint", "s.pickle",
                       "--mg_interp", "roll", "--history_full", "2"])
    assert (b.frames, b.checkpoint, b.mg_interp, b.history_full) == \
        (3, "s.pickle", "roll", 2)
    assert (b.report_every, b.plot_every, b.checkpoint_every,
            b.history_every, b.every_factor, b.plotext, b.multigrid,
            b.nn_initializer) == (10, 5, 5, 1, 1, "pdf", 0, "legacy")
    # util.py:147-150, 168-171: seeded by default, single precision by default
    assert (b.seed, b.double, b.epoch_start, b.optimizer) == (0, 0, 0, "newton")


def test_unknown_names_raise_value_error():
    from odil_gb300.optimizer import make_optimizer
    from odil_gb300 import linsolver
    with pytest.raises(ValueError):
        make_optimizer("sgd")
    with pytest.raises(ValueError):
        linsolver.solve(None, torch.zeros(1), linsolver="nope")


def test_history_csv_rows_backfill_and_errors(tmp_path):
    """History (util_history.py:7-108): rows, zero back-fill of a late
    column, warm-up, the header fixed at the first write, pickle round trip."""
    from odil_gb300.history import History
    path = tmp_path / "train.csv"
    h = History(str(path), warmup=1)
    h.append("epoch", 0)
    h.append("loss", 1.5)
    h.write()  # count 1 <= warmup: nothing written yet
    assert path.read_text() == ""
    h.append("epoch", 1)
    h.append("loss", 0.25)
    h.write()
    assert path.read_text() == "epoch,loss\n0,1.5\n1,0.25\n"
    h.append("epoch", 2)
    h.append("loss", None)  # repeats the kind of the last value as zero
    h.write()
    assert path.read_text().splitlines()[-1] == "2,0.0"
    h.append("epoch", 3)
    h.append("loss", 0.125)
    h.append("err", 1e-3)  # new column: back-filled, but the header is fixed
    assert h.get("err") == [0.0, 0.0, 0.0, 1e-3]
    with pytest.raises(RuntimeError, match="'err' appeared after the CSV header"):
        h.write()
    h.close()
    h2 = History()
    h2.append("a", 1)
    h2.append("b", 2.0)
    h2.commit()
    h2.append("a", 2)
    with pytest.raises(RuntimeError, match="row 1 has no value for 'b'"):
        h2.commit()
    with pytest.raises(TypeError):
        h2.append("a", [1])
    pk = tmp_path / "hist.pickle"
    h3 = History()
    h3.append_dict({"x": 1, "y": 0.5})
    h3.commit()
    h3.save(str(pk))
    out = tmp_path / "re.csv"
    h4 = History(str(out))
    h4.load(str(pk))
    h4.close()
    assert out.read_text() == "x,y\n1,0.5\n"
    assert h4.count == 1 and h4.get("y") == [0.5]


@pytest.mark.parametrize("shape", [(12, 9), (1, 4), (3, 1), (7, 2)])
def test_stencil_to_csr_reference_layout(shape):
    """StencilOp.to_csr() with the oracle's per-shift coefficients gives the
    CSR matrix the reference assembles (util_op.py:877-896), exactly."""
    from odil_gb300.stencil import StencilOp
    from odil_gb300.wave import WaveKernels
    rng = np.random.default_rng(0)
    s = W.WaveSetup(*shape, rng.standard_normal(shape[1]),
                    rng.standard_normal(shape[1]), rng.standard_normal(shape[0]),
                    rng.standard_normal(shape[0]), c=1.3)
    co = W.slot_coefficients(s)
    coef = torch.as_tensor(np.stack([co[sh] for sh in WaveKernels.SLOT_SHIFTS]))
    J = StencilOp(WaveKernels.SLOT_SHIFTS, coef, shape).to_csr().to_dense()
    _, Jo = W.linearize(s, np.zeros(shape))
    assert np.array_equal(J.numpy(), Jo.toarray())


def _dense_of(op):
    """Dense matrix of a StencilOp from its definition: output cell i, input
    cell stride*i + dw, dropped outside the grid on non-periodic axes and
    wrapped on periodic ones."""
    import itertools
    nw, nwh = op.nw, op.nwh
    M = np.zeros((int(np.prod(nwh)), int(np.prod(nw))))
    coef = op.coef.double().cpu().numpy()
    for k, dw in enumerate(op.shifts):
        for i in itertools.product(*[range(n) for n in nwh]):
            j = []
            for a in range(len(nw)):
                v = op.stride * i[a] + dw[a]
                if op.periodic[a]:
                    v %= nw[a]
                elif not 0 <= v < nw[a]:
                    break
                j.append(v)
            else:
                M[np.ravel_multi_index(i, nwh),
                  np.ravel_multi_index(tuple(j), nw)] += coef[(k, ) + i]
    return M


@pytest.mark.parametrize("periodic", [(False, False), (True, False)])
def test_stencil_coefficient_algebra(periodic):
    """The SparseOperator algebra of multigrid.py:923-1216 on coefficient
    fields (torch ops, checked here on CPU tensors against dense matrices
    built from the operator definition)."""
    import torch
    from odil_gb300.stencil import StencilOp
    rng = np.random.default_rng(1)
    nw = (6, 5)
    sh_a = [(0, 0), (-1, 0), (1, 0), (0, 1), (1, -1)]
    sh_b = [(0, 0), (0, 1), (2, 0)]
    A = StencilOp(sh_a, torch.as_tensor(rng.standard_normal((5, ) + nw)), nw,
                  periodic=periodic)
    B = StencilOp(sh_b, torch.as_tensor(rng.standard_normal((3, ) + nw)), nw,
                  periodic=periodic)
    dA, dB = _dense_of(A), _dense_of(B)
    n = int(np.prod(nw))
    u = rng.standard_normal(nw)
    I = StencilOp.eye(nw, periodic=periodic, device="cpu")
    assert np.array_equal(_dense_of(I), np.eye(n))
    I2 = StencilOp.eye(nw, stride=2, device="cpu")
    assert np.array_equal(_dense_of(I2) @ u.ravel(), u[::2, ::2].ravel())
    c = torch.as_tensor(rng.standard_normal(nw))
    assert np.allclose(_dense_of(StencilOp.from_diag(c, nw)),
                       np.diag(c.numpy().ravel()))
    assert np.allclose(_dense_of(A.add_elementwise(B)), dA + dB)
    if not any(periodic):
        # Shifts that alias under the periodic wrap would merge entries.
        assert np.allclose(_dense_of(A.mul_elementwise(B)), dA * dB)
    assert A.mul_elementwise(B).shifts == [(0, 0), (0, 1)]
    # shift_left: the output shifted, (A' u)[i] = (A u)[i + s].
    for s in [(1, 0), (-1, 2), (0, -1)]:
        Au = (dA @ u.ravel()).reshape(nw)
        ref = StencilOp.apply_shift(torch.as_tensor(Au), s, periodic).numpy()
        got = (_dense_of(A.shift_left(s)) @ u.ravel()).reshape(nw)
        assert np.allclose(got, ref), s
    # shift_right: the input shifted, (A' u)[i] = sum c_dw[i] u[i + dw + s].
    for s in [(1, 0), (0, -2)]:
        Ar = A.shift_right(s)
        assert Ar.shifts == [(a + s[0], b + s[1]) for a, b in sh_a]
        assert torch.equal(Ar.coef, A.coef)
    # eliminate_zeros drops the all-zero shifts in place.
    coef = A.coef.clone()
    coef[2] = 0
    Z = StencilOp(sh_a, coef, nw, periodic=periodic).eliminate_zeros()
    assert Z.shifts == [s for k, s in enumerate(sh_a) if k != 2]
    assert np.allclose(_dense_of(Z), _dense_of(StencilOp(sh_a, coef, nw,
                                                         periodic=periodic)))
    with pytest.raises(NotImplementedError):
        A.mul_op(B)
    # apply_stride / apply_shift conventions (u[::s], u[i + dw]).
    ut = torch.as_tensor(u)
    assert torch.equal(StencilOp.apply_stride(ut, 2), ut[::2, ::2])
    sh = StencilOp.apply_shift(ut, (1, -1)).numpy()
    assert sh[0, 1] == u[1, 0] and sh[0, 0] == 0 and sh[-1, 2] == 0


def test_solve_regularized_host_logic(monkeypatch):
    """linsolver.solve_regularized (linsolver.py:35-41 relaxed normal
    equations) on CPU tensors through a small matrix-free Jacobian: the
    dense path and the conjugate-gradient path against numpy."""
    import argparse
    import torch
    from odil_gb300 import linsolver
    rng = np.random.default_rng(11)
    A = rng.standard_normal((30, 20)) + 3 * np.eye(30, 20)
    At = torch.as_tensor(A)

    class J:
        shape = A.shape

        def matvec(self, v):
            return At @ v

        def rmatvec(self, w):
            return At.T @ w

        def to_csr(self):
            return At.to_sparse_csr()

    b = rng.standard_normal(30)
    for beta, bd in ((0.0, 0.0), (0.5, 0.0), (0.0, 0.7), (0.4, 0.3)):
        M = A.T @ A + beta**2 * np.eye(20)
        M += bd**2 * np.diag(np.diag(M))
        ref = np.linalg.solve(M, A.T @ b)
        got = linsolver.solve_regularized(J(), torch.as_tensor(b), beta, bd)
        assert np.allclose(got.numpy(), ref, rtol=1e-10, atol=1e-12)
        monkeypatch.setattr(linsolver, "DENSE_MAX", 0)
        got = linsolver.solve_regularized(J(), torch.as_tensor(b), beta, bd,
                                          tol=1e-14)
        assert np.allclose(got.numpy(), ref, rtol=1e-8, atol=1e-10)
        monkeypatch.setattr(linsolver, "DENSE_MAX", 16384)
    args = argparse.Namespace(beta=0.5, betadiag=0.0)
    out = linsolver.solve(J(), torch.as_tensor(b), args, None, "direct")
    M = A.T @ A + 0.25 * np.eye(20)
    assert np.allclose(out.numpy(), np.linalg.solve(M, A.T @ b))


def test_util_op_helpers():
    """util_op.py:1017-1098 and util.py:46-106, 373-379 host helpers."""
    import io
    import torch
    from odil_gb300 import util
    from odil_gb300.domain import Domain, State
    from odil_gb300.problem import (extrap_linear, extrap_quad, extrap_quadh,
                                    latin_hypercube)
    # Extrapolations are exact on polynomials of their degree.
    assert extrap_linear(1.0, 3.0) == 5.0
    assert extrap_quad(1.0, 4.0, 9.0) == 16.0            # x^2 at 1, 2, 3 -> 4
    f = lambda x: 2 * x * x - x + 1  # noqa: E731
    assert abs(extrap_quadh(f(0), f(1), f(1.5)) - f(2)) < 1e-12
    # Latin hypercube: one point per stratum on every axis.
    rng = np.random.default_rng(0)
    pts = latin_hypercube(3, 50, rng)
    assert pts.shape == (50, 3) and pts.min() >= 0 and pts.max() < 1
    for j in range(3):
        assert sorted(np.floor(pts[:, j] * 50).astype(int)) == list(range(50))
    np.random.seed(1)
    a = latin_hypercube(2, 10)
    np.random.seed(1)
    assert np.array_equal(a, latin_hypercube(2, 10))
    dom = Domain(ndim=2, shape=(8, 6), lower=(0, -1), upper=(2, 1),
                 varnames=("x", "y"), fieldnames=["u"], device="cpu")
    xs, ys = dom.random_inner(20, rng)
    assert xs.min() >= 0 and xs.max() <= 2 and ys.min() >= -1 and ys.max() <= 1
    bx, by = dom.random_boundary(1, 1, 7, rng)
    assert np.all(by == 1) and bx.min() >= 0 and bx.max() <= 2
    assert np.allclose(dom.cell_node_by_name("y"), np.linspace(-1, 1, 7))
    assert dom.cell_node_by_name("z") is None
    assert float(dom.custom_by_name("ones").sum()) == 48
    assert dom.custom_by_name("other") is None
    st = State(fields={"u": torch.zeros(8, 6, dtype=torch.float64)})
    dom.add_field_to_state(torch.ones(8, 6, dtype=torch.float64), "u", st)
    assert float(dom.state_to_field("u", st).sum()) == 48
    # util: error norms, logging, memory.
    e1, e2, ei = util.get_error(np.array([1.0, 2.0]), np.array([1.0, 4.0]))
    assert (e1, ei) == (1.0, 2.0) and abs(e2 - 2**0.5) < 1e-15
    buf = io.StringIO()
    util.set_log_file(buf)
    util.printlog("a", 1)
    util.TIMECLEAR()
    util.TIME()
    util.set_log_file(__import__("sys").stderr)
    lines = buf.getvalue().splitlines()
    assert lines[0] == "a 1" and lines[1].startswith("test_host.py:")
    assert util.get_memory_usage_kb() > 0


def test_operator_laplace_is_traced():
    """The reference's sample operator (util_op.py:1038-1079) traces into
    the stencil compiler: three terms, the zero term constant."""
    from odil_gb300 import jit
    from odil_gb300.domain import Domain
    from odil_gb300.problem import operator_laplace
    dom = Domain(ndim=2, shape=(10, 12), lower=(0, 0), upper=(1, 1),
                 varnames=("x", "y"), fieldnames=["u", "v"], device="cpu")
    g, terms = jit.trace(operator_laplace, dom)
    assert len(terms) == 3 and terms[2].op == "const"
    assert {n for n, _ in jit.reads(terms[0])} == {"u"}
    assert len(jit.reads(terms[1])) == 5


def test_minimal_domain_pickles():
    """Domain.get_minimal (util_op.py:112-113, util_min.py:5-28)."""
    import pickle
    from odil_gb300.domain import Domain
    dom = Domain(ndim=2, shape=(8, 6), lower=(0, -1), upper=(2, 1),
                 varnames=("x", "y"), fieldnames=["u"], device="cpu")
    m = pickle.loads(pickle.dumps(dom.get_minimal()))
    assert m.shape == (8, 6) and m.step_by_dim(1) == dom.step(1)
    x, y = m.cell_center_all()
    assert np.allclose(x[:, 0], dom.cell_center_1d(0))
    assert np.allclose(y[0], dom.cell_center_1d(1))


def test_batch_instances_stay_below_the_stability_limit():
    """Batch instances keep the Courant number c dt / dx <= 0.9 (high wave
    speeds get a refined time grid): the wave operator's boundary closure
    makes forward substitution unstable above ~0.93, where the FP64
    oracle's own march grows without bound.  With it, the oracle solution of
    every instance is finite and close to the exact one."""
    from odil_gb300.workloads import wave_batch_instances
    from oracle import wave as W
    insts = wave_batch_instances(count=48, seed=7, nmin=24, nmax=96)
    assert any(i["nt"] != i["nx"] for i in insts)  # some were refined
    for i in insts:
        assert i["c"] * i["dt"] / i["dx"] <= 0.9 + 1e-12
        s = W.WaveSetup(i["nt"], i["nx"], i["init_u"], i["init_ut"],
                        i["left_u"], i["right_u"], c=i["c"])
        u = W.solve_march(s, rounds=1)
        assert np.isfinite(u).all()
        assert W.rel_err(u, i["exact_u"]) < 0.05, (i["nt"], i["nx"], i["c"])
