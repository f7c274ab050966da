"""CPU tests: the oracle is pinned to the reference's own shipped outputs
before anything is compared against it."""
import json
import os

import numpy as np
import pytest

from oracle import wave as W
from oracle import autodiff as AD

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def test_wave_newton_error_table_matches_reference():
    """wave.py --optimizer newton, 2 epochs, error vs exact (ref_du_l2), for
    every grid in the reference's fd_newton/lines.pickle (N = Nt * Nx,
    Nt = Nx).  Tolerance: 1e-8 relative (normal-equation conditioning grows
    with N; the largest grids agree to ~2e-10)."""
    g = _load("wave_fd_newton.json")
    assert len(g["N"]) == 36
    for N, err in zip(g["N"], g["error"]):
        n = int(round(N**0.5))
        assert n * n == N
        s = W.make_setup(n, n, "cos")
        u = W.newton(s, epochs=2)
        e = W.l2_error(u, s.exact_u)
        assert abs(e - err) <= 1e-8 * err, (n, e, err)


def test_wave_march_equals_normal_equations():
    """Forward substitution = SuperLU normal-equation solve (linsolver.py:35-45)."""
    for n, prof, c in [(16, "cos", 1.0), (33, "sine", 1.0), (20, "sine", 0.8)]:
        s = W.make_setup(n, n + 3, prof, seed=5, nmodes=5, c=c)
        # Two epochs as the reference runs them (the second refines the
        # normal-equation solve, whose condition number is squared).
        un = W.newton(s, epochs=2)
        um = W.solve_march(s, rounds=1)
        assert W.rel_err(um, un) < 1e-12


def test_wave_residual_affine_and_jacobian():
    """const + J u == F(u) for the CSR of util_op.py:859-937, incl. degenerate
    nx = 1, 2 (aliasing of the rolled x-neighbours)."""
    rng = np.random.default_rng(0)
    shapes = [(7, 5), (4, 1), (5, 2), (3, 3), (1, 4), (2, 6)]
    for nt, nx in shapes:
        s = W.WaveSetup(nt, nx, rng.standard_normal(nx), rng.standard_normal(nx),
                        rng.standard_normal(nt), rng.standard_normal(nt), c=1.4)
        u = rng.standard_normal((nt, nx))
        const, J = W.linearize(s, u)
        f0 = W.residual(s, np.zeros((nt, nx)))
        lin = J.dot(u.ravel()).reshape(nt, nx) + f0
        assert np.abs(lin - const[0]).max() <= 1e-10 * (1 + np.abs(const[0]).max())


def test_wave_gradient_matches_autodiff():
    """Analytic (2/N) J^T f vs reverse-mode autodiff of the op-by-op operator
    (stand-in for the reference's tf.GradientTape), FP64."""
    rng = np.random.default_rng(1)
    for nt, nx in [(9, 7), (4, 1), (6, 2), (12, 12)]:
        s = W.WaveSetup(nt, nx, rng.standard_normal(nx), rng.standard_normal(nx),
                        rng.standard_normal(nt), rng.standard_normal(nt), c=0.8)
        u = rng.standard_normal((nt, nx))
        l1, g1 = W.loss_grad(s, u)
        l2, g2 = AD.wave_loss_grad_autodiff(s, u)
        assert abs(l1 - l2) <= 1e-12 * l2
        assert np.abs(g1 - g2).max() <= 1e-11 * np.abs(g2).max()


def test_sine_profile_exact_solution_properties():
    """Benchmark profile: zero Dirichlet values, u_t(x,0) = 0, d'Alembert."""
    s = W.make_setup(64, 64, "sine", seed=0, nmodes=5)
    assert np.abs(s.left_u).max() < 1e-12
    assert np.abs(s.right_u).max() < 1e-12
    assert np.abs(s.init_ut).max() < 1e-12
    u = W.solve_march(s)
    # Second-order scheme: error vs exact of the order of the discretisation.
    assert W.l2_error(u, s.exact_u) < 0.05


def test_lbfgsb_error_table_is_consistent():
    """fd_lbfgsb/lines.pickle: the L-BFGS-B errors approach the Newton
    (discrete-solution) errors; the oracle's Newton errors bound them below."""
    gn = _load("wave_fd_newton.json")
    gl = _load("wave_fd_lbfgsb.json")
    newton = dict(zip(gn["N"], gn["error"]))
    for N, e in zip(gl["N"], gl["error"]):
        if N in newton and N >= 256:
            assert e >= newton[N] * 0.95
            assert e <= newton[N] * 1.2


def test_ns_oracle_reference_solutions():
    """ns_steady.py restated: the reference's shipped FP64 Newton cavity
    solutions (N=128, Re=100 and 400) are roots of the restated operator to
    the level the reference converged them (rms residual ~1e-6 against
    terms of O(10)); a wrong operator leaves O(1e-1 .. 10) residuals."""
    from oracle import ns as NS
    gold = np.load(os.path.join(GOLDEN, "cavity_N128.npz"))
    for Re in (100, 400):
        st = {k: gold["Re%d_%s" % (Re, k)] for k in "uvp"}
        ff = NS.residual(NS.NsSetup(128, Re), st)
        for f in ff:
            assert np.sqrt(np.mean(f**2)) < 1e-5
        # Sensitivity: another Reynolds number is not a root.
        ff2 = NS.residual(NS.NsSetup(128, 2 * Re), st)
        assert max(np.sqrt(np.mean(f**2)) for f in ff2) > 1e-3


def test_ns_oracle_jacobian_is_affine():
    """const + J (w - w0) reproduces F(w) for the live part of the operator
    (the frozen copies held at w0), as the reference's linearize assumes."""
    from oracle import ns as NS
    import torch
    n = 10
    rng = np.random.default_rng(0)
    s = NS.NsSetup(n, 400, kreg=1e-4, pin=(3, 4), pin_weight=2.0)
    w0 = {k: rng.standard_normal((n, n)) for k in "uvp"}
    w1 = {k: w0[k] + rng.standard_normal((n, n)) for k in "uvp"}
    const, J = NS.linearize(s, w0)
    frozen = {k: torch.as_tensor(w0[k]) for k in "uvp"}
    live = NS._live_from(w1)
    with torch.no_grad():
        f1 = [f.numpy() for f in NS.operator(s, live, frozen)]
    dw = np.concatenate([(w1[k] - w0[k]).ravel() for k in "uvp"])
    lin = np.concatenate([c.ravel() for c in const]) + J @ dw
    assert np.allclose(lin, np.concatenate([f.ravel() for f in f1]),
                       atol=1e-9 * np.abs(lin).max())
