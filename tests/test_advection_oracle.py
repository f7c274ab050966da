"""The advection oracle (oracle/advection.py) pinned to the reference.

* tests/golden/advection_ref.npz holds residuals computed by the
  reference's own `operator` function of advection_2d.py:103-223 (its body
  run on NumPy stand-ins for `mod` and the Context; make_golden.py,
  make_advection), so the restated residual is checked against the
  reference's code, not against itself;
* a cell-by-cell restatement of the upwind rule (advection_2d.py:129-138)
  and of the first time row (advection_2d.py:196-202) in plain loops;
* the discrete solution converges to the exact translated solution at
  first order, as the first-order upwind / backward-Euler scheme must.
"""
import os

import numpy as np
import pytest

from oracle import advection as A

G = np.load(os.path.join(os.path.dirname(__file__), "golden",
                         "advection_ref.npz"))
CASES = sorted({k.rsplit("_", 1)[0] for k in G.files if k.endswith("_fp")})


def _setup(name, vel=None):
    p = G[name + "_p"]
    nt, nx, ny = p.shape
    ax, ay = vel if vel is not None else (0.0, 0.0)
    s = A.AdvectSetup(nt, nx, ny, ax, ay, G[name + "_exact_pp"][0],
                      tmax=float(G[name + "_tmax"]))
    return s


def test_cases_present():
    assert len(CASES) == 7
    assert {"const_pp", "const_pm", "const_mp", "const_mm"} <= set(CASES)


@pytest.mark.parametrize("name", CASES)
def test_residual_matches_reference_operator(name):
    """fp, fu, fv of the oracle equal the reference operator's to rounding,
    with per-cell velocity fields of both signs and exact zeros."""
    s = _setup(name)
    f = A.residual_uvp(s, G[name + "_u"], G[name + "_v"], G[name + "_p"],
                       G[name + "_exact_uu"], G[name + "_exact_vv"])
    for got, key in zip(f, ("fp", "fu", "fv")):
        ref = G[name + "_" + key]
        np.testing.assert_allclose(got, ref, rtol=1e-13,
                                   atol=1e-13 * np.abs(ref).max())


@pytest.mark.parametrize("name", [c for c in CASES if c.startswith("const")])
def test_constant_velocity_residual_matches_reference(name):
    """residual_p (constant velocity, the form the GPU kernels implement)
    equals the reference operator's fp for each sign pair of (ax, ay), and
    the oracle's CSR Jacobian is its linear part."""
    u, v = G[name + "_u"], G[name + "_v"]
    s = _setup(name, (float(u.flat[0]), float(v.flat[0])))
    p = G[name + "_p"]
    ref = G[name + "_fp"]
    np.testing.assert_allclose(A.residual_p(s, p), ref, rtol=1e-13,
                               atol=1e-13 * np.abs(ref).max())
    jp = (A.jacobian(s) @ p.ravel()).reshape(p.shape)
    lin = ref - A.residual_p(s, np.zeros_like(p))
    np.testing.assert_allclose(jp, lin, rtol=1e-12,
                               atol=1e-12 * np.abs(lin).max())
    np.testing.assert_allclose(A.jv(s, p), lin, rtol=1e-12,
                               atol=1e-12 * np.abs(lin).max())


def _residual_loops(u, v, p, exact_pp, dt, dx, dy):
    """The direct problem's fp cell by cell: backward difference in t with
    the exact field as the value before row 0, and in x (y) the backward
    difference where the velocity is positive, else the forward one, with
    periodic neighbours."""
    nt, nx, ny = p.shape
    f = np.empty_like(p)
    for i in range(nt):
        for j in range(nx):
            for k in range(ny):
                prev = p[i - 1, j, k] if i > 0 else exact_pp[0, j, k]
                if u[i, j, k] > 0:
                    px = (p[i, j, k] - p[i, (j - 1) % nx, k]) / dx
                else:
                    px = (p[i, (j + 1) % nx, k] - p[i, j, k]) / dx
                if v[i, j, k] > 0:
                    py = (p[i, j, k] - p[i, j, (k - 1) % ny]) / dy
                else:
                    py = (p[i, j, (k + 1) % ny] - p[i, j, k]) / dy
                f[i, j, k] = ((p[i, j, k] - prev) / dt + u[i, j, k] * px +
                              v[i, j, k] * py)
    return f


@pytest.mark.parametrize("name", CASES)
def test_reference_operator_matches_cell_by_cell_rule(name):
    p = G[name + "_p"]
    nt, nx, ny = p.shape
    f = _residual_loops(G[name + "_u"], G[name + "_v"], p,
                        G[name + "_exact_pp"], float(G[name + "_tmax"]) / nt,
                        1.0 / nx, 1.0 / ny)
    np.testing.assert_allclose(f, G[name + "_fp"], rtol=1e-13,
                               atol=1e-13 * np.abs(f).max())


def _smooth_setup(n, ax=0.6, ay=-0.3):
    """p0 = sin(2 pi x) cos(2 pi y) advected by (ax, ay) on an n^3 grid;
    returns the setup and the exact solution at the cell centres."""
    from oracle.wave import cell_center_1d
    t1 = cell_center_1d(0.0, 1.0, n)
    x1 = cell_center_1d(0.0, 1.0, n)
    xx, yy = np.meshgrid(x1, x1, indexing="ij")

    def exact(t):
        return np.sin(2 * np.pi * (xx - ax * t)) * np.cos(
            2 * np.pi * (yy - ay * t))

    return (A.AdvectSetup(n, n, n, ax, ay, exact(t1[0])),
            np.stack([exact(t) for t in t1]))


def test_first_order_convergence_to_exact_solution():
    """Errors of the discrete solution against the exact translated
    solution of a smooth profile at 32^3, 64^3 and 128^3 fall by a factor
    that approaches 2 per refinement (first order in dt, dx, dy).  The
    benchmark's blobs (widths down to 0.05) are still pre-asymptotic at
    these sizes (factors 1.3-1.6), so the check uses a smooth field."""
    errs = []
    for n in (32, 64, 128):
        s, ex = _smooth_setup(n)
        p = A.solve(s)
        errs.append(np.linalg.norm(p - ex) / np.linalg.norm(ex))
        # the FFT solve is the discrete solution: its residual is zero
        assert np.abs(A.residual_p(s, p)).max() < 1e-9 * np.abs(
            A.residual_p(s, np.zeros_like(p))).max()
    r1, r2 = errs[0] / errs[1], errs[1] / errs[2]
    assert 1.6 < r1 < 2.1 and 1.75 < r2 < 2.1 and r2 > r1, errs


def test_newton_direct_equals_fft_solve():
    """The reference's method (normal equations + SuperLU MMD_ATA) and the
    FFT solve give the same discrete solution."""
    s = A.make_setup(8, seed=3)
    np.testing.assert_allclose(A.newton_direct(s, epochs=1), A.solve(s),
                               rtol=1e-10, atol=1e-12)
