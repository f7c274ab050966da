"""CPU tests: the oracle's multigrid decomposition (oracle/multigrid.py)
reproduces the reference's MultigridDecomp outputs
(tests/golden/mgdecomp_ref.npz, made by tests/golden/make_golden.py from
the reference's own code with every interpolation method it defines)."""
import os

import numpy as np
import pytest

from oracle import multigrid as M

G = np.load(os.path.join(os.path.dirname(__file__), "golden",
                         "mgdecomp_ref.npz"))
NODE = ["5", "9", "5x9", "3x5x5"]
CELL = ["4", "6", "3x5", "2x3x4"]


@pytest.mark.parametrize("key", ["node_" + k for k in NODE] +
                         ["cell_" + k for k in CELL])
@pytest.mark.parametrize("depth", [1, 2])
def test_interp_matches_reference(key, depth):
    u = G[key + "_u"]
    r = M.interp_field(u, depth, cell=key.startswith("cell"))
    np.testing.assert_allclose(r, G["%s_d%d" % (key, depth)], rtol=0,
                               atol=1e-13)


@pytest.mark.parametrize("kind", ["node", "cell"])
def test_weights_to_field_matches_reference(kind):
    uw = G["w2f_%s_uw" % kind]
    nnw = [tuple(v) for v in G["w2f_%s_nnw" % kind]]
    factors = [1.0, 0.5, 2.0]
    cell = kind == "cell"
    np.testing.assert_allclose(
        M.weights_to_field(uw, nnw, factors, cell), G["w2f_%s_field" % kind],
        rtol=0, atol=1e-13)
    for i, f in enumerate(M.weights_to_fields(uw, nnw, factors, cell)):
        np.testing.assert_allclose(f, G["w2f_%s_fields%d" % (kind, i)],
                                   rtol=0, atol=1e-13)
    np.testing.assert_array_equal(M.weights_coarse_ones(nnw),
                                  G["w2f_%s_ones" % kind])


def test_interp_reproduces_linear_functions():
    """Both refinements are exact on linear functions (node: multilinear
    interpolation; cell: linear interpolation with linear extrapolation)."""
    x, y = np.meshgrid(np.arange(5.0), np.arange(4.0), indexing="ij")
    lin = 2 * x - 3 * y + 1
    xf, yf = np.meshgrid(np.arange(9) / 2, np.arange(7) / 2, indexing="ij")
    np.testing.assert_allclose(M.interp_node(lin), 2 * xf - 3 * yf + 1)
    xc, yc = np.meshgrid((np.arange(10) - 0.5) / 2, (np.arange(8) - 0.5) / 2,
                         indexing="ij")
    np.testing.assert_allclose(M.interp_cell(lin), 2 * xc - 3 * yc + 1,
                               atol=1e-13)
