"""The device arithmetic of the multigrid decomposition, run on the CPU.

odil_gb300/csrc/mgdecomp.cuh holds the per-point refinement, its adjoint and
the owned-point copy that the kernels of mgdecomp.cu call; it is plain C++,
so here g++ builds it with a loop over points in place of the grid.  The
refinement is compared with the oracle (pinned to the reference's own
MultigridDecomp outputs) and with the fixture itself, and the adjoint with
the transpose of the refinement matrix assembled from the oracle."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import multigrid as M

pytestmark = pytest.mark.skipif(shutil.which("g++") is None,
                                reason="g++ not available")

HERE = os.path.dirname(os.path.abspath(__file__))
HDR = os.path.join(HERE, "..", "odil_gb300", "csrc", "mgdecomp.cuh")
G = np.load(os.path.join(HERE, "golden", "mgdecomp_ref.npz"))

_DRIVER = r"""
#include "%s"
using namespace odil::mgd;
static Grid make(int dim, const int64_t* n, int cell) {
    Grid g; g.dim = dim; g.cell = cell;
    for (int d = 0; d < 3; ++d) { g.n[d] = d < dim ? n[d] : 1;
                                  g.m[d] = d < dim ? fine_size(n[d], cell) : 1; }
    return g;
}
template <typename T>
static void refine(int dim, const int64_t* n, int cell, const T* in, T* out) {
    Grid g = make(dim, n, cell);
    for (int64_t i = 0; i < g.m[0] * g.m[1] * g.m[2]; ++i) {
        int64_t o[3] = {0, 0, 0};
        unflatten(g.m, g.dim, i, o);
        out[i] = refine_point(g, in, o);
    }
}
template <typename T>
static void refine_t(int dim, const int64_t* n, int cell, const T* gf, T* gc,
                     T* wf, double beta) {
    Grid g = make(dim, n, cell);
    for (int64_t i = 0; i < g.n[0] * g.n[1] * g.n[2]; ++i) {
        int64_t q[3] = {0, 0, 0};
        unflatten(g.n, g.dim, i, q);
        gc[i] = refine_adjoint_point(g, gf, q);
        scale_owned(g, gf, wf, (T)beta, q);
    }
}
extern "C" void emu_refine_f64(int dim, const int64_t* n, int cell,
                               const double* in, double* out) {
    refine<double>(dim, n, cell, in, out);
}
extern "C" void emu_refine_f32(int dim, const int64_t* n, int cell,
                               const float* in, float* out) {
    refine<float>(dim, n, cell, in, out);
}
extern "C" void emu_refine_t_f64(int dim, const int64_t* n, int cell,
                                 const double* gf, double* gc, double* wf,
                                 double beta) {
    refine_t<double>(dim, n, cell, gf, gc, wf, beta);
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    d = tmp_path_factory.mktemp("mgd")
    src = os.path.join(str(d), "emu.cpp")
    so = os.path.join(str(d), "emu.so")
    with open(src, "w") as f:
        f.write(_DRIVER % os.path.abspath(HDR))
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", src,
                        "-o", so], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    L = ctypes.CDLL(so)
    for name in ("emu_refine_f64", "emu_refine_f32"):
        getattr(L, name).argtypes = [ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_void_p]
    L.emu_refine_t_f64.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                   ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_double]
    return L


def _n(shape):
    return np.array(shape, np.int64)


def _fine(shape, cell):
    return tuple(2 * v if cell else 2 * v - 1 for v in shape)


def refine(L, u, cell, dtype=np.float64):
    u = np.ascontiguousarray(u, dtype)
    out = np.zeros(_fine(u.shape, cell), dtype)
    n = _n(u.shape)
    fn = L.emu_refine_f64 if dtype == np.float64 else L.emu_refine_f32
    fn(u.ndim, n.ctypes.data, int(cell), u.ctypes.data, out.ctypes.data)
    return out


def refine_t(L, g, coarse, cell, beta=1.0):
    g = np.ascontiguousarray(g, np.float64)
    gc = np.zeros(coarse)
    wf = np.full(g.shape, np.nan)
    n = _n(coarse)
    L.emu_refine_t_f64(len(coarse), n.ctypes.data, int(cell), g.ctypes.data,
                       gc.ctypes.data, wf.ctypes.data, beta)
    return gc, wf


@pytest.mark.parametrize("key", ["node_5", "node_9", "node_5x9", "node_3x5x5",
                                 "cell_4", "cell_6", "cell_3x5",
                                 "cell_2x3x4"])
def test_refine_matches_reference(lib, key):
    cell = key.startswith("cell")
    u = G[key + "_u"]
    r1 = refine(lib, u, cell)
    np.testing.assert_allclose(r1, G[key + "_d1"], rtol=0, atol=1e-13)
    r2 = refine(lib, r1, cell)
    np.testing.assert_allclose(r2, G[key + "_d2"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(r1, M.interp_field(u, 1, cell), rtol=0,
                               atol=1e-14)
    r32 = refine(lib, u, cell, np.float32)
    np.testing.assert_allclose(r32, G[key + "_d1"], rtol=2e-6, atol=2e-6)


@pytest.mark.parametrize("shape,cell", [((5, ), False), ((2, ), True),
                                        ((3, ), True), ((6, ), True),
                                        ((4, 3), False), ((2, 3), True),
                                        ((3, 4), True), ((2, 2, 3), True),
                                        ((3, 2, 4), False), ((4, 3, 2), True)])
def test_adjoint_is_transpose(lib, shape, cell):
    """refine^T from the per-point adjoint equals the transpose of the
    refinement matrix (columns = oracle refinement of unit vectors),
    including the halo corners of small cell grids; the owned-point copy
    covers every fine point once."""
    n = int(np.prod(shape))
    P = np.stack([M.interp_field(np.eye(n)[k].reshape(shape), 1, cell)
                  .reshape(-1) for k in range(n)], axis=1)
    fine = _fine(shape, cell)
    g = np.random.default_rng(3).standard_normal(fine)
    gc, wf = refine_t(lib, g, shape, cell, beta=-1.5)
    np.testing.assert_allclose(gc.reshape(-1), P.T @ g.reshape(-1), rtol=0,
                               atol=1e-13)
    np.testing.assert_array_equal(wf, -1.5 * g)


@pytest.mark.parametrize("nw", [(9, ), (9, 9), (9, 9, 9)])
def test_node_refinement_is_interpolation_matrix(lib, nw):
    """test_multigrid.py:422-459: refining the coarse node field equals the
    interpolation matrix T of the CSR multigrid (Multigrid.get_T) applied
    to it, to 1e-14, in 1, 2 and 3 dimensions."""
    import torch
    from odil_gb300.multigrid import Multigrid
    nwh = tuple(n // 2 + 1 for n in nw)
    uh = np.sin(0.123 + np.linspace(0, 1, int(np.prod(nwh)))).reshape(nwh)
    T = Multigrid.get_T(nw, device="cpu")
    ub = (T @ torch.as_tensor(uh.reshape(-1))).numpy().reshape(nw)
    assert np.linalg.norm(refine(lib, uh, False) - ub) <= 1e-14
    assert np.linalg.norm(M.interp_node(uh) - ub) <= 1e-14
