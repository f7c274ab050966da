"""The stencil compiler's generated kernels, run on the CPU.

The CUDA source the compiler writes is turned into plain C++ (the CUDA
qualifiers become no-ops, blockIdx/threadIdx become loop variables), built
with g++ and run over every cell.  Residual, the two-pass gradient (pass-1
products, pass-2 gather) and the Jacobian coefficients are compared with the
op-by-op torch path and autograd on CPU tensors.  This checks the generated
indexing (periodic offsets, wrapped index and array leaves of rolled
expressions, broadcast strides) without a GPU; the per-block loss reduction,
which needs warp shuffles, is left to the GPU tests."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.skipif(shutil.which("g++") is None,
                                reason="g++ not available")

_EMU = r"""
#include <cmath>
#include <cstdint>
#include <algorithm>
using std::fmax; using std::fmin; using std::fabs; using std::sqrt;
struct EmuDim { unsigned x, y, z; };
static EmuDim blockIdx, threadIdx, blockDim, gridDim;
#define __device__
#define __forceinline__ inline
#define __global__
#define __launch_bounds__(n)
#define __shared__ static
static inline double __shfl_down_sync(unsigned, double, int) { return 0.0; }
static inline void __syncthreads() {}
"""

_DRIVER = r"""
extern "C" void emu_run(Args* a, long long ncell, int which) {
    const unsigned nb = (unsigned)((ncell + 255) / 256);
    blockDim = {256, 1, 1};
    gridDim = {nb, 1, 1};
    for (unsigned b = 0; b < nb; ++b) {
        for (unsigned t = 0; t < 256; ++t) {
            blockIdx = {b, 0, 0};
            threadIdx = {t, 0, 0};
            if (which == 0) residual_kernel(*a);
            else if (which == 1) contrib_kernel(*a);
            else if (which == 2) gather_kernel(*a);
            else jacobian_kernel(*a);
        }
    }
}
"""


def _emulate(J, tmp_path):
    code = J.code
    code = code[:code.index("static int launch_status()")]
    code = code.replace("#include <cuda_runtime.h>", _EMU)
    src = os.path.join(str(tmp_path), "emu.cpp")
    so = os.path.join(str(tmp_path), "emu.so")
    with open(src, "w") as f:
        f.write(code + _DRIVER)
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", src,
                        "-o", so], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    lib = ctypes.CDLL(so)
    lib.emu_run.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int]
    return lib


def _args(J, fields, keep):
    """Args over numpy buffers (kept alive in `keep`)."""
    g = J.graph
    a = J._Args()
    for i, name in enumerate(J.fields):
        arr = np.ascontiguousarray(fields[name], np.float64)
        keep.append(arr)
        a.f[i] = arr.ctypes.data
    shp = list(g.shape) + [1] * (3 - len(g.shape))
    for d in range(3):
        a.n[d] = shp[d]
    for i, (arr, _) in enumerate(g.ext):
        arr = np.ascontiguousarray(arr, np.float64)
        keep.append(arr)
        a.e[i] = arr.ctypes.data
        st, stride = [0, 0, 0], 1
        for d in reversed(range(len(g.shape))):
            if arr.shape[d] != 1:
                st[d] = stride
            stride *= arr.shape[d]
        for d in range(3):
            a.es[i][d] = st[d]
    n = int(np.prod(g.shape))
    for k in range(len(J.terms)):
        a.scale[k] = 2.0 / n
    a.epoch = 0
    return a, n


def _cases():
    from odil_gb300.domain import Domain
    from odil_gb300.ns import NsCavityOperator
    from odil_gb300.workloads import WaveInstance
    import test_jit as T
    out = []
    inst = WaveInstance(12, 10, profile="sine", seed=3, nmodes=3, c=0.9,
                        device="cpu")
    out.append(("wave", inst.domain, lambda m, c: inst.operator(m, c)))
    out.append(("nonlinear", T._nonlinear_domain("cpu"), T._nonlinear))
    out.append(("roll", T._dom((9, 7), ("x", "y"), "cpu", ["u"]), T._op_roll))
    out.append(("rank3", T._dom((4, 6, 5), ("t", "x", "y"), "cpu", ["p"]),
                T._op3d))
    rng = np.random.default_rng(5)
    n = 8
    ns = NsCavityOperator(400.0, mask=(rng.random((n, n)) < 0.3) * 1.0,
                          u_imp=rng.standard_normal((n, n)),
                          v_imp=rng.standard_normal((n, n)), kreg=1e-3,
                          pin=(2, 3))
    out.append(("ns", Domain(ndim=2, shape=(n, n), lower=(0, 0),
                             upper=(1, 1), varnames=("x", "y"),
                             fieldnames=["u", "v", "p"], device="cpu"),
                lambda m, c: ns(m, c)))
    return out


@pytest.mark.parametrize("case", ["wave", "nonlinear", "roll", "rank3", "ns"])
def test_generated_kernels_on_cpu(case, tmp_path):
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    from odil_gb300 import jit
    from odil_gb300.problem import Problem, StencilJacobian
    name, dom, op = [c for c in _cases() if c[0] == case][0]
    J = jit.JitOperator(op, dom)
    lib = _emulate(J, tmp_path)
    rng = np.random.default_rng(11)
    fields = {k: rng.uniform(-1, 1, dom.shape) for k in dom.fieldnames}
    pt = Problem(op, dom, jit=False)
    tf = {k: torch.as_tensor(v).requires_grad_(True)
          for k, v in fields.items()}
    ref = pt._generic(tf, 0)
    keep = []
    a, n = _args(J, fields, keep)
    # residual
    outs = [np.zeros(dom.shape) for _ in J.terms]
    for k, o in enumerate(outs):
        a.out[k] = o.ctypes.data
    lib.emu_run(ctypes.byref(a), n, 0)
    for o, r in zip(outs, ref):
        r = np.broadcast_to(torch.as_tensor(r).detach().numpy(), dom.shape)
        assert np.allclose(o, r, rtol=1e-12, atol=1e-12 * np.abs(r).max())
    # gradient: pass-1 products, pass-2 gather
    contrib = np.zeros((max(1, J.ncontrib), ) + tuple(dom.shape))
    grads = {k: np.zeros(dom.shape) for k in dom.fieldnames}
    partial = np.zeros(((n + 255) // 256, len(J.terms)))
    for q in range(J.ncontrib):
        a.contrib[q] = contrib[q].ctypes.data
    for i, k in enumerate(J.fields):
        a.grad[i] = grads[k].ctypes.data
    a.partial = partial.ctypes.data
    lib.emu_run(ctypes.byref(a), n, 1)
    lib.emu_run(ctypes.byref(a), n, 2)
    loss = sum(torch.mean(torch.as_tensor(r).reshape(-1).expand(n)**2)
               if torch.as_tensor(r).numel() == 1 else torch.mean(r**2)
               for r in ref)
    gt = torch.autograd.grad(loss, [tf[k] for k in J.fields],
                             allow_unused=True)
    for k, g in zip(J.fields, gt):
        g = np.zeros(dom.shape) if g is None else g.numpy()
        assert np.allclose(grads[k], g, rtol=1e-10,
                           atol=1e-10 * max(np.abs(g).max(), 1e-300)), k
    # Jacobian coefficients, assembled in the reference's CSR layout
    coef = np.zeros_like(contrib)
    for q in range(J.ncontrib):
        a.contrib[q] = coef[q].ctypes.data
    lib.emu_run(ctypes.byref(a), n, 3)
    blocks = {}
    q = 0
    for k, rd in enumerate(J.term_reads):
        for fname, sh in rd:
            blocks.setdefault((k, J.fields.index(fname)), []).append((q, sh))
            q += 1
    S = StencilJacobian(torch.as_tensor(coef), blocks, len(J.terms),
                        len(J.fields), dom.shape)
    D = S.to_csr().to_dense().numpy()
    packed = torch.cat([torch.as_tensor(fields[k]).reshape(-1)
                        for k in J.fields])

    def res(x):
        fs = {k: x[i * n:(i + 1) * n].reshape(dom.shape)
              for i, k in enumerate(J.fields)}
        return torch.cat([torch.as_tensor(r).expand(dom.shape).reshape(-1)
                          if torch.as_tensor(r).numel() == 1
                          else r.reshape(-1) for r in pt._generic(fs, 0)])

    Jref = torch.autograd.functional.jacobian(res, packed).numpy()
    assert np.allclose(D, Jref, rtol=1e-11, atol=1e-11 * np.abs(Jref).max())
