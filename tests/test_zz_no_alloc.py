"""The allocation-free fused loss entry point, called through the C ABI.

Collected near the end on purpose: it shares one device array across
calls, so a stop at the first failure has already run the other parity
tests (only the GPU runs of code also checked on the CPU come after it).  Callers that
cannot allocate device memory use this variant; it must agree with the
workspace-taking entry point on consecutive calls (the array keeps the
previous call's contents, which must not leak into the next result)."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _params(nt, nx, dev, seed):
    from odil_gb300 import _capi
    rng = np.random.default_rng(seed)
    bc = [torch.as_tensor(rng.standard_normal(n), dtype=torch.float32,
                          device=dev) for n in (nx, nx, nt, nt)]
    p = _capi.OdilWaveParams()
    p.nt, p.nx, p.dt, p.dx, p.c = nt, nx, 1.0 / nt, 2.0 / nx, 1.1
    p.init_u, p.init_ut, p.left_u, p.right_u = [t.data_ptr() for t in bc]
    return p, bc


@pytest.mark.parametrize("shape", [(64, 64), (1024, 1024), (300, 77)])
def test_noalloc_matches_workspace_entry_point(cuda, shape):
    from odil_gb300 import _capi
    lib = _capi.load()
    nt, nx = shape
    p, keep = _params(nt, nx, cuda, nt + nx)
    ws_bytes = lib.odil_wave_workspace_bytes(ctypes.byref(p))
    ws = torch.zeros(ws_bytes, dtype=torch.uint8, device=cuda)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(1)
    for call in range(2):  # two calls in a row on different inputs
        u = torch.as_tensor(rng.standard_normal(shape), dtype=torch.float32,
                            device=cuda)
        g_ref = torch.empty_like(u)
        g_na = torch.full_like(u, float("nan"))
        l_ref = torch.zeros(1, dtype=torch.float64, device=cuda)
        l_na = torch.full((1, ), float("nan"), dtype=torch.float64,
                          device=cuda)
        st = lib.odil_wave_loss_grad_f32(ctypes.byref(p), u.data_ptr(),
                                         g_ref.data_ptr(), l_ref.data_ptr(),
                                         ws.data_ptr(), ws_bytes, stream)
        assert st == 0
        st = lib.odil_wave_loss_grad_f32_noalloc(ctypes.byref(p), u.data_ptr(),
                                                 g_na.data_ptr(),
                                                 l_na.data_ptr(), stream)
        assert st == 0
        torch.cuda.synchronize()
        # Same kernel and reduction order: equal to FP32 test tolerance
        # (bitwise in practice).
        assert abs(l_na.item() - l_ref.item()) <= 1e-12 * abs(l_ref.item())
        assert torch.allclose(g_na, g_ref, rtol=1e-6, atol=0)


def test_noalloc_rejects_oversized_grids(cuda):
    from odil_gb300 import _capi
    lib = _capi.load()
    maxb = lib.odil_wave_loss_grad_noalloc_max_blocks()
    assert maxb > 10000
    nt, nx = 65536, 8192  # needs more reduction blocks than the limit
    p, keep = _params(nt, nx, cuda, 0)
    # Full-size buffers, so that the call would stay in bounds even if the
    # size check were missing.
    u = torch.zeros((nt, nx), dtype=torch.float32, device=cuda)
    g = torch.zeros_like(u)
    loss = torch.zeros(1, dtype=torch.float64, device=cuda)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.odil_wave_loss_grad_f32_noalloc(ctypes.byref(p), u.data_ptr(),
                                             g.data_ptr(), loss.data_ptr(),
                                             stream)
    torch.cuda.synchronize()
    assert st == -7  # ODIL_ERR_WORKSPACE, returned before any launch
    assert loss.item() == 0.0
