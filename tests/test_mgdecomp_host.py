"""CPU tests of the multigrid decomposition's host side: argument checks of
odil_gb300.multigrid.MultigridDecomp and of the C-ABI entry points (which
return before any device work on invalid arguments)."""
import ctypes

import numpy as np
import pytest
import torch

from odil_gb300 import _capi
from odil_gb300.multigrid import MultigridDecomp as D


def test_cpu_tensor_is_refused():
    with pytest.raises(ValueError, match="CUDA"):
        D.interp_field(torch.zeros(5, dtype=torch.float64), 1)
    with pytest.raises(ValueError, match="CUDA"):
        D.weights_to_field(torch.zeros(9 + 5, dtype=torch.float64),
                           [(9, ), (5, )])


def test_method_checks_follow_the_reference():
    """multigrid.py:1254-1287: unknown methods raise NotImplementedError,
    'manual' covers 1-3 axes for nodes and 1-2 for cells."""
    u = torch.zeros((3, 3, 3), dtype=torch.float64)
    with pytest.raises(NotImplementedError, match="Unknown method"):
        D.interp_field(u, 1, method="spline")
    with pytest.raises(NotImplementedError):
        D.interp_cell_field(u, 1, method="manual")
    assert D.interp_field(u, 0) is u  # depth 0 returns the input


def test_level_chain_is_checked():
    uw = torch.zeros(9 * 9 + 4 * 4, dtype=torch.float64)
    with pytest.raises(ValueError, match="does not refine"):
        D.weights_to_field(uw, [(9, 9), (4, 4)])
    with pytest.raises(ValueError, match="does not refine"):
        D.weights_to_fields(uw, [(8, 8), (5, 5)], cell=True)
    with pytest.raises(NotImplementedError):
        D.weights_to_field(uw, [(3, 3, 3, 3)])


def test_capi_argument_checks(built_lib):
    lib = _capi.load()
    n = (ctypes.c_int64 * 3)(5, 1, 7)
    dummy = ctypes.c_void_p(16)  # never dereferenced: the checks come first
    f = lib.odil_mgdecomp_refine_f64
    assert f(0, n, 0, dummy, dummy, 1.0, None, 0.0, None) == _capi.ODIL_ERR_ARG
    assert f(4, n, 0, dummy, dummy, 1.0, None, 0.0, None) == _capi.ODIL_ERR_ARG
    assert f(2, n, 2, dummy, dummy, 1.0, None, 0.0, None) == _capi.ODIL_ERR_ARG
    # a cell axis of one cell cannot be extrapolated
    assert f(2, n, 1, dummy, dummy, 1.0, None, 0.0, None) == \
        _capi.ODIL_ERR_SHAPE
    assert f(1, n, 0, None, dummy, 1.0, None, 0.0, None) == _capi.ODIL_ERR_ARG
    ft = lib.odil_mgdecomp_refine_t_f32
    assert ft(1, n, 0, dummy, None, None, 0.0, None, 0.0, None) == \
        _capi.ODIL_ERR_ARG
    zero = (ctypes.c_int64 * 1)(0)
    assert ft(1, zero, 0, dummy, dummy, None, 0.0, None, 0.0, None) == \
        _capi.ODIL_ERR_SHAPE
    assert np.all(np.array(n[:]) == [5, 1, 7])
