"""ctypes binding of libodil_gb300.so (the C ABI declared in include/odil_gb300.h).

The library is the only compute path: if it is missing, every call raises.
Arguments are raw device pointers (``tensor.data_ptr()``), sizes and the
current torch stream handle; nothing here copies or allocates on its own.
"""
import ctypes
import os

import torch

from . import _build

ODIL_OK = 0
ODIL_ERR_SHAPE = -1
ODIL_ERR_ARG = -8
_STATUS = {
    -1: "ODIL_ERR_SHAPE",
    -2: "ODIL_ERR_DTYPE",
    -3: "ODIL_ERR_ALIGN",
    -4: "ODIL_ERR_LAUNCH",
    -5: "ODIL_ERR_TIMEOUT",
    -6: "ODIL_ERR_NONFINITE",
    -7: "ODIL_ERR_WORKSPACE",
    -8: "ODIL_ERR_ARG",
}


class OdilError(RuntimeError):
    """A libodil_gb300 entry point returned a negative status."""

    def __init__(self, fn, status, text):
        super().__init__("%s failed: %s (%d): %s" %
                         (fn, _STATUS.get(status, "?"), status, text))
        self.status = status


class OdilWaveParams(ctypes.Structure):
    _fields_ = [
        ("nt", ctypes.c_int64),
        ("nx", ctypes.c_int64),
        ("dt", ctypes.c_double),
        ("dx", ctypes.c_double),
        ("c", ctypes.c_double),
        ("init_u", ctypes.c_void_p),
        ("init_ut", ctypes.c_void_p),
        ("left_u", ctypes.c_void_p),
        ("right_u", ctypes.c_void_p),
    ]


class OdilAdvectParams(ctypes.Structure):
    _fields_ = [
        ("nt", ctypes.c_int64),
        ("nx", ctypes.c_int64),
        ("ny", ctypes.c_int64),
        ("dt", ctypes.c_double),
        ("dx", ctypes.c_double),
        ("dy", ctypes.c_double),
        ("ax", ctypes.c_double),
        ("ay", ctypes.c_double),
        ("p_init", ctypes.c_void_p),
    ]


class OdilWaveInstance(ctypes.Structure):
    _fields_ = [
        ("nt", ctypes.c_int64),
        ("nx", ctypes.c_int64),
        ("dt", ctypes.c_double),
        ("dx", ctypes.c_double),
        ("c", ctypes.c_double),
        ("offset", ctypes.c_int64),
        ("offset_x", ctypes.c_int64),
        ("offset_t", ctypes.c_int64),
        ("inv_dt", ctypes.c_double),
        ("inv_dx2", ctypes.c_double),
        ("c2", ctypes.c_double),
        ("dt2", ctypes.c_double),
        ("lam2", ctypes.c_double),
        ("a", ctypes.c_double),
        ("b", ctypes.c_double),
        ("half_dt", ctypes.c_double),
        ("ah", ctypes.c_float),
        ("al", ctypes.c_float),
        ("ch", ctypes.c_float),
        ("cl", ctypes.c_float),
        ("bh", ctypes.c_float),
        ("bl", ctypes.c_float),
    ]


class OdilWaveBatch(ctypes.Structure):
    _fields_ = [
        ("ninst", ctypes.c_int32),
        ("max_nx", ctypes.c_int32),
        ("total_cells", ctypes.c_int64),
        ("inst", ctypes.c_void_p),
        ("order", ctypes.c_void_p),
        ("init_u", ctypes.c_void_p),
        ("init_ut", ctypes.c_void_p),
        ("left_u", ctypes.c_void_p),
        ("right_u", ctypes.c_void_p),
        ("row_inst", ctypes.c_void_p),
        ("total_rows", ctypes.c_int64),
        ("bnd_off", ctypes.c_void_p),
        ("total_bnd", ctypes.c_int64),
    ]


class OdilNsParams(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64),
        ("re", ctypes.c_double),
        ("kreg", ctypes.c_double),
        ("mask", ctypes.c_void_p),
        ("u_imp", ctypes.c_void_p),
        ("v_imp", ctypes.c_void_p),
        ("imp_coeff", ctypes.c_double),
        ("pin", ctypes.c_int64),
        ("pin_weight", ctypes.c_double),
    ]


STENCIL_MAXS = 128


class OdilStencil(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("stride", ctypes.c_int32),
        ("periodic", ctypes.c_int32 * 3),
        ("nw", ctypes.c_int64 * 3),
        ("nshift", ctypes.c_int32),
        ("shifts", (ctypes.c_int32 * 3) * STENCIL_MAXS),
        ("coef", ctypes.c_void_p),
    ]


_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_D = ctypes.c_double
_INT = ctypes.c_int

# name -> (restype, argtypes)
SIGNATURES = {
    "odil_version": (_INT, []),
    "odil_status_string": (ctypes.c_char_p, [_INT]),
    "odil_wave_workspace_bytes": (_I64, [_P]),
    "odil_wave_residual_f32": (_INT, [_P, _P, _P, _P]),
    "odil_wave_residual_f64": (_INT, [_P, _P, _P, _P]),
    "odil_wave_loss_grad_f32": (_INT, [_P, _P, _P, _P, _P, _I64, _P]),
    "odil_wave_loss_grad_f64": (_INT, [_P, _P, _P, _P, _P, _I64, _P]),
    "odil_wave_loss_grad_noalloc_max_blocks": (_I64, []),
    "odil_wave_loss_grad_f32_noalloc": (_INT, [_P, _P, _P, _P, _P]),
    "odil_wave_jv_f32": (_INT, [_P, _P, _P, _P]),
    "odil_wave_jv_f64": (_INT, [_P, _P, _P, _P]),
    "odil_wave_jtv_f32": (_INT, [_P, _P, _P, _P]),
    "odil_wave_jtv_f64": (_INT, [_P, _P, _P, _P]),
    "odil_wave_jtj_workspace_bytes": (_I64, [_P]),
    "odil_wave_jtj_v_f32": (_INT, [_P, _P, _P, _P, _I64, _P]),
    "odil_wave_jtj_v_f64": (_INT, [_P, _P, _P, _P, _I64, _P]),
    "odil_wave_jtj_diag_f32": (_INT, [_P, _P, _P]),
    "odil_wave_jtj_diag_f64": (_INT, [_P, _P, _P]),
    "odil_wave_march_f32": (_INT, [_P, _P, _P, _P]),
    "odil_wave_march_f64": (_INT, [_P, _P, _P, _P]),
    "odil_wave_initial_rhs_mixed": (_INT, [_P, _P, _P]),
    "odil_wave_boundary_cells": (_I64, [_P]),
    "odil_wave_initial_table_mixed": (_INT, [_P, _P, _P]),
    "odil_wave_march_tiled_table_f32": (_INT, [_P, _P, _P]
                                        + [ctypes.c_int32] * 5 + [_P]),
    "odil_wave_march_shape_f32": (_INT, [_P, _P, _P, ctypes.c_int32,
                                         ctypes.c_int32, _P]),
    "odil_wave_march_tiled_f32": (_INT, [_P, _P, _P] + [ctypes.c_int32] * 5
                                  + [_P]),
    "odil_wave_march_tiled_f64": (_INT, [_P, _P, _P] + [ctypes.c_int32] * 5
                                  + [_P]),
    "odil_wave_march_tiled_planted_wait_f32": (_INT, [_P, _P, _P]
                                               + [ctypes.c_int32] * 5 + [_P]),
    "odil_wave_march_tiled_wait_failures": (_INT, [_P, ctypes.c_int32]),
    "odil_add_f32_to_f64": (_INT, [_P, _P, _P, _I64, _P]),
    "odil_pair_to_f64": (_INT, [_P, _P, _P, _I64, _P]),
    "odil_bicgstab_scalars": (_INT, [_P, _P, ctypes.c_int32, _P]),
    "odil_bicgstab_update_p": (_INT, [_P, _P, _P, _P, _I64, _P]),
    "odil_bicgstab_update_s": (_INT, [_P, _P, _P, _P, _I64, _P]),
    "odil_bicgstab_update_xr": (_INT, [_P, _P, _P, _P, _P, _P, _P, _I64,
                                       ctypes.c_int32, _P]),
    "odil_ns_direct_workspace_bytes": (_I64, [_I64]),
    "odil_ns_direct_factor": (_INT, [_I64, _P, _I64, _P, _I64, _P]),
    "odil_ns_direct_check": (_INT, [_I64, _P, _P]),
    "odil_ns_direct_solve": (_INT, [_I64, _P, _I64, _P, _I64, _P, _P, _P]),
    "odil_ns_direct_solve_t": (_INT, [_I64, _P, _I64, _P, _I64, _P, _P, _P]),
    "odil_dense_inverse_workspace_bytes": (_I64, [_I64]),
    "odil_dense_inverse_f64": (_INT, [_I64, _P, _P, _P, _I64, _P]),
    "odil_wave_pair_residual_mixed": (_INT, [_P, _P, _P, _P, _P]),
    "odil_wave_batch_initial_rhs_mixed": (_INT, [_P, _P, _P]),
    "odil_wave_batch_pair_residual_mixed": (_INT, [_P, _P, _P, _P, _P]),
    "odil_wave_update_residual_workspace_bytes": (_I64, [_P]),
    "odil_wave_update_residual_mixed": (_INT, [_P, _P, _P, _P, _P, _P, _P, _I64,
                                               _P]),
    "odil_wave_batch_setup": (_INT, [_P, ctypes.c_int32, _P]),
    "odil_wave_batch_workspace_bytes": (_I64, [_P]),
    "odil_wave_batch_update_residual_mixed": (_INT, [_P, _P, _P, _P, _P, _P]),
    "odil_wave_batch_march_f32": (_INT, [_P, _P, _P, ctypes.c_int32,
                                         ctypes.c_int32, ctypes.c_int32,
                                         ctypes.c_int32, _P, _I64, _P]),
    "odil_wave_batch_solve_mixed": (_INT, [_P, ctypes.c_int32, _P, _P, _P,
                                           _P] + [ctypes.c_int32] * 4 +
                                    [_P, _I64, _P]),
    "odil_nsmg_jx_f32": (_INT, [_I64, ctypes.c_int32, _P, _P, _P, _P]),
    "odil_nsmg_jx_f64": (_INT, [_I64, ctypes.c_int32, _P, _P, _P, _P]),
    "odil_nsmg_jtw_f32": (_INT, [_I64, ctypes.c_int32, _P, _P, _P, _P, _P, _P,
                                 ctypes.c_float, ctypes.c_int32, _P]),
    "odil_nsmg_jtw_f64": (_INT, [_I64, ctypes.c_int32, _P, _P, _P, _P]),
    "odil_nsmg_fine_ata": (_INT, [_I64, ctypes.c_int32, _P, _P, _P, _P]),
    "odil_nsmg_galerkin": (_INT, [_I64, _P, _P, _P, _P]),
    "odil_nsmg_smooth": (_INT, [_I64, _P, _P, _P, _P, _P, ctypes.c_float,
                                ctypes.c_int32, _P]),
    "odil_nsmg_jacobi0": (_INT, [_I64, _P, _P, _P, ctypes.c_float, _P]),
    "odil_nsmg_restrict": (_INT, [_I64, _P, _P, _P]),
    "odil_nsmg_prolong_add": (_INT, [_I64, _P, _P, _P]),
    "odil_nsmg_coarse_inverse": (_INT, [_I64, _P, _P, _P]),
    "odil_nsmg_coarse_apply": (_INT, [_I64, _P, _P, _P, _P]),
    "odil_pcg_scalars": (_INT, [_P, _P, ctypes.c_int32, _P]),
    "odil_pcg_update_xr": (_INT, [_I64, _P, _P, _P, _P, _P, _P]),
    "odil_pcg_update_p": (_INT, [_I64, _P, _P, _P, _P]),
    "odil_lbfgs_coef": (_INT, [ctypes.c_int32, ctypes.c_int32, _P, _P, _P, _P,
                               _P, _P, _P]),
    "odil_lbfgs_trial_f32": (_INT, [_I64, _P, _P, _P, _P, _P, _P, _P]),
    "odil_lbfgs_trial_f64": (_INT, [_I64, _P, _P, _P, _P, _P, _P, _P]),
    "odil_lbfgs_accept": (_INT, [_P, _P, _P, _P]),
    "odil_lbfgs_pair_f32": (_INT, [_I64, _P, _P, _P, _P, _P, _P]),
    "odil_lbfgs_pair_f64": (_INT, [_I64, _P, _P, _P, _P, _P, _P]),
    "odil_lbfgs_pair_dots_workspace_bytes": (_I64, [_I64]),
    "odil_lbfgs_pair_dots_f32": (_INT, [_I64, _P, _P, _P, _P, _P,
                                        ctypes.c_int32, _P, _P, _P, _I64,
                                        _P]),
    "odil_lbfgs_pair_dots_f64": (_INT, [_I64, _P, _P, _P, _P, _P,
                                        ctypes.c_int32, _P, _P, _P, _I64,
                                        _P]),
    "odil_lbfgs_update": (_INT, [_P, _P, _P, _P, _P, _P, ctypes.c_int32, _P,
                                 _P]),
    "odil_lbfgs_commit_f32": (_INT, [_I64, _P, _I64, _P, _P, _P, _P, _P, _P]),
    "odil_lbfgs_commit_f64": (_INT, [_I64, _P, _I64, _P, _P, _P, _P, _P, _P]),
    "odil_wave_batch_loss_grad_items": (_I64, [_I64, _I64]),
    "odil_wave_batch_loss_grad_f32": (_INT, [_P, _P, _P, _I64, _P, _P, _P, _P,
                                             _P, _P, _P, _P, _P, _P]),
    "odil_ns_num_equations": (_INT, [_P]),
    "odil_ns_residual_f32": (_INT, [_P, _P, _P, _P, _P, _P]),
    "odil_ns_residual_f64": (_INT, [_P, _P, _P, _P, _P, _P]),
    "odil_ns_jacobian_f32": (_INT, [_P, _P, _P, _P, _P, _P]),
    "odil_ns_jacobian_f64": (_INT, [_P, _P, _P, _P, _P, _P]),
    "odil_advect_workspace_bytes": (_I64, [_P]),
    "odil_advect_residual_f32": (_INT, [_P, _P, _P, _P]),
    "odil_advect_residual_f64": (_INT, [_P, _P, _P, _P]),
    "odil_advect_jv_f32": (_INT, [_P, _P, _P, _P]),
    "odil_advect_jv_f64": (_INT, [_P, _P, _P, _P]),
    "odil_advect_jtv_f32": (_INT, [_P, _P, _P, _P]),
    "odil_advect_jtv_f64": (_INT, [_P, _P, _P, _P]),
    "odil_advect_loss_grad_f32": (_INT, [_P, _P, _P, _P, _P, _I64, _P]),
    "odil_advect_loss_grad_f64": (_INT, [_P, _P, _P, _P, _P, _I64, _P]),
    "odil_advect_update_residual_mixed": (_INT, [_P, _P, _P, _P, _P, _P, _P,
                                                 _I64, _P]),
    "odil_advect_mg_jacobi": (_INT, [_P, _P, _P, _P, ctypes.c_float, _P, _P]),
    "odil_advect_mg_restrict": (_INT, [_I64, _I64, _I64, _P, _P, _P]),
    "odil_advect_mg_prolong_add": (_INT, [_I64, _I64, _I64, _P, _P, _P]),
    "odil_advect_dense": (_INT, [_P, _P, _P]),
    "odil_dense_apply_f64": (_INT, [_I64, _P, _P, _P, _P]),
    "odil_stencil_apply_f32": (_INT, [_P, _P, _P, _D, _D, _P]),
    "odil_stencil_apply_f64": (_INT, [_P, _P, _P, _D, _D, _P]),
    "odil_stencil_apply_t_f32": (_INT, [_P, _P, _P, _D, _D, _P]),
    "odil_stencil_apply_t_f64": (_INT, [_P, _P, _P, _D, _D, _P]),
    "odil_stencil_pair_workspace_bytes": (_I64, []),
    "odil_stencil_mul_transpose_op_f32": (_INT, [_P, _P, _P, _P, _I64, _P]),
    "odil_stencil_mul_transpose_op_f64": (_INT, [_P, _P, _P, _P, _I64, _P]),
    "odil_stencil_galerkin_f32": (_INT, [_P, _P, _P, _P, _P, _I64, _P]),
    "odil_stencil_galerkin_f64": (_INT, [_P, _P, _P, _P, _P, _I64, _P]),
    "odil_stencil_block_row_f32": (_INT, [_INT, _P, _P, _P, _P, _P, _P, _P, _D,
                                          _P]),
    "odil_stencil_block_row_f64": (_INT, [_INT, _P, _P, _P, _P, _P, _P, _P, _D,
                                          _P]),
    "odil_adam_step_f32": (_INT, [_P, _P, _P, _P, _I64, _D, _D, _D, _D, _P]),
    "odil_adam_step_f64": (_INT, [_P, _P, _P, _P, _I64, _D, _D, _D, _D, _P]),
    "odil_axpby_f32": (_INT, [_P, _P, _P, _I64, _D, _D, _P]),
    "odil_axpby_f64": (_INT, [_P, _P, _P, _I64, _D, _D, _P]),
    "odil_multidot_workspace_bytes": (_I64, [_I64, _INT, _INT]),
    "odil_multidot_f32": (_INT, [_P, _I64, _INT, _P, _INT, _I64, _P, _P, _I64,
                                 _P]),
    "odil_multidot_f64": (_INT, [_P, _I64, _INT, _P, _INT, _I64, _P, _P, _I64,
                                 _P]),
    "odil_lincomb_f32": (_INT, [_P, _P, _P, _I64, _INT, _P, _I64, _P]),
    "odil_lincomb_f64": (_INT, [_P, _P, _P, _I64, _INT, _P, _I64, _P]),
    "odil_lincomb_dot_workspace_bytes": (_I64, [_I64]),
    "odil_lincomb_dot_f32": (_INT, [_P, _P, _P, _I64, ctypes.c_int, _P, _I64,
                                    _P, _P, _I64, _P]),
    "odil_lincomb_dot_f64": (_INT, [_P, _P, _P, _I64, ctypes.c_int, _P, _I64,
                                    _P, _P, _I64, _P]),
    "odil_mgdecomp_refine_f32": (_INT, [ctypes.c_int32, _P, ctypes.c_int32, _P,
                                        _P, _D, _P, _D, _P]),
    "odil_mgdecomp_refine_f64": (_INT, [ctypes.c_int32, _P, ctypes.c_int32, _P,
                                        _P, _D, _P, _D, _P]),
    "odil_mgdecomp_refine_t_f32": (_INT, [ctypes.c_int32, _P, ctypes.c_int32,
                                          _P, _P, _P, _D, _P, _D, _P]),
    "odil_mgdecomp_refine_t_f64": (_INT, [ctypes.c_int32, _P, ctypes.c_int32,
                                          _P, _P, _P, _D, _P, _D, _P]),
}

_lib = None


def lib_path():
    return os.path.join(_build.LIBDIR, _build.LIBNAME)


def load():
    """Loads libodil_gb300.so once; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError(
            "libodil_gb300.so is not built (%s); run "
            "`python -c 'import __graft_entry__ as g; g.build()'` first. "
            "There is no CPU fallback." % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(SIGNATURES)


def stream_handle(device=None):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def call(name, *args):
    """Calls entry point `name`; raises OdilError on a negative status."""
    lib = load()
    st = getattr(lib, name)(*args)
    if st != ODIL_OK:
        text = lib.odil_status_string(st).decode()
        raise OdilError(name, st, text)
    return st


def ptr(t):
    """Device pointer of a CUDA tensor (None -> NULL)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor, got device %s" % t.device)
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return ctypes.c_void_p(t.data_ptr())
