"""ctypes binding of the C ABI in include/xflow.h (libxflow.so, built in-tree).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libxflow.so")

XF_OK, XF_ERR_ARG, XF_ERR_CUDA, XF_ERR_MASK, XF_ERR_NOMEM, XF_ERR_STATE, XF_ERR_UNSUPPORTED = 0, 1, 2, 3, 4, 5, 6
XF_ERR_CHECK = 7
XF_STALL, XF_DIVERGED, XF_NAN, XF_MAXIT, XF_BREAKDOWN = 10, 11, 12, 13, 14
XF_F64, XF_F32 = 0, 1
XF_OP_LAPLACE, XF_OP_VARDIV, XF_OP_PACK, XF_OP_ADVDIFF = 0, 1, 2, 3
XF_ADV_CONVECTIVE, XF_ADV_DIFFUSIVE, XF_ADV_UPWIND = 1, 2, 4
XF_EXACT, XF_ZERO_INACTIVE = 1, 2
XF_CG, XF_CG_REFERENCE, XF_BICGSTAB, XF_MINRES, XF_BICG, XF_FCG = 0, 1, 2, 3, 4, 5
XF_PREC_FP64, XF_PREC_MIXED = 0, 1
XF_PRECOND_NONE, XF_PRECOND_JACOBI, XF_PRECOND_UNET, XF_PRECOND_CHEB, XF_PRECOND_UNET2 = 0, 1, 2, 3, 4
XF_IB_ELASTIC, XF_IB_TARGET, XF_IB_FIXED_ELASTIC, XF_IB_PLAIN, XF_IB_FIXED_STRETCHING = 0, 1, 2, 3, 4
XF_IB_POS, XF_IB_VEL, XF_IB_FORCE = 0, 1, 2

# Every symbol include/xflow.h declares (checked by tests/test_abi.py).
EXPORTS = [
    "xf_create", "xf_destroy", "xf_last_error", "xf_status_string", "xf_synchronize", "xf_stream",
    "xf_grid_create", "xf_grid_destroy", "xf_grid_end_index", "xf_grid_rn_map", "xf_grid_space_mask",
    "xf_grid_check", "xf_vec_create", "xf_vec_destroy", "xf_vec_upload", "xf_vec_download", "xf_vec_assign",
    "xf_vec_fill", "xf_vec_data", "xf_op_create", "xf_op_destroy", "xf_op_set_density", "xf_op_set_advection", "xf_op_set_diffusion_field", "xf_pack_create", "xf_op_transpose",
    "xf_pack_size", "xf_pack_download", "xf_matvec",
    "xf_lincomb", "xf_dot", "xf_norm", "xf_dot_op", "xf_absmax", "xf_solve_opts_default", "xf_solve",
    "xf_solve_host", "xf_pressure_rhs", "xf_velocity_correct", "xf_divergence_max", "xf_momentum_rhs", "xf_vtk_write", "xf_format_fixed6", "xf_npy_write", "xf_thomas_lines", "xf_ib_create", "xf_ib_destroy", "xf_ib_download", "xf_ib_upload",
    "xf_ib_interpolate", "xf_ib_update_position", "xf_ib_compute_forces", "xf_ib_spread",
    "xf_tc_gemm_bf16", "xf_conv3d_bf16", "xf_conv_status", "xf_unet_create", "xf_unet_destroy",
    "xf_unet_param_count", "xf_unet_set_params", "xf_unet_get_params", "xf_unet_get_grads", "xf_unet_apply",
    "xf_unet_train_step", "xf_solve_fcg", "xf_profile_cg_kernels", "xf_selftest_division", "xf_voxelize_mesh", "xf_cheb_factors_host", "xf_dot_noalloc", "xf_transfer_rhs", "xf_border_recalc", "xf_border_follow",
    "xf_conc_transfer", "xf_outflow_convective",
]


class SolveOpts(C.Structure):
    _fields_ = [("method", C.c_int), ("precision", C.c_int), ("precond", C.c_int), ("maxit", C.c_int),
                ("rtol", C.c_double), ("atol", C.c_double), ("replace_every", C.c_int),
                ("check_every", C.c_int), ("exact", C.c_int), ("reserved", C.c_int * 7)]


class SolveStats(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("replacements", C.c_int), ("fallbacks", C.c_int),
                ("rel_resid", C.c_double), ("abs_resid", C.c_double), ("ms", C.c_double),
                ("reserved", C.c_double * 4)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run `python -m xflow_gb300.build` (no CPU fallback exists)")
        L = C.CDLL(LIB_PATH)
        vp, i64p = C.c_void_p, C.POINTER(C.c_int64)
        L.xf_last_error.restype = C.c_char_p
        L.xf_last_error.argtypes = [vp]
        L.xf_status_string.restype = C.c_char_p
        L.xf_create.argtypes = [C.c_int, C.POINTER(vp)]
        L.xf_destroy.argtypes = [vp]
        L.xf_synchronize.argtypes = [vp]
        L.xf_stream.restype = vp
        L.xf_stream.argtypes = [vp]
        L.xf_grid_create.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp, C.POINTER(vp)]
        L.xf_grid_destroy.argtypes = [vp]
        L.xf_grid_end_index.argtypes = [vp, i64p]
        L.xf_grid_rn_map.argtypes = [vp, vp, vp]
        L.xf_grid_space_mask.argtypes = [vp, vp]
        L.xf_grid_check.argtypes = [vp, C.c_int, i64p]
        L.xf_vec_create.argtypes = [vp, C.c_int, C.POINTER(vp)]
        L.xf_vec_destroy.argtypes = [vp]
        L.xf_vec_upload.argtypes = [vp, vp]
        L.xf_vec_download.argtypes = [vp, vp]
        L.xf_vec_assign.argtypes = [vp, vp]
        L.xf_vec_fill.argtypes = [vp, C.c_double]
        L.xf_vec_data.restype = vp
        L.xf_vec_data.argtypes = [vp]
        L.xf_op_create.argtypes = [vp, C.c_int, C.POINTER(vp)]
        L.xf_op_destroy.argtypes = [vp]
        L.xf_op_set_density.argtypes = [vp, vp]
        L.xf_op_set_advection.argtypes = [vp, vp, vp, vp, C.c_double, C.c_double, C.c_int]
        L.xf_pack_create.argtypes = [vp, C.POINTER(vp)]
        L.xf_op_transpose.argtypes = [vp]
        L.xf_pack_size.argtypes = [vp, i64p, i64p, i64p]
        L.xf_pack_download.argtypes = [vp, C.c_int, vp, vp, vp]
        L.xf_matvec.argtypes = [vp, vp, vp, vp, C.c_int, C.c_int, vp, C.POINTER(C.c_double)]
        L.xf_lincomb.argtypes = [C.c_double, vp, C.c_double, vp, vp]
        L.xf_dot.argtypes = [vp, vp, C.POINTER(C.c_double)]
        L.xf_norm.argtypes = [vp, C.POINTER(C.c_double)]
        L.xf_dot_op.argtypes = [vp, vp, vp, C.POINTER(C.c_double)]
        L.xf_absmax.argtypes = [vp, C.POINTER(C.c_double), i64p]
        L.xf_solve_opts_default.argtypes = [C.POINTER(SolveOpts)]
        L.xf_solve.argtypes = [vp, C.POINTER(SolveOpts), vp, vp, C.POINTER(SolveStats)]
        L.xf_solve_host.argtypes = [vp, C.POINTER(SolveOpts), vp, vp, C.POINTER(SolveStats)]
        L.xf_transfer_rhs.argtypes = [vp, vp, C.c_double, vp]
        L.xf_border_recalc.argtypes = [vp, vp]
        L.xf_border_follow.argtypes = [vp, vp, C.c_int, C.c_int]
        L.xf_dot_noalloc.argtypes = [vp, vp, vp, C.c_int64, vp, vp]
        L.xf_profile_cg_kernels.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
        L.xf_selftest_division.argtypes = [vp, C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong)]
        L.xf_cheb_factors_host.argtypes = [C.c_double, C.c_double, C.c_int, C.POINTER(C.c_float)]
        L.xf_voxelize_mesh.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, C.c_longlong, vp, C.c_longlong,
                                       C.c_int32, vp]
        L.xf_tc_gemm_bf16.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp, C.c_int]
        L.xf_conv3d_bf16.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, C.c_int64, C.c_int, vp, vp, C.c_int, vp, vp,
                                     C.c_int64, C.c_int, C.c_int, C.c_int]
        L.xf_conv_status.argtypes = [vp]
        L.xf_unet_create.argtypes = [vp, C.POINTER(vp)]
        L.xf_unet_destroy.argtypes = [vp]
        L.xf_unet_param_count.argtypes = [vp, i64p]
        L.xf_unet_set_params.argtypes = [vp, vp]
        L.xf_unet_get_params.argtypes = [vp, vp]
        L.xf_unet_get_grads.argtypes = [vp, vp]
        L.xf_unet_apply.argtypes = [vp, vp, vp]
        L.xf_unet_train_step.argtypes = [vp, vp, vp, vp, C.c_double, C.c_int, C.POINTER(C.c_double)]
        L.xf_solve_fcg.argtypes = [vp, vp, C.POINTER(SolveOpts), vp, vp, C.POINTER(SolveStats)]
        L.xf_pressure_rhs.argtypes = [vp, vp, vp, vp, vp, C.c_double, vp, vp]
        L.xf_velocity_correct.argtypes = [C.c_int, vp, vp, vp, C.c_double, vp, vp]
        L.xf_divergence_max.argtypes = [vp, vp, vp, vp, C.POINTER(C.c_double), vp]
        L.xf_momentum_rhs.argtypes = [C.c_int] + [vp] * 11
        L.xf_conc_transfer.argtypes = [vp] * 9
        L.xf_outflow_convective.argtypes = [vp, vp, C.c_int, C.c_double, C.c_double]
        L.xf_vtk_write.argtypes = [C.c_char_p] + [vp] * 12
        L.xf_format_fixed6.argtypes = [vp, vp, C.c_int64, vp, C.c_int64, C.POINTER(C.c_int64)]
        L.xf_npy_write.argtypes = [C.c_char_p, vp]
        L.xf_op_set_diffusion_field.argtypes = [vp, vp]
        L.xf_thomas_lines.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int64, C.c_int64, C.c_int64,
                                      vp, vp, vp, vp, vp]
        L.xf_ib_create.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, vp, C.POINTER(vp)]
        L.xf_ib_destroy.argtypes = [vp]
        L.xf_ib_download.argtypes = [vp, C.c_int, vp]
        L.xf_ib_upload.argtypes = [vp, C.c_int, vp]
        L.xf_ib_interpolate.argtypes = [vp, vp, vp, C.c_int]
        L.xf_ib_update_position.argtypes = [vp, C.c_int, C.c_double]
        L.xf_ib_compute_forces.argtypes = [vp, C.c_int]
        L.xf_ib_spread.argtypes = [vp, vp, vp, C.c_int]
        _lib = L
    return _lib


class XFError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"xflow status {status}: {msg}")
        self.status = status


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None
