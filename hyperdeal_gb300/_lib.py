"""ctypes binding of the C ABI in include/hyperdeal_gb300.h.

The shared library is built in-tree (hyperdeal_gb300/build.py).  There is no
fallback: if the library cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

MAX_DIM = 6
HD_OK, HD_ERR_INVALID, HD_ERR_UNSUPPORTED, HD_ERR_CUDA, HD_ERR_ALLOC, HD_ERR_DEVICE = range(6)
HD_F64, HD_F32 = 0, 1
HD_BC_HOMOGENEOUS, HD_BC_FUNCTION = 0, 1
HD_QUAD_GAUSS_LOBATTO, HD_QUAD_GAUSS = 0, 1

#: every symbol the C header declares
EXPORTED_SYMBOLS = (
    "hd_last_error", "hd_version", "hd_adv_create", "hd_adv_destroy", "hd_adv_n_dofs", "hd_adv_apply",
    "hd_adv_critical_time_step", "hd_interpolate", "hd_norm_and_error", "hd_lsrk_create", "hd_lsrk_destroy",
    "hd_lsrk_n_stages", "hd_lsrk_step", "hd_lsrk_step_unfused", "hd_lsrk_stage_update", "hd_lsrk_coefficients",
    "hd_adv_set_kernel", "hd_adv_kernel", "hd_adv_device_status", "hd_norm_and_error_noalloc",
    "hd_vp_create", "hd_vp_destroy", "hd_vp_n_dofs", "hd_vp_n_dofs_x", "hd_vp_interpolate", "hd_vp_solve_field",
    "hd_vp_apply", "hd_vp_lsrk_step", "hd_vp_diagnostics", "hd_vp_fields", "hd_vp_cg_stats", "hd_vp_set_guess",
    "hd_vp_learn_loss_grad", "hd_adv_set_tile", "hd_adv_tile_limits",
    "hd_batch_create", "hd_batch_destroy", "hd_batch_n_classes", "hd_batch_class_info", "hd_batch_set_tile",
    "hd_batch_apply", "hd_batch_lsrk_step", "hd_batch_graph_capture", "hd_batch_graph_launch", "hd_batch_autotune",
    "hd_adv_autotune", "hd_vp_lsrk_step_fused", "hd_adv_set_arithmetic", "hd_adv_arithmetic",
    "hd_batch_class_arithmetic", "hd_vp_set_arithmetic", "hd_vp_set_kernel", "hd_vp_kernel", "hd_vp_device_status",
    "hd_vp_set_wait_test",
    "hd_part_layout_get", "hd_adv_create_part", "hd_adv_part_layout", "hd_adv_pack_faces", "hd_adv_apply_cells",
    "hd_lsrk_stage", "hd_lsrk_stage_input", "hd_adv_set_wait_test",
)
HD_KERNEL_AUTO, HD_KERNEL_GENERIC, HD_KERNEL_PIPELINED = 0, 1, 2
HD_ARITH_NATIVE, HD_ARITH_FP32X2 = 0, 1
HD_VP_GUESS_ZERO, HD_VP_GUESS_PREVIOUS, HD_VP_GUESS_LEARNED = 0, 1, 2
HD_CELLS_ALL, HD_CELLS_INTERIOR, HD_CELLS_BOUNDARY = 0, 1, 2
HD_VP_PRECOND_NONE, HD_VP_PRECOND_BLOCK_JACOBI = 0, 1
HD_VP_SOLVER_CG, HD_VP_SOLVER_DIRECT = 0, 1
HD_VP_FIT_LEAST_SQUARES, HD_VP_FIT_ADAM = 0, 1


class HdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("hyperdeal_gb300 error %d: %s" % (code, msg))
        self.code = code


class hd_function(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("amp", ctypes.c_double),
                ("omega", ctypes.c_double * MAX_DIM), ("speed", ctypes.c_double * MAX_DIM),
                ("phase", ctypes.c_double * MAX_DIM), ("cosine", ctypes.c_int * MAX_DIM)]


class hd_adv_desc(ctypes.Structure):
    _fields_ = [("dim_x", ctypes.c_int), ("dim_v", ctypes.c_int), ("degree", ctypes.c_int),
                ("n_points", ctypes.c_int), ("dtype", ctypes.c_int),
                ("cells_x", ctypes.c_int * 3), ("cells_v", ctypes.c_int * 3),
                ("lo_x", ctypes.c_double * 3), ("hi_x", ctypes.c_double * 3),
                ("lo_v", ctypes.c_double * 3), ("hi_v", ctypes.c_double * 3),
                ("periodic_x", ctypes.c_int), ("periodic_v", ctypes.c_int),
                ("velocity", ctypes.c_double * MAX_DIM), ("skew", ctypes.c_double),
                ("bc_kind", ctypes.c_int), ("bc", hd_function), ("quadrature", ctypes.c_int)]


class hd_vp_desc(ctypes.Structure):
    _fields_ = [("dim_x", ctypes.c_int), ("dim_v", ctypes.c_int), ("degree", ctypes.c_int), ("dtype", ctypes.c_int),
                ("cells_x", ctypes.c_int * 3), ("cells_v", ctypes.c_int * 3),
                ("lo_x", ctypes.c_double * 3), ("hi_x", ctypes.c_double * 3),
                ("lo_v", ctypes.c_double * 3), ("hi_v", ctypes.c_double * 3),
                ("cg_tol", ctypes.c_double), ("cg_max_iter", ctypes.c_int), ("guess", ctypes.c_int),
                ("learn_rank", ctypes.c_int), ("learn_history", ctypes.c_int), ("cg_rhs_relative", ctypes.c_int),
                ("learn_every", ctypes.c_int), ("cg_precond", ctypes.c_int), ("learn_fit", ctypes.c_int),
                ("quadrature", ctypes.c_int), ("poisson_solver", ctypes.c_int)]


class hd_part_layout(ctypes.Structure):
    _fields_ = [("first_cell", ctypes.c_longlong), ("n_cells", ctypes.c_longlong),
                ("layer_cells", ctypes.c_longlong), ("face_values", ctypes.c_longlong),
                ("ghost_values", ctypes.c_longlong), ("recv_from", ctypes.c_int), ("send_to", ctypes.c_int),
                ("send_first_cell", ctypes.c_longlong), ("send_slab", ctypes.c_int),
                ("boundary_first", ctypes.c_longlong), ("boundary_cells", ctypes.c_longlong)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


_lib = None


def lib_path() -> str:
    """The library this process loads: the in-tree build, or its bounds-checked variant when the
    environment sets HYPERDEAL_GB300_CHECK=1 (hyperdeal_gb300/build.py --check)."""
    return _build.CHECK_LIB_PATH if os.environ.get("HYPERDEAL_GB300_CHECK") == "1" else _build.LIB_PATH


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load the CUDA library (building it first when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise HdError(HD_ERR_UNSUPPORTED, "CUDA library %s is not built" % path)
        _build.build(check=path == _build.CHECK_LIB_PATH)
    L = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    L.hd_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.hd_version.restype = ctypes.c_char_p
    L.hd_adv_create.argtypes = [ctypes.POINTER(hd_adv_desc), ctypes.POINTER(vp)]
    L.hd_adv_destroy.argtypes = [vp]
    L.hd_adv_n_dofs.argtypes = [vp]
    L.hd_adv_n_dofs.restype = ctypes.c_longlong
    L.hd_adv_apply.argtypes = [vp, vp, vp, ctypes.c_double, vp]
    L.hd_adv_set_kernel.argtypes = [vp, ctypes.c_int]
    L.hd_adv_kernel.argtypes = [vp]
    L.hd_adv_set_arithmetic.argtypes = [vp, ctypes.c_int]
    L.hd_adv_arithmetic.argtypes = [vp]
    L.hd_adv_device_status.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    L.hd_adv_set_tile.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.hd_adv_autotune.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                  dp, vp]
    L.hd_adv_tile_limits.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.hd_adv_critical_time_step.argtypes = [vp]
    L.hd_adv_critical_time_step.restype = ctypes.c_double
    L.hd_interpolate.argtypes = [vp, ctypes.POINTER(hd_function), ctypes.c_double, vp, vp]
    L.hd_norm_and_error.argtypes = [vp, ctypes.POINTER(hd_function), ctypes.c_double, vp, dp, vp]
    L.hd_norm_and_error_noalloc.argtypes = [ctypes.POINTER(hd_adv_desc), ctypes.POINTER(hd_function),
                                            ctypes.c_double, vp, dp, vp]
    L.hd_lsrk_create.argtypes = [ctypes.c_char_p, ctypes.POINTER(vp)]
    L.hd_lsrk_destroy.argtypes = [vp]
    L.hd_lsrk_n_stages.argtypes = [vp]
    L.hd_lsrk_step.argtypes = [vp, vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp),
                               ctypes.c_double, ctypes.c_double, vp]
    L.hd_lsrk_step_unfused.argtypes = [vp, vp, vp, vp, vp, ctypes.c_double, ctypes.c_double, vp]
    L.hd_lsrk_stage_update.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.c_double, ctypes.c_double,
                                       vp, vp, vp, vp]
    L.hd_lsrk_coefficients.argtypes = [vp, dp, dp, dp]
    llp = ctypes.POINTER(ctypes.c_longlong)
    L.hd_vp_create.argtypes = [ctypes.POINTER(hd_vp_desc), ctypes.POINTER(vp)]
    L.hd_vp_destroy.argtypes = [vp]
    L.hd_vp_n_dofs.argtypes = [vp]
    L.hd_vp_n_dofs.restype = ctypes.c_longlong
    L.hd_vp_n_dofs_x.argtypes = [vp]
    L.hd_vp_n_dofs_x.restype = ctypes.c_longlong
    L.hd_vp_interpolate.argtypes = [vp, ctypes.POINTER(hd_function), ctypes.c_double, vp, vp]
    L.hd_vp_solve_field.argtypes = [vp, vp, vp]
    L.hd_vp_apply.argtypes = [vp, vp, vp, ctypes.c_double, vp]
    L.hd_vp_lsrk_step.argtypes = [vp, vp, vp, vp, vp, ctypes.c_double, ctypes.c_double, vp]
    L.hd_vp_lsrk_step_fused.argtypes = [vp, vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp),
                                        ctypes.c_double, ctypes.c_double, vp]
    L.hd_vp_diagnostics.argtypes = [vp, vp, dp, vp]
    L.hd_vp_fields.argtypes = [vp, vp, vp, vp, vp]
    L.hd_vp_cg_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_int), llp, llp, dp, llp]
    L.hd_vp_set_guess.argtypes = [vp, ctypes.c_int]
    L.hd_vp_set_arithmetic.argtypes = [vp, ctypes.c_int]
    L.hd_vp_set_kernel.argtypes = [vp, ctypes.c_int]
    L.hd_vp_kernel.argtypes = [vp]
    L.hd_vp_device_status.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    L.hd_vp_set_wait_test.argtypes = [vp, ctypes.c_uint, ctypes.c_int]
    L.hd_vp_learn_loss_grad.argtypes = [ctypes.c_longlong, ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp, vp, vp,
                                        vp]
    vpp = ctypes.POINTER(vp)
    ip = ctypes.POINTER(ctypes.c_int)
    L.hd_batch_create.argtypes = [vpp, ctypes.c_int, vp, vpp]
    L.hd_batch_destroy.argtypes = [vp]
    L.hd_batch_n_classes.argtypes = [vp]
    L.hd_batch_class_info.argtypes = [vp, ctypes.c_int, ip, ip, ip, ip, ip, ip, ip]
    L.hd_batch_class_arithmetic.argtypes = [vp, ctypes.c_int]
    L.hd_batch_set_tile.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.hd_batch_apply.argtypes = [vp, vpp, vpp, dp, vp]
    L.hd_batch_lsrk_step.argtypes = [vp, vpp, vpp, vpp, dp, dp, vp]
    L.hd_batch_graph_capture.argtypes = [vp, vpp, vpp, vpp, dp, dp]
    L.hd_batch_graph_launch.argtypes = [vp, vp]
    L.hd_batch_autotune.argtypes = [vp, vpp, vpp, ctypes.c_int, vp]
    L.hd_part_layout_get.argtypes = [ctypes.POINTER(hd_adv_desc), ctypes.c_int, ctypes.c_int,
                                     ctypes.POINTER(hd_part_layout)]
    L.hd_adv_create_part.argtypes = [ctypes.POINTER(hd_adv_desc), ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]
    L.hd_adv_part_layout.argtypes = [vp, ctypes.POINTER(hd_part_layout)]
    L.hd_adv_pack_faces.argtypes = [vp, vp, vp, vp]
    L.hd_adv_apply_cells.argtypes = [vp, vp, vp, ctypes.c_double, ctypes.c_int, vp]
    L.hd_lsrk_stage.argtypes = [vp, vp, ctypes.c_int, vpp, ctypes.c_double, ctypes.c_double, ctypes.c_int, vp]
    L.hd_lsrk_stage_input.argtypes = [vp, ctypes.c_int]
    L.hd_adv_set_wait_test.argtypes = [vp, ctypes.c_uint, ctypes.c_int]
    _lib = L
    return L


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    load().hd_last_error(buf, 1024)
    return buf.value.decode()


def check(rc: int) -> None:
    if rc != HD_OK:
        raise HdError(rc, last_error())
