"""ctypes binding of libminiaero_gpu.so (declarations in include/miniaero_gpu.h).

The library is the product: there is no Python or CPU fallback. Loading fails
with an error when the shared library has not been built.
"""
import ctypes
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libminiaero_gpu.so")

MA_OK, MA_EINVAL, MA_ENOMEM, MA_ECUDA, MA_EBUDGET, MA_ETIMEDOUT, MA_ENUMERIC, MA_ESTATE, MA_EIO, MA_ENOTFOUND = range(10)
MA_BC_EXTRAPOLATE, MA_BC_TANGENT, MA_BC_INFLOW, MA_BC_NOSLIP = range(4)
MA_LIMITER_VENKAT, MA_LIMITER_VANALBADA = 0, 1
MA_VISC_SUTHERLAND, MA_VISC_CONSTANT = 0, 1
MA_PREC_FP64, MA_PREC_MIXED, MA_PREC_FP64_FMA = 0, 1, 2
MA_HOST_MESH_DEVICE_GEOMETRY = 1
MA_GATHER_ATOMICS, MA_GATHER_CELL_FLUX = 0, 1
MA_MESH_CELL_FLUX = 1
MA_LAYOUT_AOS, MA_LAYOUT_SOA = 0, 1
MA_IC_REFERENCE, MA_IC_SOD, MA_IC_CONSTANT = 0, 1, 2
MA_MAX_BC_SETS = 16
MA_PROFILE_KINDS = 4
KERNEL_KINDS = ("sweep_gradient_limiter", "internal_face_flux", "boundary_face_flux", "residual_rk_update")

c_int32 = ctypes.c_int32
c_double = ctypes.c_double
c_void_p = ctypes.c_void_p
P_i32 = ctypes.POINTER(ctypes.c_int32)
P_f64 = ctypes.POINTER(ctypes.c_double)


class ma_options(ctypes.Structure):
    _fields_ = [
        ("problem_type", c_int32),
        ("lx", c_double), ("ly", c_double), ("lz", c_double), ("angle", c_double),
        ("nx", c_int32), ("ny", c_int32), ("nz", c_int32),
        ("ntimesteps", c_int32),
        ("dt", c_double),
        ("output_results", c_int32),
        ("output_frequency", c_int32),
        ("second_order_space", c_int32),
        ("viscous", c_int32),
        ("limiter", c_int32),
        ("viscosity_model", c_int32),
        ("mu", c_double),
        ("prandtl", c_double),
        ("precision", c_int32),
        ("cfl", c_double),
        ("ic", c_int32),
        ("sod_left", c_double * 2),
        ("sod_right", c_double * 2),
        ("sod_split", c_double),
        ("inflow_given", c_int32),
        ("inflow_state", c_double * 5),
        ("bc_override", c_int32 * 6),
        ("keep_residual", c_int32),
        ("gather", c_int32),
    ]


class ma_face_set(ctypes.Structure):
    _fields_ = [
        ("nfaces", c_int32),
        ("type", c_int32),
        ("conn", P_i32),
        ("flux_index", P_i32),
        ("coords", P_f64),
        ("normal", P_f64),
        ("tangent", P_f64),
        ("binormal", P_f64),
        ("permutation", P_i32),
    ]


class ma_mesh_view(ctypes.Structure):
    _fields_ = [
        ("ncells", c_int32),
        ("cell_coords", P_f64),
        ("cell_volumes", P_f64),
        ("internal", ma_face_set),
        ("nbc", c_int32),
        ("bc", ma_face_set * MA_MAX_BC_SETS),
    ]


MA_PATH_MAX = 512


class ma_run_options(ctypes.Structure):
    _fields_ = [
        ("checkpoint_path", ctypes.c_char * MA_PATH_MAX),
        ("checkpoint_frequency", c_int32),
        ("restart_path", ctypes.c_char * MA_PATH_MAX),
    ]


class ma_checkpoint_info(ctypes.Structure):
    _fields_ = [
        ("ncells", ctypes.c_int64), ("steps_done", ctypes.c_int64),
        ("time", c_double), ("dt", c_double), ("mesh_hash", ctypes.c_uint64),
    ]


class ma_request(ctypes.Structure):
    _fields_ = [
        ("nx", c_int32), ("ny", c_int32), ("nz", c_int32), ("problem_type", c_int32),
        ("lx", c_double), ("ly", c_double), ("lz", c_double), ("angle", c_double),
        ("inflow_state", c_double * 5),
        ("nsteps", c_int32),
        ("dt", c_double),
        ("keep_result", c_int32),
    ]


class ma_request_info(ctypes.Structure):
    _fields_ = [
        ("state", c_int32), ("error", c_int32),
        ("steps_done", ctypes.c_int64), ("cells", ctypes.c_int64),
        ("t_submit_ns", ctypes.c_int64), ("t_admit_ns", ctypes.c_int64), ("t_finish_ns", ctypes.c_int64),
        ("state_sq_norm", c_double * 5),
    ]


class ma_server_stats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_int64), ("admitted", ctypes.c_int64), ("completed", ctypes.c_int64),
        ("failed", ctypes.c_int64), ("cancelled", ctypes.c_int64),
        ("ticks", ctypes.c_int64), ("cell_stages", ctypes.c_int64),
        ("bytes_in_use", ctypes.c_int64), ("peak_bytes", ctypes.c_int64),
        ("running", c_int32), ("queued", c_int32), ("peak_running", c_int32), ("capacity", c_int32),
        ("cached_meshes", c_int32),
        ("busy_seconds", c_double),
    ]


MA_SERVER_THREAD, MA_SERVER_DRYRUN = 1, 2
MA_REQ_QUEUED, MA_REQ_RUNNING, MA_REQ_DONE, MA_REQ_CANCELLED, MA_REQ_FAILED = range(5)


class MiniaeroError(RuntimeError):
    """A C-ABI call returned a non-zero ma_status."""

    def __init__(self, status, message):
        super().__init__("%s (status %d)" % (message, status))
        self.status = status


_lib = None

# name: (restype, argtypes)
_SIGNATURES = {
    "ma_abi_version": (c_int32, []),
    "ma_last_error": (ctypes.c_char_p, []),
    "ma_status_string": (ctypes.c_char_p, [c_int32]),
    "ma_device_count": (c_int32, []),
    "ma_options_default": (None, [ctypes.POINTER(ma_options)]),
    "ma_options_read": (c_int32, [ctypes.c_char_p, ctypes.POINTER(ma_options)]),
    "ma_run_options_default": (None, [ctypes.POINTER(ma_run_options)]),
    "ma_run_options_read": (c_int32, [ctypes.c_char_p, ctypes.POINTER(ma_run_options)]),
    "ma_mesh_hash": (ctypes.c_uint64, [ctypes.POINTER(ma_mesh_view)]),
    "ma_checkpoint_write": (c_int32, [ctypes.c_char_p, ctypes.POINTER(ma_checkpoint_info), P_f64, c_int32]),
    "ma_checkpoint_read": (c_int32, [ctypes.c_char_p, ctypes.POINTER(ma_checkpoint_info), P_f64, ctypes.c_int64,
                                     c_int32]),
    "ma_host_mesh_build": (c_int32, [ctypes.POINTER(ma_options), ctypes.POINTER(c_void_p)]),
    "ma_host_mesh_build_ex": (c_int32, [ctypes.POINTER(ma_options), c_int32, ctypes.POINTER(c_void_p)]),
    "ma_host_mesh_view": (c_int32, [c_void_p, ctypes.POINTER(ma_mesh_view)]),
    "ma_host_mesh_free": (None, [c_void_p]),
    "ma_host_initial_state": (c_int32, [c_void_p, ctypes.POINTER(ma_options), P_f64]),
    "ma_mesh_upload": (c_int32, [ctypes.POINTER(ma_mesh_view), ctypes.POINTER(c_void_p)]),
    "ma_mesh_upload_ex": (c_int32, [ctypes.POINTER(ma_mesh_view), c_int32, ctypes.POINTER(c_void_p)]),
    "ma_mesh_free": (None, [c_void_p]),
    "ma_mesh_device_bytes": (ctypes.c_size_t, [c_void_p]),
    "ma_solver_create": (c_int32, [c_void_p, ctypes.POINTER(ma_options), ctypes.POINTER(c_void_p)]),
    "ma_solver_free": (None, [c_void_p]),
    "ma_solver_init_state": (c_int32, [c_void_p, c_void_p]),
    "ma_solver_set_state": (c_int32, [c_void_p, P_f64, c_int32]),
    "ma_solver_get_state": (c_int32, [c_void_p, P_f64, c_int32]),
    "ma_solver_get_residual": (c_int32, [c_void_p, P_f64, c_int32]),
    "ma_solver_step": (c_int32, [c_void_p, c_int32]),
    "ma_solver_synchronize": (c_int32, [c_void_p]),
    "ma_solver_profile_steps": (c_int32, [c_void_p, c_int32, P_f64, P_i32]),
    "ma_solver_stream": (c_void_p, [c_void_p]),
    "ma_solver_dt": (c_double, [c_void_p]),
    "ma_solver_steps_done": (ctypes.c_int64, [c_void_p]),
    "ma_solver_launches_per_step": (c_int32, [c_void_p]),
    "ma_solver_set_dt": (c_int32, [c_void_p, c_double]),
    "ma_solver_check_state": (c_int32, [c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "ma_solver_solve": (c_int32, [c_void_p, c_void_p]),
    "ma_cfl_dt_noalloc": (c_int32, [c_void_p, c_void_p, c_double, P_f64, c_void_p]),
    "ma_batch_create": (c_int32, [ctypes.POINTER(ma_options), c_int32, ctypes.c_size_t, ctypes.POINTER(c_void_p)]),
    "ma_batch_free": (None, [c_void_p]),
    "ma_batch_member_bytes": (ctypes.c_size_t, [c_void_p, c_void_p]),
    "ma_batch_add": (c_int32, [c_void_p, c_void_p, P_f64, c_int32, c_double, P_f64, P_i32]),
    "ma_batch_remove": (c_int32, [c_void_p, c_int32]),
    "ma_batch_get_state": (c_int32, [c_void_p, c_int32, P_f64, c_int32]),
    "ma_batch_step": (c_int32, [c_void_p, c_int32]),
    "ma_batch_synchronize": (c_int32, [c_void_p]),
    "ma_batch_stream": (c_void_p, [c_void_p]),
    "ma_batch_cells": (ctypes.c_int64, [c_void_p]),
    "ma_batch_size": (c_int32, [c_void_p]),
    "ma_batch_device_bytes": (ctypes.c_size_t, [c_void_p]),
    "ma_batch_member_steps": (ctypes.c_int64, [c_void_p, c_int32]),
    "ma_batch_member_dt": (c_double, [c_void_p, c_int32]),
    "ma_batch_get_launch": (c_int32, [c_void_p, P_i32, P_i32]),
    "ma_batch_set_launch": (c_int32, [c_void_p, P_i32, P_i32]),
    "ma_batch_set_single_launch": (c_int32, [c_void_p, c_int32, P_i32]),
    "ma_debug_barrier_timeout": (c_int32, [c_double, P_i32, P_i32, ctypes.POINTER(c_double)]),
    "ma_batch_autotune": (c_int32, [c_void_p, c_int32, P_f64]),
    "ma_batch_profile_steps": (c_int32, [c_void_p, c_int32, P_f64, P_i32]),
    "ma_server_create": (c_int32, [ctypes.POINTER(ma_options), ctypes.c_size_t, c_int32, c_int32, c_int32,
                                   ctypes.POINTER(c_void_p)]),
    "ma_server_free": (None, [c_void_p]),
    "ma_server_submit": (c_int32, [c_void_p, ctypes.POINTER(ma_request), ctypes.POINTER(ctypes.c_int64)]),
    "ma_server_set_launch": (c_int32, [c_void_p, P_i32, P_i32]),
    "ma_server_set_max_running_cells": (c_int32, [c_void_p, ctypes.c_int64]),
    "ma_server_preload_mesh": (c_int32, [c_void_p, ctypes.POINTER(ma_request)]),
    "ma_server_poll": (c_int32, [c_void_p, P_i32]),
    "ma_server_cancel": (c_int32, [c_void_p, ctypes.c_int64]),
    "ma_server_query": (c_int32, [c_void_p, ctypes.c_int64, ctypes.POINTER(ma_request_info)]),
    "ma_server_result": (c_int32, [c_void_p, ctypes.c_int64, P_f64]),
    "ma_server_wait": (c_int32, [c_void_p, ctypes.c_int64, c_double]),
    "ma_server_get_stats": (c_int32, [c_void_p, ctypes.POINTER(ma_server_stats)]),
    "ma_debug_glibc_rand": (c_int32, [ctypes.c_uint32, c_int32, P_i32]),
    "ma_debug_binsort": (c_int32, [P_i32, c_int32, P_i32]),
    "ma_debug_check_division": (c_int32, [c_int32, ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64),
                                          P_f64]),
    "ma_debug_fp64_rate": (c_int32, [c_int32, P_f64]),
    "ma_op_roe_flux": (c_int32, [c_int32, P_f64, P_f64, P_f64, P_f64, P_f64, P_f64]),
    "ma_op_viscous_flux": (c_int32, [c_int32, P_f64, P_f64, P_f64, c_int32, c_double, c_double, P_f64]),
    "ma_op_limiter": (c_int32, [c_int32, c_int32, P_f64, P_f64, P_f64, P_f64, P_f64]),
    "ma_op_primitives": (c_int32, [c_int32, P_f64, P_f64]),
    "ma_op_green_gauss": (c_int32, [c_void_p, P_f64, c_int32, P_f64]),
    "ma_op_stencil_limiter": (c_int32, [c_void_p, c_int32, P_f64, c_int32, P_f64]),
    "ma_op_bc_flux": (c_int32, [c_void_p, ctypes.POINTER(ma_options), P_f64, c_int32, P_f64]),
    "ma_op_apply_cell_flux": (c_int32, [c_int32, c_double, P_f64, P_f64, P_f64]),
    "ma_op_rk_update": (c_int32, [ctypes.c_int64, c_double, P_f64, P_f64, P_f64]),
}


def lib():
    """Loads the shared library once; raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                "libminiaero_gpu.so is not built (%s); run `python -c \"import __graft_entry__ as g; g.build()\"`"
                % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status):
    if status != MA_OK:
        L = lib()
        msg = (L.ma_last_error() or b"").decode() or L.ma_status_string(status).decode()
        raise MiniaeroError(status, msg)


def f64p(a):
    return a.ctypes.data_as(P_f64)


def i32p(a):
    return a.ctypes.data_as(P_i32)
