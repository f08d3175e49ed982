"""ctypes binding of the C ABI declared in ``include/fv_gb300.h``.

This module only loads ``_lib/libfvgb300.so`` (built in-tree by
``finitevolume_gb300.build``) and declares its entry points; it performs no
computation of its own.  If the library is missing, :func:`lib` raises:
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libfvgb300.so")

FV_OK, FV_ERR_BAD_ARG, FV_ERR_CUDA, FV_ERR_NONFINITE, FV_ERR_TIMEOUT, FV_ERR_BAD_MESH, FV_ERR_UNSUPPORTED = range(7)
STATUS_NAMES = {0: "FV_OK", 1: "FV_ERR_BAD_ARG", 2: "FV_ERR_CUDA", 3: "FV_ERR_NONFINITE", 4: "FV_ERR_TIMEOUT",
                5: "FV_ERR_BAD_MESH", 6: "FV_ERR_UNSUPPORTED"}
REORDER = {"none": 0, "morton": 1, "rcm": 2}


class FVError(RuntimeError):
    """A non-FV_OK status from the C ABI."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class NewtonOpts(C.Structure):
    _fields_ = [("limiter_mode", C.c_int32), ("max_newton", C.c_int32), ("tol", C.c_double), ("cfl0", C.c_double),
                ("cfl_max", C.c_double), ("cfl_growth", C.c_double), ("krylov_dim", C.c_int32),
                ("krylov_rtol", C.c_double), ("precond_sweeps", C.c_int32), ("precond_kind", C.c_int32),
                ("max_rel_change", C.c_double)]


class BC(C.Structure):
    _fields_ = [("type", C.c_int32), ("isothermal", C.c_int32), ("state", C.c_double * 4),
                ("wall_u", C.c_double), ("wall_v", C.c_double), ("wall_T", C.c_double), ("nut", C.c_double)]


class IC(C.Structure):
    _fields_ = [("two_region", C.c_int32), ("pad", C.c_int32),
                ("rho", C.c_double), ("u", C.c_double), ("v", C.c_double), ("p", C.c_double),
                ("rho_l", C.c_double), ("u_l", C.c_double), ("v_l", C.c_double), ("p_l", C.c_double),
                ("rho_r", C.c_double), ("u_r", C.c_double), ("v_r", C.c_double), ("p_r", C.c_double),
                ("x0", C.c_double)]


class Options(C.Structure):
    _fields_ = [("flux", C.c_int32), ("order", C.c_int32), ("gradient", C.c_int32), ("limiter", C.c_int32),
                ("venkat_k", C.c_double), ("rk_stages", C.c_int32), ("dt_mode", C.c_int32),
                ("precision", C.c_int32), ("strict", C.c_int32), ("exact_tol", C.c_double),
                ("exact_max_iter", C.c_int32), ("viscous", C.c_int32), ("gas_constant", C.c_double),
                ("mu", C.c_double), ("prandtl", C.c_double), ("prandtl_t", C.c_double),
                ("initial_nut", C.c_double), ("sa", C.c_double * 9)]


class NoAllocMesh(C.Structure):
    """fv_noalloc_mesh_t: device pointers in the caller's numbering."""
    _fields_ = [("n_cells", C.c_int32), ("n_faces", C.c_int32), ("face_left", C.c_void_p),
                ("face_right", C.c_void_p), ("face_patch", C.c_void_p), ("face_geom", C.c_void_p),
                ("cell_face_off", C.c_void_p), ("cell_faces", C.c_void_p), ("cell_volume", C.c_void_p)]


NOALLOC_MAX_FACES = 131072
NOALLOC_MAX_CELLS = 131072

_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_I64 = C.POINTER(C.c_int64)

# name -> (restype, argtypes); every function declared in include/fv_gb300.h
SIGNATURES = {
    "fv_last_error": (C.c_char_p, []),
    "fv_abi_version": (C.c_int, []),
    "fv_device_count": (C.c_int, []),
    "fv_mesh_create_polygons": (C.c_int, [C.c_int32, _D, C.c_int32, _I64, _I32, C.c_int32, _I32, _I32, C.c_int32,
                                          C.c_int32, C.POINTER(_P)]),
    "fv_mesh_create_faces": (C.c_int, [C.c_int32, _D, C.c_int32, _I32, _I32, _I32, C.c_int32, _I32, _I32, _D,
                                       C.c_int32, C.c_int32, C.POINTER(_P)]),
    "fv_mesh_counts": (C.c_int, [_P, _I64]),
    "fv_mesh_export": (C.c_int, [_P, _I32, _D, _D, _I32, _I32]),
    "fv_mesh_permutation": (C.c_int, [_P, _I32]),
    "fv_mesh_dataflow_plan": (C.c_int, [_P, _I32, C.c_int32, _I32, _I32, _I32, _I32, _I32, _I32, _I32, _I32, _I32]),
    "fv_mesh_agglomerate": (C.c_int, [_P, _I32, _I32, _D, _I32, _D]),
    "fv_mesh_destroy": (C.c_int, [_P]),
    "fv_options_default": (None, [C.POINTER(Options)]),
    "fv_solver_create": (C.c_int, [_P, C.POINTER(BC), C.c_int32, C.c_double, C.c_double, C.POINTER(IC),
                                   C.POINTER(Options), C.POINTER(_P)]),
    "fv_solver_destroy": (C.c_int, [_P]),
    "fv_solver_set_stream": (C.c_int, [_P, _P]),
    "fv_step": (C.c_int, [_P, C.c_int32, _D]),
    "fv_step_async": (C.c_int, [_P, C.c_int32]),
    "fv_get_history": (C.c_int, [_P, C.c_int32, _D]),
    "fv_step_timed": (C.c_int, [_P, C.c_int32, _D, _I32]),
    "fv_get_field": (C.c_int, [_P, _D]),
    "fv_set_field": (C.c_int, [_P, _D]),
    "fv_get_residual": (C.c_int, [_P, _D]),
    "fv_set_cfl": (C.c_int, [_P, C.c_double]),
    "fv_get_nut": (C.c_int, [_P, _D]),
    "fv_set_nut": (C.c_int, [_P, _D]),
    "fv_get_nut_residual": (C.c_int, [_P, _D]),
    "fv_get_wall_distance": (C.c_int, [_P, _D]),
    "fv_solver_set_launch": (C.c_int, [_P, _I32]),
    "fv_solver_freeze_limiter": (C.c_int, [_P, C.c_int32]),
    "fv_solver_set_persistent": (C.c_int, [_P, C.c_int32]),
    "fv_solver_persistent": (C.c_int, [_P, _I32, _I32]),
    "fv_solver_set_wait_limit": (C.c_int, [_P, C.c_int64, C.c_int32]),
    "fv_newton_default": (None, [C.POINTER(NewtonOpts)]),
    "fv_steady_newton": (C.c_int, [_P, C.POINTER(NewtonOpts), _D, _I32, _I32]),
    "fv_adjoint_solve_krylov": (C.c_int, [_P, _D, C.c_double, C.c_int32, C.c_int32, C.c_double, C.c_int32, _D, _D,
                                          _D, _I32, _D]),
    "fv_solver_limiter_values": (C.c_int, [_P, _D, _D]),
    "fv_solver_update_nodes": (C.c_int, [_P, _P, _D]),
    "fv_solver_multigrid": (C.c_int, [_P, _P, C.c_int32, C.c_int32, C.c_double]),
    "fv_solver_autotune": (C.c_int, [_P, C.c_int32, _I32]),
    "fv_get_gamma": (C.c_int, [_P, _D]),
    "fv_device_state": (C.c_int, [_P, C.POINTER(_P), C.POINTER(_P)]),
    "fv_wall_forces": (C.c_int, [_P, _D, _D]),
    "fv_step_noalloc": (C.c_int, [C.POINTER(NoAllocMesh), C.POINTER(BC), C.c_int32, C.c_double, C.c_double,
                                  C.c_int32, _P, _D, _P]),
    "fv_diffusion_create": (C.c_int, [_P, C.c_double, C.c_double, C.c_double, C.c_double, _I32, _D,
                                      C.POINTER(_P)]),
    "fv_diffusion_destroy": (C.c_int, [_P]),
    "fv_diffusion_step": (C.c_int, [_P, C.c_int32, _D]),
    "fv_diffusion_get_field": (C.c_int, [_P, _D]),
    "fv_diffusion_set_field": (C.c_int, [_P, _D]),
    "fv_diffusion_residual": (C.c_int, [_P, _D]),
    "fv_gradient_create": (C.c_int, [_P, C.c_int32, C.POINTER(_P)]),
    "fv_gradient_destroy": (C.c_int, [_P]),
    "fv_gradient_compute": (C.c_int, [_P, _D, _D, _D, _D]),
    "fv_mesh_create_batch": (C.c_int, [C.c_int32, C.POINTER(_P), C.c_int32, C.POINTER(_P)]),
    "fv_batch_create": (C.c_int, [_P, C.POINTER(BC), C.c_int32, _D, C.c_double, C.c_double, C.POINTER(Options),
                                  C.POINTER(_P)]),
    "fv_batch_set_tolerance": (C.c_int, [_P, C.c_double]),
    "fv_batch_status": (C.c_int, [_P, _I32, _I32, _D]),
    "fv_batch_wall_forces": (C.c_int, [_P, C.c_int32, _D, _D]),
    "fv_batch_set_active": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "fv_adjoint_create": (C.c_int, [_P, C.c_int32, C.POINTER(_P)]),
    "fv_adjoint_destroy": (C.c_int, [_P]),
    "fv_residual_forward": (C.c_int, [_P, _D, _D]),
    "fv_residual_jvp": (C.c_int, [_P, _D, _D, _D]),
    "fv_residual_backward": (C.c_int, [_P, _D, _D, _D]),
    "fv_adjoint_solve": (C.c_int, [_P, _D, C.c_int32, C.c_double, _D, _D, _D, C.POINTER(C.c_int32)]),
    "fv_adjoint_solve_gmres": (C.c_int, [_P, _D, C.c_int32, C.c_int32, C.c_double, _D, _D, _D,
                                         C.POINTER(C.c_int32), _D]),
    "fv_force_gradient": (C.c_int, [_P, C.c_int32, _D, _D, _D]),
    "fv_adjoint_shape_gradient": (C.c_int, [_P, _P, C.c_int32, _D, _D]),
    "fv_residual_shape_vjp": (C.c_int, [_P, _P, _D, _D]),
    "fv_checkpoint_write": (C.c_int, [C.c_char_p, C.c_int32, C.c_int64, C.c_uint64, C.c_int64, _D]),
    "fv_checkpoint_read": (C.c_int, [C.c_char_p, C.c_int32, C.c_int64, C.POINTER(C.c_int64),
                                     C.POINTER(C.c_uint64), _D]),
}

_lib = None
_lock = threading.Lock()


def lib() -> C.CDLL:
    """Load the library once; raise if it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"{LIB_PATH} not built: run __graft_entry__.build() (no CPU fallback exists)")
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
        return _lib


def check(status: int) -> None:
    if status != FV_OK:
        raise FVError(status, lib().fv_last_error().decode(errors="replace"))


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


def i32ptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_I32)


def i64ptr(a: np.ndarray):
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(_I64)


def default_options() -> Options:
    o = Options()
    lib().fv_options_default(C.byref(o))
    return o
