"""ctypes binding of libopenmhd_gb300.so (the C ABI in include/openmhd_gb300.h).

The shared library is built in-tree by openmhd_gb300.build.  There is no CPU
fallback: importing the bindings without the library raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libopenmhd_gb300.so")

_lib = None

c_double_p = C.POINTER(C.c_double)
c_int_p = C.POINTER(C.c_int)


class ErrorInfo(C.Structure):
    _fields_ = [("code", C.c_int), ("i", C.c_int), ("j", C.c_int), ("k", C.c_int),
                ("instance", C.c_int), ("value", C.c_double), ("message", C.c_char * 160)]


class Config(C.Structure):
    _fields_ = [("nd", C.c_int), ("ix", C.c_int), ("jx", C.c_int), ("kx", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("x0", C.c_double), ("y0", C.c_double), ("z0", C.c_double),
                ("cfl", C.c_double), ("gamma", C.c_double),
                ("lm_type", C.c_int), ("flux_type", C.c_int), ("time_type", C.c_int),
                ("eta_kind", C.c_int), ("bc_kind", C.c_int * 6), ("bc_flip", C.c_int * 6),
                ("precision", C.c_int), ("tend", C.c_double)]


class StepInfo(C.Structure):
    _fields_ = [("t", C.c_double), ("dt", C.c_double), ("ch", C.c_double),
                ("vmax_next", C.c_double), ("steps", C.c_longlong), ("done", C.c_int),
                ("status", C.c_int)]


class Model(C.Structure):
    _fields_ = [("kind", C.c_int), ("amp", C.c_double), ("bx0", C.c_double),
                ("phase_x", C.c_double), ("phase_y", C.c_double), ("beta", C.c_double),
                ("pert", C.c_double), ("seed", C.c_uint64)]


P = C.c_void_p  # array arguments are passed as raw addresses (host or device)
I = C.c_int
D = C.c_double

# (name, restype, argtypes) for every symbol declared in include/openmhd_gb300.h
SIGNATURES = [
    ("omhd_u2v_2d", I, [P, P, I, I]),
    ("omhd_u2v_3d", I, [P, P, I, I, I]),
    ("omhd_limiter_2d", I, [P, P, P, I, I, I, I]),
    ("omhd_limiter_3d", I, [P, P, P, I, I, I, I, I]),
    ("omhd_flux_solver_2d", I, [P, P, P, D, I, I, I, I]),
    ("omhd_flux_solver_3d", I, [P, P, P, D, I, I, I, I, I]),
    ("omhd_rk_tvd21_2d", I, [P, P, P, P, D, D, I, I]),
    ("omhd_rk_tvd22_2d", I, [P, P, P, P, D, D, I, I]),
    ("omhd_rk_std21_2d", I, [P, P, P, P, D, D, I, I]),
    ("omhd_rk_std22_2d", I, [P, P, P, D, D, I, I]),
    ("omhd_rk_tvd21_3d", I, [P, P, P, P, P, D, D, I, I, I]),
    ("omhd_rk_tvd22_3d", I, [P, P, P, P, P, D, D, I, I, I]),
    ("omhd_rk_std21_3d", I, [P, P, P, P, P, D, D, I, I, I]),
    ("omhd_rk_std22_3d", I, [P, P, P, P, D, D, I, I, I]),
    ("omhd_glm_ss2_2d", I, [P, D, D, I, I]),
    ("omhd_glm_ss2_3d", I, [P, D, D, I, I, I]),
    ("omhd_set_dt_2d", I, [P, P, c_double_p, c_double_p, D, D, I, I]),
    ("omhd_set_dt_3d", I, [P, P, c_double_p, c_double_p, D, D, I, I, I]),
    ("omhd_set_dt_resistive", I, [c_double_p, D, D, I]),
    ("omhd_bc_2d", I, [P, I, I, c_int_p, c_int_p]),
    ("omhd_bc_3d", I, [P, I, I, I, c_int_p, c_int_p]),
    ("omhd_facefix_2d", I, [P, P, I, I, I, I, I, I, I]),
    ("omhd_facefix_3d", I, [P, P, I, I, I, I, I, I, I, I]),
    ("omhd_flux_resistive_2d", I, [P, P, P, P, D, I, I, I, I]),
    ("omhd_flux_resistive_3d", I, [P, P, P, P, P, D, I, I, I, I, I]),
    ("u2v_", None, [P, P, c_int_p, c_int_p]),
    ("limiter_", None, [P, P, P, c_int_p, c_int_p, c_int_p, c_int_p]),
    ("flux_solver_", None, [P, P, P, c_double_p, c_int_p, c_int_p, c_int_p, c_int_p]),
    ("rk_tvd21_", None, [P, P, P, P, c_double_p, c_double_p, c_int_p, c_int_p]),
    ("rk_tvd22_", None, [P, P, P, P, c_double_p, c_double_p, c_int_p, c_int_p]),
    ("rk_std21_", None, [P, P, P, P, c_double_p, c_double_p, c_int_p, c_int_p]),
    ("rk_std22_", None, [P, P, P, c_double_p, c_double_p, c_int_p, c_int_p]),
    ("glm_ss2_", None, [P, c_double_p, c_double_p, c_int_p, c_int_p]),
    ("set_dt_", None, [P, P, c_double_p, c_double_p, c_double_p, c_double_p, c_int_p, c_int_p]),
    ("bc_", None, [P, c_int_p, c_int_p]),
    ("flux_resistive_", None, [P, P, P, P, c_double_p, c_int_p, c_int_p, c_int_p]),
    ("set_dt_resistive_", None, [c_double_p, c_double_p, c_double_p]),
    ("omhd_abi_version", I, []),
    ("omhd_set_stream", I, [P]),
    ("omhd_set_abort_on_error", None, [I]),
    ("omhd_last_error", I, [C.POINTER(ErrorInfo)]),
    ("omhd_clear_error", None, []),
    ("omhd_release_host_mirrors", None, []),
    ("omhd_probe_fp64_peak", I, [c_double_p]),
    ("omhd_probe_fp32_peak", I, [c_double_p]),
    ("omhd_set_tma_staging", None, [I]),
    ("omhd_set_3d_pipeline", None, [I]),
    ("omhd_set_2d_pipeline", None, [I]),
    ("omhd_probe_fastmath", I, [P, C.c_longlong, P]),
    ("omhd_probe_convert", I, [P, P, P, P, C.c_longlong]),
    ("omhd_solver_create", I, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
    ("omhd_solver_destroy", I, [P]),
    ("omhd_solver_set_stream", I, [P, P]),
    ("omhd_solver_bind", I, [P, P, P]),
    ("omhd_solver_state_ptr", I, [P, C.POINTER(C.c_void_p)]),
    ("omhd_solver_put_state", I, [P, P, D]),
    ("omhd_solver_get_state", I, [P, P]),
    ("omhd_solver_step_host", I, [P, P, P, D, I]),
    ("omhd_solver_init_model", I, [P, C.POINTER(Model)]),
    ("omhd_solver_coords", I, [P, P, P, P]),
    ("omhd_solver_set_tend", I, [P, D]),
    ("omhd_solver_step", I, [P, I]),
    ("omhd_solver_step_graph", I, [P, I, I]),
    ("omhd_solver_sync", I, [P, C.POINTER(StepInfo)]),
    ("omhd_solver_last_error", I, [P, C.POINTER(ErrorInfo)]),
    ("omhd_solver_launches_per_step", I, [P]),
    ("omhd_ensemble_create", I, [C.POINTER(Config), I, C.POINTER(C.c_void_p)]),
    ("omhd_ensemble_destroy", I, [P]),
    ("omhd_ensemble_size", I, [P]),
    ("omhd_ensemble_set_stream", I, [P, P]),
    ("omhd_ensemble_member", I, [P, I, C.POINTER(C.c_void_p)]),
    ("omhd_ensemble_init_models", I, [P, C.POINTER(Model)]),
    ("omhd_ensemble_set_tiling", I, [P, I, I]),
    ("omhd_ensemble_autotune", I, [P, I, c_int_p, c_int_p, c_double_p]),
    ("omhd_ensemble_step", I, [P, I]),
    ("omhd_ensemble_step_graph", I, [P, I, I]),
    ("omhd_ensemble_sync", I, [P, C.POINTER(StepInfo)]),
    ("omhd_step2d_noalloc", I, [P, C.POINTER(Config), D, I, P, C.POINTER(StepInfo)]),
    ("omhd_step2d_noalloc_max_doubles", C.c_size_t, []),
    ("omhd_fileio_output", I, [C.c_char_p, I, I, I, I, D, P, P, P, P, P]),
    ("omhd_fileio_input", I, [C.c_char_p, I, I, I, I, c_double_p, P, P, P, P]),
    ("omhd_solver_write", I, [P, C.c_char_p]),
    ("omhd_solver_read", I, [P, C.c_char_p]),
    ("omhd_adjoint_create", I, [C.POINTER(Config), I, I, C.POINTER(C.c_void_p)]),
    ("omhd_adjoint_destroy", I, [P]),
    ("omhd_adjoint_set_stream", I, [P, P]),
    ("omhd_adjoint_forward", I, [P, P, P]),
    ("omhd_adjoint_backward", I, [P, P, P]),
    ("omhd_adjoint_record", I, [P, P, P]),
    ("omhd_adjoint_replay", I, [P, P, P]),
    ("omhd_adjoint_step_vjp", I, [P, P, P, P, P, P]),
    ("omhd_adjoint_sync", I, [P]),
    ("omhd_adjoint_step_log", I, [P, P]),
    ("omhd_adjoint_memory", I, [P, C.POINTER(C.c_size_t)]),
]


def load(path: str | None = None):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"{p} is missing: build the CUDA extension first "
            "(python -c 'import __graft_entry__ as g; g.build()' or python -m openmhd_gb300.build)")
    lib = C.CDLL(p)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
