"""ctypes binding of libhdg.so (the C ABI declared in include/hdg.h).

The library is built in-tree (``build.py``) and loaded from this package directory.  There is
no fallback: if the library cannot be built or loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libhdg.so")

HDG_OK = 0
ERRORS = {
    -1: "HDG_ERR_ARG", -2: "HDG_ERR_NEG_DETJ", -3: "HDG_ERR_BAD_ORDER", -4: "HDG_ERR_NOT_BOUNDARY",
    -5: "HDG_ERR_NO_CONVERGENCE", -6: "HDG_ERR_OOM", -7: "HDG_ERR_CUDA", -8: "HDG_ERR_SINGULAR",
    -9: "HDG_ERR_BREAKDOWN", -10: "HDG_ERR_UNKNOWN_SET", -11: "HDG_ERR_TIMEOUT", -12: "HDG_ERR_CAPACITY",
}
PREC_FP64, PREC_MIXED = 0, 1
PRECOND_JACOBI, PRECOND_AMG = 0, 1
STEP_ASSEMBLE, STEP_APPLY, STEP_RECOVER, STEP_DOWNLOAD = 1, 2, 4, 8  # hdg_batch_step flags
FIELD_CONST, FIELD_SINSIN, FIELD_BUMPS, FIELD_FOURIER, FIELD_EXP_FOURIER = 0, 1, 2, 3, 4


class HDGError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class hdg_field(C.Structure):
    _fields_ = [("kind", C.c_int), ("nparams", C.c_int), ("params", C.POINTER(C.c_double))]


class hdg_solver(C.Structure):
    _fields_ = [("tol", C.c_double), ("maxit", C.c_int), ("precision", C.c_int), ("chunk", C.c_int),
                ("inner_tol", C.c_double), ("preconditioner", C.c_int)]


class hdg_timings(C.Structure):
    _fields_ = [("element_ms", C.c_double), ("gather_ms", C.c_double), ("apply_ms", C.c_double),
                ("cg_ms", C.c_double), ("cg_a_ms", C.c_double), ("cg_b_ms", C.c_double), ("cg_samples", C.c_int),
                ("cg_iterations", C.c_int), ("recover_ms", C.c_double), ("cg_a_bytes", C.c_double),
                ("cg_b_bytes", C.c_double), ("cg_bytes", C.c_double)]


class hdg_stats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("outer", C.c_int), ("rel_residual", C.c_double), ("converged", C.c_int)]


vp = C.c_void_p
ip = C.c_int
dp = C.POINTER(C.c_double)
i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
intp = C.POINTER(C.c_int)

# name -> (argtypes, restype); every symbol declared in include/hdg.h
SIGNATURES = {
    "hdg_ctx_create": ([ip, C.POINTER(vp)], ip),
    "hdg_ctx_destroy": ([vp], ip),
    "hdg_last_error": ([vp], C.c_char_p),
    "hdg_ctx_set_stream": ([vp, vp], ip),
    "hdg_ctx_launch_count": ([vp], C.c_int64),
    "hdg_ctx_set_profiling": ([vp, ip], ip),
    "hdg_system_timings": ([vp, C.POINTER(hdg_timings)], ip),
    "hdg_mesh_rectangle": ([vp, ip, ip, dp, dp, C.POINTER(vp)], ip),
    "hdg_mesh_from_cells": ([vp, ip, dp, ip, i32p, ip, i32p, C.POINTER(vp)], ip),
    "hdg_mesh_set_coordinates": ([vp, dp], ip),
    "hdg_mesh_jitter": ([vp, C.c_double, C.c_uint64], ip),
    "hdg_mesh_sizes": ([vp, intp, intp, intp], ip),
    "hdg_mesh_get_topology": ([vp, dp, i32p, i32p, i32p], ip),
    "hdg_mesh_faceset": ([vp, C.c_char_p, i32p, intp], ip),
    "hdg_mesh_destroy": ([vp], ip),
    "hdg_space_create": ([vp, ip, ip, C.POINTER(vp)], ip),
    "hdg_space_info": ([vp, intp, intp, intp, intp, intp], ip),
    "hdg_space_tables": ([vp, dp, dp, dp, dp, dp, dp, dp, dp], ip),
    "hdg_space_cell_geometry": ([vp, ip, dp, dp, dp, dp], ip),
    "hdg_space_destroy": ([vp], ip),
    "hdg_assemble_condense": ([vp, C.c_double, C.POINTER(hdg_field), C.POINTER(hdg_field), dp, ip, C.POINTER(vp)], ip),
    "hdg_system_reassemble": ([vp, C.c_double, C.POINTER(hdg_field), C.POINTER(hdg_field), dp], ip),
    "hdg_system_reassemble_resident": ([vp], ip),
    "hdg_system_sizes": ([vp, intp, i64p, intp, intp], ip),
    "hdg_system_get_csc": ([vp, ip, i64p, i64p, dp, dp], ip),
    "hdg_system_get_element_blocks": ([vp, dp, dp, dp, dp], ip),
    "hdg_dirichlet": ([vp, C.c_char_p, C.POINTER(hdg_field), i32p, dp, intp], ip),
    "hdg_apply_dirichlet": ([vp, i32p, dp, ip], ip),
    "hdg_dirichlet_l2": ([vp, C.c_char_p, C.POINTER(hdg_field), i32p, dp, intp], ip),
    "hdg_space_set_he_tau": ([vp, ip], ip),
    "hdg_solve": ([vp, C.POINTER(hdg_solver), dp, C.POINTER(hdg_stats)], ip),
    "hdg_system_kernel_sample": ([vp, ip, dp, dp, intp], ip),
    "hdg_refine": ([vp, C.POINTER(hdg_solver), ip, C.c_double, dp, C.POINTER(hdg_stats)], ip),
    "hdg_recover": ([vp, dp, dp, dp], ip),
    "hdg_errornorm_l2sq": ([vp, C.POINTER(hdg_field), dp], ip),
    "hdg_nodal_avg": ([vp, dp], ip),
    "hdg_system_destroy": ([vp], ip),
    "hdg_errornorm_l2sq_noalloc": ([ip, vp, ip, ip, ip, vp, vp, vp, C.POINTER(hdg_field), dp], ip),
    "hdg_noalloc_last_error": ([], C.c_char_p),
    "hdg_solve_poisson": ([vp, C.c_double, C.POINTER(hdg_field), C.POINTER(hdg_field), dp, C.c_char_p,
                           C.POINTER(hdg_field), C.POINTER(hdg_solver), dp, dp, dp, C.POINTER(hdg_stats)], ip),
    "hdg_mesh_concat": ([vp, ip, C.POINTER(vp), C.POINTER(vp)], ip),
    "hdg_mesh_problems": ([vp, intp, i32p, i32p, i32p], ip),
    "hdg_assemble_condense_batch": ([vp, dp, C.POINTER(hdg_field), C.POINTER(hdg_field), dp, ip, C.POINTER(vp)], ip),
    "hdg_system_reassemble_batch": ([vp, dp, C.POINTER(hdg_field), C.POINTER(hdg_field), dp], ip),
    "hdg_solve_batch": ([ip, C.POINTER(vp), C.POINTER(hdg_solver), C.POINTER(hdg_stats)], ip),
    "hdg_system_set_coefficients_batch": ([vp, dp, C.POINTER(hdg_field), C.POINTER(hdg_field), dp], ip),
    "hdg_system_set_dirichlet": ([vp, i32p, dp, ip], ip),
    "hdg_batch_step": ([ip, C.POINTER(vp), C.POINTER(hdg_solver), ip, C.POINTER(hdg_stats)], ip),
    "hdg_host_alloc": ([C.c_size_t, C.POINTER(vp)], ip),
    "hdg_lagrange_create": ([vp, vp, ip, ip, ip, i32p, C.c_int64, i64p, i64p, C.POINTER(vp)], ip),
    "hdg_lagrange_assemble": ([vp, C.POINTER(hdg_field), dp], ip),
    "hdg_lagrange_get_csc": ([vp, dp, dp], ip),
    "hdg_lagrange_apply_dirichlet": ([vp, i32p, dp, ip], ip),
    "hdg_lagrange_solve": ([vp, C.POINTER(hdg_solver), dp, C.POINTER(hdg_stats)], ip),
    "hdg_lagrange_errornorm_l2sq": ([vp, dp, C.POINTER(hdg_field), C.POINTER(C.c_double)], ip),
    "hdg_lagrange_destroy": ([vp], ip),
    "hdg_host_free": ([vp], ip),
    "hdg_system_set_download": ([vp, dp, dp], ip),
    "hdg_system_get_solution": ([vp, dp, dp], ip),
    "hdg_engine_create": ([vp, C.c_double, ip, ip, C.POINTER(hdg_solver), C.POINTER(vp)], ip),
    "hdg_engine_add_resident_mesh": ([vp, vp, ip, intp], ip),
    "hdg_engine_submit": ([vp, ip, vp, ip, ip, C.POINTER(hdg_field), dp, C.c_double, i64p], ip),
    "hdg_engine_step": ([vp, intp, intp], ip),
    "hdg_engine_poll": ([vp, ip, i64p, dp, intp, dp, intp, intp], ip),
    "hdg_engine_result": ([vp, C.c_int64, dp, dp, dp, intp, intp, intp], ip),
    "hdg_engine_set_keep_results": ([vp, ip], ip),
    "hdg_engine_destroy": ([vp], ip),
    "hdg_dofhandler_create": ([vp, ip, intp, intp, intp, intp, C.POINTER(vp)], ip),
    "hdg_dofhandler_sizes": ([vp, intp, i64p], ip),
    "hdg_dofhandler_cell_dofs": ([vp, i32p, i32p], ip),
    "hdg_dofhandler_field_range": ([vp, ip, intp, intp], ip),
    "hdg_dofhandler_sparsity": ([vp, ip, ip, i64p, i64p, i64p], ip),
    "hdg_dofhandler_dirichlet": ([vp, C.c_char_p, ip, i32p, i32p, i32p, intp], ip),
    "hdg_dofhandler_destroy": ([vp], ip),
    "hdg_dofhandler_last_error": ([], C.c_char_p),
    "hdg_csc_assemble": ([C.c_int64, i64p, i64p, ip, dp, dp, ip, ip, ip, i64p, dp, dp], ip),
    "hdg_assembler_create": ([C.c_int64, C.POINTER(vp)], ip),
    "hdg_assembler_add": ([vp, ip, i64p, dp], ip),
    "hdg_assembler_finish": ([vp, i64p, i64p, i64p], ip),
    "hdg_assembler_get_csc": ([vp, ip, i64p, i64p, dp], ip),
    "hdg_assembler_destroy": ([vp], ip),
}

_lock = threading.Lock()
_lib = None


def load(build_if_needed: bool = True):
    """Load libhdg.so (building it first if it is missing or stale)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build_if_needed:
            from . import build as _build
            if _build.needs_build():
                _build.build()
        if not os.path.exists(LIBPATH):
            raise RuntimeError(f"libhdg.so not found at {LIBPATH}; build it with build.py (needs nvcc)")
        lib = C.CDLL(LIBPATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
        return lib


def check(rc: int, ctx=None):
    if rc != HDG_OK:
        msg = load().hdg_last_error(ctx)
        raise HDGError(rc, msg.decode() if msg else "")


def dptr(a):
    return None if a is None else a.ctypes.data_as(dp)


def i32ptr(a):
    return None if a is None else a.ctypes.data_as(i32p)


def i64ptr(a):
    return None if a is None else a.ctypes.data_as(i64p)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)
