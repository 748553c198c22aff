"""ctypes binding of libbemgpu.so (the C ABI declared in include/bemgpu.h).

Loading fails loudly: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libbemgpu.so")

OK, EINVAL, ETOPOLOGY, ENOMEM_BUDGET, ESINGULAR, ENOTCONVERGED, ETIMEOUT, ECUDA, ENODEV, EBUSY = \
    range(10)
RIGID, PRESSURE_RELEASE, FLUID = 0, 1, 2
FORMULATION_DEFAULT, BURTON_MILLER, CBIE, MULLER = -1, 0, 1, 2
DOUBLE, MIXED = 0, 1
ASSEMBLY = {None: 0, "default": 0, "double": 1, "single": 2}
DISCRETIZATION = {"collocation": 0, "nystrom": 1}
NODES_PER_PANEL = {"collocation": 1, "nystrom": 7}
REASONS = ("none", "conversion", "single_singular", "condition", "nonfinite",
           "iteration_limit", "stagnation")
FIELDS = {"total": 0, "scattered": 1, "incident": 2, "interior": 3}


class Problem(ctypes.Structure):
    _fields_ = [("boundary", ctypes.c_int32), ("formulation", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("equilibrate", ctypes.c_int32),
                ("k", ctypes.c_double), ("density_contrast", ctypes.c_double),
                ("soundspeed_contrast", ctypes.c_double),
                ("refine_tolerance", ctypes.c_double), ("refine_maxiter", ctypes.c_int32),
                ("assembly", ctypes.c_int32), ("condition_guard", ctypes.c_double),
                ("near_eta", ctypes.c_double), ("discretization", ctypes.c_int32),
                ("condition_limit", ctypes.c_int32), ("norm_floor", ctypes.c_double)]


class ServerOptions(ctypes.Structure):
    _fields_ = [("max_batch", ctypes.c_int32), ("queue_limit", ctypes.c_int32),
                ("cache_bytes", ctypes.c_uint64), ("lanes", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64),
                ("failed", ctypes.c_int64), ("items", ctypes.c_int64),
                ("factorizations", ctypes.c_int64), ("cache_hits", ctypes.c_int64),
                ("batches", ctypes.c_int64), ("evictions", ctypes.c_int64),
                ("busy_ms", ctypes.c_double), ("cached_bytes", ctypes.c_uint64),
                ("retries", ctypes.c_int64)]


class Diagnostics(ctypes.Structure):
    _fields_ = [("unknown_count", ctypes.c_int64), ("quadrature_nodes", ctypes.c_int64),
                ("near_pairs", ctypes.c_int64), ("formulation", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("factor_precision", ctypes.c_int32),
                ("refinement_reason", ctypes.c_int32),
                ("refinement_iterations", ctypes.c_int32), ("equilibrate", ctypes.c_int32),
                ("coupling_re", ctypes.c_double), ("coupling_im", ctypes.c_double),
                ("absolute_residual", ctypes.c_double), ("relative_residual", ctypes.c_double),
                ("scaled_absolute_residual", ctypes.c_double),
                ("scaled_relative_residual", ctypes.c_double),
                ("normwise_backward_error", ctypes.c_double),
                ("componentwise_backward_error", ctypes.c_double),
                ("single_reciprocal_condition", ctypes.c_double),
                ("assemble_ms", ctypes.c_double), ("factor_ms", ctypes.c_double),
                ("solve_ms", ctypes.c_double), ("total_ms", ctypes.c_double),
                ("device_bytes", ctypes.c_int64), ("nrhs", ctypes.c_int32),
                ("info", ctypes.c_int32), ("condition_number", ctypes.c_double),
                ("scaled_condition_number", ctypes.c_double), ("conditioning", ctypes.c_int32),
                ("condition_limit", ctypes.c_int32), ("derivative_exterior", ctypes.c_int32),
                ("derivative_interior", ctypes.c_int32)]


class HmatrixOptions(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("eta", ctypes.c_double),
                ("leaf_size", ctypes.c_int32), ("restart", ctypes.c_int32),
                ("reltol", ctypes.c_double), ("abstol", ctypes.c_double),
                ("maxiter", ctypes.c_int32), ("neighbours", ctypes.c_int32)]


class HmatrixStats(ctypes.Structure):
    _fields_ = [("lowrank_blocks", ctypes.c_int64), ("dense_blocks", ctypes.c_int64),
                ("densified_blocks", ctypes.c_int64), ("lowrank_entries", ctypes.c_int64),
                ("dense_entries", ctypes.c_int64), ("max_rank", ctypes.c_int32),
                ("depth", ctypes.c_int32), ("leaves", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("compression", ctypes.c_double), ("gmres_iterations", ctypes.c_int32),
                ("gmres_converged", ctypes.c_int32), ("build_ms", ctypes.c_double),
                ("gmres_ms", ctypes.c_double)]


_vp = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64

# name -> (restype, argtypes)
SIGNATURES = {
    "bemgpu_version": (ctypes.c_char_p, []),
    "bemgpu_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "bemgpu_problem_init": (None, [ctypes.POINTER(Problem)]),
    "bemgpu_mesh_validate": (ctypes.c_int, [_dp, _i64, _i64p, _i64, _dp, ctypes.c_char_p,
                                            ctypes.c_size_t]),
    "bemgpu_mesh_hash": (ctypes.c_int, [_dp, _i64, _i64p, _i64, ctypes.c_char_p]),
    "bemgpu_near_pairs": (ctypes.c_int, [_dp, _i64, _i64p, _i64, ctypes.c_double, _i64p, _i64p,
                                         _i64, _i64p]),
    "bemgpu_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(_vp)]),
    "bemgpu_ctx_destroy": (ctypes.c_int, [_vp]),
    "bemgpu_last_error": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_size_t]),
    "bemgpu_ctx_memory": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_uint64),
                                         ctypes.POINTER(ctypes.c_uint64)]),
    "bemgpu_ctx_synchronize": (ctypes.c_int, [_vp]),
    "bemgpu_mesh_upload": (ctypes.c_int, [_vp, _dp, _i64, _i64p, _i64, ctypes.POINTER(_vp)]),
    "bemgpu_mesh_info": (ctypes.c_int, [_vp, _i64p, _dp, ctypes.c_char_p]),
    "bemgpu_mesh_destroy": (ctypes.c_int, [_vp]),
    "bemgpu_factor_create": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(Problem),
                                            ctypes.POINTER(_vp)]),
    "bemgpu_factor_create_batch": (ctypes.c_int, [_vp, _i32, ctypes.POINTER(_vp),
                                                  ctypes.POINTER(Problem), ctypes.POINTER(_vp)]),
    "bemgpu_factor_solve": (ctypes.c_int, [_vp, _i32, _dp, ctypes.POINTER(_vp)]),
    "bemgpu_factor_solve_batch": (ctypes.c_int, [_vp, _i32, ctypes.POINTER(_vp),
                                                 ctypes.POINTER(_i32), ctypes.POINTER(_dp),
                                                 ctypes.POINTER(_vp)]),
    "bemgpu_factor_destroy": (ctypes.c_int, [_vp]),
    "bemgpu_factor_diagnostics": (ctypes.c_int, [_vp, ctypes.POINTER(Diagnostics)]),
    "bemgpu_solve": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(Problem), _i32, _dp,
                                    ctypes.POINTER(_vp)]),
    "bemgpu_far_field": (ctypes.c_int, [_vp, _i32, _i64, _dp, _dp]),
    "bemgpu_target_strength": (ctypes.c_int, [_vp, _i32, _i64, _dp, _dp]),
    "bemgpu_traces": (ctypes.c_int, [_vp, _i32, _dp, _dp]),
    "bemgpu_region_solve": (ctypes.c_int, [_vp, _i32, ctypes.POINTER(_vp), _dp, _dp,
                                           ctypes.POINTER(_i32), ctypes.POINTER(Problem), _i32,
                                           _dp, ctypes.POINTER(_vp)]),
    "bemgpu_region_traces": (ctypes.c_int, [_vp, _i32, _dp, _dp]),
    "bemgpu_hmatrix_options_init": (None, [ctypes.POINTER(HmatrixOptions)]),
    "bemgpu_hmatrix_plan": (ctypes.c_int, [_dp, _i64, _i64p, _i64, ctypes.c_double,
                                           ctypes.POINTER(HmatrixOptions), _i64p,
                                           ctypes.POINTER(_i32), _i64, ctypes.POINTER(_i32)]),
    "bemgpu_hmatrix_solve": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(Problem),
                                            ctypes.POINTER(HmatrixOptions), _i32, _dp,
                                            ctypes.POINTER(_vp)]),
    "bemgpu_hmatrix_stats_get": (ctypes.c_int, [_vp, ctypes.POINTER(HmatrixStats)]),
    "bemgpu_gmres_history": (ctypes.c_int, [_vp, _i32, _dp, _i32, ctypes.POINTER(_i32)]),
    "bemgpu_hmatrix_apply": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(Problem),
                                            ctypes.POINTER(HmatrixOptions), _i32, _i32, _dp,
                                            _dp, ctypes.POINTER(HmatrixStats)]),
    "bemgpu_ctx_set_autotune": (ctypes.c_int, [_vp, _i32]),
    "bemgpu_solution_diagnostics": (ctypes.c_int, [_vp, ctypes.POINTER(Diagnostics)]),
    "bemgpu_pressure": (ctypes.c_int, [_vp, _i32, _i64, _dp, _i32, _dp]),
    "bemgpu_pressure_region": (ctypes.c_int, [_vp, _i32, _i64, _dp, _i32, _i32, _dp]),
    "bemgpu_solution_destroy": (ctypes.c_int, [_vp]),
    "bemgpu_dense_solve": (ctypes.c_int, [_vp, _i64, _dp, _i32, _dp, _i32, _i32,
                                          ctypes.c_double, _i32, ctypes.c_double,
                                          ctypes.POINTER(Diagnostics)]),
    "bemgpu_assemble_dense": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(Problem), _dp, _dp]),
    "bemgpu_profile_enable": (ctypes.c_int, [_vp, _i32]),
    "bemgpu_profile_reset": (ctypes.c_int, [_vp]),
    "bemgpu_profile_read": (ctypes.c_int, [_vp, ctypes.c_char_p, _i64p, _dp]),
    "bemgpu_launch_count": (ctypes.c_int, [_vp, _i64p]),
    "bemgpu_timer_start": (ctypes.c_int, [_vp]),
    "bemgpu_server_options_init": (None, [ctypes.POINTER(ServerOptions)]),
    "bemgpu_server_create": (ctypes.c_int, [_vp, ctypes.POINTER(ServerOptions),
                                            ctypes.POINTER(_vp)]),
    "bemgpu_server_submit": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(Problem), _i32, _dp, _i32,
                                            _dp, _i64p]),
    "bemgpu_server_wait": (ctypes.c_int, [_vp, _i64, _i32, _dp, _dp]),
    "bemgpu_server_stats_get": (ctypes.c_int, [_vp, ctypes.POINTER(ServerStats)]),
    "bemgpu_server_destroy": (ctypes.c_int, [_vp]),
    "bemgpu_cgemm_update_noalloc": (ctypes.c_int, [_vp, _i64, _i64, _i32, _vp, _i64, _vp, _i64,
                                                   _vp, _i64]),
    "bemgpu_ctx_set_tensor_lu": (ctypes.c_int, [_vp, _i32]),
    "bemgpu_ctx_set_graphs": (ctypes.c_int, [_vp, _i32]),
    "bemgpu_ctx_inject_alloc_failures": (ctypes.c_int, [_vp, _i32]),
    "bemgpu_schwarz_neighbourhoods": (ctypes.c_int, [_dp, _i64, _i64p, _i64, _i32,
                                                     ctypes.POINTER(ctypes.c_int32)]),
    "bemgpu_ctx_graph_stats": (ctypes.c_int, [_vp, _i64p, _i64p]),
    "bemgpu_debug_cgemm": (ctypes.c_int, [_vp, _i64, _i64, _i32,
                                          ctypes.POINTER(ctypes.c_float),
                                          ctypes.POINTER(ctypes.c_float),
                                          ctypes.POINTER(ctypes.c_float)]),
    "bemgpu_timer_stop": (ctypes.c_int, [_vp, _dp]),
}

_LIB = None


def lib():
    """The loaded library; raises if libbemgpu.so has not been built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"libbemgpu.so not found at {LIB_PATH}: build it with "
                "`python acousticscattering.jl_gb300/build.py` (nvcc, sm_103a)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def dptr(a):
    """double* of a contiguous float64 / complex128 numpy array (any memory order)."""
    assert a.flags.c_contiguous or a.flags.f_contiguous
    return ctypes.cast(a.ctypes.data, _dp)


def fptr(a):
    """float* of a contiguous float32 / complex64 numpy array (any memory order)."""
    assert a.flags.c_contiguous or a.flags.f_contiguous
    return ctypes.cast(a.ctypes.data, ctypes.POINTER(ctypes.c_float))


def i64ptr(a):
    assert a.flags.c_contiguous or a.flags.f_contiguous
    return ctypes.cast(a.ctypes.data, _i64p)
