"""ctypes bindings of the two C-ABI libraries.

``host()`` returns libuchol_host.so (matrix construction, symbolic phase),
``gpu()`` returns libuchol_gpu.so (device numeric phase).  Both are built
in-tree (``magla_gb300/build.py``).  There is no fallback: when the device
library is missing or cannot be loaded, ``gpu()`` raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import build as _build

_LOCK = threading.Lock()
_HOST = None
_GPU = None

c_int_p = C.POINTER(C.c_int)
c_double_p = C.POINTER(C.c_double)
c_void_pp = C.POINTER(C.c_void_p)

# status codes (include/uchol_host.h, include/uchol_gpu.h)
OK = 0
BAD_ARG = 1
PATTERN_MISMATCH = 2
NOT_SPD = 3
OOM = 4
TIMEOUT = 5
CUDA_ERROR = 6
TOO_DENSE = 7
NO_CONVERGENCE = 8
INTERNAL = 9
OUT_OF_RANGE = 10
NOT_IN_PATTERN = 11

PRECISION_FP64 = 0
PRECISION_TF32 = 1
PRECISION_BF16 = 2


class AnalysisInfo(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("nnz", C.c_int), ("supernode_count", C.c_int), ("max_front_size", C.c_int),
        ("max_supernode_width", C.c_int), ("pattern_entries", C.c_int), ("lower_entries", C.c_int),
        ("front_row_entries", C.c_int), ("child_entries", C.c_int), ("slab_count", C.c_int),
        ("factor_entry_count", C.c_int64), ("strict_factor_nonzero_count", C.c_int64),
        ("factor_operation_count", C.c_int64), ("peak_contribution_entries", C.c_int64),
    ]


class SymbolicDesc(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("nnz", C.c_int), ("row_ptr", c_int_p), ("col", c_int_p), ("permutation", c_int_p),
        ("diag_value_index", c_int_p), ("pattern_ptr", c_int_p), ("pattern_rows", c_int_p),
        ("lower_start", c_int_p), ("lower_value_ptr", c_int_p), ("lower_value_index", c_int_p),
        ("supernode_count", C.c_int), ("first_column", c_int_p), ("parent", c_int_p), ("child_ptr", c_int_p),
        ("children", c_int_p), ("front_ptr", c_int_p), ("front_rows", c_int_p),
    ]


class Options(C.Structure):
    _fields_ = [
        ("allow_diagonal_regularization", C.c_int), ("pivot_tolerance", C.c_double),
        ("diagonal_regularization", C.c_double), ("panel_width", C.c_int), ("precision", C.c_int),
        ("block_width", C.c_int), ("small_front_buckets", C.c_int), ("chain_merge_width", C.c_int),
        ("inverse_block_width", C.c_int), ("device_memory_budget", C.c_int64), ("split_min_kblocks", C.c_int),
        ("extend_add_overlap", C.c_int), ("chain_merge_fill", C.c_double),
    ]


class FactorStats(C.Structure):
    _fields_ = [
        ("regularized_pivot_count", C.c_int), ("negative_pivot_count", C.c_int),
        ("smallest_pivot_magnitude", C.c_double), ("largest_pivot_magnitude", C.c_double),
        ("failed_pivot", C.c_int), ("factor_ms", C.c_double), ("device_bytes", C.c_int64),
    ]


class AutotuneReport(C.Structure):
    _fields_ = [("candidates", C.c_int), ("default_ms", C.c_double), ("best_ms", C.c_double),
                ("small_front_buckets", C.c_int), ("block_width", C.c_int), ("chain_merge_width", C.c_int),
                ("split_min_kblocks", C.c_int)]


class RefineOptions(C.Structure):
    _fields_ = [("tolerance", C.c_double), ("max_iterations", C.c_int), ("method", C.c_int)]


class RefineStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("relative_residual", C.c_double),
                ("initial_relative_residual", C.c_double), ("solve_ms", C.c_double)]


class PhaseTimes(C.Structure):
    _fields_ = [("pivot_block_ms", C.c_double), ("extend_add_ms", C.c_double), ("small_fronts_ms", C.c_double),
                ("panel_ms", C.c_double), ("schur_ms", C.c_double), ("total_ms", C.c_double),
                ("launches", C.c_int), ("schur_tensor_flops", C.c_double), ("schur_tensor_ms", C.c_double),
                ("schur_tensor_launches", C.c_int), ("solve_kind_ms", C.c_double * 14), ("solve_total_ms", C.c_double),
                ("solve_launches", C.c_int)]

class CgOptions(C.Structure):
    _fields_ = [("relative_tolerance", C.c_double), ("max_iterations", C.c_int), ("use_preconditioner", C.c_int),
                ("use_initial_guess", C.c_int), ("pivot_tolerance", C.c_double)]


class CgResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("residual_norm", C.c_double),
                ("relative_residual", C.c_double), ("ms", C.c_double)]


# launch kinds of PhaseTimes.solve_kind_ms
SOLVE_KINDS = ("fwd_gather", "fwd_solo", "fwd_level", "bwd_gather", "bwd_cols", "bwd_solo", "bwd_level", "fwd_tail",
               "bwd_cols_reduce", "fwd_inv_diag", "fwd_inv_tail", "bwd_inv_cols", "bwd_inv_diag",
               "bwd_inv_reduce")


HOST_SYMBOLS = {
    "uchol_csr_from_triplets": (C.c_int, [C.c_int, C.c_int64, c_int_p, c_int_p, c_double_p, c_void_pp]),
    "uchol_csr_grid": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, c_void_pp]),
    "uchol_csr_laplacian3d": (C.c_int, [C.c_int, C.c_int, C.c_int, c_void_pp]),
    "uchol_csr_laplacian2d": (C.c_int, [C.c_int, C.c_int, c_double_p, c_void_pp]),
    "uchol_csr_elasticity": (C.c_int, [C.c_int, C.c_int, C.c_int, c_double_p, C.c_double, C.c_int, c_double_p,
                                       c_void_pp]),
    "uchol_csr_shape": (C.c_int, [C.c_void_p, c_int_p, c_int_p]),
    "uchol_csr_copy": (C.c_int, [C.c_void_p, c_int_p, c_int_p, c_double_p, c_int_p]),
    "uchol_csr_destroy": (None, [C.c_void_p]),
    "uchol_analyze": (C.c_int, [C.c_int, C.c_int, c_int_p, c_int_p, C.c_int, C.c_int, c_void_pp]),
    "uchol_analysis_get_info": (C.c_int, [C.c_void_p, C.POINTER(AnalysisInfo)]),
    "uchol_analysis_copy": (C.c_int, [C.c_void_p, C.c_int, c_int_p]),
    "uchol_analysis_destroy": (None, [C.c_void_p]),
    "uchol_amd_order": (C.c_int, [C.c_int, c_int_p, c_int_p, c_int_p]),
    "uchol_batch_csr": (C.c_int, [C.c_int, c_int_p, C.POINTER(c_int_p), C.POINTER(c_int_p), C.POINTER(c_double_p),
                                  c_void_pp]),
    "uchol_batch_analyze": (C.c_int, [C.c_int, c_int_p, C.POINTER(c_int_p), C.POINTER(c_int_p), C.c_int, C.c_int,
                                      c_void_pp]),
    "uchol_host_last_error": (C.c_char_p, []),
}

GPU_SYMBOLS = {
    "uchol_default_options": (None, [C.POINTER(Options)]),
    "uchol_symbolic_create": (C.c_int, [C.POINTER(SymbolicDesc), c_void_pp]),
    "uchol_symbolic_destroy": (C.c_int, [C.c_void_p]),
    "uchol_symbolic_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "uchol_factorize": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.POINTER(Options), c_void_pp,
                                  C.POINTER(FactorStats)]),
    "uchol_factorize_device": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.POINTER(Options), c_void_pp,
                                         C.POINTER(FactorStats)]),
    "uchol_refactorize": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(FactorStats)]),
    "uchol_factor_destroy": (C.c_int, [C.c_void_p]),
    "uchol_factor_diagonal": (C.c_int, [C.c_void_p, c_double_p]),
    "uchol_factor_get_stats": (C.c_int, [C.c_void_p, C.POINTER(FactorStats)]),
    "uchol_solve": (C.c_int, [C.c_void_p, C.c_int, C.c_int, c_double_p, C.c_int, c_double_p, C.c_int]),
    "uchol_solve_device": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    "uchol_solve_refined": (C.c_int, [C.c_void_p, C.c_int, C.c_int, c_double_p, C.c_int, c_double_p, C.c_int,
                                      C.POINTER(RefineOptions), C.POINTER(RefineStats)]),
    "uchol_solve_refined_device": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                             C.POINTER(RefineOptions), C.POINTER(RefineStats)]),
    "uchol_residual_norms": (C.c_int, [C.c_void_p, C.c_int, C.c_int, c_double_p, C.c_int, c_double_p, C.c_int,
                                       c_double_p]),
    "uchol_factor_phase_times": (C.c_int, [C.c_void_p, C.POINTER(PhaseTimes)]),
    "uchol_estimate_device_bytes": (C.c_int, [C.POINTER(SymbolicDesc), C.POINTER(Options), C.POINTER(C.c_int64),
                                              C.POINTER(C.c_int64), C.POINTER(C.c_int64), c_int_p, c_int_p]),
    "uchol_residual_norms_static": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "uchol_residual_norms_static_error": (C.c_char_p, []),
    "uchol_autotune": (C.c_int, [C.c_void_p, C.c_int, C.c_int, c_double_p, C.POINTER(Options), C.POINTER(Options),
                                 C.POINTER(AutotuneReport)]),
    "uchol_check_schur_update": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                           C.POINTER(C.c_int64), c_int_p]),
    "uchol_check_diag_panel": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_void_p,
                                         C.c_void_p, C.c_void_p, c_int_p]),
    "uchol_check_plan": (C.c_int, [C.POINTER(SymbolicDesc), C.POINTER(Options), C.c_int, c_int_p]),
    "uchol_set_wait_limits": (C.c_int, [C.c_double, C.c_double]),
    "uchol_check_solve_wait": (C.c_int, [C.c_void_p, C.c_double]),
    "uchol_dmatrix_create": (C.c_int, [C.c_int, C.c_int, c_int_p, c_int_p, C.c_void_p, C.c_void_p, c_void_pp]),
    "uchol_dmatrix_destroy": (C.c_int, [C.c_void_p]),
    "uchol_dmatrix_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "uchol_dmatrix_values": (C.c_int, [C.c_void_p, c_void_pp]),
    "uchol_dmatrix_set_values": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "uchol_dmatrix_get_values": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "uchol_dmatrix_clear_values": (C.c_int, [C.c_void_p]),
    "uchol_accumulate_plan_create": (C.c_int, [C.c_void_p, C.c_int, c_int_p, c_int_p, c_void_pp]),
    "uchol_accumulate": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "uchol_line_cross_plan_create": (C.c_int, [C.c_void_p, C.c_int, c_int_p, c_void_pp]),
    "uchol_line_cross": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int,
                                   C.c_int]),
    "uchol_values_plan_destroy": (C.c_int, [C.c_void_p]),
    "uchol_dmatrix_multiply": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int]),
    "uchol_default_cg_options": (None, [C.POINTER(CgOptions)]),
    "uchol_jacobi_pcg": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int,
                                   C.POINTER(CgOptions), C.POINTER(CgResult)]),
    "uchol_refactorize_dmatrix": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(FactorStats)]),
    "uchol_kernel_launches": (C.c_int64, []),
    "uchol_set_phase_timing": (None, [C.c_int]),
    "uchol_last_error": (C.c_char_p, []),
}


def _bind(lib, table):
    for name, (res, args) in table.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def host():
    """libuchol_host.so, built on first use."""
    global _HOST
    with _LOCK:
        if _HOST is None:
            path = _build.HOST_LIB
            if not path.exists():
                _build.build_host()
            _HOST = _bind(C.CDLL(str(path)), HOST_SYMBOLS)
        return _HOST


def gpu():
    """libuchol_gpu.so.  Raises when it has not been built or cannot be loaded."""
    global _GPU
    with _LOCK:
        if _GPU is None:
            path: Path = _build.GPU_LIB
            if not path.exists():
                raise RuntimeError(
                    f"the CUDA library {path} is missing: build it with `python -m magla_gb300.build` "
                    "(there is no CPU fallback)")
            _GPU = _bind(C.CDLL(str(path)), GPU_SYMBOLS)
        return _GPU


def ptr(a, ctype=C.c_int):
    """ctypes pointer into a contiguous numpy array (None for None)."""
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))
