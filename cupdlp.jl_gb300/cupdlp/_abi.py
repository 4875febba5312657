"""ctypes mirror of include/gpdhg.h and the loader of libgpdhg.so.

Every structure here matches the C header field for field; tests check the sizes
against the library (gpdhg_abi_version) and the header. The library is required: if it
is missing or cannot be loaded, `load()` raises — there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

_PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(os.path.dirname(_PKG_DIR), "lib")
LIB_PATH = os.path.join(LIB_DIR, "libgpdhg.so")

ABI_VERSION = 1

# gpdhg_status
OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_INVALID_PROBLEM = 2
ERR_OUT_OF_MEMORY = 3
ERR_CUDA = 4
ERR_NOT_SUPPORTED = 5
ERR_ADMISSION = 6
ERR_NOT_READY = 7
ERR_DEVICE_TIMEOUT = 8
ERR_INTERNAL = 9

STATUS_NAMES = {
    0: "OK", 1: "INVALID_ARGUMENT", 2: "INVALID_PROBLEM", 3: "OUT_OF_MEMORY", 4: "CUDA",
    5: "NOT_SUPPORTED", 6: "ADMISSION", 7: "NOT_READY", 8: "DEVICE_TIMEOUT", 9: "INTERNAL",
}

PRECISION_FP64 = 0
PRECISION_FP32_REFINE = 1
PRECISION_FP32 = 2

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_int64)


class Params(C.Structure):
    _fields_ = [
        ("l_inf_ruiz_iterations", C.c_int32),
        ("l2_norm_rescaling", C.c_int32),
        ("pock_chambolle_alpha", C.c_double),
        ("primal_importance", C.c_double),
        ("scale_invariant_initial_primal_weight", C.c_int32),
        ("verbosity", C.c_int32),
        ("record_iteration_stats", C.c_int32),
        ("termination_evaluation_frequency", C.c_int32),
        ("optimality_norm", C.c_int32),
        ("iteration_limit", C.c_int32),
        ("eps_optimal_absolute", C.c_double),
        ("eps_optimal_relative", C.c_double),
        ("eps_primal_infeasible", C.c_double),
        ("eps_dual_infeasible", C.c_double),
        ("time_sec_limit", C.c_double),
        ("kkt_matrix_pass_limit", C.c_double),
        ("restart_scheme", C.c_int32),
        ("restart_to_current_metric", C.c_int32),
        ("restart_frequency_if_fixed", C.c_int64),
        ("artificial_restart_threshold", C.c_double),
        ("sufficient_reduction_for_restart", C.c_double),
        ("necessary_reduction_for_restart", C.c_double),
        ("primal_weight_update_smoothing", C.c_double),
        ("step_size_policy", C.c_int32),
        ("precision", C.c_int32),
        ("reduction_exponent", C.c_double),
        ("growth_exponent", C.c_double),
        ("fp64_handoff_relative_kkt", C.c_double),
        ("fp64_handoff_stall_evaluations", C.c_int32),
        ("profile_kernels", C.c_int32),
        ("reserved", C.c_double * 6),
    ]


class ConvergenceInformation(C.Structure):
    _fields_ = [("candidate_type", C.c_int32), ("pad0", C.c_int32)] + [
        (name, C.c_double) for name in (
            "primal_objective", "dual_objective", "corrected_dual_objective",
            "l_inf_primal_residual", "l2_primal_residual", "l_inf_dual_residual",
            "l2_dual_residual", "relative_l_inf_primal_residual", "relative_l2_primal_residual",
            "relative_l_inf_dual_residual", "relative_l2_dual_residual",
            "relative_optimality_gap", "l_inf_primal_variable", "l2_primal_variable",
            "l_inf_dual_variable", "l2_dual_variable")
    ]


class InfeasibilityInformation(C.Structure):
    _fields_ = [("candidate_type", C.c_int32), ("pad0", C.c_int32)] + [
        (name, C.c_double) for name in (
            "max_primal_ray_infeasibility", "primal_ray_linear_objective",
            "max_dual_ray_infeasibility", "dual_ray_objective")
    ]


class IterationStats(C.Structure):
    _fields_ = [
        ("iteration_number", C.c_int32),
        ("cumulative_rejected_steps", C.c_int32),
        ("restart_used", C.c_int32),
        ("precision", C.c_int32),
        ("convergence_information", ConvergenceInformation),
        ("infeasibility_information", InfeasibilityInformation),
        ("cumulative_kkt_matrix_passes", C.c_double),
        ("cumulative_time_sec", C.c_double),
        ("step_size", C.c_double),
        ("primal_weight", C.c_double),
        ("time_spent_doing_basic_algorithm", C.c_double),
    ]


class Result(C.Structure):
    _fields_ = [
        ("termination_reason", C.c_int32),
        ("iteration_count", C.c_int32),
        ("total_number_iterations", C.c_int64),
        ("cumulative_kkt_matrix_passes", C.c_double),
        ("solve_time_sec", C.c_double),
        ("num_iteration_stats", C.c_int32),
        ("fp64_handoff_iteration", C.c_int32),
        ("last_iteration_stats", IterationStats),
        ("step_loop_device_sec", C.c_double),
        ("accepted_steps", C.c_int64),
        ("rejected_steps", C.c_int64),
        ("primal_kernel_sec", C.c_double),
        ("dual_kernel_sec", C.c_double),
        ("primal_kernel_launches", C.c_int64),
        ("primal_spmv_launches", C.c_int64),
        ("kernels_launched", C.c_int64),
    ]


class LpDesc(C.Structure):
    _fields_ = [
        ("num_variables", C.c_int32),
        ("num_constraints", C.c_int32),
        ("num_equalities", C.c_int32),
        ("pad0", C.c_int32),
        ("nnz", C.c_int64),
        ("row_ptr", _ip),
        ("col_idx", _ip),
        ("values", _dp),
        ("variable_lower_bound", _dp),
        ("variable_upper_bound", _dp),
        ("objective_vector", _dp),
        ("right_hand_side", _dp),
        ("objective_constant", C.c_double),
        ("original_variable_lower_bound", _dp),
        ("original_variable_upper_bound", _dp),
        ("original_objective_vector", _dp),
        ("original_right_hand_side", _dp),
        ("constraint_rescaling", _dp),
        ("variable_rescaling", _dp),
    ]


class TwoSidedDesc(C.Structure):
    _fields_ = [
        ("num_variables", C.c_int32),
        ("num_constraints", C.c_int32),
        ("nnz", C.c_int64),
        ("variable_lower_bound", _dp),
        ("variable_upper_bound", _dp),
        ("constraint_lower_bound", _dp),
        ("constraint_upper_bound", _dp),
        ("objective_vector", _dp),
        ("objective_offset", C.c_double),
    ]


class ServerConfig(C.Structure):
    _fields_ = [
        ("hbm_budget_bytes", C.c_double),
        ("max_resident", C.c_int32),
        ("max_cohort", C.c_int32),
        ("workers", C.c_int32),
        ("reserved_int", C.c_int32),
        ("linger_sec", C.c_double),
        ("reserved", C.c_double * 2),
    ]


# Every exported symbol of include/gpdhg.h, with its ctypes signature.
SIGNATURES = {
    "gpdhg_abi_version": (C.c_int32, []),
    "gpdhg_last_error": (C.c_char_p, []),
    "gpdhg_default_params": (None, [C.POINTER(Params)]),
    "gpdhg_problem_create": (C.c_int, [C.POINTER(LpDesc), C.POINTER(C.c_void_p)]),
    "gpdhg_problem_create_unscaled": (C.c_int, [C.POINTER(LpDesc), C.POINTER(Params),
                                                C.POINTER(C.c_void_p)]),
    "gpdhg_get_rescaling": (C.c_int, [C.c_void_p, _dp, _dp]),
    "gpdhg_problem_create_csc": (C.c_int, [C.POINTER(LpDesc), _lp, _lp, _dp, C.c_int32, C.POINTER(Params),
                                           C.POINTER(C.c_void_p)]),
    "gpdhg_problem_create_two_sided": (C.c_int, [C.POINTER(TwoSidedDesc), _lp, _lp, _dp, C.c_int32,
                                                 C.POINTER(Params), C.POINTER(C.c_void_p)]),
    "gpdhg_get_standard_form": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                          C.POINTER(C.c_int32), _ip]),
    "gpdhg_solve": (C.c_int, [C.c_void_p, C.POINTER(Params), C.POINTER(Result), _dp, _dp]),
    "gpdhg_get_stats": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(IterationStats)]),
    "gpdhg_set_warm_start": (C.c_int, [C.c_void_p, _dp, _dp]),
    "gpdhg_get_current_iterate": (C.c_int, [C.c_void_p, _dp, _dp]),
    "gpdhg_problem_destroy": (C.c_int, [C.c_void_p]),
    "gpdhg_problem_stream": (C.c_void_p, [C.c_void_p]),
    "gpdhg_batch_create": (C.c_int, [C.c_int32, C.POINTER(LpDesc), C.POINTER(C.c_void_p)]),
    "gpdhg_batch_solve": (C.c_int, [C.c_void_p, C.POINTER(Params), C.POINTER(Result),
                                    C.POINTER(_dp), C.POINTER(_dp)]),
    "gpdhg_batch_destroy": (C.c_int, [C.c_void_p]),
    "gpdhg_convergence_noalloc": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_double] + [_dp] * 8
                                  + [C.c_double, C.c_double, C.c_void_p, C.POINTER(ConvergenceInformation)]),
    "gpdhg_set_tile_override": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "gpdhg_server_footprint": (C.c_double, [C.POINTER(LpDesc), C.POINTER(Params)]),
    "gpdhg_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
    "gpdhg_server_submit": (C.c_int, [C.c_void_p, C.POINTER(LpDesc), C.POINTER(Params),
                                      C.POINTER(C.c_uint64)]),
    "gpdhg_server_poll": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(Result), _dp, _dp]),
    "gpdhg_server_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.c_double, C.POINTER(Result),
                                    _dp, _dp]),
    "gpdhg_server_destroy": (C.c_int, [C.c_void_p]),
}

_lib = None


class GpdhgError(RuntimeError):
    """A non-OK gpdhg_status, with the library's last-error text."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"gpdhg {STATUS_NAMES.get(status, status)}: {message}")


def load(path: str | None = None):
    """Loads libgpdhg.so (built in-tree by cupdlp.build). Raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"libgpdhg.so not found at {p}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.gpdhg_abi_version() != ABI_VERSION:
        raise RuntimeError("libgpdhg.so ABI version mismatch")
    if path is None:
        _lib = lib
    return lib


def check(status: int, lib=None) -> None:
    if status != OK:
        lib = lib or _lib
        msg = lib.gpdhg_last_error().decode() if lib is not None else ""
        raise GpdhgError(status, msg)


def lptr(a):
    """int64_t* of a contiguous int64 numpy array (or NULL for None)."""
    if a is None:
        return C.cast(None, _lp)
    return a.ctypes.data_as(_lp)


def dptr(a):
    """double* of a contiguous float64 numpy array (or NULL for None)."""
    if a is None:
        return C.cast(None, _dp)
    return a.ctypes.data_as(_dp)


def iptr(a):
    if a is None:
        return C.cast(None, _ip)
    return a.ctypes.data_as(_ip)
