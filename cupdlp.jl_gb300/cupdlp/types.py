"""Host-side types mirroring cuPDLP.jl's public API, field for field.

  QuadraticProgrammingProblem   src/quadratic_programming.jl:25-67
  ScaledQpProblem               src/quadratic_programming.jl:284-289
  TerminationCriteria           src/termination.jl:9-99
  RestartParameters             src/saddle_point_gpu.jl:353-414
  AdaptiveStepsizeParams,
  ConstantStepsizeParams,
  PdhgParameters                src/primal_dual_hybrid_gradient_gpu.jl:2-24
  ConvergenceInformation,
  InfeasibilityInformation,
  IterationStats, SolveLog      src/solve_log.jl:51-413
  SaddlePointOutput             src/saddle_point_gpu.jl:3-34
Enums keep the reference's names and 0-based values.
"""
from __future__ import annotations

import dataclasses
import enum
import math
from typing import Dict, List, Optional, Union

import numpy as np
import scipy.sparse as sp

from . import _abi


class OptimalityNorm(enum.IntEnum):
    L_INF = 0
    L2 = 1


class RestartScheme(enum.IntEnum):
    NO_RESTARTS = 0
    FIXED_FREQUENCY = 1
    ADAPTIVE_KKT = 2


class RestartToCurrentMetric(enum.IntEnum):
    NO_RESTART_TO_CURRENT = 0
    KKT_GREEDY = 1


class RestartChoice(enum.IntEnum):
    RESTART_CHOICE_UNSPECIFIED = 0
    RESTART_CHOICE_NO_RESTART = 1
    RESTART_CHOICE_WEIGHTED_AVERAGE_RESET = 2
    RESTART_CHOICE_RESTART_TO_AVERAGE = 3


class PointType(enum.IntEnum):
    POINT_TYPE_UNSPECIFIED = 0
    POINT_TYPE_CURRENT_ITERATE = 1
    POINT_TYPE_ITERATE_DIFFERENCE = 2
    POINT_TYPE_AVERAGE_ITERATE = 3
    POINT_TYPE_NONE = 4


class TerminationReason(enum.IntEnum):
    TERMINATION_REASON_UNSPECIFIED = 0
    TERMINATION_REASON_OPTIMAL = 1
    TERMINATION_REASON_PRIMAL_INFEASIBLE = 2
    TERMINATION_REASON_DUAL_INFEASIBLE = 3
    TERMINATION_REASON_TIME_LIMIT = 4
    TERMINATION_REASON_ITERATION_LIMIT = 5
    TERMINATION_REASON_KKT_MATRIX_PASS_LIMIT = 6
    TERMINATION_REASON_NUMERICAL_ERROR = 7
    TERMINATION_REASON_INVALID_PROBLEM = 8
    TERMINATION_REASON_OTHER = 9


class Precision(enum.IntEnum):
    """Arithmetic of the bulk iteration (an addition; the reference is FP64 only)."""
    FP64 = _abi.PRECISION_FP64
    FP32_REFINE = _abi.PRECISION_FP32_REFINE
    FP32 = _abi.PRECISION_FP32


# Module-level aliases so call sites read like the reference (cuPDLP.ADAPTIVE_KKT ...).
L_INF, L2 = OptimalityNorm.L_INF, OptimalityNorm.L2
NO_RESTARTS, FIXED_FREQUENCY, ADAPTIVE_KKT = (RestartScheme.NO_RESTARTS, RestartScheme.FIXED_FREQUENCY,
                                              RestartScheme.ADAPTIVE_KKT)
NO_RESTART_TO_CURRENT, KKT_GREEDY = (RestartToCurrentMetric.NO_RESTART_TO_CURRENT,
                                     RestartToCurrentMetric.KKT_GREEDY)
globals().update({m.name: m for m in TerminationReason})
globals().update({m.name: m for m in PointType})
globals().update({m.name: m for m in RestartChoice})


def termination_reason_to_string(reason: TerminationReason) -> str:
    """src/termination.jl:248-251: the enum name without TERMINATION_REASON_."""
    return TerminationReason(reason).name[len("TERMINATION_REASON_"):]


@dataclasses.dataclass
class QuadraticProgrammingProblem:
    """min c'x + c0  s.t.  A[:neq] x = b[:neq],  A[neq:] x >= b[neq:],  l <= x <= u."""
    variable_lower_bound: np.ndarray
    variable_upper_bound: np.ndarray
    objective_matrix: sp.spmatrix
    objective_vector: np.ndarray
    objective_constant: float
    constraint_matrix: sp.spmatrix
    right_hand_side: np.ndarray
    num_equalities: int

    @property
    def num_variables(self) -> int:
        return int(self.constraint_matrix.shape[1])

    @property
    def num_constraints(self) -> int:
        return int(self.constraint_matrix.shape[0])


@dataclasses.dataclass
class TwoSidedQpProblem:
    """TwoSidedQpProblem (src/quadratic_programming_io.jl:5-22) of an LP: l <= x <= u and
    constraint_lower_bound <= A x <= constraint_upper_bound (the MPS reader's form)."""
    variable_lower_bound: np.ndarray
    variable_upper_bound: np.ndarray
    constraint_lower_bound: np.ndarray
    constraint_upper_bound: np.ndarray
    constraint_matrix: sp.spmatrix
    objective_offset: float
    objective_vector: np.ndarray

    @property
    def num_variables(self) -> int:
        return int(self.constraint_matrix.shape[1])

    @property
    def num_constraints(self) -> int:
        return int(self.constraint_matrix.shape[0])


@dataclasses.dataclass
class ScaledQpProblem:
    original_qp: QuadraticProgrammingProblem
    scaled_qp: QuadraticProgrammingProblem
    constraint_rescaling: np.ndarray
    variable_rescaling: np.ndarray


@dataclasses.dataclass
class TerminationCriteria:
    optimality_norm: OptimalityNorm = OptimalityNorm.L2
    eps_optimal_absolute: float = 1.0e-6
    eps_optimal_relative: float = 1.0e-6
    eps_primal_infeasible: float = 1.0e-8
    eps_dual_infeasible: float = 1.0e-8
    time_sec_limit: float = math.inf
    iteration_limit: int = 2**31 - 1
    kkt_matrix_pass_limit: float = math.inf


def construct_termination_criteria(*, optimality_norm=OptimalityNorm.L2, eps_optimal_absolute=1.0e-6,
                                   eps_optimal_relative=1.0e-6, eps_primal_infeasible=1.0e-8,
                                   eps_dual_infeasible=1.0e-8, time_sec_limit=math.inf,
                                   iteration_limit=2**31 - 1, kkt_matrix_pass_limit=math.inf):
    """src/termination.jl:79-99 (same keyword defaults)."""
    return TerminationCriteria(optimality_norm, eps_optimal_absolute, eps_optimal_relative,
                               eps_primal_infeasible, eps_dual_infeasible, time_sec_limit,
                               int(iteration_limit), kkt_matrix_pass_limit)


def validate_termination_criteria(criteria: TerminationCriteria) -> None:
    """src/termination.jl:101-117."""
    if criteria.eps_primal_infeasible < 0:
        raise ValueError("eps_primal_infeasible must be nonnegative")
    if criteria.eps_dual_infeasible < 0:
        raise ValueError("eps_dual_infeasible must be nonnegative")
    if criteria.time_sec_limit <= 0:
        raise ValueError("time_sec_limit must be positive")
    if criteria.iteration_limit <= 0:
        raise ValueError("iteration_limit must be positive")
    if criteria.kkt_matrix_pass_limit <= 0:
        raise ValueError("kkt_matrix_pass_limit must be positive")


@dataclasses.dataclass
class RestartParameters:
    restart_scheme: RestartScheme
    restart_to_current_metric: RestartToCurrentMetric
    restart_frequency_if_fixed: int
    artificial_restart_threshold: float
    sufficient_reduction_for_restart: float
    necessary_reduction_for_restart: float
    primal_weight_update_smoothing: float


def construct_restart_parameters(restart_scheme, restart_to_current_metric, restart_frequency_if_fixed,
                                 artificial_restart_threshold, sufficient_reduction_for_restart,
                                 necessary_reduction_for_restart, primal_weight_update_smoothing):
    """src/saddle_point_gpu.jl:388-414, with its assertions."""
    assert restart_frequency_if_fixed > 1
    assert 0.0 < artificial_restart_threshold <= 1.0
    assert 0.0 < sufficient_reduction_for_restart <= necessary_reduction_for_restart <= 1.0
    assert 0.0 <= primal_weight_update_smoothing <= 1.0
    return RestartParameters(RestartScheme(restart_scheme), RestartToCurrentMetric(restart_to_current_metric),
                             int(restart_frequency_if_fixed), float(artificial_restart_threshold),
                             float(sufficient_reduction_for_restart), float(necessary_reduction_for_restart),
                             float(primal_weight_update_smoothing))


@dataclasses.dataclass
class AdaptiveStepsizeParams:
    reduction_exponent: float
    growth_exponent: float


@dataclasses.dataclass
class ConstantStepsizeParams:
    pass


@dataclasses.dataclass
class PdhgParameters:
    """Positional order as src/primal_dual_hybrid_gradient_gpu.jl:9-24; `precision`,
    `fp64_handoff_relative_kkt` and `fp64_handoff_stall_evaluations` are appended
    additions, so old positional call sites stay valid."""
    l_inf_ruiz_iterations: int
    l2_norm_rescaling: bool
    pock_chambolle_alpha: Optional[float]
    primal_importance: float
    scale_invariant_initial_primal_weight: bool
    verbosity: int
    record_iteration_stats: bool
    termination_evaluation_frequency: int
    termination_criteria: TerminationCriteria
    restart_params: RestartParameters
    step_size_policy_params: Union[AdaptiveStepsizeParams, ConstantStepsizeParams]
    precision: Precision = Precision.FP64
    fp64_handoff_relative_kkt: float = 1.0e-6
    fp64_handoff_stall_evaluations: int = 20


def default_restart_parameters() -> RestartParameters:
    """The restart parameters of scripts/solve.jl:163-171 and src/MOI_wrapper.jl:68-76."""
    return construct_restart_parameters(ADAPTIVE_KKT, KKT_GREEDY, 1000, 0.36, 0.2, 0.8, 0.5)


def default_parameters(tolerance: float = 1e-4, time_sec_limit: float = 3600.0, verbosity: int = 0,
                       iteration_limit: int = 2**31 - 1, precision: Precision = Precision.FP64,
                       record_iteration_stats: bool = True) -> PdhgParameters:
    """PdhgParameters exactly as scripts/solve.jl:173-196 builds them for --tolerance."""
    tc = construct_termination_criteria(eps_optimal_absolute=tolerance, eps_optimal_relative=tolerance,
                                        eps_primal_infeasible=1.0e-8, eps_dual_infeasible=1.0e-8,
                                        time_sec_limit=time_sec_limit, iteration_limit=iteration_limit,
                                        kkt_matrix_pass_limit=math.inf)
    return PdhgParameters(10, False, 1.0, 1.0, True, verbosity, record_iteration_stats, 64, tc,
                          default_restart_parameters(), AdaptiveStepsizeParams(0.3, 0.6),
                          precision=Precision(precision))


def params_to_c(p: PdhgParameters) -> _abi.Params:
    """Flattens PdhgParameters into the C gpdhg_params struct."""
    c = _abi.Params()
    c.l_inf_ruiz_iterations = int(p.l_inf_ruiz_iterations)
    c.l2_norm_rescaling = int(bool(p.l2_norm_rescaling))
    c.pock_chambolle_alpha = math.nan if p.pock_chambolle_alpha is None else float(p.pock_chambolle_alpha)
    c.primal_importance = float(p.primal_importance)
    c.scale_invariant_initial_primal_weight = int(bool(p.scale_invariant_initial_primal_weight))
    c.verbosity = int(p.verbosity)
    c.record_iteration_stats = int(bool(p.record_iteration_stats))
    c.termination_evaluation_frequency = int(p.termination_evaluation_frequency)
    tc = p.termination_criteria
    c.optimality_norm = int(tc.optimality_norm)
    c.iteration_limit = int(min(tc.iteration_limit, 2**31 - 1))
    c.eps_optimal_absolute = float(tc.eps_optimal_absolute)
    c.eps_optimal_relative = float(tc.eps_optimal_relative)
    c.eps_primal_infeasible = float(tc.eps_primal_infeasible)
    c.eps_dual_infeasible = float(tc.eps_dual_infeasible)
    c.time_sec_limit = float(tc.time_sec_limit)
    c.kkt_matrix_pass_limit = float(tc.kkt_matrix_pass_limit)
    rp = p.restart_params
    c.restart_scheme = int(rp.restart_scheme)
    c.restart_to_current_metric = int(rp.restart_to_current_metric)
    c.restart_frequency_if_fixed = int(rp.restart_frequency_if_fixed)
    c.artificial_restart_threshold = float(rp.artificial_restart_threshold)
    c.sufficient_reduction_for_restart = float(rp.sufficient_reduction_for_restart)
    c.necessary_reduction_for_restart = float(rp.necessary_reduction_for_restart)
    c.primal_weight_update_smoothing = float(rp.primal_weight_update_smoothing)
    sp_ = p.step_size_policy_params
    if isinstance(sp_, AdaptiveStepsizeParams):
        c.step_size_policy = 0
        c.reduction_exponent = float(sp_.reduction_exponent)
        c.growth_exponent = float(sp_.growth_exponent)
    else:
        c.step_size_policy = 1
        c.reduction_exponent = 0.3
        c.growth_exponent = 0.6
    c.precision = int(p.precision)
    c.fp64_handoff_relative_kkt = float(p.fp64_handoff_relative_kkt)
    c.fp64_handoff_stall_evaluations = int(p.fp64_handoff_stall_evaluations)
    return c


@dataclasses.dataclass
class ConvergenceInformation:
    candidate_type: PointType = PointType.POINT_TYPE_UNSPECIFIED
    primal_objective: float = 0.0
    dual_objective: float = 0.0
    corrected_dual_objective: float = 0.0
    l_inf_primal_residual: float = 0.0
    l2_primal_residual: float = 0.0
    l_inf_dual_residual: float = 0.0
    l2_dual_residual: float = 0.0
    relative_l_inf_primal_residual: float = 0.0
    relative_l2_primal_residual: float = 0.0
    relative_l_inf_dual_residual: float = 0.0
    relative_l2_dual_residual: float = 0.0
    relative_optimality_gap: float = 0.0
    l_inf_primal_variable: float = 0.0
    l2_primal_variable: float = 0.0
    l_inf_dual_variable: float = 0.0
    l2_dual_variable: float = 0.0


@dataclasses.dataclass
class InfeasibilityInformation:
    candidate_type: PointType = PointType.POINT_TYPE_UNSPECIFIED
    max_primal_ray_infeasibility: float = 0.0
    primal_ray_linear_objective: float = 0.0
    max_dual_ray_infeasibility: float = 0.0
    dual_ray_objective: float = 0.0


@dataclasses.dataclass
class IterationStats:
    iteration_number: int = 0
    convergence_information: List[ConvergenceInformation] = dataclasses.field(default_factory=list)
    infeasibility_information: List[InfeasibilityInformation] = dataclasses.field(default_factory=list)
    cumulative_kkt_matrix_passes: float = 0.0
    cumulative_rejected_steps: int = 0
    cumulative_time_sec: float = 0.0
    restart_used: RestartChoice = RestartChoice.RESTART_CHOICE_UNSPECIFIED
    step_size: float = 0.0
    primal_weight: float = 0.0
    method_specific_stats: Dict[str, float] = dataclasses.field(default_factory=dict)


def stats_from_c(s: _abi.IterationStats) -> IterationStats:
    ci = s.convergence_information
    ii = s.infeasibility_information
    conv = ConvergenceInformation(PointType(ci.candidate_type), *[
        getattr(ci, f.name) for f in dataclasses.fields(ConvergenceInformation)[1:]])
    inf = InfeasibilityInformation(PointType(ii.candidate_type), *[
        getattr(ii, f.name) for f in dataclasses.fields(InfeasibilityInformation)[1:]])
    return IterationStats(
        iteration_number=s.iteration_number, convergence_information=[conv], infeasibility_information=[inf],
        cumulative_kkt_matrix_passes=s.cumulative_kkt_matrix_passes,
        cumulative_rejected_steps=s.cumulative_rejected_steps, cumulative_time_sec=s.cumulative_time_sec,
        restart_used=RestartChoice(s.restart_used), step_size=s.step_size, primal_weight=s.primal_weight,
        method_specific_stats={"time_spent_doing_basic_algorithm": s.time_spent_doing_basic_algorithm,
                               "precision": float(s.precision)})


@dataclasses.dataclass
class SaddlePointOutput:
    primal_solution: np.ndarray
    dual_solution: np.ndarray
    termination_reason: TerminationReason
    termination_string: str
    iteration_count: int
    iteration_stats: List[IterationStats]
    # additions: the raw C result (KKT passes, attempts, device loop time, FP64 hand-off)
    result: Optional[_abi.Result] = None


@dataclasses.dataclass
class SolveLog:
    """src/solve_log.jl:336-407."""
    instance_name: str = ""
    command_line_invocation: str = ""
    termination_reason: TerminationReason = TerminationReason.TERMINATION_REASON_UNSPECIFIED
    termination_string: str = ""
    iteration_count: int = 0
    solve_time_sec: float = 0.0
    solution_stats: IterationStats = dataclasses.field(default_factory=IterationStats)
    solution_type: PointType = PointType.POINT_TYPE_UNSPECIFIED
    iteration_stats: List[IterationStats] = dataclasses.field(default_factory=list)
