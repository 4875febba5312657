"""cupdlp — host-side mirror of cuPDLP.jl's API over libgpdhg.so (GB300, sm_103a).

The names follow the Julia module (src/cuPDLP.jl): `optimize`, `PdhgParameters`,
`QuadraticProgrammingProblem`, `rescale_problem`, `construct_termination_criteria`,
`construct_restart_parameters`, the enums, and the result types. The solve loop itself
runs in libgpdhg.so; this package never computes it on the CPU.
"""
from .types import *  # noqa: F401,F403
from .types import (AdaptiveStepsizeParams, ConstantStepsizeParams, ConvergenceInformation,  # noqa: F401
                    InfeasibilityInformation, IterationStats, PdhgParameters, Precision,
                    QuadraticProgrammingProblem, RestartParameters, SaddlePointOutput, ScaledQpProblem,
                    SolveLog, TerminationCriteria, TerminationReason, TwoSidedQpProblem, construct_restart_parameters,
                    construct_termination_criteria, default_parameters, default_restart_parameters,
                    params_to_c, termination_reason_to_string, validate_termination_criteria)
from .preprocess import (InfeasibleProblemError, InvalidProblemError, PresolveInfo,  # noqa: F401
                         l2_norm_rescaling, pock_chambolle_rescaling, presolve, rescale_problem, ruiz_rescaling,
                         scale_problem, undo_presolve, unscale_problem, validate)
from .solver import (DeviceBatch, DeviceProblem, Server, optimize, optimize_batch, scaled_desc,  # noqa: F401
                     unscaled_desc)
from . import _abi  # noqa: F401
from . import layout  # noqa: F401

__all__ = [n for n in dir() if not n.startswith("_")]
