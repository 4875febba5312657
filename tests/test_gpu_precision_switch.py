"""GPU tests of the FP64 workspace of a handle used for several precisions: an FP32_REFINE
solve gives the same result, bit for bit, whether its FP64 workspace existed before the solve
or was built at the hand-off, and an FP64 solve after an FP32_REFINE solve that ended in its
FP32 phase equals the FP64 solve of a fresh handle."""
import numpy as np
import pytest

import cupdlp
from cupdlp import synthetic
from cupdlp.solver import DeviceProblem, scaled_desc

pytestmark = pytest.mark.gpu


def _scaled(seed=21):
    p = synthetic.known_optimum_lp(seed, m=800, n=1600, density=0.01).problem
    return cupdlp.rescale_problem(10, False, 1.0, 0, p)


def _params(precision, tol):
    return cupdlp.default_parameters(tolerance=tol, precision=precision, iteration_limit=60_000,
                                     time_sec_limit=300.0)


def _same(a, b):
    (ra, xa, ya), (rb, xb, yb) = a, b
    assert ra.termination_reason == rb.termination_reason
    assert ra.iteration_count == rb.iteration_count
    assert ra.fp64_handoff_iteration == rb.fp64_handoff_iteration
    assert np.array_equal(xa, xb) and np.array_equal(ya, yb)


def test_refine_result_does_not_depend_on_when_the_fp64_workspace_was_built():
    d = scaled_desc(_scaled())
    refine = _params(cupdlp.Precision.FP32_REFINE, 1e-8)
    with DeviceProblem(d) as dp:
        fresh = dp.solve(refine)              # FP64 workspace built at the hand-off
    with DeviceProblem(d) as dp:
        dp.solve(_params(cupdlp.Precision.FP64, 1e-4))   # FP64 workspace built up front
        warm = dp.solve(refine)
        again = dp.solve(refine)              # both workspaces cached
    assert fresh[0].fp64_handoff_iteration > 0
    _same(fresh, warm)
    _same(fresh, again)


def test_fp64_solve_after_a_refine_solve_that_ended_in_fp32():
    d = scaled_desc(_scaled(22))
    p64 = _params(cupdlp.Precision.FP64, 1e-6)
    with DeviceProblem(d) as dp:
        early = dp.solve(_params(cupdlp.Precision.FP32_REFINE, 1e-3))   # ends in the FP32 phase
        assert early[0].fp64_handoff_iteration < 0
        after = dp.solve(p64)
    with DeviceProblem(d) as dp:
        alone = dp.solve(p64)
    _same(after, alone)
