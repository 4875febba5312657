"""GPU tests of the batched solve (gpdhg_batch_*): every instance of a packed batch
terminates exactly as it does alone (same kernels, same per-CTA schedule, same
reduction order, so bit for bit), and mixed-size batches reach the planted optimum."""
import numpy as np
import pytest

import cupdlp
from cupdlp import synthetic
from cupdlp.solver import DeviceBatch, DeviceProblem, scaled_desc

import instances

pytestmark = pytest.mark.gpu

OPT = cupdlp.TerminationReason.TERMINATION_REASON_OPTIMAL


def _params(**kw):
    kw.setdefault("time_sec_limit", 120.0)
    return cupdlp.default_parameters(**kw)


def _mix(seed=21, count=12):
    lps = synthetic.batch_lps(seed, count=count, median_m=400, m_range=(60, 3000))
    lps.append(synthetic.known_optimum_lp(5, m=50, n=80, neq=50, density=0.1))   # equalities only
    lps.append(synthetic.known_optimum_lp(6, m=50, n=80, neq=0, density=0.1))    # inequalities only
    return lps


@pytest.mark.parametrize("precision", [cupdlp.Precision.FP64, cupdlp.Precision.FP32])
def test_batch_equals_alone_bitwise(precision):
    lps = _mix()
    # FP32 runs at its own tolerance; the iteration limit keeps every instance's end
    # independent of the wall clock, so the two runs must match exactly either way
    tol = 1e-6 if precision == cupdlp.Precision.FP64 else 1e-4
    params = _params(tolerance=tol, precision=precision, iteration_limit=100_000)
    scaled = [cupdlp.rescale_problem(10, False, 1.0, 0, lp.problem) for lp in lps]
    with DeviceBatch([scaled_desc(sq) for sq in scaled]) as db:
        results, xs, ys = db.solve(params)
    for k, sq in enumerate(scaled):
        with DeviceProblem(scaled_desc(sq)) as dp:
            r, x, y = dp.solve(params)
        assert results[k].termination_reason == r.termination_reason, k
        assert results[k].iteration_count == r.iteration_count, k
        assert results[k].total_number_iterations == r.total_number_iterations, k
        assert np.array_equal(xs[k], x), k
        assert np.array_equal(ys[k], y), k
        gb = results[k].last_iteration_stats.convergence_information
        ga = r.last_iteration_stats.convergence_information
        assert gb.primal_objective == ga.primal_objective and gb.dual_objective == ga.dual_objective


def test_batch_reaches_planted_optimum():
    lps = _mix(seed=22, count=16)
    outs = cupdlp.optimize_batch(_params(tolerance=1e-8), [lp.problem for lp in lps])
    for lp, out in zip(lps, outs):
        assert out.termination_reason == OPT, lp.name
        if lp.optimal_objective is not None:
            ci = out.iteration_stats[-1].convergence_information[0]
            assert ci.primal_objective == pytest.approx(lp.optimal_objective, rel=1e-6), lp.name


def test_batch_with_edge_instances():
    """Instances without constraints, infeasible and unbounded ones, next to normal LPs:
    each one terminates with its own reason."""
    probs = [instances.no_constraints(), instances.primal_infeasible(), instances.dual_infeasible(),
             instances.tiny()[0], synthetic.known_optimum_lp(7, m=100, n=200, density=0.05).problem]
    outs = cupdlp.optimize_batch(_params(tolerance=1e-6), probs)
    reasons = [o.termination_reason for o in outs]
    assert reasons == [OPT, cupdlp.TERMINATION_REASON_PRIMAL_INFEASIBLE, cupdlp.TERMINATION_REASON_DUAL_INFEASIBLE,
                       OPT, OPT]
