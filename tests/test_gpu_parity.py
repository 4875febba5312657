"""GPU parity: libgpdhg.so (through its C ABI) against the CPU oracle.

Both sides get the same scaled problem (the host package's rescale_problem) and the
same parameters. The reference loop is chaotic in floating point: the oracle rebuilt
with another summation order drifts from itself to ~1e-6 relative objective by
iteration 1,000 and needs up to 30% more or fewer iterations, although every decision
it takes is well away from its threshold. So parity is checked in three layers:
  * short horizon (first 30 iterations): statistics, iterates and every restart
    decision agree to rtol 1e-9;
  * longer horizon: each statistic stays within 100x the distance between the oracle
    and its perturbed-summation twin (the round-off envelope);
  * converged: at tolerance 1e-8 the primal and dual objectives agree to 1e-6
    relative, the correctness bar of the task, and the solution meets the reference's
    relative-KKT criteria when recomputed independently in numpy.
"""
import json
import os

import numpy as np
import pytest

import cupdlp
from cupdlp import synthetic
from cupdlp.solver import DeviceProblem, scaled_desc

import instances
from golden.make_golden import make
from kkt import kkt_measures, meets_tolerance

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))
OPT = cupdlp.TerminationReason.TERMINATION_REASON_OPTIMAL


def _params(**kw):
    """The CLI's parameters with a 120 s time limit, so a regression cannot run for an hour."""
    kw.setdefault("time_sec_limit", 120.0)
    return cupdlp.default_parameters(**kw)


def solve_both(problem, params, perturbed=False):
    import oracle
    sq = cupdlp.rescale_problem(params.l_inf_ruiz_iterations, params.l2_norm_rescaling,
                                params.pock_chambolle_alpha, 0, problem)
    with DeviceProblem(scaled_desc(sq)) as dp:
        res, xa, ya = dp.solve(params)
        stats = dp.stats(res.num_iteration_stats)
        xc, yc = dp.current_iterate()
    orc = oracle.solve_scaled(sq, params)
    pert = oracle.solve_scaled(sq, params, perturbed=True) if perturbed else None
    return sq, (res, xa, ya, stats, xc, yc), orc, pert


FIELDS = ["primal_objective", "dual_objective", "l2_primal_residual", "l2_dual_residual",
          "l_inf_primal_residual", "l_inf_dual_residual", "l2_primal_variable", "l2_dual_variable"]


def _rel(a, b):
    d = abs(a - b)
    s = max(abs(a), abs(b))
    return d / s if s > 0 else 0.0


def same_restart(g, o, equivalent):
    if equivalent:   # a KKT_GREEDY tie between numerically identical points
        return (g > 1) == (o > 1)
    return g == o


def compare_strict(gpu_stats, orc, rtol):
    assert len(gpu_stats) == len(orc.stats)
    for k, (g, o) in enumerate(zip(gpu_stats, orc.stats)):
        assert g.iteration_number == o.iteration_number
        assert same_restart(int(g.restart_used), o.restart_used, orc.greedy_equivalent[k]), (k, g.restart_used,
                                                                                             o.restart_used)
        assert g.cumulative_kkt_matrix_passes == o.cumulative_kkt_matrix_passes
        assert _rel(g.step_size, o.step_size) <= rtol and _rel(g.primal_weight, o.primal_weight) <= rtol
        gi, oi = g.convergence_information[0], o.convergence_information
        for f in FIELDS:
            assert _rel(getattr(gi, f), getattr(oi, f)) <= rtol, (k, f, getattr(gi, f), getattr(oi, f))


def compare_envelope(gpu_stats, orc, pert, factor=100.0, floor=1e-10):
    """Each statistic within `factor` x the running oracle-vs-perturbed distance."""
    n = min(len(gpu_stats), len(orc.stats), len(pert.stats))
    env = dict.fromkeys(FIELDS, 0.0)
    worst = 0.0
    for k in range(n):
        gi = gpu_stats[k].convergence_information[0]
        oi, qi = orc.stats[k].convergence_information, pert.stats[k].convergence_information
        for f in FIELDS:
            env[f] = max(env[f], _rel(getattr(oi, f), getattr(qi, f)))
            d = _rel(getattr(gi, f), getattr(oi, f))
            assert d <= factor * env[f] + floor, (k, f, d, env[f])
            worst = max(worst, d)
    return worst


@pytest.mark.parametrize("iters", [1, 5, 10, 30])
def test_fp64_trajectory_short_horizon(iters):
    p = synthetic.known_optimum_lp(0).problem
    params = _params(tolerance=1e-10, iteration_limit=iters)
    sq, (res, xa, ya, stats, xc, yc), orc, _ = solve_both(p, params)
    assert res.termination_reason == orc.result.termination_reason
    assert res.iteration_count == orc.result.iteration_count
    assert res.total_number_iterations == orc.result.total_number_iterations
    compare_strict(stats, orc, rtol=1e-9)
    scale = lambda v: 1e-9 * max(1.0, np.abs(v).max())
    np.testing.assert_allclose(xa, orc.x_avg, rtol=0, atol=scale(orc.x_avg))
    np.testing.assert_allclose(ya, orc.y_avg, rtol=0, atol=scale(orc.y_avg))
    np.testing.assert_allclose(xc, orc.x_cur, rtol=0, atol=scale(orc.x_cur))
    np.testing.assert_allclose(yc, orc.y_cur, rtol=0, atol=scale(orc.y_cur))


@pytest.mark.parametrize("entry", GOLDEN["instances"], ids=lambda e: f"{e['gen']}-{e['seed']}")
@pytest.mark.parametrize("iters", [100, 300])
def test_fp64_trajectory_within_roundoff_envelope(entry, iters):
    p = make(entry).problem
    params = _params(tolerance=1e-10, iteration_limit=iters)
    sq, (res, *_rest), orc, pert = solve_both(p, params, perturbed=True)
    stats = _rest[2]
    compare_envelope(stats, orc, pert)


@pytest.mark.parametrize("entry", GOLDEN["instances"], ids=lambda e: f"{e['gen']}-{e['seed']}")
def test_fp64_full_solve_matches_oracle(entry):
    p = make(entry).problem
    params = _params(tolerance=1e-8)
    sq, (res, xa, ya, stats, xc, yc), orc, _ = solve_both(p, params)
    assert res.termination_reason == OPT and orc.result.termination_reason == OPT
    g = res.last_iteration_stats.convergence_information
    o = orc.result.last_iteration_stats.convergence_information
    assert _rel(g.primal_objective, o.primal_objective) <= 1e-6
    assert _rel(g.dual_objective, o.dual_objective) <= 1e-6
    assert 0.5 * orc.result.iteration_count <= res.iteration_count <= 2.0 * orc.result.iteration_count + 64


def test_fp64_tolerance_1e4_against_fp64_oracle():
    """At 1e-4 two correct runs stop at different points; each result is held to the
    FP64 oracle at 1e-8 (objective error stated), and to the oracle at 1e-4 within the
    oracle's own round-off envelope."""
    lp = synthetic.known_optimum_lp(0)
    p = lp.problem
    sq, (res, xa, ya, *_), orc, pert = solve_both(p, _params(tolerance=1e-4), perturbed=True)
    assert res.termination_reason == OPT
    g = res.last_iteration_stats.convergence_information
    ref8 = GOLDEN["instances"][0]["highs_objective"]
    assert _rel(g.primal_objective, ref8) <= 2e-4
    o = orc.result.last_iteration_stats.convergence_information
    q = pert.result.last_iteration_stats.convergence_information
    assert _rel(g.primal_objective, o.primal_objective) <= max(1e-6, 10 * _rel(o.primal_objective, q.primal_objective))
    ok, k = meets_tolerance(p, xa / sq.variable_rescaling, ya / sq.constraint_rescaling, 1e-4, slack=1.01)
    assert ok, k


@pytest.mark.parametrize("entry", GOLDEN["instances"], ids=lambda e: f"{e['gen']}-{e['seed']}")
def test_golden_instances_reach_highs_optimum(entry):
    p = make(entry).problem
    out = cupdlp.optimize(_params(tolerance=1e-8), p)
    assert out.termination_reason == OPT
    ci = out.iteration_stats[-1].convergence_information[0]
    assert ci.primal_objective == pytest.approx(entry["highs_objective"], rel=1e-6)
    assert ci.dual_objective == pytest.approx(entry["highs_objective"], rel=1e-6)
    ok, k = meets_tolerance(p, out.primal_solution, out.dual_solution, 1e-8, slack=1.01)
    assert ok, k


@pytest.mark.parametrize("entry", GOLDEN["instances"], ids=lambda e: f"{e['gen']}-{e['seed']}")
def test_golden_fixed_iterations(entry):
    """100 iterations against the committed fixtures, within the fixtures' own envelope."""
    p = make(entry).problem
    out = cupdlp.optimize(_params(tolerance=1e-8, iteration_limit=100), p)
    g, q = entry["oracle_it100"], entry["oracle_it100_perturbed"]
    ci = out.iteration_stats[-1].convergence_information[0]
    for f in ("primal_objective", "l2_dual_residual"):
        env = _rel(g[f], q[f])
        assert _rel(getattr(ci, f), g[f]) <= 100 * env + 1e-10, (f, getattr(ci, f), g[f], env)
    assert out.iteration_stats[-1].cumulative_kkt_matrix_passes == g["kkt_passes"]


def test_no_constraints():
    out = cupdlp.optimize(_params(tolerance=1e-8), instances.no_constraints())
    assert out.termination_reason == OPT
    np.testing.assert_allclose(out.primal_solution, [-1.0, 3.0, -1.0], atol=1e-6)


def test_primal_infeasible():
    out = cupdlp.optimize(_params(tolerance=1e-6), instances.primal_infeasible())
    assert out.termination_reason == cupdlp.TERMINATION_REASON_PRIMAL_INFEASIBLE


def test_dual_infeasible():
    out = cupdlp.optimize(_params(tolerance=1e-6), instances.dual_infeasible())
    assert out.termination_reason == cupdlp.TERMINATION_REASON_DUAL_INFEASIBLE


def test_free_variables():
    p, obj = instances.free_variables()
    out = cupdlp.optimize(_params(tolerance=1e-8), p)
    assert out.termination_reason == OPT
    assert out.iteration_stats[-1].convergence_information[0].primal_objective == pytest.approx(obj, rel=1e-6, abs=1e-6)


def test_tiny_and_empty_rows():
    p, obj = instances.tiny()
    out = cupdlp.optimize(_params(tolerance=1e-8), p)
    assert out.termination_reason == OPT and out.primal_solution[0] == pytest.approx(1.0, abs=1e-6)
    p = instances.empty_rows_and_columns()
    import oracle
    params = _params(tolerance=1e-8)
    out = cupdlp.optimize(params, p)
    res, x, y, _ = oracle.optimize(p, params)
    assert out.termination_reason == res.termination_reason == OPT
    np.testing.assert_allclose(out.primal_solution, x, atol=1e-6)


def test_constant_step_policy_matches_oracle():
    p = synthetic.known_optimum_lp(11, m=200, n=400, density=0.03).problem
    params = _params(tolerance=1e-6)
    params.step_size_policy_params = cupdlp.ConstantStepsizeParams()
    sq, (res, *_), orc, _ = solve_both(p, params)
    assert res.termination_reason == orc.result.termination_reason == OPT
    g = res.last_iteration_stats.convergence_information
    o = orc.result.last_iteration_stats.convergence_information
    assert g.primal_objective == pytest.approx(o.primal_objective, rel=1e-6)


def test_repeat_solve_is_bitwise_deterministic():
    p = synthetic.known_optimum_lp(11, m=200, n=400, density=0.03).problem
    sq = cupdlp.rescale_problem(10, False, 1.0, 0, p)
    params = _params(tolerance=1e-6)
    with DeviceProblem(scaled_desc(sq)) as dp:
        r1, x1, y1 = dp.solve(params)
        r2, x2, y2 = dp.solve(params)
    assert r1.iteration_count == r2.iteration_count
    assert np.array_equal(x1, x2) and np.array_equal(y1, y2)


def test_warm_start_from_solution_converges_fast():
    lp = synthetic.known_optimum_lp(11, m=200, n=400, density=0.03)
    sq = cupdlp.rescale_problem(10, False, 1.0, 0, lp.problem)
    params = _params(tolerance=1e-6)
    with DeviceProblem(scaled_desc(sq)) as dp:
        r0, xs, ys = dp.solve(params)
        dp.set_warm_start(xs, ys)
        r1, _, _ = dp.solve(params)
    assert r1.termination_reason == OPT
    assert r1.iteration_count < r0.iteration_count


@pytest.mark.parametrize("precision", [cupdlp.Precision.FP32])
def test_fp32_bulk_reaches_1e4(precision):
    lp = synthetic.known_optimum_lp(0)
    params = _params(tolerance=1e-4, precision=precision)
    out = cupdlp.optimize(params, lp.problem)
    assert out.termination_reason == OPT
    ok, k = meets_tolerance(lp.problem, out.primal_solution, out.dual_solution, 1e-4, slack=1.05)
    assert ok, k
    assert k["primal_objective"] == pytest.approx(lp.optimal_objective, rel=1e-3)


def test_fp32_refine_reaches_1e8():
    lp = synthetic.known_optimum_lp(0)
    params = _params(tolerance=1e-8, precision=cupdlp.Precision.FP32_REFINE)
    out = cupdlp.optimize(params, lp.problem)
    assert out.termination_reason == OPT
    assert out.result.fp64_handoff_iteration > 0
    ci = out.iteration_stats[-1].convergence_information[0]
    assert ci.primal_objective == pytest.approx(lp.optimal_objective, rel=1e-6)
    ok, k = meets_tolerance(lp.problem, out.primal_solution, out.dual_solution, 1e-8, slack=1.01)
    assert ok, k


def test_transportation_full_size_property():
    """Full-size transportation LP (1M columns): size-independent properties only —
    termination under the reference's own relative-KKT criteria, recomputed in numpy."""
    lp = synthetic.transportation_lp(1)
    params = _params(tolerance=1e-4)
    out = cupdlp.optimize(params, lp.problem)
    assert out.termination_reason == OPT
    ok, k = meets_tolerance(lp.problem, out.primal_solution, out.dual_solution, 1e-4, slack=1.01)
    assert ok, k
