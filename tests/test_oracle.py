"""The oracle (CPU FP64 restatement of the reference loop) against independent pins."""
import json
import os

import numpy as np
import pytest

import cupdlp
from cupdlp import synthetic
from cupdlp.preprocess import csr_arrays

import instances
from golden.make_golden import checksum, make

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


@pytest.mark.parametrize("entry", GOLDEN["instances"], ids=lambda e: f"{e['gen']}-{e['seed']}")
def test_generator_reproduces_golden(entry):
    p = make(entry).problem
    assert checksum(p) == entry["checksum"]
    assert (p.num_constraints, p.num_variables, p.constraint_matrix.nnz) == (entry["m"], entry["n"], entry["nnz"])


@pytest.mark.parametrize("entry", GOLDEN["instances"], ids=lambda e: f"{e['gen']}-{e['seed']}")
def test_planted_optimum_matches_highs(entry):
    if entry["planted_objective"] is not None:
        assert entry["planted_objective"] == pytest.approx(entry["highs_objective"], rel=1e-9, abs=1e-9)


@pytest.mark.parametrize("entry", GOLDEN["instances"], ids=lambda e: f"{e['gen']}-{e['seed']}")
def test_oracle_converges_to_highs_optimum(entry, oracle_mod):
    p = make(entry).problem
    res, x, y, st = oracle_mod.optimize(p, cupdlp.default_parameters(tolerance=1e-8))
    assert res.termination_reason == cupdlp.TERMINATION_REASON_OPTIMAL
    ci = res.last_iteration_stats.convergence_information
    hi = entry["highs_objective"]
    assert ci.primal_objective == pytest.approx(hi, rel=1e-6)
    assert ci.dual_objective == pytest.approx(hi, rel=1e-6)
    assert res.iteration_count == entry["oracle_1e8"]["iteration_count"]
    assert ci.primal_objective == pytest.approx(entry["oracle_1e8"]["primal_objective"], rel=1e-12)


@pytest.mark.parametrize("entry", GOLDEN["instances"], ids=lambda e: f"{e['gen']}-{e['seed']}")
def test_oracle_fixed_iterations_golden(entry, oracle_mod):
    p = make(entry).problem
    res, _, _, _ = oracle_mod.optimize(p, cupdlp.default_parameters(tolerance=1e-8, iteration_limit=100))
    g = entry["oracle_it100"]
    ci = res.last_iteration_stats.convergence_information
    assert res.termination_reason == cupdlp.TERMINATION_REASON_ITERATION_LIMIT
    assert ci.primal_objective == pytest.approx(g["primal_objective"], rel=1e-12)
    assert ci.l2_dual_residual == pytest.approx(g["l2_dual_residual"], rel=1e-10)
    assert res.last_iteration_stats.step_size == pytest.approx(g["step_size"], rel=1e-12)
    assert res.cumulative_kkt_matrix_passes == g["kkt_passes"]


def test_oracle_deterministic_across_thread_counts(oracle_mod):
    p = synthetic.known_optimum_lp(11, m=200, n=400, density=0.03).problem
    params = cupdlp.default_parameters(tolerance=1e-6)
    oracle_mod.set_threads(1)
    r1, x1, y1, _ = oracle_mod.optimize(p, params)
    oracle_mod.set_threads(4)
    r4, x4, y4, _ = oracle_mod.optimize(p, params)
    oracle_mod.set_threads(min(8, os.cpu_count() or 1))
    assert r1.iteration_count == r4.iteration_count
    assert np.array_equal(x1, x4) and np.array_equal(y1, y4)


def test_python_rescaling_matches_oracle(oracle_mod):
    p = synthetic.known_optimum_lp(0).problem
    sq = cupdlp.rescale_problem(10, False, 1.0, 0, p)
    vals_o, l_o, u_o, c_o, b_o, con_o, var_o = oracle_mod.rescale(p)
    _, _, vals = csr_arrays(sq.scaled_qp.constraint_matrix, sq._pattern)
    np.testing.assert_allclose(vals, vals_o, rtol=1e-14)
    np.testing.assert_allclose(sq.constraint_rescaling, con_o, rtol=1e-14)
    np.testing.assert_allclose(sq.variable_rescaling, var_o, rtol=1e-14)
    np.testing.assert_allclose(sq.scaled_qp.objective_vector, c_o, rtol=1e-14)
    np.testing.assert_allclose(sq.scaled_qp.right_hand_side, b_o, rtol=1e-14)


def test_python_l2_rescaling_matches_oracle(oracle_mod):
    p = synthetic.known_optimum_lp(11, m=200, n=400, density=0.03).problem
    sq = cupdlp.rescale_problem(3, True, None, 0, p)
    vals_o, *_, con_o, var_o = oracle_mod.rescale(p, ruiz=3, l2=True, alpha=None)
    _, _, vals = csr_arrays(sq.scaled_qp.constraint_matrix, sq._pattern)
    np.testing.assert_allclose(vals, vals_o, rtol=1e-13)
    np.testing.assert_allclose(sq.variable_rescaling, var_o, rtol=1e-13)


def test_oracle_detects_primal_infeasible(oracle_mod):
    res, *_ = oracle_mod.optimize(instances.primal_infeasible(), cupdlp.default_parameters(tolerance=1e-6))
    assert res.termination_reason == cupdlp.TERMINATION_REASON_PRIMAL_INFEASIBLE


def test_oracle_detects_dual_infeasible(oracle_mod):
    res, *_ = oracle_mod.optimize(instances.dual_infeasible(), cupdlp.default_parameters(tolerance=1e-6))
    assert res.termination_reason == cupdlp.TERMINATION_REASON_DUAL_INFEASIBLE


def test_oracle_no_constraints(oracle_mod):
    res, x, y, _ = oracle_mod.optimize(instances.no_constraints(), cupdlp.default_parameters(tolerance=1e-8))
    assert res.termination_reason == cupdlp.TERMINATION_REASON_OPTIMAL
    np.testing.assert_allclose(x, [-1.0, 3.0, -1.0], atol=1e-6)


def test_oracle_free_variables(oracle_mod):
    p, obj = instances.free_variables()
    res, *_ = oracle_mod.optimize(p, cupdlp.default_parameters(tolerance=1e-8))
    assert res.termination_reason == cupdlp.TERMINATION_REASON_OPTIMAL
    assert res.last_iteration_stats.convergence_information.primal_objective == pytest.approx(obj, rel=1e-6, abs=1e-6)


def test_oracle_constant_step_policy(oracle_mod):
    p = synthetic.known_optimum_lp(11, m=200, n=400, density=0.03)
    params = cupdlp.default_parameters(tolerance=1e-6)
    params.step_size_policy_params = cupdlp.ConstantStepsizeParams()
    res, *_ = oracle_mod.optimize(p.problem, params)
    assert res.termination_reason == cupdlp.TERMINATION_REASON_OPTIMAL
    assert res.last_iteration_stats.convergence_information.primal_objective == pytest.approx(
        p.optimal_objective, rel=1e-5)


# ---- reduced power-law LPs (the large power-law generator at m = 300 and m = 2,000) ------------

POWER_LAW = GOLDEN["power_law"]


@pytest.mark.parametrize("entry", POWER_LAW, ids=lambda e: f"{e['gen']}-{e['seed']}-m{e['m']}")
def test_power_law_generator_and_planted_optimum(entry):
    lp = make(entry)
    assert checksum(lp.problem) == entry["checksum"]
    assert lp.optimal_objective == pytest.approx(entry["planted_objective"], rel=1e-15)
    assert entry["planted_objective"] == pytest.approx(entry["highs_objective"], rel=1e-9)


@pytest.mark.parametrize("entry", [e for e in POWER_LAW if e["kind"] == "converge"],
                         ids=lambda e: f"{e['gen']}-{e['seed']}")
def test_oracle_reaches_power_law_optimum(entry, oracle_mod):
    p = make(entry).problem
    res, *_ = oracle_mod.optimize(p, cupdlp.default_parameters(tolerance=1e-8, iteration_limit=400000))
    g = entry["oracle_1e8"]
    ci = res.last_iteration_stats.convergence_information
    assert res.termination_reason == cupdlp.TERMINATION_REASON_OPTIMAL
    assert res.iteration_count == g["iteration_count"]
    assert ci.primal_objective == pytest.approx(g["primal_objective"], rel=1e-12)
    assert ci.primal_objective == pytest.approx(entry["highs_objective"], rel=1e-6)
    assert ci.dual_objective == pytest.approx(entry["highs_objective"], rel=1e-6)


@pytest.mark.parametrize("entry", [e for e in POWER_LAW if e["kind"] == "study"],
                         ids=lambda e: f"{e['gen']}-{e['seed']}-m{e['m']}")
def test_oracle_power_law_budget_state(entry, oracle_mod):
    """The m = 2,000 instance: the planted optimum is HiGHS', but after 20,000 iterations the
    oracle is still far from 1e-4 (relative gap ~0.57): the slow convergence is the method's on
    this family, not a defect of the generator."""
    p = make(entry).problem
    res, *_ = oracle_mod.optimize(p, cupdlp.default_parameters(tolerance=1e-4, iteration_limit=entry["budget"]))
    g = entry["oracle_budget"]
    ci = res.last_iteration_stats.convergence_information
    assert res.termination_reason == cupdlp.TERMINATION_REASON_ITERATION_LIMIT
    assert ci.primal_objective == pytest.approx(g["primal_objective"], rel=1e-12)
    assert ci.relative_optimality_gap == pytest.approx(g["relative_optimality_gap"], rel=1e-10)
    assert ci.relative_optimality_gap > 0.1


def test_transportation_full_size_golden(oracle_mod):
    """The transportation benchmark (1M columns): the generator reproduces the committed
    instance and the oracle its 1e-4 solve; the committed 1e-8 optimum (the reference objective
    of the benchmark) is within the 1e-4 tolerance of the 1e-4 solve's objectives."""
    g = GOLDEN["full_size"]["transportation"]
    p = make(g).problem
    assert checksum(p) == g["checksum"]
    res, *_ = oracle_mod.optimize(p, cupdlp.default_parameters(tolerance=1e-4), max_stats=1000)
    ci = res.last_iteration_stats.convergence_information
    assert res.iteration_count == g["oracle_1e4"]["iteration_count"]
    assert ci.primal_objective == pytest.approx(g["oracle_1e4"]["primal_objective"], rel=1e-12)
    opt = g["oracle_1e8"]["primal_objective"]
    assert g["oracle_1e8"]["dual_objective"] == pytest.approx(opt, rel=1e-8)
    assert ci.primal_objective == pytest.approx(opt, rel=1e-4)
    assert ci.dual_objective == pytest.approx(opt, rel=1e-4)


def test_power_law_iterations_record(oracle_mod):
    """The recorded iterations-to-tolerance of the family (tests/golden, power_law_iterations):
    the instances regenerate with the recorded sizes, and the cheapest record re-runs exactly."""
    rec = GOLDEN["power_law_iterations"]
    for e in rec:
        assert make(e).problem.constraint_matrix.nnz == e["nnz"]
    e = min((e for e in rec if e["tol_1e4"]["termination_reason"] == 1), key=lambda e: e["tol_1e4"]["iteration_count"])
    res, *_ = oracle_mod.optimize(make(e).problem, cupdlp.default_parameters(tolerance=1e-4,
                                                                                iteration_limit=e["budget"]), max_stats=10)
    assert res.iteration_count == e["tol_1e4"]["iteration_count"]
    # the family slows down as it grows: no instance with m >= 3,000 reaches 1e-4 within its budget
    assert all(e["tol_1e4"]["termination_reason"] != 1 for e in rec if e["kw"]["m"] >= 3000)
