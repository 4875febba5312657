"""The reference-form GPU baseline (baseline/ref_equiv.cu: cuSPARSE CSR_ALG2, per-kernel
synchronisation, host-side reductions, FP64) is the reference's algorithm: its statistics
match the oracle's over the first iterations and it reaches the HiGHS optimum, so the
benchmark's "reference on the same GPU" figures time the reference's loop."""
import json
import os
import sys

import pytest

import cupdlp
from cupdlp import synthetic

from golden.make_golden import make

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "baseline"))

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))
FIELDS = ["primal_objective", "dual_objective", "l2_primal_residual", "l2_dual_residual",
          "l_inf_primal_residual", "l_inf_dual_residual", "l2_primal_variable", "l2_dual_variable"]


def _rel(a, b):
    s = max(abs(a), abs(b))
    return abs(a - b) / s if s > 0 else 0.0


@pytest.mark.parametrize("iters", [1, 10, 30])
def test_ref_equiv_matches_oracle_short_horizon(iters):
    import oracle
    import ref_equiv
    p = synthetic.known_optimum_lp(0).problem
    params = cupdlp.default_parameters(tolerance=1e-10, iteration_limit=iters, time_sec_limit=120.0)
    sq = cupdlp.rescale_problem(10, False, 1.0, 0, p)
    res, xa, ya = ref_equiv.solve_scaled(sq, params)
    orc = oracle.solve_scaled(sq, params)
    assert res.termination_reason == orc.result.termination_reason
    assert res.iteration_count == orc.result.iteration_count
    assert res.total_number_iterations == orc.result.total_number_iterations
    assert res.cumulative_kkt_matrix_passes == orc.result.cumulative_kkt_matrix_passes
    g, o = res.last_iteration_stats, orc.result.last_iteration_stats
    assert _rel(g.step_size, o.step_size) <= 1e-9 and _rel(g.primal_weight, o.primal_weight) <= 1e-9
    for f in FIELDS:
        a, b = getattr(g.convergence_information, f), getattr(o.convergence_information, f)
        assert _rel(a, b) <= 1e-9, (f, a, b)


@pytest.mark.parametrize("entry", GOLDEN["instances"][:4], ids=lambda e: f"{e['gen']}-{e['seed']}")
def test_ref_equiv_reaches_highs_optimum(entry):
    import ref_equiv
    p = make(entry).problem
    params = cupdlp.default_parameters(tolerance=1e-8, time_sec_limit=120.0)
    sq = cupdlp.rescale_problem(10, False, 1.0, 0, p)
    res, _, _ = ref_equiv.solve_scaled(sq, params, want_solution=False)
    assert res.termination_reason == cupdlp.TERMINATION_REASON_OPTIMAL
    ci = res.last_iteration_stats.convergence_information
    assert ci.primal_objective == pytest.approx(entry["highs_objective"], rel=1e-6)
    assert ci.dual_objective == pytest.approx(entry["highs_objective"], rel=1e-6)
