"""FP32 trajectories against the FP64 oracle: over the first evaluations every statistic of
an FP32 solve stays within 100x the distance between the oracle and the oracle run on the
same data rounded to FP32 (the FP32 envelope), on the golden instances."""
import json
import os

import pytest

import cupdlp
from cupdlp.solver import DeviceProblem, scaled_desc

from golden.make_golden import make
from test_gpu_long_rows import _rounded_to_fp32
from test_gpu_parity import FIELDS, _params, _rel

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


@pytest.mark.parametrize("entry", GOLDEN["instances"], ids=lambda e: f"{e['gen']}-{e['seed']}")
def test_fp32_first_evaluations_within_fp32_envelope(entry):
    import oracle
    p = make(entry).problem
    sq = cupdlp.rescale_problem(10, False, 1.0, 0, p)
    params = _params(tolerance=1e-10, iteration_limit=10, precision=cupdlp.Precision.FP32)
    with DeviceProblem(scaled_desc(sq)) as dp:
        res, _, _ = dp.solve(params)
        stats = dp.stats(res.num_iteration_stats)
    p64 = _params(tolerance=1e-10, iteration_limit=10)
    orc = oracle.solve_scaled(sq, p64)
    rnd = oracle.solve_scaled(_rounded_to_fp32(sq), p64)
    assert res.iteration_count == orc.result.iteration_count
    n = min(len(stats), len(orc.stats), len(rnd.stats))
    assert n >= 10
    env = dict.fromkeys(FIELDS, 0.0)
    for k in range(n):
        g = stats[k].convergence_information[0]
        o, q = orc.stats[k].convergence_information, rnd.stats[k].convergence_information
        for f in FIELDS:
            env[f] = max(env[f], _rel(getattr(o, f), getattr(q, f)))
            d = _rel(getattr(g, f), getattr(o, f))
            assert d <= 100.0 * env[f] + 1e-6, (k, f, d, env[f])
