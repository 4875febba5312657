"""Any tile-plan parameters the planner may choose give the reference's results: with the
parameters pinned to non-default values (gpdhg_set_tile_override, the tuning sweep's hook)
the first 30 iterations still match the oracle to rtol 1e-9, and a batch instance still
equals its lone solve bit for bit."""
import numpy as np
import pytest

import cupdlp
from cupdlp import _abi, synthetic
from cupdlp.solver import DeviceBatch, DeviceProblem, scaled_desc

import instances
from test_gpu_parity import _params, compare_strict, solve_both

pytestmark = pytest.mark.gpu


@pytest.fixture
def override():
    lib = _abi.load()
    set_ = []

    def pin(precision, cfg):
        for side in (0, 1):
            _abi.check(lib.gpdhg_set_tile_override(precision, side, *cfg), lib)
        set_.append(precision)
    yield pin
    for p in set_:
        for side in (0, 1):
            lib.gpdhg_set_tile_override(p, side, 0, 0, 0)


@pytest.mark.parametrize("cfg", [(64, 1, 8), (128, 4, 24), (32, 2, 96)])
def test_pinned_fp64_plan_matches_oracle(override, cfg):
    override(_abi.PRECISION_FP64, cfg)
    lp = instances.long_rows_lp(seed=44, m=20000, n=24000, lengths=(300, 700, 3000, 17000))
    params = _params(tolerance=1e-10, iteration_limit=30)
    sq, (res, xa, ya, stats, xc, yc), orc, _ = solve_both(lp.problem, params)
    compare_strict(stats, orc, rtol=1e-9)


@pytest.mark.parametrize("cfg", [(128, 1, 8), (256, 8, 24)])
def test_pinned_fp32_plan_batch_equals_alone(override, cfg):
    override(_abi.PRECISION_FP32, cfg)
    params = _params(tolerance=1e-8, precision=cupdlp.Precision.FP32, iteration_limit=200)
    lps = [synthetic.known_optimum_lp(71, m=400, n=800, density=0.02), synthetic.transportation_lp(72, 30, 90)]
    scaled = [cupdlp.rescale_problem(10, False, 1.0, 0, lp.problem) for lp in lps]
    with DeviceBatch([scaled_desc(s) for s in scaled]) as db:
        rs, xs, ys = db.solve(params)
    for k, s in enumerate(scaled):
        with DeviceProblem(scaled_desc(s)) as dp:
            r, x, y = dp.solve(params)
        assert np.array_equal(xs[k], x) and np.array_equal(ys[k], y), k


def test_override_rejects_other_precisions():
    lib = _abi.load()
    assert lib.gpdhg_set_tile_override(_abi.PRECISION_FP32_REFINE, 0, 128, 1, 8) == _abi.ERR_INVALID_ARGUMENT
