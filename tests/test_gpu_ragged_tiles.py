"""GPU parity on an LP whose warp tiles hold empty rows, single-nonzero rows and rows that
cross lanes side by side (instances.ragged_rows_lp), in A (dual kernel) and in A' (primal
kernel): the row sums of such tiles go through every branch of the tile summation (rows
wholly inside a lane, rows ending at a lane's end, rows spanning several lanes, empty rows)."""
import numpy as np
import pytest
import scipy.sparse as sp

import cupdlp
from cupdlp.solver import DeviceProblem, scaled_desc

import instances
from test_gpu_long_rows import _rounded_to_fp32
from test_gpu_parity import FIELDS, _params, _rel, compare_envelope, compare_strict, solve_both

pytestmark = pytest.mark.gpu


def test_instance_is_ragged():
    lp = instances.ragged_rows_lp()
    a = sp.csr_matrix(lp.problem.constraint_matrix)
    rl, cl = np.diff(a.indptr), np.diff(sp.csc_matrix(a).indptr)
    for lens in (rl, cl):
        assert (lens == 0).mean() > 0.15 and (lens == 1).mean() > 0.1 and (lens >= 10).mean() > 0.1


@pytest.mark.parametrize("iters", [1, 10, 30])
def test_fp64_short_horizon_matches_oracle(iters):
    p = instances.ragged_rows_lp().problem
    params = _params(tolerance=1e-10, iteration_limit=iters)
    sq, (res, xa, ya, stats, xc, yc), orc, _ = solve_both(p, params)
    assert res.iteration_count == orc.result.iteration_count
    compare_strict(stats, orc, rtol=1e-9)
    scale = lambda v: 1e-9 * max(1.0, np.abs(v).max())
    np.testing.assert_allclose(xc, orc.x_cur, rtol=0, atol=scale(orc.x_cur))
    np.testing.assert_allclose(yc, orc.y_cur, rtol=0, atol=scale(orc.y_cur))


def test_fp32_first_evaluations_within_fp32_envelope():
    import oracle
    p = instances.ragged_rows_lp().problem
    sq = cupdlp.rescale_problem(10, False, 1.0, 0, p)
    params = _params(tolerance=1e-10, iteration_limit=10, precision=cupdlp.Precision.FP32)
    with DeviceProblem(scaled_desc(sq)) as dp:
        res, _, _ = dp.solve(params)
        stats = dp.stats(res.num_iteration_stats)
    p64 = _params(tolerance=1e-10, iteration_limit=10)
    orc = oracle.solve_scaled(sq, p64)
    rnd = oracle.solve_scaled(_rounded_to_fp32(sq), p64)
    n = min(len(stats), len(orc.stats), len(rnd.stats))
    assert n >= 10
    env = dict.fromkeys(FIELDS, 0.0)
    for k in range(n):
        g = stats[k].convergence_information[0]
        o, q = orc.stats[k].convergence_information, rnd.stats[k].convergence_information
        for f in FIELDS:
            env[f] = max(env[f], _rel(getattr(o, f), getattr(q, f)))
            assert _rel(getattr(g, f), getattr(o, f)) <= 100.0 * env[f] + 1e-6, (k, f)


def test_fp64_trajectory_within_roundoff_envelope():
    p = instances.ragged_rows_lp().problem
    params = _params(tolerance=1e-10, iteration_limit=500)
    sq, (res, *_rest), orc, pert = solve_both(p, params, perturbed=True)
    compare_envelope(_rest[2], orc, pert)
