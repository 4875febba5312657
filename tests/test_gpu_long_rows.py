"""Parity of the long-row work shapes of the step kernels against the CPU oracle.

The reference's cuSPARSE SpMV (src/primal_dual_hybrid_gradient_gpu.jl:225 for A dx, :307
for A'y) takes rows of any length. The step kernels cut rows into warp tiles, warp-streamed
rows, group tiles of 2, 4 and 8 warps and split rows whose 16,384-nonzero pieces meet in
carry slots; instances.long_rows_lp puts rows of every such length into A (the dual kernel's
A dx) and into A' (the primal kernel's A'y) next to short ones. Checked here:
  * 1-30 iterations: every statistic, iterate and restart decision to rtol 1e-9 (FP64);
  * 100 iterations: within the oracle's round-off envelope (FP64);
  * converged: the planted optimum, and the reference's relative-KKT criteria in numpy;
  * FP32: every statistic of the first evaluations within 100x the distance between the
    oracle and the oracle run on the FP32-rounded data;
  * in a batch beside other instances: bitwise equal to the lone solve (FP64 and FP32).
"""
import copy

import numpy as np
import pytest

import cupdlp
from cupdlp import synthetic
from cupdlp.solver import DeviceBatch, DeviceProblem, scaled_desc

import instances
from kkt import meets_tolerance
from test_gpu_parity import FIELDS, _params, _rel, compare_envelope, compare_strict, solve_both

pytestmark = pytest.mark.gpu

OPT = cupdlp.TerminationReason.TERMINATION_REASON_OPTIMAL


@pytest.fixture(scope="module")
def long_lp():
    return instances.long_rows_lp()


def test_instance_reaches_every_tile_shape(long_lp):
    a = long_lp.problem.constraint_matrix
    for lengths in (np.diff(a.tocsr().indptr), np.diff(a.tocsc().indptr)):
        assert ((lengths > 128) & (lengths <= 256)).any()      # warp-streamed (FP64 tiles)
        assert ((lengths > 256) & (lengths <= 512)).any()      # warp-streamed (FP32 tiles too)
        assert ((lengths > 512) & (lengths <= 1024)).any()     # 2-warp group
        assert ((lengths > 1024) & (lengths <= 2048)).any()    # 4-warp group
        assert ((lengths > 2048) & (lengths <= 16384)).any()   # 8-warp group
        assert ((lengths > 16384) & (lengths <= 32768)).any()  # split row, two pieces
        assert (lengths > 32768).any()                         # split row, three pieces


@pytest.mark.parametrize("iters", [1, 5, 10, 30])
def test_long_rows_fp64_short_horizon(long_lp, iters):
    params = _params(tolerance=1e-10, iteration_limit=iters)
    sq, (res, xa, ya, stats, xc, yc), orc, _ = solve_both(long_lp.problem, params)
    assert res.termination_reason == orc.result.termination_reason
    assert res.iteration_count == orc.result.iteration_count
    assert res.total_number_iterations == orc.result.total_number_iterations
    compare_strict(stats, orc, rtol=1e-9)
    scale = lambda v: 1e-9 * max(1.0, np.abs(v).max())
    np.testing.assert_allclose(xa, orc.x_avg, rtol=0, atol=scale(orc.x_avg))
    np.testing.assert_allclose(ya, orc.y_avg, rtol=0, atol=scale(orc.y_avg))
    np.testing.assert_allclose(xc, orc.x_cur, rtol=0, atol=scale(orc.x_cur))
    np.testing.assert_allclose(yc, orc.y_cur, rtol=0, atol=scale(orc.y_cur))


def test_long_rows_fp64_within_roundoff_envelope(long_lp):
    params = _params(tolerance=1e-10, iteration_limit=100)
    sq, (res, *rest), orc, pert = solve_both(long_lp.problem, params, perturbed=True)
    compare_envelope(rest[2], orc, pert)


def test_long_rows_fp64_reaches_planted_optimum(long_lp):
    p = long_lp.problem
    out = cupdlp.optimize(_params(tolerance=1e-6), p)
    assert out.termination_reason == OPT
    ci = out.iteration_stats[-1].convergence_information[0]
    assert ci.primal_objective == pytest.approx(long_lp.optimal_objective, rel=1e-5)
    ok, k = meets_tolerance(p, out.primal_solution, out.dual_solution, 1e-6, slack=1.01)
    assert ok, k


def _rounded_to_fp32(sq):
    r = copy.deepcopy(sq)
    s = r.scaled_qp
    f = lambda v: np.asarray(v, dtype=np.float32).astype(np.float64)
    s.constraint_matrix.data[:] = f(s.constraint_matrix.data)
    s.variable_lower_bound = f(s.variable_lower_bound)
    s.variable_upper_bound = f(s.variable_upper_bound)
    s.objective_vector = f(s.objective_vector)
    s.right_hand_side = f(s.right_hand_side)
    return r


def test_long_rows_fp32_within_fp32_envelope(long_lp):
    import oracle
    params = _params(tolerance=1e-10, iteration_limit=10, precision=cupdlp.Precision.FP32)
    sq = cupdlp.rescale_problem(10, False, 1.0, 0, long_lp.problem)
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


@pytest.mark.parametrize("precision", [cupdlp.Precision.FP64, cupdlp.Precision.FP32])
def test_long_rows_in_a_batch_equal_alone_bitwise(long_lp, precision):
    lps = [synthetic.known_optimum_lp(41, m=300, n=600, density=0.02), long_lp,
           synthetic.transportation_lp(42, supplies=30, demands=90),
           instances.long_rows_lp(seed=43, m=20000, n=24000, lengths=(700, 3000, 17000))]
    params = _params(tolerance=1e-8, precision=precision, iteration_limit=300)
    scaled = [cupdlp.rescale_problem(10, False, 1.0, 0, lp.problem) for lp in lps]
    with DeviceBatch([scaled_desc(sq) for sq in scaled]) as db:
        results, xs, ys = db.solve(params)
    for k, sq in enumerate(scaled):
        with DeviceProblem(scaled_desc(sq)) as dp:
            r, x, y = dp.solve(params)
        assert results[k].termination_reason == r.termination_reason, k
        assert results[k].iteration_count == r.iteration_count, k
        assert np.array_equal(xs[k], x), k
        assert np.array_equal(ys[k], y), k
