"""The handle's column order for skewed LPs (choose_column_order / apply_column_order in
csrc/problem.cu): when the 1% most used columns hold at least 20% of the nonzeros (and there
are at least 65,536 columns) the handle renumbers the columns by decreasing degree, so the
dual kernel's gathers of the primal candidate hit few cache lines, and maps every n-vector
back at the boundary. Checked: the renumbering happens (the handle of an LP equals, bit for
bit, the handle of the same LP whose caller already sorted the columns), results stay the
reference's (oracle, rtol 1e-9 over 10 iterations, iterates included), a batch instance
equals its lone solve, and warm starts, current iterates and device rescaling vectors come
back in the caller's order."""
import numpy as np
import scipy.sparse as sp
import pytest

import cupdlp
from cupdlp import layout, synthetic
from cupdlp.solver import DeviceBatch, DeviceProblem, scaled_desc

from test_gpu_parity import _params, compare_strict, solve_both

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def skewed():
    lp = synthetic.power_law_lp(5, m=30000, n=70000, target_nnz=300000)
    a = lp.problem.constraint_matrix.tocsc()
    deg = np.sort(np.diff(a.indptr))[::-1]
    assert deg[: (deg.size + 99) // 100].sum() >= 0.2 * deg.sum()   # the rule applies
    return lp


def _ruiz_only(**kw):
    p = _params(**kw)
    p.l_inf_ruiz_iterations = 10
    p.l2_norm_rescaling = False
    p.pock_chambolle_alpha = None   # Ruiz alone rescales by maxima: exact in any column order
    return p


@pytest.mark.parametrize("precision", [cupdlp.Precision.FP64, cupdlp.Precision.FP32])
def test_handle_order_equals_a_caller_sorted_lp(skewed, precision):
    params = _ruiz_only(tolerance=1e-10, iteration_limit=200, precision=precision)
    sq = cupdlp.rescale_problem(10, False, None, 0, skewed.problem)
    q, perm = layout.reorder_columns_by_degree(skewed.problem)
    sqq = cupdlp.rescale_problem(10, False, None, 0, q)
    with DeviceProblem(scaled_desc(sq)) as dp:
        r1, x1, y1 = dp.solve(params)
    with DeviceProblem(scaled_desc(sqq)) as dq:
        r2, x2, y2 = dq.solve(params)
    assert r1.total_number_iterations == r2.total_number_iterations
    assert np.array_equal(x1, layout.restore_primal(x2, perm))
    assert np.array_equal(y1, y2)


def test_skewed_lp_matches_oracle_short_horizon(skewed):
    params = _params(tolerance=1e-10, iteration_limit=10)
    sq, (res, xa, ya, stats, xc, yc), orc, _ = solve_both(skewed.problem, params)
    assert res.iteration_count == orc.result.iteration_count
    compare_strict(stats, orc, rtol=1e-9)
    scale = lambda v: 1e-9 * max(1.0, np.abs(v).max())
    np.testing.assert_allclose(xa, orc.x_avg, rtol=0, atol=scale(orc.x_avg))
    np.testing.assert_allclose(xc, orc.x_cur, rtol=0, atol=scale(orc.x_cur))
    np.testing.assert_allclose(yc, orc.y_cur, rtol=0, atol=scale(orc.y_cur))


@pytest.mark.parametrize("precision", [cupdlp.Precision.FP64, cupdlp.Precision.FP32])
def test_skewed_lp_in_a_batch_equals_alone(skewed, precision):
    params = _params(tolerance=1e-8, iteration_limit=150, precision=precision)
    lps = [synthetic.known_optimum_lp(61, m=200, n=400, density=0.03), skewed,
           synthetic.transportation_lp(62, supplies=20, demands=60)]
    scaled = [cupdlp.rescale_problem(10, False, 1.0, 0, lp.problem) for lp in lps]
    with DeviceBatch([scaled_desc(s) for s in scaled]) as db:
        rs, xs, ys = db.solve(params)
    for k, s in enumerate(scaled):
        with DeviceProblem(scaled_desc(s)) as dp:
            r, x, y = dp.solve(params)
        assert rs[k].total_number_iterations == r.total_number_iterations, k
        assert np.array_equal(xs[k], x) and np.array_equal(ys[k], y), k


def test_warm_start_current_iterate_and_rescaling_in_caller_order(skewed):
    p = skewed.problem
    sq = cupdlp.rescale_problem(10, False, 1.0, 0, p)
    params = _params(tolerance=1e-10, iteration_limit=40)
    with DeviceProblem(scaled_desc(sq)) as dp:
        dp.solve(params)
        xc, yc = dp.current_iterate()
        # warm start at the planted optimum (scaled): the first evaluation sees an optimal
        # point only if the handle put it into its own column order
        dp.set_warm_start(skewed.x_star * sq.variable_rescaling, skewed.y_star * sq.constraint_rescaling)
        r1, _, _ = dp.solve(_params(tolerance=1e-10, iteration_limit=1))
        first = dp.stats(1)[0].convergence_information[0]
    assert first.relative_l2_primal_residual < 1e-9
    assert first.relative_optimality_gap < 1e-9
    import oracle
    orc = oracle.solve_scaled(sq, params)
    scale = lambda v: 1e-9 * max(1.0, np.abs(v).max())
    np.testing.assert_allclose(xc, orc.x_cur, rtol=0, atol=scale(orc.x_cur))
    np.testing.assert_allclose(yc, orc.y_cur, rtol=0, atol=scale(orc.y_cur))
    uparams = cupdlp.default_parameters(tolerance=1e-6)
    with DeviceProblem.from_unscaled(p, uparams) as du:
        con, var = du.rescaling()
    np.testing.assert_allclose(con, sq.constraint_rescaling, rtol=1e-14, atol=0)
    np.testing.assert_allclose(var, sq.variable_rescaling, rtol=1e-14, atol=0)


def test_every_entry_orders_the_columns_alike(skewed):
    """The CSR, CSC and two-sided entries of the same skewed LP build the same renumbered
    handle: the same solve, bit for bit (rescaled on the GPU for the unscaled entries)."""
    from cupdlp.solver import unscaled_desc
    from cupdlp.types import TwoSidedQpProblem
    p = skewed.problem
    params = cupdlp.default_parameters(tolerance=1e-12, iteration_limit=100, time_sec_limit=60.0)
    with DeviceProblem.from_unscaled(p, params) as dp:
        r, x, y = dp.solve(params)
    a = sp.csc_matrix(p.constraint_matrix)
    a.sort_indices()
    with DeviceProblem.from_csc(unscaled_desc(p), a, index_base=1, unscaled_params=params) as dq:
        r2, x2, y2 = dq.solve(params)
    assert r2.total_number_iterations == r.total_number_iterations
    assert np.array_equal(x2, x) and np.array_equal(y2, y)
    # the same LP as an MPS reader returns it: '=' rows with equal bounds, '>=' rows open above
    m, neq = p.num_constraints, p.num_equalities
    hi = p.right_hand_side.copy()
    hi[neq:] = np.inf
    t = TwoSidedQpProblem(p.variable_lower_bound.copy(), p.variable_upper_bound.copy(), p.right_hand_side.copy(),
                          hi, a, p.objective_constant, p.objective_vector.copy())
    with DeviceProblem.from_two_sided(t, index_base=0, unscaled_params=params) as dt:
        nv, neq2, ns, order = dt.standard_form()
        r3, x3, y3 = dt.solve(params)
    assert (nv, neq2, ns) == (p.num_variables, neq, 0) and np.array_equal(order, np.arange(m))
    assert r3.total_number_iterations == r.total_number_iterations
    assert np.array_equal(x3, x) and np.array_equal(y3, y)
