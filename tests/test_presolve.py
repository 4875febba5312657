"""presolve / undo_presolve (src/preprocess.jl:105-326), which the reference defines but never
calls, mirrored on the host: pinned on a hand-worked example, by HiGHS (the presolved LP plus
its objective constant has the original's optimum), and through the GPU solve."""
import numpy as np
import pytest
import scipy.sparse as sp
from scipy.optimize import linprog

import cupdlp
from cupdlp import synthetic


def _worked():
    # rows: 0 '=' x0 + x2 = 2; 1 '=' empty, b 0; 2 '>=' x0 - x2 >= -1; 3 '>=' empty, b -0.5
    # columns 1 (c = -2, u = 4) and 3 (c = 3, l = 1) are empty
    a = sp.csc_matrix(np.array([[1.0, 0, 1.0, 0], [0, 0, 0, 0], [1.0, 0, -1.0, 0], [0, 0, 0, 0]]))
    a.eliminate_zeros()
    n = 4
    return cupdlp.QuadraticProgrammingProblem(np.array([0.0, 0.0, 0.0, 1.0]), np.array([10.0, 4.0, np.inf, 5.0]),
                                              sp.csc_matrix((n, n)), np.array([1.0, -2.0, 0.5, 3.0]), 0.5, a,
                                              np.array([2.0, 0.0, -1.0, -0.5]), 2)


def test_presolve_on_a_hand_worked_example(capsys):
    p = _worked()
    info = cupdlp.presolve(p)
    assert list(info.empty_rows) == [1, 3] and list(info.empty_columns) == [1, 3]
    assert (info.original_primal_size, info.original_dual_size) == (4, 4)
    assert p.num_equalities == 1
    assert np.array_equal(p.constraint_matrix.toarray(), [[1.0, 1.0], [1.0, -1.0]])
    assert list(p.right_hand_side) == [2.0, -1.0]
    assert list(p.objective_vector) == [1.0, 0.5]
    assert p.objective_constant == 0.5 + 4.0 * -2.0 + 1.0 * 3.0
    assert list(p.variable_lower_bound) == [0.0, 0.0] and list(p.variable_upper_bound) == [10.0, np.inf]
    assert capsys.readouterr().out == ""          # no singleton rows left
    x, y = cupdlp.undo_presolve(info, np.array([1.5, 0.5]), np.array([0.25, -0.75]))
    assert list(x) == [1.5, 0.0, 0.5, 1.0]        # removed columns are 0, then projected: x3 >= 1
    assert list(y) == [0.25, 0.0, -0.75, 0.0]


def test_presolve_detects_infeasible_empty_rows():
    p = _worked()
    p.right_hand_side[1] = 1e-9
    with pytest.raises(cupdlp.InfeasibleProblemError):
        cupdlp.presolve(p)
    p = _worked()
    p.right_hand_side[3] = 0.25
    with pytest.raises(cupdlp.InfeasibleProblemError):
        cupdlp.presolve(p)
    p = _worked()
    p.right_hand_side[3] = 0.0                    # 0 >= 0 holds
    assert list(cupdlp.presolve(p).empty_rows) == [1, 3]


def test_transform_bounds_and_singletons(capsys):
    p = _worked()
    cupdlp.presolve(p, verbosity=1, transform_bounds=True)
    # finite lower bounds of the kept columns (both), then their finite upper bounds (x0 <= 10)
    assert np.array_equal(p.constraint_matrix.toarray(),
                          [[1.0, 1.0], [1.0, -1.0], [1.0, 0.0], [0.0, 1.0], [-1.0, 0.0]])
    assert list(p.right_hand_side) == [2.0, -1.0, 0.0, 0.0, -10.0]
    assert np.isinf(p.variable_lower_bound).all() and np.isinf(p.variable_upper_bound).all()
    q = _worked()
    q.constraint_matrix = sp.csc_matrix(np.array([[1.0, 0, 1.0, 0], [0, 0, 0, 0], [1.0, 0, 0, 0], [0, 0, 0, 0]]))
    q.constraint_matrix.eliminate_zeros()
    cupdlp.presolve(q)
    assert "1 constraints involving exactly a single variable" in capsys.readouterr().out


def _with_empty_parts(seed):
    """A planted LP with two empty rows ('=' with b 0, '>=' with b -1) and three empty
    columns inserted; the optimum moves by the empty columns' best-bound costs."""
    lp = synthetic.known_optimum_lp(seed, m=150, n=400, neq=80, density=0.03)
    p = lp.problem
    a = sp.csr_matrix(p.constraint_matrix)
    m, n = a.shape
    rows = sp.vstack([a[:40], sp.csr_matrix((1, n)), a[40:100], sp.csr_matrix((1, n)), a[100:]])
    b = np.concatenate([p.right_hand_side[:40], [0.0], p.right_hand_side[40:100], [-1.0], p.right_hand_side[100:]])
    cols = sp.hstack([rows[:, :10], sp.csr_matrix((m + 2, 1)), rows[:, 10:200], sp.csr_matrix((m + 2, 2)),
                      rows[:, 200:]]).tocsc()
    c = np.concatenate([p.objective_vector[:10], [2.0], p.objective_vector[10:200], [-1.5, 0.0],
                        p.objective_vector[200:]])
    lo = np.zeros(n + 3)
    hi = np.concatenate([p.variable_upper_bound[:10], [7.0], p.variable_upper_bound[10:200], [3.0, 9.0],
                         p.variable_upper_bound[200:]])
    q = cupdlp.QuadraticProgrammingProblem(lo, hi, sp.csc_matrix((n + 3, n + 3)), c, 0.0, cols, b,
                                           p.num_equalities + 1)
    return q, lp.optimal_objective + 3.0 * -1.5


def _highs(p):
    a = sp.csr_matrix(p.constraint_matrix)
    k = p.num_equalities
    hi = np.where(np.isinf(p.variable_upper_bound), None, p.variable_upper_bound)
    r = linprog(p.objective_vector, A_ub=-a[k:], b_ub=-p.right_hand_side[k:], A_eq=a[:k],
                b_eq=p.right_hand_side[:k], bounds=list(zip(p.variable_lower_bound, hi)), method="highs")
    assert r.status == 0, r.message
    return r.fun + p.objective_constant


def test_presolve_keeps_the_optimum():
    q, want = _with_empty_parts(31)
    before = _highs(q)
    info = cupdlp.presolve(q, verbosity=0)
    assert list(info.empty_rows) == [40, 101] and {10, 201, 202} <= set(info.empty_columns.tolist())
    after = _highs(q)
    assert abs(before - want) <= 1e-7 * max(1.0, abs(want))
    assert abs(after - before) <= 1e-7 * max(1.0, abs(want))


@pytest.mark.gpu
def test_presolved_solve_matches_the_plain_solve():
    """optimize() on the presolved LP, undone, has the objective of optimize() on the LP."""
    q, want = _with_empty_parts(32)
    params = cupdlp.default_parameters(tolerance=1e-8, iteration_limit=200_000, time_sec_limit=60.0)
    plain = cupdlp.optimize(params, q)
    c = q.objective_vector.copy()
    info = cupdlp.presolve(q, verbosity=0)
    out = cupdlp.optimize(params, q)
    assert plain.termination_reason == out.termination_reason == cupdlp.TerminationReason.TERMINATION_REASON_OPTIMAL
    x, y = cupdlp.undo_presolve(info, out.primal_solution, out.dual_solution)
    assert x.size == c.size and y.size == info.original_dual_size
    # the undone primal sets removed columns to 0 (then projects); the objective constant
    # carries their best-bound costs instead, so compare the optimal values
    assert abs((q.objective_vector @ out.primal_solution + q.objective_constant) - want) <= 1e-6 * max(1.0, abs(want))
    assert abs((c @ plain.primal_solution) - want) <= 1e-6 * max(1.0, abs(want))
