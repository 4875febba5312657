"""cupdlp.layout: the degree-ordered LP is the same LP (CPU: structure and HiGHS optimum)."""
import numpy as np
import scipy.sparse as sp
from scipy.optimize import linprog

from cupdlp import layout, synthetic


def _highs(p):
    a = sp.csr_matrix(p.constraint_matrix)
    k = p.num_equalities
    hi = np.where(np.isinf(p.variable_upper_bound), None, p.variable_upper_bound)
    r = linprog(p.objective_vector, A_ub=-a[k:], b_ub=-p.right_hand_side[k:], A_eq=a[:k],
                b_eq=p.right_hand_side[:k], bounds=list(zip(p.variable_lower_bound, hi)), method="highs")
    assert r.status == 0, r.message
    return r.fun, r.x


def test_reorder_by_degree_is_a_column_permutation():
    lp = synthetic.power_law_lp(4, m=300, n=900, target_nnz=9000)
    p = lp.problem
    q, perm = layout.reorder_columns_by_degree(p)
    deg = np.diff(sp.csc_matrix(q.constraint_matrix).indptr)
    assert (np.diff(deg) <= 0).all()                       # decreasing degree
    assert np.array_equal(np.sort(perm), np.arange(p.num_variables))
    a = sp.csc_matrix(p.constraint_matrix)
    assert (abs(sp.csc_matrix(q.constraint_matrix) - a[:, perm]) > 0).nnz == 0
    assert np.array_equal(q.objective_vector, p.objective_vector[perm])
    assert np.array_equal(q.right_hand_side, p.right_hand_side) and q.num_equalities == p.num_equalities
    x = np.arange(p.num_variables, dtype=float)
    assert np.array_equal(layout.restore_primal(x[perm], perm), x)


def test_reordered_lp_has_the_same_optimum():
    lp = synthetic.power_law_lp(5, m=200, n=600, target_nnz=5000)
    q, perm = layout.reorder_columns_by_degree(lp.problem)
    f0, _ = _highs(lp.problem)
    f1, x1 = _highs(q)
    assert abs(f1 - f0) <= 1e-9 * max(1.0, abs(f0))
    assert abs(f0 - lp.optimal_objective) <= 1e-7 * max(1.0, abs(f0))
    x = layout.restore_primal(x1, perm)
    assert abs(lp.problem.objective_vector @ x - f0) <= 1e-7 * max(1.0, abs(f0))
