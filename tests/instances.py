"""Small hand-made LPs for edge cases (shared by CPU and GPU tests)."""
import numpy as np
import scipy.sparse as sp

from cupdlp import QuadraticProgrammingProblem


def lp(A, b, c, l, u, neq, c0=0.0):
    A = sp.csc_matrix(np.asarray(A, dtype=np.float64)) if not sp.issparse(A) else sp.csc_matrix(A)
    n = A.shape[1]
    return QuadraticProgrammingProblem(np.asarray(l, float), np.asarray(u, float), sp.csc_matrix((n, n)),
                                       np.asarray(c, float), float(c0), A, np.asarray(b, float), neq)


def primal_infeasible():
    # x1 + x2 = -1, x >= 0
    return lp([[1.0, 1.0]], [-1.0], [1.0, 1.0], [0, 0], [np.inf, np.inf], 1)


def dual_infeasible():
    # min -x1 - x2  s.t.  x1 - x2 = 0, x >= 0  (unbounded)
    return lp([[1.0, -1.0]], [0.0], [-1.0, -1.0], [0, 0], [np.inf, np.inf], 1)


def no_constraints():
    # min c'x over a box: the reference crashes here (empty launch grid)
    return lp(sp.csc_matrix((0, 3)), [], [1.0, -2.0, 0.5], [-1, -1, -1], [2, 3, 4], 0)


def free_variables(seed=7):
    rng = np.random.default_rng(seed)
    m, n = 40, 60
    A = sp.random(m, n, density=0.2, random_state=seed, format="csc") + sp.eye(m, n, format="csc")
    x = rng.standard_normal(n)
    b = A @ x
    y = rng.standard_normal(m)
    c = A.T @ y
    return lp(A, b, c, np.full(n, -np.inf), np.full(n, np.inf), m), float(c @ x)


def tiny():
    # min x s.t. x >= 1, 0 <= x <= 5 -> x = 1
    return lp([[1.0]], [1.0], [1.0], [0.0], [5.0], 0), 1.0


def empty_rows_and_columns(seed=8):
    # a zero row (equality, rhs 0) and a zero column with a bounded variable
    A = sp.csc_matrix(np.array([[1.0, 2.0, 0.0, 0.0], [0.0, 0.0, 0.0, 0.0], [1.0, -1.0, 0.0, 1.0]]))
    return lp(A, [2.0, 0.0, 0.5], [1.0, 1.0, -1.0, 0.5], [0, 0, 0, 0], [10, 10, 3, 10], 2)
