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


# Row lengths that reach every work shape of the step kernels' tile plans, in A (dual kernel)
# and in A' (primal kernel): warp-streamed rows (FP64 tiles hold 128 nonzeros, FP32 tiles 256;
# up to 512), group tiles of 2, 4 and 8 warps (513-1,024, 1,025-2,048, 2,049-16,384) and
# split rows cut into 16,384-nonzero pieces (20,000: two pieces, 40,000: three).
LONG_ROW_LENGTHS = (150, 300, 600, 1500, 4000, 20000, 40000)


def long_rows_lp(seed=31, m=45000, n=45000, per_column=2, lengths=LONG_ROW_LENGTHS):
    """A planted-optimum LP (bounds [0, 10]) whose short rows and columns (about
    `per_column` nonzeros per column) surround a few rows of A and a few columns of A (rows of
    A') of the given lengths, spread over equality and inequality rows; values N(0,1)."""
    from cupdlp import synthetic
    rng = np.random.default_rng(seed)
    rows = [rng.integers(0, m, per_column * n)]
    cols = [np.repeat(np.arange(n), per_column)]
    long_r = rng.choice(m, size=len(lengths), replace=False)
    long_c = rng.choice(n, size=len(lengths), replace=False)
    for r, c, k in zip(long_r, long_c, lengths):
        rows.append(np.full(k, r))
        cols.append(rng.choice(n, size=k, replace=False))
        rows.append(rng.choice(m, size=k, replace=False))
        cols.append(np.full(k, c))
    rows, cols = np.concatenate(rows), np.concatenate(cols)
    a = sp.csc_matrix((rng.standard_normal(rows.size), (rows, cols)), shape=(m, n))
    a.sum_duplicates()
    a.sort_indices()
    return synthetic._planted(rng, a, int(round(0.6 * m)), np.full(n, 10.0), f"long_rows_m{m}_n{n}_s{seed}")


def ragged_rows_lp(seed=61, m=4000, n=3000):
    """A planted-optimum LP (bounds [0, 10]) whose warp tiles mix every row shape inside one
    warp's run: a quarter of the rows empty, a quarter with one nonzero, a quarter with 2-6 and
    a quarter with 10-80; a fifth of the columns empty and the rest drawn with skewed
    popularity, so that A' (the primal kernel's rows) is as ragged. Values N(0,1)."""
    from cupdlp import synthetic
    rng = np.random.default_rng(seed)
    kind = rng.integers(0, 4, m)
    lens = np.where(kind == 0, 0, np.where(kind == 1, 1, np.where(kind == 2, rng.integers(2, 7, m),
                                                                   rng.integers(10, 81, m))))
    w = 1.0 / np.arange(1, n + 1) ** 1.5
    w[rng.permutation(n)[: n // 5]] = 0.0
    w /= w.sum()
    rows = np.repeat(np.arange(m), lens)
    cols = np.concatenate([rng.choice(n, size=k, replace=False, p=w) for k in lens if k > 0])
    a = sp.csc_matrix((rng.standard_normal(rows.size), (rows, cols)), shape=(m, n))
    a.sort_indices()
    return synthetic._planted(rng, a, int(round(0.6 * m)), np.full(n, 10.0), f"ragged_rows_m{m}_n{n}_s{seed}")


def infeasible_planted_lp(kind, seed=51, m=400, n=800, density=0.01):
    """A planted-optimum LP made infeasible: kind "primal" repeats equality row 0 with its
    right-hand side raised by 1 (two contradictory equalities); kind "dual" appends a column
    with cost -1, no constraint coefficients and no upper bound (the objective is unbounded
    below along it)."""
    from cupdlp import synthetic
    base = synthetic.known_optimum_lp(seed, m=m, n=n, density=density).problem
    a = sp.csr_matrix(base.constraint_matrix)
    l, u, c, b, neq = (base.variable_lower_bound, base.variable_upper_bound, base.objective_vector,
                       base.right_hand_side, base.num_equalities)
    if kind == "primal":
        a = sp.vstack([a[:neq], a[0:1], a[neq:]], format="csc")
        b = np.concatenate([b[:neq], [b[0] + 1.0], b[neq:]])
        return lp(a, b, c, l, u, neq + 1)
    a = sp.hstack([a, sp.csr_matrix((a.shape[0], 1))], format="csc")
    return lp(a, b, np.append(c, -1.0), np.append(l, 0.0), np.append(u, np.inf), neq)
