"""Host preprocessing: validate and rescale_problem, as cuPDLP.jl keeps them on the host.

  validate                  src/preprocess.jl:8-74
  l2_norm                   src/preprocess.jl:89-103
  l2_norm_rescaling         src/preprocess.jl:344-358
  ruiz_rescaling (p = Inf)  src/preprocess.jl:398-463
  pock_chambolle_rescaling  src/preprocess.jl:494-525
  scale_problem             src/preprocess.jl:541-561
  rescale_problem           src/preprocess.jl:619-675
  presolve / undo_presolve  src/preprocess.jl:105-326 (defined by the reference, never called)

Matrices are scipy CSC, as the reference's SparseMatrixCSC. Row-wise reductions go
through a fixed CSC->CSR permutation of the nonzeros (the pattern never changes while
rescaling), so each Ruiz pass is a handful of vectorised segment reductions.
Only the LP case (objective_matrix == 0) is supported, as on the solve path.
"""
from __future__ import annotations

import copy
import dataclasses
import math

import numpy as np
import scipy.sparse as sp

from .types import QuadraticProgrammingProblem, ScaledQpProblem


class InvalidProblemError(ValueError):
    """validate() failure (the reference raises `error(...)`, src/preprocess.jl:68-71)."""


def validate(p: QuadraticProgrammingProblem) -> bool:
    msgs = []
    n = len(p.objective_vector)
    if len(p.variable_lower_bound) != len(p.variable_upper_bound):
        msgs.append("length(variable_lower_bound) != length(variable_upper_bound)")
    if len(p.variable_lower_bound) != n:
        msgs.append("length(variable_lower_bound) != length(objective_vector)")
    if p.constraint_matrix.shape[0] != len(p.right_hand_side):
        msgs.append("size(constraint_matrix,1) != length(right_hand_side)")
    if p.constraint_matrix.shape[1] != n:
        msgs.append("size(constraint_matrix,2) != length(objective_vector)")
    if p.objective_matrix is not None and tuple(p.objective_matrix.shape) != (n, n):
        msgs.append("objective_matrix is not square with length(objective_vector)")
    lb = np.asarray(p.variable_lower_bound, dtype=np.float64)
    ub = np.asarray(p.variable_upper_bound, dtype=np.float64)
    if np.any(lb == np.inf):
        msgs.append("variable_lower_bound contains +Inf")
    if np.any(ub == -np.inf):
        msgs.append("variable_upper_bound contains -Inf")
    if np.any(np.isnan(lb)) or np.any(np.isnan(ub)):
        msgs.append("NaN found in variable bounds")
    if not np.all(np.isfinite(p.right_hand_side)):
        msgs.append("NaN or Inf found in right hand side")
    if not np.all(np.isfinite(p.objective_vector)):
        msgs.append("NaN or Inf found in objective vector")
    if not np.all(np.isfinite(sp.csc_matrix(p.constraint_matrix).data)):
        msgs.append("NaN or Inf found in constraint matrix")
    if p.objective_matrix is not None and p.objective_matrix.nnz and not np.all(
            np.isfinite(sp.csc_matrix(p.objective_matrix).data)):
        msgs.append("NaN or Inf found in objective matrix")
    if not (0 <= p.num_equalities <= p.constraint_matrix.shape[0]):
        msgs.append("num_equalities out of range")
    if msgs:
        raise InvalidProblemError("Error found when validating QuadraticProgrammingProblem: " + "; ".join(msgs))
    return True


def is_linear_programming_problem(p: QuadraticProgrammingProblem) -> bool:
    """src/quadratic_programming.jl:273-275."""
    return p.objective_matrix is None or p.objective_matrix.nnz == 0


class _Pattern:
    """Index maps of a CSC matrix: column of each nonzero and the CSR ordering."""

    def __init__(self, a: sp.csc_matrix):
        m, n = a.shape
        self.m, self.n = m, n
        counts = np.diff(a.indptr)
        self.col_of = np.repeat(np.arange(n, dtype=np.int64), counts)
        self.row_of = a.indices.astype(np.int64)
        self.perm = np.argsort(self.row_of, kind="stable")
        self.rptr = np.zeros(m + 1, dtype=np.int64)
        np.cumsum(np.bincount(self.row_of, minlength=m), out=self.rptr[1:])
        self.cptr = a.indptr.astype(np.int64)

    @staticmethod
    def _seg(ufunc, vals, ptr, empty):
        nseg = len(ptr) - 1
        out = np.full(nseg, empty, dtype=np.float64)
        if vals.size == 0 or nseg == 0:
            return out
        nonempty = ptr[:-1] < ptr[1:]
        out[nonempty] = ufunc.reduceat(vals, ptr[:-1][nonempty])
        return out

    def col_reduce(self, ufunc, vals, empty=0.0):
        return self._seg(ufunc, vals, self.cptr, empty)

    def row_reduce(self, ufunc, vals, empty=0.0):
        return self._seg(ufunc, vals[self.perm], self.rptr, empty)


def _ensure_csc(p: QuadraticProgrammingProblem) -> None:
    a = sp.csc_matrix(p.constraint_matrix, dtype=np.float64)
    a.sort_indices()
    p.constraint_matrix = a


def scale_problem(p: QuadraticProgrammingProblem, constraint_rescaling, variable_rescaling, pattern=None):
    """In place: c ./= D, bounds .*= D, b ./= E, A <- ((1/E_i) a_ij)(1/D_j)."""
    con = np.asarray(constraint_rescaling, dtype=np.float64)
    var = np.asarray(variable_rescaling, dtype=np.float64)
    assert np.all(con > 0) and np.all(var > 0)
    pat = pattern or _Pattern(p.constraint_matrix)
    p.objective_vector = p.objective_vector / var
    p.variable_upper_bound = p.variable_upper_bound * var
    p.variable_lower_bound = p.variable_lower_bound * var
    p.right_hand_side = p.right_hand_side / con
    a = p.constraint_matrix
    a.data = ((1.0 / con)[pat.row_of] * a.data) * (1.0 / var)[pat.col_of]


def ruiz_rescaling(p: QuadraticProgrammingProblem, num_iterations: int, pnorm: float = math.inf, pattern=None):
    if pnorm != math.inf:
        raise NotImplementedError("only the p = Inf Ruiz variant is on the solve path")
    pat = pattern or _Pattern(p.constraint_matrix)
    m, n = p.constraint_matrix.shape
    cum_con = np.ones(m)
    cum_var = np.ones(n)
    for _ in range(num_iterations):
        absdata = np.abs(p.constraint_matrix.data)
        var = np.sqrt(pat.col_reduce(np.maximum, absdata))
        var[var == 0.0] = 1.0
        if m == 0:
            con = np.zeros(0)
        else:
            con = np.sqrt(pat.row_reduce(np.maximum, absdata))
            con[con == 0.0] = 1.0
        scale_problem(p, con, var, pat)
        cum_con *= con
        cum_var *= var
    return cum_con, cum_var


def l2_norm(p_matrix_data, pat: _Pattern, dimension: int):
    """Row (dimension=2) or column (dimension=1) 2-norms, scaled by the max |a| first."""
    absdata = np.abs(p_matrix_data)
    if dimension == 1:
        sf = pat.col_reduce(np.maximum, absdata)
        sf[sf == 0.0] = 1.0
        t = p_matrix_data * (1.0 / sf)[pat.col_of]
        return sf * np.sqrt(pat.col_reduce(np.add, t * t))
    sf = pat.row_reduce(np.maximum, absdata)
    sf[sf == 0.0] = 1.0
    t = (1.0 / sf)[pat.row_of] * p_matrix_data
    return sf * np.sqrt(pat.row_reduce(np.add, t * t))


def l2_norm_rescaling(p: QuadraticProgrammingProblem, pattern=None):
    pat = pattern or _Pattern(p.constraint_matrix)
    rows = l2_norm(p.constraint_matrix.data, pat, 2)
    cols = l2_norm(p.constraint_matrix.data, pat, 1)
    rows[rows == 0.0] = 1.0
    cols[cols == 0.0] = 1.0
    col_f = np.sqrt(cols)
    row_f = np.sqrt(rows)
    scale_problem(p, row_f, col_f, pat)
    return row_f, col_f


def pock_chambolle_rescaling(p: QuadraticProgrammingProblem, alpha: float, pattern=None):
    assert 0 <= alpha <= 2
    pat = pattern or _Pattern(p.constraint_matrix)
    absdata = np.abs(p.constraint_matrix.data)
    var = np.sqrt(pat.col_reduce(np.add, np.power(absdata, 2.0 - alpha)))
    con = np.sqrt(pat.row_reduce(np.add, np.power(absdata, alpha)))
    var[var == 0.0] = 1.0
    con[con == 0.0] = 1.0
    scale_problem(p, con, var, pat)
    return con, var


def rescale_problem(l_inf_ruiz_iterations: int, l2_norm_rescaling_flag: bool, pock_chambolle_alpha,
                    verbosity: int, original_problem: QuadraticProgrammingProblem) -> ScaledQpProblem:
    """Returns ScaledQpProblem(original, scaled, constraint_rescaling, variable_rescaling);
    `original_problem` is not modified."""
    problem = copy.deepcopy(original_problem)
    _ensure_csc(problem)
    problem.variable_lower_bound = np.asarray(problem.variable_lower_bound, dtype=np.float64)
    problem.variable_upper_bound = np.asarray(problem.variable_upper_bound, dtype=np.float64)
    problem.objective_vector = np.asarray(problem.objective_vector, dtype=np.float64)
    problem.right_hand_side = np.asarray(problem.right_hand_side, dtype=np.float64)
    pat = _Pattern(problem.constraint_matrix)
    m, n = problem.constraint_matrix.shape
    con = np.ones(m)
    var = np.ones(n)
    if l_inf_ruiz_iterations > 0:
        c1, v1 = ruiz_rescaling(problem, l_inf_ruiz_iterations, math.inf, pat)
        con *= c1
        var *= v1
    if l2_norm_rescaling_flag:
        c1, v1 = l2_norm_rescaling(problem, pat)
        con *= c1
        var *= v1
    if pock_chambolle_alpha is not None:
        c1, v1 = pock_chambolle_rescaling(problem, float(pock_chambolle_alpha), pat)
        con *= c1
        var *= v1
    out = ScaledQpProblem(original_problem, problem, con, var)
    out._pattern = pat  # reused to emit CSR without re-sorting
    return out


def unscale_problem(p: QuadraticProgrammingProblem, constraint_rescaling, variable_rescaling):
    """src/preprocess.jl:568-575 (testing only)."""
    scale_problem(p, 1.0 / np.asarray(constraint_rescaling), 1.0 / np.asarray(variable_rescaling))


def csr_arrays(a, pattern: _Pattern | None = None):
    """(row_ptr int32, col_idx int32, values float64) of a sparse matrix, CSR order."""
    if pattern is not None and isinstance(a, sp.csc_matrix):
        vals = np.ascontiguousarray(a.data[pattern.perm], dtype=np.float64)
        cols = np.ascontiguousarray(pattern.col_of[pattern.perm], dtype=np.int32)
        rptr = np.ascontiguousarray(pattern.rptr, dtype=np.int32)
        return rptr, cols, vals
    c = sp.csr_matrix(a, dtype=np.float64)
    c.sort_indices()
    if c.nnz >= 2**31:
        raise ValueError("nnz must fit int32")
    return (np.ascontiguousarray(c.indptr, dtype=np.int32), np.ascontiguousarray(c.indices, dtype=np.int32),
            np.ascontiguousarray(c.data, dtype=np.float64))


# ---- presolve (src/preprocess.jl:105-326) --------------------------------------------------
# The reference defines presolve / undo_presolve but optimize() never calls them; they are
# mirrored here so a caller that wants them finds them with the same behaviour (indices are
# 0-based here, 1-based in Julia).

class InfeasibleProblemError(ValueError):
    """remove_empty_rows' `error("The problem is infeasible.")` (src/preprocess.jl:118-123)."""


@dataclasses.dataclass
class PresolveInfo:
    """src/preprocess.jl:210-217."""
    original_primal_size: int
    original_dual_size: int
    empty_rows: np.ndarray
    empty_columns: np.ndarray
    variable_lower_bound: np.ndarray
    variable_upper_bound: np.ndarray


def remove_empty_rows(p: QuadraticProgrammingProblem) -> np.ndarray:
    """Drops rows without nonzeros; an empty '=' row needs b = 0 and an empty '>=' row b <= 0,
    else the problem is infeasible (src/preprocess.jl:112-133)."""
    _ensure_csc(p)
    a = p.constraint_matrix
    seen = np.zeros(a.shape[0], dtype=bool)
    seen[a.indices] = True
    empty = np.flatnonzero(~seen)
    b = p.right_hand_side
    for row in empty:
        if row >= p.num_equalities and b[row] > 0.0:
            raise InfeasibleProblemError("The problem is infeasible.")
        if row < p.num_equalities and b[row] != 0.0:
            raise InfeasibleProblemError("The problem is infeasible.")
    if empty.size:
        p.constraint_matrix = sp.csc_matrix(a[seen, :])
        p.right_hand_side = b[seen]
        p.num_equalities -= int((empty < p.num_equalities).sum())
    return empty


def remove_empty_columns(p: QuadraticProgrammingProblem) -> np.ndarray:
    """Drops variables without nonzeros, fixing each at its best bound in the objective
    constant: the lower bound when c_j >= 0, else the upper (src/preprocess.jl:143-171; an
    infinite best bound makes the constant infinite, and 0 * Inf NaN, as there)."""
    assert is_linear_programming_problem(p)
    _ensure_csc(p)
    a = p.constraint_matrix
    is_empty = np.diff(a.indptr) == 0
    empty = np.flatnonzero(is_empty)
    if empty.size == 0:
        return empty
    const = float(p.objective_constant)
    for col in empty:   # one addition at a time, in column order, as the reference's loop
        coef = p.objective_vector[col]
        const += (p.variable_lower_bound[col] if coef >= 0 else p.variable_upper_bound[col]) * coef
    p.objective_constant = const
    keep = ~is_empty
    p.constraint_matrix = sp.csc_matrix(a[:, keep])
    p.objective_vector = p.objective_vector[keep]
    p.variable_lower_bound = p.variable_lower_bound[keep]
    p.variable_upper_bound = p.variable_upper_bound[keep]
    n = int(keep.sum())
    p.objective_matrix = sp.csc_matrix((n, n), dtype=np.float64)
    return empty


def transform_bounds_into_linear_constraints(p: QuadraticProgrammingProblem) -> None:
    """Appends a '>=' row x_j >= l_j per finite lower bound, then -x_j >= -u_j per finite upper
    bound, and frees the variables (src/preprocess.jl:176-207)."""
    _ensure_csc(p)
    lo = np.flatnonzero(np.isfinite(p.variable_lower_bound))
    hi = np.flatnonzero(np.isfinite(p.variable_upper_bound))
    k = lo.size + hi.size
    n = p.constraint_matrix.shape[1]
    block = sp.csc_matrix((np.concatenate([np.ones(lo.size), -np.ones(hi.size)]),
                           (np.arange(k), np.concatenate([lo, hi]))), shape=(k, n))
    p.constraint_matrix = sp.csc_matrix(sp.vstack([p.constraint_matrix, block], format="csc"))
    p.right_hand_side = np.concatenate([p.right_hand_side, p.variable_lower_bound[lo], -p.variable_upper_bound[hi]])
    p.variable_lower_bound = np.full(n, -np.inf)
    p.variable_upper_bound = np.full(n, np.inf)


def check_for_singleton_constraints(p: QuadraticProgrammingProblem) -> int:
    """Counts (and reports) rows with exactly one nonzero (src/preprocess.jl:262-276)."""
    _ensure_csc(p)
    per_row = np.bincount(p.constraint_matrix.indices, minlength=p.constraint_matrix.shape[0])
    single = int((per_row == 1).sum())
    if single > 0:
        print(f"{single} constraints involving exactly a single variable")
    return single


def presolve(p: QuadraticProgrammingProblem, verbosity: int = 1, transform_bounds: bool = False) -> PresolveInfo:
    """Modifies p in place; the returned record undoes it (src/preprocess.jl:223-258)."""
    saved_lo = p.variable_lower_bound.copy()
    saved_hi = p.variable_upper_bound.copy()
    original_dual_size, original_primal_size = p.constraint_matrix.shape
    empty_rows = remove_empty_rows(p)
    if is_linear_programming_problem(p):
        empty_columns = remove_empty_columns(p)
    else:
        empty_columns = np.zeros(0, dtype=np.int64)
    if verbosity >= 1:
        check_for_singleton_constraints(p)
    if transform_bounds:
        transform_bounds_into_linear_constraints(p)
    return PresolveInfo(original_primal_size, original_dual_size, empty_rows, empty_columns, saved_lo, saved_hi)


def recover_original_solution(solution: np.ndarray, empty_indices: np.ndarray, original_size: int) -> np.ndarray:
    """Zeros at the removed indices, the solution's leading entries elsewhere in order
    (src/preprocess.jl:290-299)."""
    keep = np.ones(original_size, dtype=bool)
    keep[np.asarray(empty_indices, dtype=np.int64)] = False
    out = np.zeros(original_size)
    out[keep] = np.asarray(solution)[: int(keep.sum())]
    return out


def undo_presolve(info: PresolveInfo, primal_solution: np.ndarray, dual_solution: np.ndarray):
    """(primal, dual) of the problem before presolve; the primal is projected onto the saved
    bounds (src/preprocess.jl:301-326)."""
    primal = recover_original_solution(primal_solution, info.empty_columns, info.original_primal_size)
    primal = np.minimum(np.maximum(primal, info.variable_lower_bound), info.variable_upper_bound)
    dual = recover_original_solution(dual_solution, info.empty_rows, info.original_dual_size)
    return primal, dual
