"""CPU restatement of the MPS reader's conversion of a two-sided LP into cuPDLP's standard form.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of gpdhg_problem_create_two_sided,
never by the `cupdlp` package. Follows, step by step:

  two_sided_rows_to_slacks    src/quadratic_programming_io.jl:85-121
  transform_to_standard_form  src/quadratic_programming_io.jl:33-76
  row_permute_in_place        src/preprocess.jl:586-611
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


class StandardFormError(ValueError):
    pass


def two_sided_rows_to_slacks(l, u, lc, uc, a: sp.csc_matrix, c):
    """Rows with finite, unequal bounds become `a'x - s = 0` with a new column s in [lc, uc]
    (:85-121): slack j sits in row two_sided[j] with coefficient -1, the new variables'
    bounds are the rows' bounds, their costs 0, and those rows' bounds become 0."""
    two_sided = np.flatnonzero(np.isfinite(lc) & np.isfinite(uc) & (lc != uc))            # :86-90
    if two_sided.size == 0:                                                               # :91-93
        return l, u, lc, uc, a, c, two_sided
    k = two_sided.size
    slack = sp.csc_matrix((np.full(k, -1.0), (two_sided, np.arange(k))), shape=(a.shape[0], k))  # :95-101
    l = np.concatenate([l, lc[two_sided]])                                                # :102-103
    u = np.concatenate([u, uc[two_sided]])                                                # :104-105
    c = np.concatenate([c, np.zeros(k)])                                                  # :106
    a = sp.hstack([a, slack], format="csc")                                               # :107
    lc = lc.copy()
    uc = uc.copy()
    lc[two_sided] = 0.0                                                                   # :108
    uc[two_sided] = 0.0                                                                   # :109
    return l, u, lc, uc, a, c, two_sided


def row_permute(a: sp.csc_matrix, old_row_to_new: np.ndarray) -> sp.csc_matrix:
    """Renumbers the rows and sorts each column's entries by their new row (:586-611)."""
    out = a.copy()
    out.indices = old_row_to_new[out.indices].astype(out.indices.dtype)
    out.has_sorted_indices = False
    out.sort_indices()
    return out


def transform_to_standard_form(l, u, lc, uc, a, c, offset):
    """(l, u, c, offset, A, b, num_equalities, new_row_to_old, num_slacks) of the standard
    form: equality rows first, then ">=" rows; "<=" rows negated (:33-76)."""
    l, u, c = (np.asarray(v, dtype=np.float64).copy() for v in (l, u, c))
    lc, uc = (np.asarray(v, dtype=np.float64).copy() for v in (lc, uc))
    a = sp.csc_matrix(a, dtype=np.float64, copy=True)
    a.sort_indices()
    l, u, lc, uc, a, c, two_sided = two_sided_rows_to_slacks(l, u, lc, uc, a, c)          # :34
    is_eq = lc == uc                                                                      # :36
    is_geq = ~is_eq & np.isfinite(lc)                                                     # :37
    is_leq = ~is_eq & np.isfinite(uc)                                                     # :38
    assert not (is_geq & is_leq).any()                                                    # :40-41
    num_eq = int(is_eq.sum())                                                             # :43
    if num_eq + int(is_geq.sum()) + int(is_leq.sum()) != lc.size:                         # :45-48
        raise StandardFormError("Not all constraints have finite bounds on at least one side.")
    flip = is_leq[a.indices]                                                              # :52-56
    a.data[flip] *= -1
    new_row_to_old = np.concatenate([np.flatnonzero(is_eq), np.flatnonzero(~is_eq)])      # :58
    if not np.array_equal(new_row_to_old, np.arange(lc.size)):                            # :59-61
        a = row_permute(a, np.argsort(new_row_to_old))
    rhs = lc.copy()                                                                       # :63
    rhs[is_leq] = -uc[is_leq]                                                             # :64
    rhs = rhs[new_row_to_old]                                                             # :65
    return dict(l=l, u=u, c=c, offset=float(offset), A=a, b=rhs, num_equalities=num_eq,
                new_row_to_old=new_row_to_old, num_slacks=int(two_sided.size))
