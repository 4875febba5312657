"""Column order of an LP for the GPU's gathers (an addition; the reference has no counterpart).

The library applies this order itself inside a problem handle when the column degrees are
skewed (at least 65,536 columns, the 1% most used columns holding at least 20% of the
nonzeros), and maps solutions back; this module is the same renumbering on the host, for
callers who want the reordered LP itself.

The dual step kernel gathers the primal candidate by column index once per nonzero. On a
matrix with skewed column degrees (the power-law LP: the 1% most used columns hold 44% of
the nonzeros) the hot entries are scattered over the whole vector, one 32-byte sector each.
Renumbering the columns by decreasing degree packs them into a few hundred kilobytes that
stay in L1/L2, and groups the long rows of A' for the primal kernel. On one GB300 the
power-law LP's FP32 phase ran at 3,048 KKT passes/s reordered against 2,742 in its own
order, measured before the tile plans grouped warp-streamed rows by themselves, which now
gives the original order 2,869 of that gain. The LP is the same up to the permutation (the
solver's reductions over n run in the new order, so results agree to round-off); rows keep
their order, so duals need no mapping.

    q, perm = reorder_columns_by_degree(p)
    out = cupdlp.optimize(params, q)
    x = restore_primal(out.primal_solution, perm)
"""
from __future__ import annotations

import dataclasses
from typing import Tuple

import numpy as np
import scipy.sparse as sp

from .types import QuadraticProgrammingProblem


def reorder_columns_by_degree(p: QuadraticProgrammingProblem) -> Tuple[QuadraticProgrammingProblem, np.ndarray]:
    """(the LP with column k = column perm[k] of p, perm); columns in decreasing order of
    their nonzero counts, ties in their original order."""
    a = sp.csc_matrix(p.constraint_matrix)
    deg = np.diff(a.indptr)
    perm = np.argsort(-deg, kind="stable")
    b = a[:, perm]
    b.sort_indices()
    n = perm.size
    q = dataclasses.replace(
        p, variable_lower_bound=np.asarray(p.variable_lower_bound)[perm],
        variable_upper_bound=np.asarray(p.variable_upper_bound)[perm],
        objective_vector=np.asarray(p.objective_vector)[perm], constraint_matrix=sp.csc_matrix(b),
        objective_matrix=sp.csc_matrix((n, n)) if p.objective_matrix is None or p.objective_matrix.nnz == 0
        else sp.csc_matrix(p.objective_matrix)[perm][:, perm])
    return q, perm


def restore_primal(x: np.ndarray, perm: np.ndarray) -> np.ndarray:
    """The primal vector in the original column order."""
    out = np.empty_like(np.asarray(x))
    out[perm] = x
    return out
