"""ctypes wrapper of the CPU oracle (oracle/pdhg_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
CPU legs, never by the `cupdlp` package. It reuses the product's descriptor and
struct definitions so both sides are compared field for field.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_PKG_ROOT = os.path.join(os.path.dirname(_HERE), "cupdlp.jl_gb300")
if _PKG_ROOT not in sys.path:
    sys.path.insert(0, _PKG_ROOT)

from cupdlp import _abi  # noqa: E402
from cupdlp.solver import scaled_desc, unscaled_desc  # noqa: E402
from cupdlp.types import params_to_c  # noqa: E402

sys.path.insert(0, _HERE)
import build_oracle  # noqa: E402

_libs = {}


def load(perturbed: bool = False):
    """The oracle library; `perturbed` selects the build with another summation order."""
    if perturbed not in _libs:
        build_oracle.build()
        lib = C.CDLL(build_oracle.LIB_PERTURBED if perturbed else build_oracle.LIB)
        dp = C.POINTER(C.c_double)
        lib.oracle_set_threads.restype = C.c_int
        lib.oracle_set_threads.argtypes = [C.c_int]
        lib.oracle_rescale_problem.restype = C.c_int
        lib.oracle_rescale_problem.argtypes = [C.POINTER(_abi.LpDesc), C.c_int, C.c_int, C.c_double] + [dp] * 7
        lib.oracle_solve_scaled.restype = C.c_int
        lib.oracle_solve_scaled.argtypes = [C.POINTER(_abi.LpDesc), C.POINTER(_abi.Params),
                                            C.POINTER(_abi.Result), dp, dp, dp, dp,
                                            C.POINTER(_abi.IterationStats), C.c_int, dp]
        lib.oracle_optimize.restype = C.c_int
        lib.oracle_optimize.argtypes = [C.POINTER(_abi.LpDesc), C.POINTER(_abi.Params), C.POINTER(_abi.Result),
                                        dp, dp, C.POINTER(_abi.IterationStats), C.c_int]
        _libs[perturbed] = lib
    return _libs[perturbed]


def set_threads(n: int) -> int:
    load(True).oracle_set_threads(int(n))
    return load().oracle_set_threads(int(n))


def rescale(problem, ruiz=10, l2=False, alpha=1.0):
    """Oracle rescale_problem: (scaled CSR values, l, u, c, b, con, var)."""
    lib = load()
    d = unscaled_desc(problem)
    n, m, nnz = d.desc.num_variables, d.desc.num_constraints, d.desc.nnz
    out = [np.empty(nnz), np.empty(n), np.empty(n), np.empty(n), np.empty(m), np.empty(m), np.empty(n)]
    rc = lib.oracle_rescale_problem(d.ref, ruiz, int(l2), float("nan") if alpha is None else alpha,
                                    *[_abi.dptr(a) for a in out])
    if rc:
        raise ValueError(f"oracle rescale failed: {rc}")
    return out


class OracleRun:
    """margins[k]: smallest relative distance of any discrete decision to its threshold
    between evaluation k-1 and k; greedy_equivalent[k]: the restart at evaluation k was a
    KKT_GREEDY tie between numerically identical points (either label is correct)."""

    def __init__(self, result, x_avg, y_avg, x_cur, y_cur, stats, margins):
        self.result, self.x_avg, self.y_avg, self.x_cur, self.y_cur = result, x_avg, y_avg, x_cur, y_cur
        self.greedy_equivalent = [s.cumulative_rejected_steps == -1 for s in stats]
        for s in stats:
            s.cumulative_rejected_steps = 0
        self.stats = stats
        self.margins = margins

    def comparable_prefix(self, threshold=1e-9):
        """Number of leading evaluations reached without a decision closer than
        `threshold` (relative) to its threshold."""
        for k, mg in enumerate(self.margins):
            if mg < threshold:
                return k
        return len(self.margins)


def solve_scaled(scaled_problem, params, max_stats=100000, perturbed=False) -> OracleRun:
    """The loop on a ScaledQpProblem (same inputs the library gets)."""
    lib = load(perturbed)
    d = scaled_desc(scaled_problem)
    n, m = d.desc.num_variables, d.desc.num_constraints
    cp = params_to_c(params)
    res = _abi.Result()
    xa, ya, xc, yc = np.empty(n), np.empty(m), np.empty(n), np.empty(m)
    st = (_abi.IterationStats * max_stats)()
    mg = np.full(max_stats, np.inf)
    rc = lib.oracle_solve_scaled(d.ref, C.byref(cp), C.byref(res), *[_abi.dptr(a) for a in (xa, ya, xc, yc)],
                                 st, max_stats, _abi.dptr(mg))
    if rc:
        raise ValueError(f"oracle solve failed: {rc}")
    k = res.num_iteration_stats
    return OracleRun(res, xa, ya, xc, yc, [st[i] for i in range(k)], mg[:k].copy())


def optimize(problem, params, max_stats=100000):
    """Oracle optimize(): rescale + loop + unscale. Returns (result, x, y, stats)."""
    lib = load()
    d = unscaled_desc(problem)
    n, m = d.desc.num_variables, d.desc.num_constraints
    cp = params_to_c(params)
    res = _abi.Result()
    x, y = np.empty(n), np.empty(m)
    st = (_abi.IterationStats * max_stats)()
    rc = lib.oracle_optimize(d.ref, C.byref(cp), C.byref(res), _abi.dptr(x), _abi.dptr(y), st, max_stats)
    if rc:
        raise ValueError(f"oracle optimize failed: {rc}")
    return res, x, y, [st[i] for i in range(res.num_iteration_stats)]
