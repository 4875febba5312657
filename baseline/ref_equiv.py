"""ctypes wrapper of libref_equiv.so, the reference's solve loop in its own GPU form
(cuSPARSE CSR_ALG2, per-kernel synchronisation, host-side reductions, FP64): the
"reference on the same GPU" baseline that the benchmark measures beside the library.

Used by bench.py and its tests only, never by the `cupdlp` package.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.join(os.path.dirname(_HERE), "cupdlp.jl_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)
sys.path.insert(0, _HERE)

from cupdlp import _abi  # noqa: E402
from cupdlp.solver import scaled_desc  # noqa: E402
from cupdlp.types import params_to_c  # noqa: E402

import build_ref_equiv  # noqa: E402

_lib = None


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build_ref_equiv.build())
        lib.refeq_solve.restype = C.c_int
        lib.refeq_solve.argtypes = [C.POINTER(_abi.LpDesc), C.POINTER(_abi.Params), C.POINTER(_abi.Result),
                                    C.POINTER(C.c_double), C.POINTER(C.c_double)]
        lib.refeq_last_error.restype = C.c_char_p
        _lib = lib
    return _lib


def solve_scaled(scaled_problem, params, want_solution=True):
    """(result, x_avg, y_avg) of the scaled problem, the same inputs gpdhg_problem_create gets."""
    lib = load()
    d = scaled_desc(scaled_problem)
    n, m = d.desc.num_variables, d.desc.num_constraints
    res = _abi.Result()
    x = np.empty(n) if want_solution else None
    y = np.empty(max(m, 1)) if want_solution else None
    rc = lib.refeq_solve(d.ref, C.byref(params_to_c(params)), C.byref(res),
                         _abi.dptr(x) if x is not None else None, _abi.dptr(y) if y is not None else None)
    if rc:
        raise RuntimeError(f"refeq_solve failed: {lib.refeq_last_error().decode()}")
    return res, x, (y[:m] if y is not None else None)
