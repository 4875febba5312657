"""optimize(params, problem) -> SaddlePointOutput, through libgpdhg.so.

Mirrors optimize() of src/primal_dual_hybrid_gradient_gpu.jl:457-798: the host keeps
validate (:461), rescale_problem (:465) and the primal_importance check (:483-485);
the library takes over from the host->device transfer (:488) to the copy of the
averaged iterate back to the host (:713-720); unscaled_saddle_point_output
(src/saddle_point_gpu.jl:40-61) runs here again.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from typing import List, Optional

import numpy as np
import scipy.sparse as sp

from . import _abi
from .preprocess import csr_arrays, is_linear_programming_problem, rescale_problem, validate
from .types import (PdhgParameters, QuadraticProgrammingProblem, SaddlePointOutput, ScaledQpProblem,
                    TerminationReason, TwoSidedQpProblem, params_to_c, stats_from_c, termination_reason_to_string)


class _Desc:
    """A gpdhg_lp_desc plus the numpy arrays it points into (kept alive with it)."""

    def __init__(self, n, m, neq, rptr, cols, vals, l, u, c, b, c0, ol=None, ou=None, oc=None, ob=None,
                 con=None, var=None):
        f64 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        self.arrays = dict(rptr=np.ascontiguousarray(rptr, dtype=np.int32),
                           cols=np.ascontiguousarray(cols, dtype=np.int32), vals=f64(vals), l=f64(l), u=f64(u),
                           c=f64(c), b=f64(b), ol=f64(ol), ou=f64(ou), oc=f64(oc), ob=f64(ob), con=f64(con),
                           var=f64(var))
        a = self.arrays
        d = _abi.LpDesc()
        d.num_variables = int(n)
        d.num_constraints = int(m)
        d.num_equalities = int(neq)
        d.nnz = int(a["vals"].size)
        d.row_ptr = _abi.iptr(a["rptr"])
        d.col_idx = _abi.iptr(a["cols"])
        d.values = _abi.dptr(a["vals"])
        d.variable_lower_bound = _abi.dptr(a["l"])
        d.variable_upper_bound = _abi.dptr(a["u"])
        d.objective_vector = _abi.dptr(a["c"])
        d.right_hand_side = _abi.dptr(a["b"])
        d.objective_constant = float(c0)
        d.original_variable_lower_bound = _abi.dptr(a["ol"])
        d.original_variable_upper_bound = _abi.dptr(a["ou"])
        d.original_objective_vector = _abi.dptr(a["oc"])
        d.original_right_hand_side = _abi.dptr(a["ob"])
        d.constraint_rescaling = _abi.dptr(a["con"])
        d.variable_rescaling = _abi.dptr(a["var"])
        self.desc = d

    @property
    def ref(self):
        return C.byref(self.desc)


def scaled_desc(sq: ScaledQpProblem) -> _Desc:
    """Descriptor of a ScaledQpProblem: scaled CSR + vectors, original vectors, scalings."""
    s, o = sq.scaled_qp, sq.original_qp
    rptr, cols, vals = csr_arrays(s.constraint_matrix, getattr(sq, "_pattern", None))
    return _Desc(s.num_variables, s.num_constraints, s.num_equalities, rptr, cols, vals,
                 s.variable_lower_bound, s.variable_upper_bound, s.objective_vector, s.right_hand_side,
                 s.objective_constant, o.variable_lower_bound, o.variable_upper_bound, o.objective_vector,
                 o.right_hand_side, sq.constraint_rescaling, sq.variable_rescaling)


def unscaled_desc(p: QuadraticProgrammingProblem) -> _Desc:
    """Descriptor of an unscaled problem (no original_* vectors, no rescaling)."""
    rptr, cols, vals = csr_arrays(p.constraint_matrix)
    return _Desc(p.num_variables, p.num_constraints, p.num_equalities, rptr, cols, vals,
                 p.variable_lower_bound, p.variable_upper_bound, p.objective_vector, p.right_hand_side,
                 p.objective_constant)


class DeviceProblem:
    """A gpdhg_problem handle: the scaled LP resident on the GPU, solvable many times."""

    def __init__(self, desc: _Desc, lib=None):
        self.lib = lib or _abi.load()
        self.n = desc.desc.num_variables
        self.m = desc.desc.num_constraints
        h = C.c_void_p()
        _abi.check(self.lib.gpdhg_problem_create(desc.ref, C.byref(h)), self.lib)
        self.handle = h

    @classmethod
    def from_csc(cls, desc: _Desc, a_csc, index_base: int = 0, unscaled_params: Optional[PdhgParameters] = None,
                 lib=None):
        """gpdhg_problem_create_csc: the matrix as compressed sparse columns (scipy's csc
        indptr / indices / data, or Julia's 1-based colptr / rowval / nzval with index_base 1);
        `desc` supplies the vectors (its CSR arrays are not read). With unscaled_params the
        data are unscaled and rescaled on the GPU."""
        self = cls.__new__(cls)
        self.lib = lib or _abi.load()
        self.n, self.m = desc.desc.num_variables, desc.desc.num_constraints
        colptr = np.ascontiguousarray(a_csc.indptr, dtype=np.int64) + index_base
        rowval = np.ascontiguousarray(a_csc.indices, dtype=np.int64) + index_base
        nzval = np.ascontiguousarray(a_csc.data, dtype=np.float64)
        d = _abi.LpDesc()
        C.pointer(d)[0] = desc.desc
        d.row_ptr = C.cast(None, _abi._ip)
        d.col_idx = C.cast(None, _abi._ip)
        d.values = C.cast(None, _abi._dp)
        d.nnz = int(nzval.size)
        cp = params_to_c(unscaled_params) if unscaled_params is not None else None
        h = C.c_void_p()
        _abi.check(self.lib.gpdhg_problem_create_csc(C.byref(d), _abi.lptr(colptr), _abi.lptr(rowval),
                                                     _abi.dptr(nzval), int(index_base),
                                                     C.byref(cp) if cp is not None else None, C.byref(h)), self.lib)
        self.handle = h
        return self

    @classmethod
    def from_two_sided(cls, qp: TwoSidedQpProblem, index_base: int = 0,
                       unscaled_params: Optional[PdhgParameters] = None, lib=None):
        """gpdhg_problem_create_two_sided: transform_to_standard_form
        (src/quadratic_programming_io.jl:33-121) while the problem is built, the matrix work on
        the GPU; with unscaled_params the standard form is then rescaled on the GPU. The
        handle solves the standard form: see standard_form() for its size and row order."""
        self = cls.__new__(cls)
        self.lib = lib or _abi.load()
        a = sp.csc_matrix(qp.constraint_matrix)
        f64 = lambda v: np.ascontiguousarray(v, dtype=np.float64)
        keep = dict(l=f64(qp.variable_lower_bound), u=f64(qp.variable_upper_bound),
                    lc=f64(qp.constraint_lower_bound), uc=f64(qp.constraint_upper_bound),
                    c=f64(qp.objective_vector), colptr=np.ascontiguousarray(a.indptr, dtype=np.int64) + index_base,
                    rowval=np.ascontiguousarray(a.indices, dtype=np.int64) + index_base, nzval=f64(a.data))
        d = _abi.TwoSidedDesc()
        d.num_variables, d.num_constraints = a.shape[1], a.shape[0]
        d.nnz = int(keep["nzval"].size)
        d.variable_lower_bound = _abi.dptr(keep["l"])
        d.variable_upper_bound = _abi.dptr(keep["u"])
        d.constraint_lower_bound = _abi.dptr(keep["lc"])
        d.constraint_upper_bound = _abi.dptr(keep["uc"])
        d.objective_vector = _abi.dptr(keep["c"])
        d.objective_offset = float(qp.objective_offset)
        cp = params_to_c(unscaled_params) if unscaled_params is not None else None
        h = C.c_void_p()
        _abi.check(self.lib.gpdhg_problem_create_two_sided(C.byref(d), _abi.lptr(keep["colptr"]),
                                                           _abi.lptr(keep["rowval"]), _abi.dptr(keep["nzval"]),
                                                           int(index_base), C.byref(cp) if cp is not None else None,
                                                           C.byref(h)), self.lib)
        self.handle = h
        self.m = a.shape[0]
        self.n = self.standard_form()[0]
        return self

    def standard_form(self):
        """(variables, equalities, slacks, new_row_to_old) of the problem the handle solves."""
        nv, neq, ns = C.c_int32(), C.c_int32(), C.c_int32()
        order = np.empty(self.m, dtype=np.int32)
        _abi.check(self.lib.gpdhg_get_standard_form(self.handle, C.byref(nv), C.byref(neq), C.byref(ns),
                                                    _abi.iptr(order)), self.lib)
        return nv.value, neq.value, ns.value, order

    @classmethod
    def from_unscaled(cls, p: QuadraticProgrammingProblem, params: PdhgParameters, lib=None):
        """Rescaling on the GPU (gpdhg_problem_create_unscaled)."""
        self = cls.__new__(cls)
        self.lib = lib or _abi.load()
        d = unscaled_desc(p)
        self.n, self.m = d.desc.num_variables, d.desc.num_constraints
        cp = params_to_c(params)
        h = C.c_void_p()
        _abi.check(self.lib.gpdhg_problem_create_unscaled(d.ref, C.byref(cp), C.byref(h)), self.lib)
        self.handle = h
        return self

    def rescaling(self):
        con = np.empty(self.m)
        var = np.empty(self.n)
        _abi.check(self.lib.gpdhg_get_rescaling(self.handle, _abi.dptr(con), _abi.dptr(var)), self.lib)
        return con, var

    def solve(self, params: PdhgParameters, want_solution: bool = True):
        cp = params_to_c(params)
        res = _abi.Result()
        x = np.empty(self.n) if want_solution else None
        y = np.empty(self.m) if want_solution else None
        _abi.check(self.lib.gpdhg_solve(self.handle, C.byref(cp), C.byref(res), _abi.dptr(x), _abi.dptr(y)),
                   self.lib)
        return res, x, y

    def stats(self, count: int) -> List:
        out = []
        st = _abi.IterationStats()
        for i in range(count):
            _abi.check(self.lib.gpdhg_get_stats(self.handle, i, C.byref(st)), self.lib)
            out.append(stats_from_c(st))
        return out

    def current_iterate(self):
        x = np.empty(self.n)
        y = np.empty(self.m)
        _abi.check(self.lib.gpdhg_get_current_iterate(self.handle, _abi.dptr(x), _abi.dptr(y)), self.lib)
        return x, y

    def set_warm_start(self, x0: Optional[np.ndarray], y0: Optional[np.ndarray]):
        x0 = None if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
        y0 = None if y0 is None else np.ascontiguousarray(y0, dtype=np.float64)
        _abi.check(self.lib.gpdhg_set_warm_start(self.handle, _abi.dptr(x0), _abi.dptr(y0)), self.lib)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gpdhg_problem_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _print_stats(stats, verbosity):
    if verbosity < 2:
        return
    print(f"{'#iter':7s} {'#kkt':8s} {'seconds':7s} | {'pr norm':8s} {'du norm':8s}  {'gap':7s} | "
          f"{' pr obj':9s} {'pr norm':8s} {'du norm':7s} | {'rel pr':7s} {'rel du':7s} {'rel gap':7s} |")
    for s in stats:
        ci = s.convergence_information[0]
        print(f"{s.iteration_number:<6d}  {s.cumulative_kkt_matrix_passes:.1e}  {s.cumulative_time_sec:.1e} | "
              f"{ci.l2_primal_residual:.1e}  {ci.l2_dual_residual:.1e}  "
              f"{ci.primal_objective - ci.dual_objective:8.1e} | {ci.primal_objective:8.1e}  "
              f"{ci.l2_primal_variable:.1e}  {ci.l2_dual_variable:.1e} | {ci.relative_l2_primal_residual:.1e} "
              f"{ci.relative_l2_dual_residual:.1e} {ci.relative_optimality_gap:.1e} |")


def optimize(params: PdhgParameters, original_problem: QuadraticProgrammingProblem) -> SaddlePointOutput:
    validate(original_problem)
    if not is_linear_programming_problem(original_problem):
        raise NotImplementedError("quadratic objectives are not supported (LP only, as the solve loop)")
    t0 = time.time()
    scaled = rescale_problem(params.l_inf_ruiz_iterations, params.l2_norm_rescaling,
                             params.pock_chambolle_alpha, params.verbosity, original_problem)
    if params.verbosity >= 1:
        print(f"Preconditioning Time (seconds): {time.time() - t0:.2e}")
    if params.primal_importance <= 0 or not math.isfinite(params.primal_importance):
        raise ValueError("primal_importance must be positive and finite")
    with DeviceProblem(scaled_desc(scaled)) as dp:
        res, xs, ys = dp.solve(params)
        stats = dp.stats(res.num_iteration_stats)
    _print_stats(stats, params.verbosity)
    reason = TerminationReason(res.termination_reason)
    if params.verbosity >= 1:
        print(f"Terminated after {res.iteration_count + 1} iterations: {termination_reason_to_string(reason)}")
    return SaddlePointOutput(xs / scaled.variable_rescaling, ys / scaled.constraint_rescaling, reason,
                             termination_reason_to_string(reason), int(res.iteration_count), stats, res)


class DeviceBatch:
    """A gpdhg_batch handle: many scaled LPs packed on the GPU, solved together."""

    def __init__(self, descs, lib=None):
        self.lib = lib or _abi.load()
        self.descs = list(descs)
        arr = (_abi.LpDesc * len(self.descs))(*[d.desc for d in self.descs])
        h = C.c_void_p()
        _abi.check(self.lib.gpdhg_batch_create(len(self.descs), arr, C.byref(h)), self.lib)
        self.handle = h

    def solve(self, params: PdhgParameters, want_solution: bool = True):
        k = len(self.descs)
        cp = params_to_c(params)
        results = (_abi.Result * k)()
        xs = [np.empty(d.desc.num_variables) for d in self.descs] if want_solution else None
        ys = [np.empty(max(d.desc.num_constraints, 1)) for d in self.descs] if want_solution else None
        xp = (_abi._dp * k)(*[_abi.dptr(x) for x in xs]) if want_solution else None
        yp = (_abi._dp * k)(*[_abi.dptr(y) for y in ys]) if want_solution else None
        _abi.check(self.lib.gpdhg_batch_solve(self.handle, C.byref(cp), results, xp, yp), self.lib)
        if want_solution:
            ys = [y[:d.desc.num_constraints] for y, d in zip(ys, self.descs)]
        return [results[i] for i in range(k)], xs, ys

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gpdhg_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def optimize_batch(params: PdhgParameters, problems) -> List[SaddlePointOutput]:
    """optimize() for many LPs at once: host validation and rescaling per problem, then
    one packed solve on the GPU (every instance keeps its own step size, primal weight,
    restarts and termination)."""
    scaled = []
    for p in problems:
        validate(p)
        if not is_linear_programming_problem(p):
            raise NotImplementedError("quadratic objectives are not supported")
        scaled.append(rescale_problem(params.l_inf_ruiz_iterations, params.l2_norm_rescaling,
                                      params.pock_chambolle_alpha, params.verbosity, p))
    with DeviceBatch([scaled_desc(sq) for sq in scaled]) as db:
        results, xs, ys = db.solve(params)
    out = []
    for sq, r, x, y in zip(scaled, results, xs, ys):
        reason = TerminationReason(r.termination_reason)
        out.append(SaddlePointOutput(x / sq.variable_rescaling, y / sq.constraint_rescaling, reason,
                                     termination_reason_to_string(reason), int(r.iteration_count),
                                     [stats_from_c(r.last_iteration_stats)], r))
    return out


class Server:
    """A gpdhg_server: continuous batching of arriving scaled LPs on the GPU.

    submit() copies the LP and returns a ticket at once; poll() / wait() hand back
    (result, x, y) once the request has terminated (each ticket once). Requests are packed
    into device batches by worker threads as memory and workers free up, so results are
    bit-identical to solving each LP alone with the same parameters."""

    def __init__(self, hbm_budget_bytes: float = 0.0, max_resident: int = 0, max_cohort: int = 0,
                 workers: int = 0, linger_sec: float = 0.0, lib=None):
        self.lib = lib or _abi.load()
        cfg = _abi.ServerConfig()
        cfg.hbm_budget_bytes = hbm_budget_bytes
        cfg.max_resident = max_resident
        cfg.max_cohort = max_cohort
        cfg.workers = workers
        cfg.linger_sec = linger_sec
        h = C.c_void_p()
        _abi.check(self.lib.gpdhg_server_create(C.byref(cfg), C.byref(h)), self.lib)
        self.handle = h
        self._shapes = {}

    def footprint(self, desc: "_Desc", params: PdhgParameters) -> float:
        cp = params_to_c(params)
        return float(self.lib.gpdhg_server_footprint(desc.ref, C.byref(cp)))

    def submit(self, desc: "_Desc", params: PdhgParameters) -> int:
        cp = params_to_c(params)
        t = C.c_uint64()
        _abi.check(self.lib.gpdhg_server_submit(self.handle, desc.ref, C.byref(cp), C.byref(t)), self.lib)
        self._shapes[t.value] = (desc.desc.num_variables, desc.desc.num_constraints)
        return t.value

    def _take(self, ticket: int, timeout: float | None):
        n, m = self._shapes.get(ticket, (0, 0))   # unknown tickets are reported by the library
        res = _abi.Result()
        x = np.empty(n)
        y = np.empty(max(m, 1))
        if timeout is None:
            st = self.lib.gpdhg_server_poll(self.handle, ticket, C.byref(res), _abi.dptr(x), _abi.dptr(y))
        else:
            st = self.lib.gpdhg_server_wait(self.handle, ticket, float(timeout), C.byref(res), _abi.dptr(x),
                                            _abi.dptr(y))
        if st == _abi.ERR_NOT_READY:
            return None
        self._shapes.pop(ticket, None)
        _abi.check(st, self.lib)
        return res, x, y[:m]

    def poll(self, ticket: int):
        """(result, x, y) if the request has terminated, else None."""
        return self._take(ticket, None)

    def wait(self, ticket: int, timeout: float = 3600.0):
        """Blocks until the request terminates (None after `timeout` seconds)."""
        return self._take(ticket, timeout)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gpdhg_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
