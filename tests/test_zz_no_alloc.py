"""gpdhg_convergence_noalloc: the reference's termination statistics of a candidate
solution, computed by the library without allocating any GPU memory (its scratch is a
fixed device array inside the library), for callers that may not allocate at that moment —
code recording a CUDA graph, or a host whose own memory pool owns the device.

The statistics must match the ones gpdhg_solve reports for the same averaged iterate, on
two calls in a row (the second call reuses the scratch the first one left behind). This
file is collected last, so a run that stops at the first failure has run everything else.
"""
import ctypes as C

import numpy as np
import pytest

import cupdlp
from cupdlp import _abi, synthetic
from cupdlp.solver import DeviceProblem, scaled_desc

pytestmark = pytest.mark.gpu

FIELDS = ["primal_objective", "dual_objective", "l2_primal_residual", "l2_dual_residual",
          "l_inf_primal_residual", "l_inf_dual_residual", "relative_l2_primal_residual",
          "relative_l2_dual_residual", "relative_optimality_gap", "l2_primal_variable",
          "l_inf_primal_variable", "l2_dual_variable", "l_inf_dual_variable"]


def test_noalloc_statistics_match_solver_twice():
    torch = pytest.importorskip("torch")
    lib = _abi.load()
    lp = synthetic.known_optimum_lp(11, m=200, n=400, density=0.03)
    p = lp.problem
    # no rescaling: the solver's averaged iterate is the unscaled candidate itself
    params = cupdlp.default_parameters(tolerance=1e-6, time_sec_limit=120.0)
    params.l_inf_ruiz_iterations = 0
    params.pock_chambolle_alpha = None
    sq = cupdlp.rescale_problem(0, False, None, 0, p)
    with DeviceProblem(scaled_desc(sq)) as dp:
        res, x, y = dp.solve(params)
    want = res.last_iteration_stats.convergence_information
    a = p.constraint_matrix.tocsr()
    dev = torch.device("cuda")
    t = lambda v: torch.as_tensor(np.ascontiguousarray(v, dtype=np.float64), device=dev)
    bufs = [t(p.variable_lower_bound), t(p.variable_upper_bound), t(p.objective_vector), t(p.right_hand_side),
            t(x), t(y), t(a @ x), t(a.T @ y)]
    torch.cuda.synchronize()
    ptr = lambda b: C.cast(C.c_void_p(b.data_ptr()), _abi._dp)
    fn = lib.gpdhg_convergence_noalloc
    for call in range(2):
        out = _abi.ConvergenceInformation()
        st = fn(p.num_variables, p.num_constraints, p.num_equalities, p.objective_constant,
                *[ptr(b) for b in bufs], 1e-6, 1e-6, None, C.byref(out))
        assert st == _abi.OK, lib.gpdhg_last_error().decode()
        for f in FIELDS:
            w, g = getattr(want, f), getattr(out, f)
            assert g == pytest.approx(w, rel=1e-6, abs=1e-9), (call, f, g, w)


def test_noalloc_rejects_oversized_input():
    lib = _abi.load()
    out = _abi.ConvergenceInformation()
    null = C.cast(None, _abi._dp)
    one = (C.c_double * 1)()
    p1 = C.cast(one, _abi._dp)
    st = lib.gpdhg_convergence_noalloc((1 << 24) + 1, 0, 0, 0.0, p1, p1, p1, null, p1, null, null, p1,
                                       1e-6, 1e-6, None, C.byref(out))
    assert st == _abi.ERR_INVALID_ARGUMENT
    assert "16,777,216" in lib.gpdhg_last_error().decode()
