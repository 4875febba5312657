"""gpdhg_convergence_noalloc: the reference's termination statistics of a candidate
solution, computed by the library without allocating any GPU memory (its scratch is a fixed
device array inside the library), for callers that may not allocate at that moment — a host
whose own memory pool owns the device, or a serving path with a fixed memory budget.

Checked against an independent numpy restatement of compute_convergence_information and
against the statistics gpdhg_solve reports for the same averaged iterate, on two calls in a
row (the second call reuses the scratch the first one left behind), at sizes that use one
and many 4,096-element items (with a ragged last item), with the device's free memory
unchanged across the calls. The call is synchronous, so a capturing stream is refused and
the caller's capture stays usable. This file is collected last, so a run that stops at the
first failure has run everything else.
"""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

import cupdlp
from cupdlp import _abi, synthetic
from cupdlp.solver import DeviceProblem, scaled_desc
from kkt import convergence_information

pytestmark = pytest.mark.gpu

FIELDS = ["primal_objective", "dual_objective", "l2_primal_residual", "l2_dual_residual",
          "l_inf_primal_residual", "l_inf_dual_residual", "relative_l2_primal_residual",
          "relative_l2_dual_residual", "relative_l_inf_primal_residual", "relative_l_inf_dual_residual",
          "relative_optimality_gap", "l2_primal_variable", "l_inf_primal_variable", "l2_dual_variable",
          "l_inf_dual_variable"]


def _device_buffers(torch, p, x, y):
    a = sp.csr_matrix(p.constraint_matrix)
    dev = torch.device("cuda")
    t = lambda v: torch.as_tensor(np.ascontiguousarray(v, dtype=np.float64), device=dev)
    bufs = [t(p.variable_lower_bound), t(p.variable_upper_bound), t(p.objective_vector), t(p.right_hand_side),
            t(x), t(y), t(a @ x), t(a.T @ y)]
    torch.cuda.synchronize()
    return bufs


def _call(lib, p, bufs, eps, stream=None):
    ptr = lambda b: C.cast(C.c_void_p(b.data_ptr()), _abi._dp)
    out = _abi.ConvergenceInformation()
    st = lib.gpdhg_convergence_noalloc(p.num_variables, p.num_constraints, p.num_equalities, p.objective_constant,
                                       *[ptr(b) for b in bufs], eps, eps, stream, C.byref(out))
    return st, out


def test_noalloc_statistics_match_solver_and_numpy_twice():
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
    ref = convergence_information(p, x, y, 1e-6, 1e-6)
    bufs = _device_buffers(torch, p, x, y)
    for call in range(2):
        st, out = _call(lib, p, bufs, 1e-6)
        assert st == _abi.OK, lib.gpdhg_last_error().decode()
        for f in FIELDS:
            g = getattr(out, f)
            assert g == pytest.approx(getattr(want, f), rel=1e-6, abs=1e-9), (call, f, g, getattr(want, f))
            assert g == pytest.approx(ref[f], rel=1e-10, abs=1e-12), (call, f, g, ref[f])


def _random_candidate(n, m, neq, seed):
    """A candidate that is no solution: bound violations on both sides, negative duals on
    inequality rows, infinite bounds on some columns, so that every statistic is non-trivial."""
    rng = np.random.default_rng(seed)
    a = sp.random(m, n, density=8.0 / n, format="csr", random_state=rng, data_rvs=rng.standard_normal)
    l = np.where(rng.random(n) < 0.2, -np.inf, rng.uniform(-5, 0, n))
    u = np.where(rng.random(n) < 0.2, np.inf, rng.uniform(1, 5, n))
    c = rng.standard_normal(n)
    b = rng.standard_normal(m)
    p = cupdlp.QuadraticProgrammingProblem(l, u, sp.csc_matrix((n, n)), c, 0.75, sp.csc_matrix(a), b, neq)
    x = rng.uniform(-7, 7, n)
    y = rng.standard_normal(m)
    return p, x, y


@pytest.mark.parametrize("n,m", [(20000, 9000), (4096 * 3 + 1, 4095)])
def test_noalloc_many_items_against_numpy_without_allocating(n, m):
    torch = pytest.importorskip("torch")
    lib = _abi.load()
    p, x, y = _random_candidate(n, m, m // 3, seed=n + m)
    ref = convergence_information(p, x, y, 1e-4, 1e-4)
    bufs = _device_buffers(torch, p, x, y)
    st, _ = _call(lib, p, bufs, 1e-4)   # the first call in this context looks the scratch address up
    assert st == _abi.OK, lib.gpdhg_last_error().decode()
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for call in range(2):
        st, out = _call(lib, p, bufs, 1e-4)
        assert st == _abi.OK, lib.gpdhg_last_error().decode()
        for f in FIELDS:
            assert getattr(out, f) == pytest.approx(ref[f], rel=1e-10, abs=1e-12), (call, f)
        assert out.corrected_dual_objective == -np.inf
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before, (free_before, free_after)


def test_noalloc_refuses_a_capturing_stream_and_leaves_the_capture_valid():
    torch = pytest.importorskip("torch")
    lib = _abi.load()
    p, x, y = _random_candidate(3000, 1000, 300, seed=5)
    bufs = _device_buffers(torch, p, x, y)
    src = torch.arange(1024, dtype=torch.float64, device="cuda")
    dst = torch.empty_like(src)
    dst.copy_(src * 2.0)   # warm up the captured op outside the capture
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        dst.copy_(src * 3.0)
        st, _ = _call(lib, p, bufs, 1e-4, stream=C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == _abi.ERR_NOT_SUPPORTED
    assert "captured" in lib.gpdhg_last_error().decode()
    dst.zero_()
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(dst, src * 3.0)
    st, out = _call(lib, p, bufs, 1e-4)   # usable again outside the capture
    assert st == _abi.OK, lib.gpdhg_last_error().decode()
    assert out.primal_objective == pytest.approx(convergence_information(p, x, y, 1e-4, 1e-4)["primal_objective"],
                                                 rel=1e-10)


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
