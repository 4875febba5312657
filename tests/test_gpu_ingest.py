"""GPU tests of the device-side ingest (csrc/ingest.cu, gpdhg_problem_create_csc). A lone
problem sorts its own A by column; a batch sorts the packed block-diagonal A of all its
instances; the CSC entry uploads A' and sorts it into A. Each instance's
block of the batch's A' must be the lone A' in the same storage order, so the same LP solved
both ways agrees bit for bit, here for column counts that take one to four 8-bit radix passes,
with empty columns, and next to other instances. (The values of A' against the
reference's are covered by the parity tests: A'y enters every primal step.)"""
import numpy as np
import pytest

import cupdlp
from cupdlp import synthetic
from cupdlp.solver import DeviceBatch, DeviceProblem, scaled_desc, unscaled_desc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n,density", [(60, 200, 0.05), (120, 5000, 0.004), (150, 70000, 0.0004),
                                         (4, (1 << 24) + 100, 40 / (4 * ((1 << 24) + 100)))],
                         ids=["1pass", "2pass", "3pass", "4pass"])
def test_lone_and_packed_transposes_agree(m, n, density):
    lp = synthetic.known_optimum_lp(11, m=m, n=n, neq=m // 2, density=density)
    a = lp.problem.constraint_matrix.tocsc()
    assert (np.diff(a.indptr) == 0).any()  # empty columns
    params = cupdlp.default_parameters(tolerance=1e-12, iteration_limit=96 if n < (1 << 20) else 24,
                                       time_sec_limit=120.0)
    sq = cupdlp.rescale_problem(10, False, 1.0, 0, lp.problem)
    with DeviceProblem(scaled_desc(sq)) as dp:
        r, x, y = dp.solve(params)
    other = cupdlp.rescale_problem(10, False, 1.0, 0, synthetic.known_optimum_lp(12, m=40, n=90).problem)
    with DeviceBatch([scaled_desc(other), scaled_desc(sq), scaled_desc(other)]) as db:
        rs, xs, ys = db.solve(params)
    assert rs[1].total_number_iterations == r.total_number_iterations
    assert np.array_equal(xs[1], x)
    assert np.array_equal(ys[1], y)
    assert rs[1].last_iteration_stats.convergence_information.primal_objective == \
        r.last_iteration_stats.convergence_information.primal_objective


@pytest.mark.parametrize("base", [0, 1])
def test_csc_entry_builds_the_csr_entry_problem(base):
    """gpdhg_problem_create_csc (the matrix as Julia's SparseMatrixCSC, 0- or 1-based) gives
    the handle gpdhg_problem_create gives for the same scaled problem: same solve, bit for bit."""
    lp = synthetic.known_optimum_lp(13, m=150, n=4000, neq=90, density=0.005)
    params = cupdlp.default_parameters(tolerance=1e-12, iteration_limit=128, time_sec_limit=60.0)
    sq = cupdlp.rescale_problem(10, False, 1.0, 0, lp.problem)
    d = scaled_desc(sq)
    with DeviceProblem(d) as dp:
        r, x, y = dp.solve(params)
    a = sq.scaled_qp.constraint_matrix.tocsc()
    a.sort_indices()
    with DeviceProblem.from_csc(d, a, index_base=base) as dq:
        r2, x2, y2 = dq.solve(params)
    assert r2.total_number_iterations == r.total_number_iterations
    assert np.array_equal(x2, x) and np.array_equal(y2, y)


def test_csc_entry_unscaled_matches_unscaled_csr_entry():
    """The CSC entry with rescaling on the GPU matches gpdhg_problem_create_unscaled."""
    lp = synthetic.known_optimum_lp(14, m=120, n=900, neq=60, density=0.02)
    params = cupdlp.default_parameters(tolerance=1e-12, iteration_limit=128, time_sec_limit=60.0)
    with DeviceProblem.from_unscaled(lp.problem, params) as dp:
        r, x, y = dp.solve(params)
        con, var = dp.rescaling()
    a = lp.problem.constraint_matrix.tocsc()
    a.sort_indices()
    with DeviceProblem.from_csc(unscaled_desc(lp.problem), a, index_base=1, unscaled_params=params) as dq:
        r2, x2, y2 = dq.solve(params)
        con2, var2 = dq.rescaling()
    assert np.array_equal(con2, con) and np.array_equal(var2, var)
    assert np.array_equal(x2, x) and np.array_equal(y2, y)
