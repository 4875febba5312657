"""GPU tests of the device-side transpose (csrc/ingest.cu). A lone problem sorts its own A
by column; a batch sorts the packed block-diagonal A of all its instances. Each instance's
block of the batch's A' must be the lone A' in the same storage order, so the same LP solved
both ways agrees bit for bit, here for column counts that take one, two and three 8-bit radix
passes, with empty columns, and next to other instances. (The values of A' against the
reference's are covered by the parity tests: A'y enters every primal step.)"""
import numpy as np
import pytest

import cupdlp
from cupdlp import synthetic
from cupdlp.solver import DeviceBatch, DeviceProblem, scaled_desc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n,density", [(60, 200, 0.05), (120, 5000, 0.004), (150, 70000, 0.0004)])
def test_lone_and_packed_transposes_agree(m, n, density):
    lp = synthetic.known_optimum_lp(11, m=m, n=n, neq=m // 2, density=density)
    a = lp.problem.constraint_matrix.tocsc()
    assert (np.diff(a.indptr) == 0).any()  # empty columns
    params = cupdlp.default_parameters(tolerance=1e-12, iteration_limit=96, time_sec_limit=60.0)
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
