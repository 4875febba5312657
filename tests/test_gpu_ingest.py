"""GPU tests of the device-side ingest (csrc/ingest.cu, gpdhg_problem_create_csc). A lone
problem sorts its own A by column; a batch sorts the packed block-diagonal A of all its
instances; the CSC entry uploads A' and sorts it into A. Each instance's
block of the batch's A' must be the lone A' in the same storage order, so the same LP solved
both ways agrees bit for bit, here for column counts that take one to four 8-bit radix passes,
with empty columns, and next to other instances. (The values of A' against the
reference's are covered by the parity tests: A'y enters every primal step.) The two-sided
entry (the MPS reader's standard-form conversion on the GPU) is checked against the oracle's
restatement of transform_to_standard_form the same way."""
import numpy as np
import pytest
import scipy.sparse as sp

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


def _oracle_standard_form(q):
    import standard_form
    sf = standard_form.transform_to_standard_form(q.variable_lower_bound, q.variable_upper_bound,
                                                  q.constraint_lower_bound, q.constraint_upper_bound,
                                                  q.constraint_matrix, q.objective_vector, q.objective_offset)
    n = sf["A"].shape[1]
    p = cupdlp.QuadraticProgrammingProblem(sf["l"], sf["u"], sp.csc_matrix((n, n)), sf["c"], sf["offset"],
                                           sp.csr_matrix(sf["A"]), sf["b"], sf["num_equalities"])
    return sf, p


@pytest.mark.parametrize("base", [0, 1])
def test_two_sided_entry_builds_the_oracle_standard_form(base):
    """gpdhg_problem_create_two_sided (slacks, '<=' flips and the row reordering on the GPU)
    gives the handle gpdhg_problem_create gives for the oracle's standard form: same size,
    row order and solve, bit for bit."""
    t = synthetic.two_sided_lp(21, m=300, n=1500, density=0.01)
    sf, p = _oracle_standard_form(t.problem)
    assert sf["num_slacks"] > 0 and not np.array_equal(sf["new_row_to_old"], np.arange(p.num_constraints))
    params = cupdlp.default_parameters(tolerance=1e-12, iteration_limit=128, time_sec_limit=60.0)
    with DeviceProblem(unscaled_desc(p)) as dp:
        r, x, y = dp.solve(params)
    with DeviceProblem.from_two_sided(t.problem, index_base=base) as dq:
        nv, neq, ns, order = dq.standard_form()
        r2, x2, y2 = dq.solve(params)
    assert (nv, neq, ns) == (p.num_variables, sf["num_equalities"], sf["num_slacks"])
    assert np.array_equal(order, sf["new_row_to_old"])
    assert r2.total_number_iterations == r.total_number_iterations
    assert np.array_equal(x2, x) and np.array_equal(y2, y)


def test_two_sided_entry_rescaled_matches_the_unscaled_entry():
    t = synthetic.two_sided_lp(23, m=200, n=700, density=0.02)
    sf, p = _oracle_standard_form(t.problem)
    params = cupdlp.default_parameters(tolerance=1e-12, iteration_limit=128, time_sec_limit=60.0)
    with DeviceProblem.from_unscaled(p, params) as dp:
        r, x, y = dp.solve(params)
        con, var = dp.rescaling()
    with DeviceProblem.from_two_sided(t.problem, index_base=1, unscaled_params=params) as dq:
        r2, x2, y2 = dq.solve(params)
        con2, var2 = dq.rescaling()
    assert np.array_equal(con2, con) and np.array_equal(var2, var)
    assert np.array_equal(x2, x) and np.array_equal(y2, y)


def test_two_sided_entry_solves_to_the_planted_optimum():
    t = synthetic.two_sided_lp(22, m=200, n=500, density=0.02)
    params = cupdlp.default_parameters(tolerance=1e-8, iteration_limit=200_000, time_sec_limit=60.0)
    with DeviceProblem.from_two_sided(t.problem, unscaled_params=params) as dq:
        r, _, _ = dq.solve(params)
    assert r.termination_reason == cupdlp.TerminationReason.TERMINATION_REASON_OPTIMAL
    po = r.last_iteration_stats.convergence_information.primal_objective
    assert abs(po - t.optimal_objective) <= 1e-6 * max(1.0, abs(t.optimal_objective))


def test_two_sided_transportation_matches_the_benchmark_problem():
    """The transportation LP (1M variables, 2M nonzeros) in its MPS form ('<=' supply rows)
    gives the benchmark's standard-form handle bit for bit; prints both creation times."""
    import time
    t = synthetic.transportation_two_sided(1)
    p = synthetic.transportation_lp(1).problem
    params = cupdlp.default_parameters(tolerance=1e-12, iteration_limit=64, time_sec_limit=60.0)
    d = unscaled_desc(p)
    with DeviceProblem(unscaled_desc(synthetic.known_optimum_lp(0, m=10, n=20, density=0.2).problem)):
        pass  # context and first-use costs out of the timings below
    t0 = time.perf_counter()
    with DeviceProblem(d) as dp:
        t1 = time.perf_counter()
        r, x, y = dp.solve(params)
    t2 = time.perf_counter()
    with DeviceProblem.from_two_sided(t.problem, index_base=1) as dq:
        t3 = time.perf_counter()
        nv, neq, ns, order = dq.standard_form()
        r2, x2, y2 = dq.solve(params)
    assert (nv, neq, ns) == (p.num_variables, p.num_equalities, 0)
    assert np.array_equal(order, np.arange(p.num_constraints))
    assert np.array_equal(x2, x) and np.array_equal(y2, y)
    print(f"\ntransportation create from CSR {1e3 * (t1 - t0):.1f} ms, from the two-sided CSC "
          f"{1e3 * (t3 - t2):.1f} ms")
