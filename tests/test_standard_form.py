"""CPU tests of the standard-form conversion (transform_to_standard_form,
src/quadratic_programming_io.jl:33-121): the oracle restatement against a hand-worked
example and against scipy's HiGHS on the two-sided LP itself, and the rejections of
gpdhg_problem_create_two_sided that happen before any GPU work."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp
from scipy.optimize import linprog

import cupdlp
from cupdlp import _abi, synthetic

import standard_form


def _worked_example():
    # row 0: 1 <= x0 + 2 x1 <= 3 (two-sided), row 1: 3 x0 <= 4, row 2: x1 = 5, row 3: x0 - x1 >= 2
    a = sp.csc_matrix(np.array([[1.0, 2.0], [3.0, 0.0], [0.0, 1.0], [1.0, -1.0]]))
    lc = np.array([1.0, -np.inf, 5.0, 2.0])
    uc = np.array([3.0, 4.0, 5.0, np.inf])
    return cupdlp.TwoSidedQpProblem(np.array([0.0, -1.0]), np.array([10.0, np.inf]), lc, uc, a, 7.0,
                                    np.array([1.0, -2.0]))


def test_oracle_on_a_hand_worked_example():
    """Row 0 gets slack column 2 (coefficient -1, bounds [1, 3], cost 0) and becomes '= 0';
    equality rows 0 and 2 move first; the '<=' row 1 is negated (rhs -4)."""
    q = _worked_example()
    sf = standard_form.transform_to_standard_form(q.variable_lower_bound, q.variable_upper_bound,
                                                  q.constraint_lower_bound, q.constraint_upper_bound,
                                                  q.constraint_matrix, q.objective_vector, q.objective_offset)
    assert sf["num_slacks"] == 1 and sf["num_equalities"] == 2
    assert list(sf["new_row_to_old"]) == [0, 2, 1, 3]
    want = np.array([[1.0, 2.0, -1.0], [0.0, 1.0, 0.0], [-3.0, 0.0, 0.0], [1.0, -1.0, 0.0]])
    assert np.array_equal(sf["A"].toarray(), want)
    assert list(sf["b"]) == [0.0, 5.0, -4.0, 2.0]
    assert list(sf["l"]) == [0.0, -1.0, 1.0] and list(sf["u"]) == [10.0, np.inf, 3.0]
    assert list(sf["c"]) == [1.0, -2.0, 0.0] and sf["offset"] == 7.0
    assert sf["A"].has_sorted_indices


def test_oracle_rejects_a_free_row():
    q = _worked_example()
    q.constraint_lower_bound[3] = -np.inf
    with pytest.raises(standard_form.StandardFormError, match="finite bounds"):
        standard_form.transform_to_standard_form(q.variable_lower_bound, q.variable_upper_bound,
                                                 q.constraint_lower_bound, q.constraint_upper_bound,
                                                 q.constraint_matrix, q.objective_vector, 0.0)


def _highs(c, a_eq, b_eq, a_ub, b_ub, lo, hi):
    r = linprog(c, A_ub=a_ub, b_ub=b_ub, A_eq=a_eq, b_eq=b_eq, bounds=list(zip(lo, hi)), method="highs")
    assert r.status == 0, r.message
    return r.fun


def test_oracle_standard_form_keeps_the_optimum():
    """HiGHS on the two-sided LP, on the oracle's standard form, and the planted optimum agree."""
    t = synthetic.two_sided_lp(5, m=120, n=300, density=0.03)
    q = t.problem
    a = sp.csr_matrix(q.constraint_matrix)
    lc, uc = q.constraint_lower_bound, q.constraint_upper_bound
    eq = lc == uc
    up = ~eq & np.isfinite(uc)
    dn = ~eq & np.isfinite(lc)
    hi = np.where(np.isinf(q.variable_upper_bound), None, q.variable_upper_bound)
    two = _highs(q.objective_vector, a[eq], lc[eq], sp.vstack([a[up], -a[dn]]),
                 np.concatenate([uc[up], -lc[dn]]), q.variable_lower_bound, hi)
    sf = standard_form.transform_to_standard_form(q.variable_lower_bound, q.variable_upper_bound, lc, uc,
                                                  q.constraint_matrix, q.objective_vector, 0.0)
    assert sf["num_slacks"] > 0 and not np.array_equal(sf["new_row_to_old"], np.arange(lc.size))
    s = sp.csr_matrix(sf["A"])
    k = sf["num_equalities"]
    hs = np.where(np.isinf(sf["u"]), None, sf["u"])
    std = _highs(sf["c"], s[:k], sf["b"][:k], -s[k:], -sf["b"][k:], sf["l"], hs)
    assert abs(two - t.optimal_objective) <= 1e-7 * max(1.0, abs(two))
    assert abs(std - two) <= 1e-7 * max(1.0, abs(two))


def test_transportation_two_sided_converts_to_the_transportation_lp():
    """The transportation LP's MPS form ('=' demand rows, '<=' supply rows) converts into the
    benchmark's standard form exactly (same matrix bits, right-hand side and row order)."""
    t = synthetic.transportation_two_sided(1, supplies=20, demands=50)
    p = synthetic.transportation_lp(1, supplies=20, demands=50).problem
    q = t.problem
    sf = standard_form.transform_to_standard_form(q.variable_lower_bound, q.variable_upper_bound,
                                                  q.constraint_lower_bound, q.constraint_upper_bound,
                                                  q.constraint_matrix, q.objective_vector, 0.0)
    a = p.constraint_matrix.tocsc()
    assert sf["num_slacks"] == 0 and sf["num_equalities"] == p.num_equalities
    assert np.array_equal(sf["A"].indptr, a.indptr) and np.array_equal(sf["A"].indices, a.indices)
    assert np.array_equal(sf["A"].data.view(np.int64), a.data.view(np.int64))
    assert np.array_equal(sf["b"], p.right_hand_side)


def _two_sided_err(lib, q, base=0, mutate=None):
    a = sp.csc_matrix(q.constraint_matrix)
    keep = dict(l=np.array(q.variable_lower_bound, dtype=np.float64), u=np.array(q.variable_upper_bound, dtype=np.float64),
                lc=np.array(q.constraint_lower_bound, dtype=np.float64),
                uc=np.array(q.constraint_upper_bound, dtype=np.float64),
                c=np.array(q.objective_vector, dtype=np.float64), cp=a.indptr.astype(np.int64) + base,
                rv=a.indices.astype(np.int64) + base, nz=a.data.astype(np.float64))
    if mutate:
        mutate(keep)
    d = _abi.TwoSidedDesc()
    d.num_variables, d.num_constraints, d.nnz = a.shape[1], a.shape[0], int(keep["nz"].size)
    d.variable_lower_bound, d.variable_upper_bound = _abi.dptr(keep["l"]), _abi.dptr(keep["u"])
    d.constraint_lower_bound, d.constraint_upper_bound = _abi.dptr(keep["lc"]), _abi.dptr(keep["uc"])
    d.objective_vector = _abi.dptr(keep["c"])
    h = C.c_void_p()
    st = lib.gpdhg_problem_create_two_sided(C.byref(d), _abi.lptr(keep["cp"]), _abi.lptr(keep["rv"]),
                                            _abi.dptr(keep["nz"]), base, None, C.byref(h))
    return st, lib.gpdhg_last_error().decode()


def test_two_sided_entry_rejects_bad_input_before_any_gpu_work(lib):
    q = _worked_example()
    st, msg = _two_sided_err(lib, q, mutate=lambda k: k["lc"].__setitem__(3, -np.inf))
    assert st == _abi.ERR_INVALID_PROBLEM and "finite bounds on at least one side" in msg
    st, msg = _two_sided_err(lib, q, mutate=lambda k: k["uc"].__setitem__(1, np.nan))
    assert st == _abi.ERR_INVALID_PROBLEM and "NaN found in constraint bounds" in msg
    st, msg = _two_sided_err(lib, q, base=1, mutate=lambda k: k["rv"].__setitem__(0, 0))
    assert st == _abi.ERR_INVALID_PROBLEM and "row index" in msg
    st, msg = _two_sided_err(lib, q, mutate=lambda k: k["nz"].__setitem__(0, np.nan))
    assert st == _abi.ERR_INVALID_PROBLEM and "constraint matrix" in msg
    # an equality row at +Inf leaves an infinite right-hand side, which validate rejects
    st, msg = _two_sided_err(lib, q, mutate=lambda k: (k["lc"].__setitem__(2, np.inf), k["uc"].__setitem__(2, np.inf)))
    assert st == _abi.ERR_INVALID_PROBLEM and "right hand side" in msg
    st, msg = _two_sided_err(lib, q, base=3)
    assert st == _abi.ERR_INVALID_ARGUMENT and "index_base" in msg
    h = C.c_void_p()
    assert lib.gpdhg_problem_create_two_sided(None, None, None, None, 0, None, C.byref(h)) == _abi.ERR_INVALID_ARGUMENT
    assert lib.gpdhg_get_standard_form(None, None, None, None, None) == _abi.ERR_INVALID_ARGUMENT


def test_oracle_pdhg_on_the_standard_form_reaches_the_planted_optimum(oracle_mod):
    """The oracle's restatement of optimize() on the oracle's standard form of a two-sided LP
    (slacks, negated and reordered rows) terminates optimal at the planted objective."""
    t = synthetic.two_sided_lp(6, m=150, n=400, density=0.03)
    q = t.problem
    sf = standard_form.transform_to_standard_form(q.variable_lower_bound, q.variable_upper_bound,
                                                  q.constraint_lower_bound, q.constraint_upper_bound,
                                                  q.constraint_matrix, q.objective_vector, q.objective_offset)
    n = sf["A"].shape[1]
    p = cupdlp.QuadraticProgrammingProblem(sf["l"], sf["u"], sp.csc_matrix((n, n)), sf["c"], sf["offset"],
                                           sp.csc_matrix(sf["A"]), sf["b"], sf["num_equalities"])
    params = cupdlp.default_parameters(tolerance=1e-8, iteration_limit=100_000, time_sec_limit=120.0)
    res, x, y, _ = oracle_mod.optimize(p, params)
    assert res.termination_reason == cupdlp.TerminationReason.TERMINATION_REASON_OPTIMAL
    po = res.last_iteration_stats.convergence_information.primal_objective
    assert abs(po - t.optimal_objective) <= 1e-6 * max(1.0, abs(t.optimal_objective))
