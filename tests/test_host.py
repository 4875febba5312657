"""CPU tests of the host package: parameter mapping, validation, generators."""
import ctypes as C
import math
import re

import numpy as np
import pytest
import scipy.sparse as sp

import cupdlp
from cupdlp import _abi, synthetic

import instances


def test_default_parameters_follow_solve_script():
    p = cupdlp.default_parameters(tolerance=1e-4)
    assert (p.l_inf_ruiz_iterations, p.l2_norm_rescaling, p.pock_chambolle_alpha, p.primal_importance,
            p.scale_invariant_initial_primal_weight, p.termination_evaluation_frequency) == (10, False, 1.0, 1.0, True, 64)
    rp = p.restart_params
    assert (rp.restart_scheme, rp.restart_to_current_metric, rp.restart_frequency_if_fixed) == (
        cupdlp.ADAPTIVE_KKT, cupdlp.KKT_GREEDY, 1000)
    assert (rp.artificial_restart_threshold, rp.sufficient_reduction_for_restart,
            rp.necessary_reduction_for_restart, rp.primal_weight_update_smoothing) == (0.36, 0.2, 0.8, 0.5)
    assert p.step_size_policy_params == cupdlp.AdaptiveStepsizeParams(0.3, 0.6)
    tc = p.termination_criteria
    assert (tc.eps_optimal_absolute, tc.eps_optimal_relative, tc.eps_primal_infeasible) == (1e-4, 1e-4, 1e-8)


def test_params_to_c_roundtrip():
    p = cupdlp.default_parameters(tolerance=1e-6, iteration_limit=77)
    p.pock_chambolle_alpha = None
    c = cupdlp.params_to_c(p)
    assert math.isnan(c.pock_chambolle_alpha)
    assert c.iteration_limit == 77 and c.eps_optimal_relative == 1e-6
    assert c.restart_scheme == 2 and c.restart_to_current_metric == 1 and c.step_size_policy == 0
    p.step_size_policy_params = cupdlp.ConstantStepsizeParams()
    assert cupdlp.params_to_c(p).step_size_policy == 1


def test_restart_parameter_assertions():
    with pytest.raises(AssertionError):
        cupdlp.construct_restart_parameters(cupdlp.ADAPTIVE_KKT, cupdlp.KKT_GREEDY, 1000, 0.36, 0.9, 0.8, 0.5)
    with pytest.raises(AssertionError):
        cupdlp.construct_restart_parameters(cupdlp.ADAPTIVE_KKT, cupdlp.KKT_GREEDY, 1, 0.36, 0.2, 0.8, 0.5)


def test_termination_reason_strings():
    assert cupdlp.termination_reason_to_string(cupdlp.TERMINATION_REASON_OPTIMAL) == "OPTIMAL"
    assert cupdlp.termination_reason_to_string(cupdlp.TerminationReason(6)) == "KKT_MATRIX_PASS_LIMIT"


@pytest.mark.parametrize("mutate,msg", [
    (lambda p: setattr(p, "right_hand_side", np.array([np.nan])), "right hand side"),
    (lambda p: setattr(p, "objective_vector", np.array([np.inf])), "objective vector"),
    (lambda p: setattr(p, "variable_lower_bound", np.array([np.inf])), "+Inf"),
    (lambda p: setattr(p, "variable_upper_bound", np.array([-np.inf])), "-Inf"),
    (lambda p: setattr(p, "variable_lower_bound", np.array([np.nan])), "NaN"),
    (lambda p: setattr(p, "right_hand_side", np.array([1.0, 2.0])), "right_hand_side"),
])
def test_validate_rejects(mutate, msg):
    p, _ = instances.tiny()
    mutate(p)
    with pytest.raises(cupdlp.InvalidProblemError, match=re.escape(msg)):
        cupdlp.validate(p)


def test_validate_rejects_nan_matrix():
    p, _ = instances.tiny()
    p.constraint_matrix = sp.csc_matrix(np.array([[np.nan]]))
    with pytest.raises(cupdlp.InvalidProblemError, match="constraint matrix"):
        cupdlp.validate(p)


def test_known_optimum_generator_shape():
    lp = synthetic.known_optimum_lp(0)
    p = lp.problem
    assert (p.num_constraints, p.num_variables, p.num_equalities) == (1000, 2000, 600)
    assert p.constraint_matrix.nnz == 10000
    assert np.all(p.variable_lower_bound == 0) and np.all(p.variable_upper_bound == 10)
    a = p.constraint_matrix
    ax = a @ lp.x_star
    assert np.allclose(ax[:600], p.right_hand_side[:600])
    assert np.all(ax[600:] >= p.right_hand_side[600:] - 1e-12)
    # complementary slackness of the planted pair
    slack = ax[600:] - p.right_hand_side[600:]
    assert np.all(lp.y_star[600:][slack > 1e-9] == 0.0)
    lam = p.objective_vector - a.T @ lp.y_star
    assert np.all(lam[lp.x_star == 0] >= -1e-12) and np.all(lam[lp.x_star == 10] <= 1e-12)
    interior = (lp.x_star > 0) & (lp.x_star < 10)
    assert np.allclose(lam[interior], 0.0, atol=1e-12)


def test_transportation_generator_shape():
    lp = synthetic.transportation_lp(1, supplies=50, demands=200)
    p = lp.problem
    assert (p.num_constraints, p.num_variables, p.num_equalities) == (250, 10000, 200)
    a = sp.csc_matrix(p.constraint_matrix)
    assert np.all(np.diff(a.indptr) == 2)
    supply = -p.right_hand_side[200:]
    assert supply.sum() == pytest.approx(1.1 * p.right_hand_side[:200].sum())


def test_power_law_generator_small():
    lp = synthetic.power_law_lp(5, m=20000, n=40000, target_nnz=400000)
    p = lp.problem
    a = sp.csr_matrix(p.constraint_matrix)
    assert 0.9 * 400000 < a.nnz <= 400000 * 1.05
    row_len = np.diff(a.indptr)
    assert row_len.max() > 20 * row_len.mean()   # skewed rows
    assert np.all(np.diff(sp.csc_matrix(a).indptr) >= 1)  # every column has an entry


def test_batch_generator_mix():
    lps = synthetic.batch_lps(3, count=24, median_m=300, m_range=(50, 2000))
    assert len(lps) == 24
    kinds = [lp.name.startswith("transportation") for lp in lps]
    assert 0 < sum(kinds) < 24
    for lp in lps:
        assert lp.problem.num_constraints >= 2


def test_serving_stream_poisson():
    reqs = synthetic.serving_stream(0, rate_per_sec=50, duration_sec=2.0, max_requests=200) if False else None
    rng = np.random.default_rng(0)
    gaps = rng.exponential(1 / 50, 10000)
    assert gaps.mean() == pytest.approx(1 / 50, rel=0.05)


def test_ctypes_struct_sizes_match_header(tmp_path):
    import subprocess, os
    src = tmp_path / "sz.c"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "gpdhg.h"\nint main(){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n",'
                   'sizeof(gpdhg_params), sizeof(gpdhg_convergence_information), sizeof(gpdhg_infeasibility_information),'
                   'sizeof(gpdhg_iteration_stats), sizeof(gpdhg_result), sizeof(gpdhg_lp_desc), sizeof(gpdhg_server_config),'
                   'offsetof(gpdhg_params, precision), offsetof(gpdhg_result, last_iteration_stats),'
                   'sizeof(gpdhg_two_sided_desc), offsetof(gpdhg_two_sided_desc, objective_offset));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", inc, str(src), "-o", str(exe)], check=True)
    got = list(map(int, subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()))
    want = [C.sizeof(_abi.Params), C.sizeof(_abi.ConvergenceInformation), C.sizeof(_abi.InfeasibilityInformation),
            C.sizeof(_abi.IterationStats), C.sizeof(_abi.Result), C.sizeof(_abi.LpDesc), C.sizeof(_abi.ServerConfig),
            _abi.Params.precision.offset, _abi.Result.last_iteration_stats.offset,
            C.sizeof(_abi.TwoSidedDesc), _abi.TwoSidedDesc.objective_offset.offset]
    assert got == want


def test_reciprocal_division_is_correctly_rounded():
    """The evaluation kernels divide by a vector or a weight sum through its reciprocal r = 1/b
    and one correction step, q = a r, q' = q + (a - q b) r with both steps fused
    multiply-adds (div_rcp in eval_kernels.cuh). The same arithmetic with libm's fma gives
    IEEE a / b on random operands over a wide exponent range."""
    libm = C.CDLL("libm.so.6")
    fma = libm.fma
    fma.restype = C.c_double
    fma.argtypes = [C.c_double, C.c_double, C.c_double]
    rng = np.random.default_rng(7)
    a = rng.standard_normal(20000) * np.exp2(rng.integers(-60, 60, 20000))
    b = np.abs(rng.standard_normal(20000)) * np.exp2(rng.integers(-60, 60, 20000)) + 1e-300
    for ai, bi in zip(a.tolist(), b.tolist()):
        r = 1.0 / bi
        q = ai * r
        q1 = fma(fma(-q, bi, ai), r, q)
        assert q1 == ai / bi, (ai, bi)
