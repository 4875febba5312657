"""GPU tests of rescale_problem on the device (gpdhg_problem_create_unscaled): the scaling
vectors match the host restatement (Ruiz bit for bit; Pock-Chambolle and the L2 rescaling,
whose sums add in another order, to 1e-14), and solving the device-rescaled problem reaches
the same optimum as solving the host-rescaled one."""
import numpy as np
import pytest

import cupdlp
from cupdlp import synthetic
from cupdlp.solver import DeviceProblem, scaled_desc

import instances

pytestmark = pytest.mark.gpu


def _lps():
    # plain, transportation-shaped, free variables, an empty row and column, no constraints
    return [synthetic.known_optimum_lp(0).problem, synthetic.transportation_lp(2, 40, 120).problem,
            instances.free_variables()[0], instances.empty_rows_and_columns(), instances.no_constraints()]


@pytest.mark.parametrize("ruiz,l2,alpha", [(10, False, None), (10, False, 1.0), (0, True, None), (10, True, 1.0),
                                           (3, False, 0.5)])
def test_device_rescaling_matches_host(ruiz, l2, alpha):
    for p in _lps():
        params = cupdlp.default_parameters(tolerance=1e-6)
        params.l_inf_ruiz_iterations = ruiz
        params.l2_norm_rescaling = l2
        params.pock_chambolle_alpha = alpha
        host = cupdlp.rescale_problem(ruiz, l2, alpha, 0, p)
        with DeviceProblem.from_unscaled(p, params) as dp:
            con, var = dp.rescaling()
        if not l2 and alpha is None:
            assert np.array_equal(con, host.constraint_rescaling)
            assert np.array_equal(var, host.variable_rescaling)
        else:
            np.testing.assert_allclose(con, host.constraint_rescaling, rtol=1e-14, atol=0)
            np.testing.assert_allclose(var, host.variable_rescaling, rtol=1e-14, atol=0)


def test_device_rescaled_solve_reaches_the_same_optimum():
    lp = synthetic.known_optimum_lp(0)
    params = cupdlp.default_parameters(tolerance=1e-8)
    host = cupdlp.rescale_problem(params.l_inf_ruiz_iterations, params.l2_norm_rescaling,
                                  params.pock_chambolle_alpha, 0, lp.problem)
    with DeviceProblem(scaled_desc(host)) as dp:
        r_host, _, _ = dp.solve(params)
    with DeviceProblem.from_unscaled(lp.problem, params) as dp:
        r_dev, x, y = dp.solve(params)
        con, var = dp.rescaling()
    assert r_dev.termination_reason == r_host.termination_reason == 1
    ph = r_host.last_iteration_stats.convergence_information.primal_objective
    pd = r_dev.last_iteration_stats.convergence_information.primal_objective
    # the two scaled problems differ at round-off level (Pock-Chambolle sums in another
    # order), so the two runs take different paths and each stops somewhere inside the
    # 1e-8 relative-KKT ball around the optimum
    assert pd == pytest.approx(ph, rel=1e-7)
    assert pd == pytest.approx(lp.optimal_objective, rel=1e-6)
    # the unscaled solution of the device path satisfies the bounds
    xu = x / var
    assert np.all(xu >= lp.problem.variable_lower_bound - 1e-6)
    assert np.all(xu <= lp.problem.variable_upper_bound + 1e-6)


def test_unscaled_descriptor_must_not_carry_scaling():
    lp = synthetic.known_optimum_lp(0)
    host = cupdlp.rescale_problem(10, False, 1.0, 0, lp.problem)
    d = scaled_desc(host)   # carries original_* and rescaling vectors
    import ctypes as C
    lib = cupdlp._abi.load()
    h = C.c_void_p()
    cp = cupdlp.params_to_c(cupdlp.default_parameters())
    assert lib.gpdhg_problem_create_unscaled(d.ref, C.byref(cp), C.byref(h)) == cupdlp._abi.ERR_INVALID_ARGUMENT
