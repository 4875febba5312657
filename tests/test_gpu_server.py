"""GPU tests of the serving loop (gpdhg_server_*): requests that arrive while others are
on the device are admitted as workers and memory free up, and every result is the same,
bit for bit, as the same LP solved alone with the same parameters."""
import time

import numpy as np
import pytest

import cupdlp
from cupdlp import synthetic
from cupdlp.solver import DeviceProblem, Server, scaled_desc

pytestmark = pytest.mark.gpu


def _params(precision, tol):
    # the iteration limit keeps every request's end independent of the wall clock
    return cupdlp.default_parameters(tolerance=tol, precision=precision, iteration_limit=60_000,
                                     time_sec_limit=300.0)


def _stream(seed, count):
    lps = synthetic.batch_lps(seed, count=count, median_m=300, m_range=(60, 2500))
    return [cupdlp.rescale_problem(10, False, 1.0, 0, lp.problem) for lp in lps]


def _alone(sq, params):
    with DeviceProblem(scaled_desc(sq)) as dp:
        return dp.solve(params)


def _same(served, alone, k):
    (rs, xs, ys), (ra, xa, ya) = served, alone
    assert rs.termination_reason == ra.termination_reason, k
    assert rs.iteration_count == ra.iteration_count, k
    assert rs.total_number_iterations == ra.total_number_iterations, k
    assert np.array_equal(xs, xa), k
    assert np.array_equal(ys, ya), k
    cs = rs.last_iteration_stats.convergence_information
    ca = ra.last_iteration_stats.convergence_information
    assert cs.primal_objective == ca.primal_objective and cs.dual_objective == ca.dual_objective, k


@pytest.mark.parametrize("precision,tol", [(cupdlp.Precision.FP64, 1e-6), (cupdlp.Precision.FP32, 1e-4)])
def test_served_equals_alone_in_a_mix(precision, tol):
    scaled = _stream(31, 12)
    params = _params(precision, tol)
    descs = [scaled_desc(sq) for sq in scaled]
    with Server(workers=2, max_cohort=4, linger_sec=0.001) as srv:
        tickets = []
        # three waves: later requests arrive while earlier cohorts are on the GPU
        for wave in range(3):
            for d in descs[4 * wave:4 * wave + 4]:
                tickets.append(srv.submit(d, params))
            time.sleep(0.05)
        served = [srv.wait(t, timeout=600.0) for t in tickets]
    for k, sq in enumerate(scaled):
        assert served[k] is not None, k
        _same(served[k], _alone(sq, params), k)


def test_backfill_under_a_tight_budget_and_mixed_parameters():
    scaled = _stream(32, 8)
    p_a = _params(cupdlp.Precision.FP64, 1e-4)
    p_b = _params(cupdlp.Precision.FP64, 1e-6)
    descs = [scaled_desc(sq) for sq in scaled]
    with Server(workers=2, max_cohort=3) as srv:
        biggest = max(srv.footprint(d, p_a) for d in descs)
    # room for about two of the largest requests at a time: the rest wait and back-fill
    with Server(hbm_budget_bytes=2.2 * biggest, workers=2, max_cohort=3) as srv:
        plist = [p_a if k % 2 == 0 else p_b for k in range(len(descs))]
        tickets = [srv.submit(d, p) for d, p in zip(descs, plist)]
        served = [srv.wait(t, timeout=600.0) for t in tickets]
    for k, (sq, p) in enumerate(zip(scaled, plist)):
        _same(served[k], _alone(sq, p), k)


def test_admission_and_ticket_lifecycle():
    sq = _stream(33, 1)[0]
    d = scaled_desc(sq)
    params = _params(cupdlp.Precision.FP64, 1e-6)
    with Server(hbm_budget_bytes=1e5, workers=1) as srv:
        with pytest.raises(cupdlp._abi.GpdhgError) as e:
            srv.submit(d, params)
        assert e.value.status == cupdlp._abi.ERR_ADMISSION
    with Server(workers=1) as srv:
        t = srv.submit(d, params)
        got = srv.wait(t, timeout=600.0)
        assert got is not None and got[0].termination_reason == 1
        with pytest.raises(cupdlp._abi.GpdhgError) as e:   # a ticket is handed out once
            srv.wait(t, timeout=1.0)
        assert e.value.status == cupdlp._abi.ERR_INVALID_ARGUMENT


def test_fp32_refine_and_constant_step_requests_are_served_alone():
    """A batch has no FP64 hand-off and only the adaptive step size; such requests are
    solved as lone problems by the worker and equal the lone solve bit for bit."""
    scaled = _stream(34, 4)
    p_ref = _params(cupdlp.Precision.FP32_REFINE, 1e-7)
    p_const = _params(cupdlp.Precision.FP64, 1e-6)
    p_const.step_size_policy_params = cupdlp.ConstantStepsizeParams()
    with Server(workers=2, max_cohort=4) as srv:
        plist = [p_ref, p_const, p_ref, _params(cupdlp.Precision.FP64, 1e-6)]
        tickets = [srv.submit(scaled_desc(sq), p) for sq, p in zip(scaled, plist)]
        served = [srv.wait(t, timeout=600.0) for t in tickets]
    for k, (sq, p) in enumerate(zip(scaled, plist)):
        _same(served[k], _alone(sq, p), k)
    assert served[0][0].fp64_handoff_iteration > 0


def test_results_are_handed_out_as_each_instance_terminates():
    """Requests packed into one cohort: the quick ones' results are collected while the slow
    one (a power-law LP that runs to the 60,000-iteration limit) is still on the device, and
    all equal their lone solves."""
    big = cupdlp.rescale_problem(10, False, 1.0, 0, synthetic.power_law_lp(1, m=300, n=600,
                                                                          target_nnz=3000).problem)
    small = [cupdlp.rescale_problem(10, False, 1.0, 0, synthetic.known_optimum_lp(36 + k, m=60, n=120,
                                                                                  density=0.05).problem)
             for k in range(3)]
    params = _params(cupdlp.Precision.FP64, 1e-8)
    with Server(workers=1, max_cohort=4, linger_sec=0.05) as srv:
        tickets = [srv.submit(scaled_desc(sq), params) for sq in [big] + small]
        got_small = [srv.wait(t, timeout=600.0) for t in tickets[1:]]
        big_pending = srv.poll(tickets[0]) is None
        got_big = srv.wait(tickets[0], timeout=600.0)
    assert big_pending
    for k, sq in enumerate(small):
        _same(got_small[k], _alone(sq, params), k)
    _same(got_big, _alone(big, params), "big")


def test_a_straggling_cohort_gives_its_slot_to_new_requests():
    """One worker slot; a cohort of one slow LP and three quick ones. Once the quick three have
    retired, the cohort is a straggler and no longer holds the slot: a request submitted then
    is packed into a new cohort and answered while the slow LP is still on the device."""
    big = cupdlp.rescale_problem(10, False, 1.0, 0, synthetic.power_law_lp(1, m=300, n=600,
                                                                          target_nnz=3000).problem)
    small = [cupdlp.rescale_problem(10, False, 1.0, 0, synthetic.known_optimum_lp(40 + k, m=60, n=120,
                                                                                  density=0.05).problem)
             for k in range(4)]
    params = cupdlp.default_parameters(tolerance=1e-8, precision=cupdlp.Precision.FP64,
                                       iteration_limit=400_000, time_sec_limit=300.0)
    with Server(workers=1, max_cohort=4, linger_sec=0.05) as srv:
        tickets = [srv.submit(scaled_desc(sq), params) for sq in [big] + small[:3]]
        for t in tickets[1:]:
            srv.wait(t, timeout=600.0)
        late = srv.submit(scaled_desc(small[3]), params)
        got_late = srv.wait(late, timeout=600.0)
        big_pending = srv.poll(tickets[0]) is None
        got_big = srv.wait(tickets[0], timeout=600.0)
    assert big_pending
    assert got_big[0].iteration_count > got_late[0].iteration_count
    _same(got_late, _alone(small[3], params), "late")
