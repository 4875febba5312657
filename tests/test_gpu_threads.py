"""GPU tests of the C ABI under concurrent host threads: the library is reentrant across
handles (one handle per thread), so LPs solved on several threads at once give the same
results, bit for bit, as the same solves one after another, and the last-error string is
per thread."""
import ctypes as C
import threading
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import cupdlp
from cupdlp import _abi, synthetic
from cupdlp.solver import DeviceProblem, scaled_desc, unscaled_desc

import instances

pytestmark = pytest.mark.gpu

PRECISIONS = [(cupdlp.Precision.FP64, 1e-6), (cupdlp.Precision.FP32, 1e-4), (cupdlp.Precision.FP32_REFINE, 1e-7)]


def _descs():
    lps = [synthetic.known_optimum_lp(60 + k, m=300 + 200 * k, n=600 + 400 * k, density=0.02) for k in range(4)]
    lps.append(synthetic.transportation_lp(7, 20, 60))
    lps.append(instances.ragged_rows_lp(62, m=1500, n=1200))
    return [scaled_desc(cupdlp.rescale_problem(10, False, 1.0, 0, lp.problem)) for lp in lps]


def _solve_all(d):
    out = []
    with DeviceProblem(d) as dp:
        for prec, tol in PRECISIONS:
            p = cupdlp.default_parameters(tolerance=tol, precision=prec, iteration_limit=40_000, time_sec_limit=300.0)
            out.append(dp.solve(p))
    return out


def test_handles_on_concurrent_threads_equal_sequential_solves():
    descs = _descs()
    seq = [_solve_all(d) for d in descs]
    with ThreadPoolExecutor(max_workers=len(descs)) as ex:
        par = list(ex.map(_solve_all, descs))
    for k, (a, b) in enumerate(zip(seq, par)):
        for (ra, xa, ya), (rb, xb, yb) in zip(a, b):
            assert ra.termination_reason == rb.termination_reason, k
            assert ra.iteration_count == rb.iteration_count, k
            assert np.array_equal(xa, xb) and np.array_equal(ya, yb), k


def test_last_error_is_per_thread():
    lib = _abi.load()
    p, _ = instances.tiny()
    bad = unscaled_desc(p)
    bad.arrays["cols"][0] = 5
    good = scaled_desc(cupdlp.rescale_problem(10, False, 1.0, 0, synthetic.known_optimum_lp(3, m=50, n=100,
                                                                                             density=0.1).problem))
    gate = threading.Barrier(2)
    seen = {}

    def failing():
        h = C.c_void_p()
        seen["bad_status"] = lib.gpdhg_problem_create(bad.ref, C.byref(h))
        gate.wait()   # the other thread now succeeds
        gate.wait()
        seen["bad_msg"] = lib.gpdhg_last_error().decode()

    def succeeding():
        gate.wait()
        with DeviceProblem(good) as dp:
            dp.solve(cupdlp.default_parameters(tolerance=1e-4))
        seen["good_msg"] = lib.gpdhg_last_error().decode()
        gate.wait()

    ts = [threading.Thread(target=failing), threading.Thread(target=succeeding)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=300)
    assert seen["bad_status"] == _abi.ERR_INVALID_PROBLEM
    assert "column index" in seen["bad_msg"]
    assert seen["good_msg"] == ""
