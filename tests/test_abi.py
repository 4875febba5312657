"""CPU tests of libgpdhg.so: it builds for sm_103a, loads, exports every declared
symbol, and rejects bad input before touching a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import cupdlp
from cupdlp import _abi
from cupdlp import synthetic
from cupdlp.solver import scaled_desc, unscaled_desc

import instances

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "gpdhg.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(gpdhg_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_what_python_binds():
    assert declared_functions() == sorted(_abi.SIGNATURES)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_abi_version(lib):
    assert lib.gpdhg_abi_version() == _abi.ABI_VERSION


def test_default_params_match_host_defaults(lib):
    c = _abi.Params()
    lib.gpdhg_default_params(C.byref(c))
    h = cupdlp.params_to_c(cupdlp.default_parameters(tolerance=1e-4, time_sec_limit=3600.0))
    for name, _ in _abi.Params._fields_:
        if name in ("verbosity", "reserved"):
            continue
        assert getattr(c, name) == getattr(h, name), name


def _create_err(lib, desc):
    h = C.c_void_p()
    st = lib.gpdhg_problem_create(desc.ref, C.byref(h))
    return st, lib.gpdhg_last_error().decode()


def test_rejects_nan_matrix_before_any_gpu_work(lib):
    p, _ = instances.tiny()
    d = unscaled_desc(p)
    d.arrays["vals"][0] = np.nan
    st, msg = _create_err(lib, d)
    assert st == _abi.ERR_INVALID_PROBLEM and "constraint matrix" in msg


def test_rejects_bad_column_index(lib):
    p, _ = instances.tiny()
    d = unscaled_desc(p)
    d.arrays["cols"][0] = 5
    st, msg = _create_err(lib, d)
    assert st == _abi.ERR_INVALID_PROBLEM and "column index" in msg


def test_rejects_infinite_lower_bound(lib):
    p, _ = instances.tiny()
    p.variable_lower_bound = np.array([np.inf])
    st, msg = _create_err(lib, unscaled_desc(p))
    assert st == _abi.ERR_INVALID_PROBLEM and "+Inf" in msg


def test_rejects_zero_variables(lib):
    p, _ = instances.tiny()
    d = unscaled_desc(p)
    d.desc.num_variables = 0
    st, _ = _create_err(lib, d)
    assert st == _abi.ERR_INVALID_PROBLEM


def test_rejects_nnz_mismatch(lib):
    p, _ = instances.tiny()
    d = unscaled_desc(p)
    d.desc.nnz = 7
    st, msg = _create_err(lib, d)
    assert st == _abi.ERR_INVALID_PROBLEM and "nnz" in msg


def test_null_arguments(lib):
    assert lib.gpdhg_problem_create(None, None) == _abi.ERR_INVALID_ARGUMENT
    assert lib.gpdhg_solve(None, None, None, None, None) == _abi.ERR_INVALID_ARGUMENT
    st = _abi.IterationStats()
    assert lib.gpdhg_get_stats(None, 0, C.byref(st)) == _abi.ERR_INVALID_ARGUMENT
    assert "NULL" in lib.gpdhg_last_error().decode()


def test_server_footprint_and_null_handling():
    """Host-only parts of the serving API: the admission footprint grows with the LP and
    the precision, and NULL handles are rejected without touching the GPU."""
    lib = _abi.load()
    small = synthetic.known_optimum_lp(0, m=100, n=200, density=0.05)
    big = synthetic.known_optimum_lp(1, m=1000, n=2000, density=0.005)
    ds = scaled_desc(cupdlp.rescale_problem(10, False, 1.0, 0, small.problem))
    db = scaled_desc(cupdlp.rescale_problem(10, False, 1.0, 0, big.problem))
    p64 = cupdlp.params_to_c(cupdlp.default_parameters(precision=cupdlp.Precision.FP64))
    p32 = cupdlp.params_to_c(cupdlp.default_parameters(precision=cupdlp.Precision.FP32))
    f_small = lib.gpdhg_server_footprint(ds.ref, C.byref(p64))
    f_big = lib.gpdhg_server_footprint(db.ref, C.byref(p64))
    assert 0 < f_small < f_big
    assert lib.gpdhg_server_footprint(db.ref, C.byref(p32)) < f_big
    assert lib.gpdhg_server_footprint(None, None) < 0
    t = C.c_uint64()
    assert lib.gpdhg_server_submit(None, ds.ref, C.byref(p64), C.byref(t)) == _abi.ERR_INVALID_ARGUMENT
    assert lib.gpdhg_server_poll(None, 1, None, None, None) == _abi.ERR_INVALID_ARGUMENT
    assert lib.gpdhg_server_wait(None, 1, 0.0, None, None, None) == _abi.ERR_INVALID_ARGUMENT
    assert lib.gpdhg_server_create(None, None) == _abi.ERR_INVALID_ARGUMENT


def _csc_err(lib, p, mutate=None, base=0, keep_csr=False):
    """gpdhg_problem_create_csc on problem p, after mutate(colptr, rowval, nzval)."""
    d = unscaled_desc(p)
    a = p.constraint_matrix.tocsc()
    colptr = np.ascontiguousarray(a.indptr, dtype=np.int64) + base
    rowval = np.ascontiguousarray(a.indices, dtype=np.int64) + base
    nzval = np.ascontiguousarray(a.data, dtype=np.float64)
    if mutate:
        mutate(colptr, rowval, nzval)
    desc = _abi.LpDesc()
    C.pointer(desc)[0] = d.desc
    if not keep_csr:
        desc.row_ptr = C.cast(None, _abi._ip)
        desc.col_idx = C.cast(None, _abi._ip)
        desc.values = C.cast(None, _abi._dp)
    h = C.c_void_p()
    st = lib.gpdhg_problem_create_csc(C.byref(desc), _abi.lptr(colptr), _abi.lptr(rowval), _abi.dptr(nzval), base,
                                      None, C.byref(h))
    return st, lib.gpdhg_last_error().decode()


def test_csc_entry_rejects_bad_input_before_any_gpu_work(lib):
    p, _ = instances.tiny()
    st, msg = _csc_err(lib, p, base=2)
    assert st == _abi.ERR_INVALID_ARGUMENT and "index_base" in msg
    st, msg = _csc_err(lib, p, keep_csr=True)
    assert st == _abi.ERR_INVALID_ARGUMENT and "CSC descriptor" in msg
    st, msg = _csc_err(lib, p, base=1, mutate=lambda cp, rv, nz: cp.__setitem__(0, 0))
    assert st == _abi.ERR_INVALID_PROBLEM and "col_ptr[0]" in msg
    st, msg = _csc_err(lib, p, base=1, mutate=lambda cp, rv, nz: rv.__setitem__(0, 0))
    assert st == _abi.ERR_INVALID_PROBLEM and "row index" in msg
    st, msg = _csc_err(lib, p, mutate=lambda cp, rv, nz: nz.__setitem__(0, np.inf))
    assert st == _abi.ERR_INVALID_PROBLEM and "constraint matrix" in msg
    st, msg = _csc_err(lib, p, mutate=lambda cp, rv, nz: cp.__setitem__(-1, cp[-1] + 1))
    assert st == _abi.ERR_INVALID_PROBLEM and "nnz" in msg


def test_batch_reports_the_first_invalid_instance(lib):
    """A batch validates its instances on host threads; the error reported is the one of the
    lowest-numbered invalid instance, as a serial loop would report."""
    p, _ = instances.tiny()
    good = unscaled_desc(p)
    nan = unscaled_desc(p)
    nan.arrays["vals"][0] = np.nan
    col = unscaled_desc(p)
    col.arrays["cols"][0] = 5
    for order, want in (((good, nan, col), "constraint matrix"), ((good, col, nan), "column index")):
        arr = (_abi.LpDesc * 3)(*[d.desc for d in order])
        h = C.c_void_p()
        assert lib.gpdhg_batch_create(3, arr, C.byref(h)) == _abi.ERR_INVALID_PROBLEM
        assert want in lib.gpdhg_last_error().decode()


def test_validation_reports_the_serial_scans_first_failure(lib):
    """Every vector check of a side runs in one threaded pass (n = 600k: several threads); the
    error reported is still the one a serial scan of the checks, in validate's order, meets."""
    from cupdlp.solver import _Desc
    n, m = 600_000, 3
    rp = np.array([0, 1, 2, 3], dtype=np.int32)
    cols = np.array([0, n // 2, n - 1], dtype=np.int32)
    vals = np.ones(3)

    def err(**bad):
        v = dict(l=np.zeros(n), u=np.full(n, 10.0), c=np.ones(n), b=np.ones(m), ol=np.zeros(n), ou=np.full(n, 10.0),
                 oc=np.ones(n), ob=np.ones(m), con=np.ones(m), var=np.ones(n))
        for key, (idx, value) in bad.items():
            v[key][idx] = value
        d = _Desc(n, m, 1, rp, cols, vals, v["l"], v["u"], v["c"], v["b"], 0.0, v["ol"], v["ou"], v["oc"], v["ob"],
                  v["con"], v["var"])
        st, msg = _create_err(lib, d)
        assert st == _abi.ERR_INVALID_PROBLEM
        return msg

    assert "objective vector" in err(c=(500_000, np.nan), var=(10, 0.0)) and "original" not in err(c=(5, np.inf))
    assert "upper_bound contains -Inf" in err(u=(400_000, -np.inf), ol=(5, np.inf))
    assert "NaN found in variable bounds" in err(l=(100_000, np.nan), u=(200_000, -np.inf))
    assert "upper_bound contains -Inf" in err(l=(300_000, np.inf), u=(200_000, -np.inf))
    assert "right hand side" in err(b=(2, np.nan), oc=(7, np.nan))
    assert "original objective vector" in err(oc=(599_999, np.inf), ob=(0, np.nan), var=(1, -1.0))
    assert "constraint_rescaling" in err(con=(1, 0.0), var=(0, np.nan))
    assert "variable_rescaling" in err(var=(300_000, 0.0))
