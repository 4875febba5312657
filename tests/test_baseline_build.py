"""The reference-form GPU baseline builds and exports its entry points (no GPU needed)."""
import ctypes as C
import os
import sys

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "baseline"))


def test_baseline_library_builds_and_exports():
    import build_ref_equiv
    lib = C.CDLL(build_ref_equiv.build())
    for name in ("refeq_solve", "refeq_last_error"):
        assert hasattr(lib, name), name


def test_product_library_does_not_link_the_baseline():
    import build as pkg_build
    with open(pkg_build.build(), "rb") as f:
        blob = f.read()
    assert b"refeq_solve" not in blob and b"libcusparse" not in blob
