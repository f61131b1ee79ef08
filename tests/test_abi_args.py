"""CPU: argument checks of C-ABI entry points that reject a call before any
CUDA call, so they run without a GPU -- the bounded-wait self-check's
selector and the library-side runLBM loop's arguments and cursor."""
import ctypes as C
import os

import pytest

from conftest import load_package


@pytest.fixture(scope="module")
def pkg():
    p = load_package()
    if not os.path.exists(p.abi.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    return p


def test_wait_selftest_rejects_unknown_selectors(pkg):
    L, a = pkg.lib(), pkg.abi
    st = C.c_int(-7)
    for which in (0, 3, -1):
        assert L.lb_wait_selftest(which, C.byref(st)) == a.LB_ERR_ARG
    assert L.lb_wait_selftest(1, None) == a.LB_ERR_ARG
    assert st.value == -7  # untouched


def _struct(pkg, W, H, D):
    d = pkg.abi.DataD3Q19()
    d.width, d.height, d.depth = W, H, D
    d.deviceCount, d.dev = 1, 0
    return d


def _params(pkg, cursor):
    prm = pkg.abi.lb_run_params_d3q19()
    prm.cursor[0], prm.cursor[1], prm.cursor[2] = cursor
    return prm


def test_run_lbm_rejects_bad_arguments(pkg):
    L, a = pkg.lib(), pkg.abi
    d = _struct(pkg, 8, 4, 4)
    prm = _params(pkg, (1, 1, 1))
    value = (C.c_float * 4)()
    assert L.lb_run_lbm_d3q19(None, None, C.byref(prm), 1, value) == a.LB_ERR_ARG
    assert L.lb_run_lbm_d3q19(C.byref(d), None, None, 1, value) == a.LB_ERR_ARG
    assert L.lb_run_lbm_d3q19(C.byref(d), None, C.byref(prm), 1, None) == a.LB_ERR_ARG
    assert L.lb_run_lbm_d3q19(C.byref(d), None, C.byref(prm), -1, value) == a.LB_ERR_ARG
    L.lb_abi_clear_error()


@pytest.mark.parametrize("cursor", [(8, 0, 0), (0, 4, 0), (0, 0, 4), (-1, 0, 0)])
def test_run_lbm_rejects_a_cursor_outside_the_lattice(pkg, cursor):
    L, a = pkg.lib(), pkg.abi
    d = _struct(pkg, 8, 4, 4)
    prm = _params(pkg, cursor)
    value = (C.c_float * 4)()
    try:
        assert L.lb_run_lbm_d3q19(C.byref(d), None, C.byref(prm), 3, value) == a.LB_ERR_ARG
        assert b"cursor outside the lattice" in L.lb_abi_last_error()
    finally:
        L.lb_abi_clear_error()


def test_run_lbm_rejects_a_struct_without_extent(pkg):
    L, a = pkg.lib(), pkg.abi
    d = _struct(pkg, 0, 4, 4)
    prm = _params(pkg, (0, 0, 0))
    value = (C.c_float * 4)()
    try:
        assert L.lb_run_lbm_d3q19(C.byref(d), None, C.byref(prm), 3, value) == a.LB_ERR_ARG
        assert b"non-positive extent" in L.lb_abi_last_error()
    finally:
        L.lb_abi_clear_error()
