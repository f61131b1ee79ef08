"""lb_reduce_d3q19_noalloc: the conservation sums without any device
allocation, for callers that cannot allocate device memory (a host whose GPU
memory all belongs to its own pool allocator, or a real-time loop where
cudaMalloc/cudaFree could synchronise the device).

Checked through the C ABI against lb_reduce_d3q19 (which allocates its
scratch) on two calls in a row with different fields, so a stale partial left
in the shared scratch array by the first call would show in the second.  The
tolerance is the one of the other FP64 reduction tests (rtol 1e-12): the two
entry points sum in a different block order.  This file is collected last on
purpose, so a run that stops at the first failure has run everything else.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu


def _sums(lib, fn, dd):
    out = (ctypes.c_double * 7)()
    rc = getattr(lib, fn)(dd.ptr(), out)
    assert rc == 0, (fn, rc, lib.lb_abi_last_error())
    return np.array(out[:])


def test_noalloc_reduce_matches_allocating_reduce():
    pkg = load_package()
    lib = pkg.lib()
    n = ctypes.c_int(0)
    assert lib.lb_device_count(ctypes.byref(n)) == 0 and n.value >= 1, "no CUDA device"
    W, H, D = 96, 40, 36  # 138 240 nodes: three first-pass blocks of the no-alloc path
    N = W * H * D
    dd = pkg.DeviceData(19, W, H, D, plot=False)
    rng = np.random.default_rng(77)
    try:
        for call in range(2):
            for name in ("rho", "ux", "uy", "uz"):
                dd.h2d(getattr(dd.s, name), rng.random(N).astype(np.float32) - 0.25 * call)
            solid = (rng.random(N) < 0.15 * (call + 1)).astype(np.uint8)
            dd.set_solid(solid, np.zeros(N, np.uint8))
            ref = _sums(lib, "lb_reduce_d3q19", dd)
            got = _sums(lib, "lb_reduce_d3q19_noalloc", dd)
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12)
            assert got[6] == N - int(solid.sum())  # fluid node count is exact
    finally:
        dd.close()


def test_noalloc_reduce_rejects_oversized_lattice():
    """The size check happens on the host, before anything touches the GPU."""
    pkg = load_package()
    lib = pkg.lib()
    d = pkg.abi.DataD3Q19()
    d.width, d.height, d.depth = 1024, 1024, 147  # 154 140 672 nodes > 153 288 704
    lib.lb_abi_clear_error()
    out = (ctypes.c_double * 7)()
    assert lib.lb_reduce_d3q19_noalloc(ctypes.byref(d), out) == pkg.abi.LB_ERR_ARG
    assert b"153288704" in lib.lb_abi_last_error()
    lib.lb_abi_clear_error()
