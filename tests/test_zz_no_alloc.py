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


class _Fields:
    """Only the arrays the reductions read (rho, ux, uy, uz, solid), allocated
    with lb_malloc, in a DataD3Q19 of the given extents."""

    def __init__(self, pkg, W, H, D):
        self.lib = pkg.lib()
        self.d = pkg.abi.DataD3Q19()
        self.d.width, self.d.height, self.d.depth = W, H, D
        self.N = W * H * D
        self.bufs = []
        for name, size in (("rho", 4), ("ux", 4), ("uy", 4), ("uz", 4), ("solid", 1)):
            p = ctypes.c_void_p()
            assert self.lib.lb_malloc(ctypes.byref(p), size * self.N) == 0
            self.bufs.append(p)
            setattr(self.d, name, p.value)

    def fill_random(self, rng, solid_frac):
        for i, name in enumerate(("rho", "ux", "uy", "uz")):
            a = (rng.random(self.N) - (0 if i == 0 else 0.5)).astype(np.float32)
            assert self.lib.lb_memcpy_h2d(ctypes.c_void_p(getattr(self.d, name)),
                                          a.ctypes.data_as(ctypes.c_void_p), a.nbytes) == 0
        s = (rng.random(self.N) < solid_frac).astype(np.uint8)
        assert self.lib.lb_memcpy_h2d(ctypes.c_void_p(self.d.solid),
                                      s.ctypes.data_as(ctypes.c_void_p), s.nbytes) == 0
        return int(s.sum())

    def sums(self, fn):
        out = (ctypes.c_double * 7)()
        rc = getattr(self.lib, fn)(ctypes.byref(self.d), out)
        assert rc == 0, (fn, rc, self.lib.lb_abi_last_error())
        return np.array(out[:])

    def close(self):
        for p in self.bufs:
            self.lib.lb_free(p)
        self.bufs = []


@pytest.mark.parametrize("extents", [(1, 1, 1), (65537, 1, 1), (17, 3, 5)])
def test_noalloc_reduce_small_and_ragged(extents):
    """One node, one node past a first-pass block (65 537 nodes: two blocks,
    the second holding a single node) and a lattice smaller than one block's
    256 threads, each on two calls in a row."""
    pkg = load_package()
    fl = _Fields(pkg, *extents)
    rng = np.random.default_rng(sum(extents))
    try:
        for call in range(2):
            n_solid = fl.fill_random(rng, 0.2 * call)
            ref = fl.sums("lb_reduce_d3q19")
            got = fl.sums("lb_reduce_d3q19_noalloc")
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12)
            assert got[6] == fl.N - n_solid
    finally:
        fl.close()


def test_noalloc_reduce_largest_lattice():
    """The largest lattice the fixed scratch array takes (153 288 704 nodes,
    2339 first-pass blocks): the 7 results then sit in the array's last slots.
    Fields are filled on the device with byte patterns (2.6 GB in all)."""
    pkg = load_package()
    lib = pkg.lib()
    W, H, D = 2339, 256, 256  # 2339 * 65536 nodes
    fl = _Fields(pkg, W, H, D)
    try:
        for call, (pat_rho, pat_u, pat_s) in enumerate([(0x3f, 0x3c, 0), (0x3e, 0xbb, 1)]):
            for name, pat in (("rho", pat_rho), ("ux", pat_u), ("uy", pat_u), ("uz", pat_u)):
                assert lib.lb_memset(ctypes.c_void_p(getattr(fl.d, name)), pat, 4 * fl.N) == 0
            assert lib.lb_memset(ctypes.c_void_p(fl.d.solid), pat_s, fl.N) == 0
            ref = fl.sums("lb_reduce_d3q19")
            got = fl.sums("lb_reduce_d3q19_noalloc")
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12)
            assert got[6] == (fl.N if pat_s == 0 else 0)
    finally:
        fl.close()


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
