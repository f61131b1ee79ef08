"""GPU: the tcgen05 pattern of the closure kernel (K-major core-matrix
operands, shared-memory descriptors, BF16 MMAs into tensor memory, commit to
an mbarrier, tensor-memory loads, a second layer over the first's columns,
several rounds) on products whose exact values the host knows."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tcgen05_selftest_rounds(pkg):
    L = pkg.lib()
    out = np.full((3, 2, 128, 64), np.nan, np.float32)
    status = ctypes.c_int(-1)
    rc = L.lb_tcgen05_selftest(out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(status))
    assert rc == 0, L.lb_abi_last_error()
    assert status.value == 0
    r, n = np.arange(128)[:, None], np.arange(64)[:, None]
    k32, k64 = np.arange(32)[None, :], np.arange(64)[None, :]
    W1 = ((n * 5 + k32) % 7 - 3).astype(np.float64)
    W2 = ((n + 2 * k64) % 5 - 2).astype(np.float64)
    for rd in range(3):
        X = (((r * 7 + k32 * 3) % 9 - 4) * (rd + 1)).astype(np.float64)
        H = ((r + 3 * k64 + rd) % 5 - 2).astype(np.float64)
        assert np.array_equal(out[rd, 0], (X @ W1.T).astype(np.float32)), rd
        assert np.array_equal(out[rd, 1], (H @ W2.T).astype(np.float32)), rd


@pytest.mark.parametrize("which", [1, 2], ids=["tcgen05_mbarrier_wait", "staged_sc_stage_wait"])
def test_bounded_waits_give_up_and_report(pkg, which):
    """A wait on an mbarrier with nothing committed, or a stage wait given no
    polls, runs out, raises the error word and returns; the GPU stays usable
    (the layout self-check runs right after)."""
    L = pkg.lib()
    status = ctypes.c_int(-1)
    assert L.lb_wait_selftest(which, ctypes.byref(status)) == 0, L.lb_abi_last_error()
    assert status.value == 1
    out = np.zeros((3, 2, 128, 64), np.float32)
    st = ctypes.c_int(-1)
    assert L.lb_tcgen05_selftest(out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(st)) == 0
    assert st.value == 0
