"""GPU: the tcgen05 operand layout (K-major core matrices, shared-memory
descriptors, BF16 MMA into tensor memory, tensor-memory loads) on a product
whose exact value the host knows."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tcgen05_layout_selftest(pkg):
    L = pkg.lib()
    out = np.full((128, 64), np.nan, np.float32)
    rc = L.lb_tcgen05_selftest(out.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0, L.lb_abi_last_error()
    r, k, n = np.arange(128)[:, None], np.arange(32)[None, :], np.arange(64)[:, None]
    X = ((r * 7 + k * 3) % 9 - 4).astype(np.float64)
    W = ((n * 5 + k) % 7 - 3).astype(np.float64)
    assert np.array_equal(out, (X @ W.T).astype(np.float32))
