"""lb_probe / lb_run_probe: the context form of the reference's per-step
cursor probe (src/read_value.cu:27-58) -- the probed value equals the moment
fields of the last step at that node, and lb_run_probe equals lb_step."""
import ctypes

import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu


def test_run_probe_matches_step_and_moments():
    pkg = load_package()
    L = pkg.lib()
    W, H, D = 40, 24, 16
    N = W * H * D
    rng = np.random.default_rng(3)
    rho = (1 + 0.02 * rng.standard_normal(N)).astype(np.float32)
    ux = (0.02 * rng.standard_normal(N)).astype(np.float32)
    flags = np.zeros(N, np.uint8)
    flags[:W * H] = 1
    out = []
    for use_probe in (True, False):
        lat = pkg.Lattice(19, W, H, D, tau_inv=1.4, force=(1e-5, 0, 0))
        lat.set_flags(flags)
        lat.init_equilibrium(rho, ux, None, None)
        if use_probe:
            v = np.zeros(4, np.float32)
            assert L.lb_run_probe(lat.h, 9, 5, 7, 3, v.ctypes.data_as(ctypes.c_void_p)) == 0
        else:
            lat.step(9)
        m = lat.moments()
        out.append((lat.populations(), m))
        if use_probe:
            o = 5 + 7 * W + 3 * W * H
            assert np.array_equal(v, np.array([m[1][o], m[2][o], m[3][o], m[0][o]], np.float32))
            bad = np.zeros(4, np.float32)
            assert L.lb_probe(lat.h, W, 0, 0, bad.ctypes.data_as(ctypes.c_void_p)) == \
                pkg.abi.LB_ERR_ARG
        lat.close()
    assert np.array_equal(out[0][0], out[1][0])
    for a, b in zip(out[0][1], out[1][1]):
        assert np.array_equal(a, b)
