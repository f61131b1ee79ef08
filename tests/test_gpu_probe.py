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


def probe_each_step(pkg, lat, n, x, y, z):
    """the per-step reference: one step with moments, then lb_probe"""
    L = pkg.lib()
    vals = []
    v = np.zeros(4, np.float32)
    for _ in range(n):
        lat.step(1)
        assert L.lb_probe(lat.h, x, y, z, v.ctypes.data_as(ctypes.c_void_p)) == 0
        vals.append(v.copy())
    return vals


CASES = {
    # lattice, extents, kwargs, probe node, steps
    "d3q19_native": (19, (36, 20, 12), dict(tau_inv=1.6, force=(1e-5, 0, 0)), (7, 9, 4), 21),
    "d3q19_native_wall_node": (19, (36, 20, 12), dict(tau_inv=1.6), (7, 0, 4), 5),
    "d3q19_reference": (19, (36, 20, 12), dict(mode=0, tau_inv=1.25, u_in=(0.03, 0, 0)),
                        (0, 9, 4), 13),
    "d3q19_shan_chen_bf16": (19, (24, 24, 24), dict(tau_inv=1.0, G=-5.0, storage=2,
                                                    rho_ref=0.693), (3, 5, 7), 11),
    # wall-free lattices that the staged single-pass Shan-Chen step tiles
    "d3q19_shan_chen_staged_f16": (19, (32, 16, 12), dict(tau_inv=1.0, G=-5.0, storage=1,
                                                          rho_ref=0.693), (31, 15, 11), 11),
    "d3q19_shan_chen_staged_f32": (19, (64, 8, 8), dict(tau_inv=1.0, G=-5.0), (5, 3, 2), 13),
    "d2q9_pdl": (9, (72, 40, 1), dict(tau_inv=1.6, wall_u=(0.1, 0, 0)), (30, 1, 0), 70),
    "d2q9_shan_chen": (9, (48, 32, 1), dict(tau_inv=1.0, G=-5.0), (10, 11, 0), 17),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_run_probe_in_step_matches_per_step_probe(name):
    """lb_run_probe's in-kernel probe (mapped host memory, graph replay) gives
    the value a per-step lb_probe gives after the last step, and the same
    state."""
    pkg = load_package()
    L = pkg.lib()
    Q, (W, H, D), kw, (x, y, z), n = CASES[name]
    N = W * H * D
    rng = np.random.default_rng(11)
    rho = ((0.693 if kw.get("G") else 1.0) * (1 + 0.01 * rng.standard_normal(N))).astype(
        np.float32)
    flags = np.zeros(N, np.uint8)
    if Q == 19 and not kw.get("G"):
        flags.reshape(D, H, W)[:, 0, :] = 1
    if Q == 9 and not kw.get("G"):
        f2 = flags.reshape(H, W)
        f2[:, 0] = f2[:, -1] = f2[-1, :] = 1
        f2[0, :] = 3

    def make():
        lat = pkg.Lattice(Q, W, H, D, graph_steps=8, **kw)
        lat.set_flags(flags)
        lat.init_equilibrium(rho, None, None, None)
        return lat

    a = make()
    vals = probe_each_step(pkg, a, n, x, y, z)
    fa, ma = a.populations(), a.moments()
    a.close()
    b = make()
    v = np.full(4, np.nan, np.float32)
    assert L.lb_run_probe(b.h, n, x, y, z, v.ctypes.data_as(ctypes.c_void_p)) == 0
    assert np.array_equal(v.view(np.uint32), vals[-1].view(np.uint32))
    assert np.array_equal(b.populations().view(np.uint32), fa.view(np.uint32))
    for p, q in zip(b.moments(), ma):
        if p is not None:
            assert np.array_equal(p.view(np.uint32), q.view(np.uint32))
    # a second call continues from there; a new cursor re-captures the graphs
    assert L.lb_run_probe(b.h, 3, x, y, z, v.ctypes.data_as(ctypes.c_void_p)) == 0
    assert L.lb_run_probe(b.h, 2, (x + 1) % W, y, z, v.ctypes.data_as(ctypes.c_void_p)) == 0
    r, ux, uy, uz = b.moments()
    o = (x + 1) % W + W * (y + H * z)
    want = [ux[o], uy[o], 0.0 if uz is None else uz[o], r[o]]
    assert np.array_equal(v, np.array(want, np.float32))
    assert b.steps_done() == n + 5
    b.close()
