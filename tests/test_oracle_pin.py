"""Pin the oracle: its float instantiation must be bit-identical to the
reference's own kernels (src/streaming.cu, src/collision.cu,
src/get_border.cu, src/apply_border.cu, src/read_value.cu) compiled for the
host by oracle/Makefile.  Runs wherever the reference sources exist."""
import ctypes

import numpy as np
import pytest

from conftest import load_package


@pytest.fixture(scope="module")
def ref(oracle):
    lib = oracle.ref_lib()
    if lib is None:
        pytest.skip("reference sources not present (pinned through tests/golden instead)")
    return lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p).value


def make_d3q19(abi, W, H, D, f, solid, sb, mom, plot=None):
    d = abi.DataD3Q19()
    N = W * H * D
    for k in range(19):
        setattr(d, "f%d" % k, _ptr(f[k]))
    d.ux, d.uy, d.uz, d.rho = [_ptr(m) for m in mom]
    d.solid, d.solid_bound = _ptr(solid), _ptr(sb)
    d.width, d.height, d.depth = W, H, D
    d.deviceCount, d.dev = 1, 0
    return d


def make_d2q9(abi, W, H, f, solid, sb, mom, sc):
    d = abi.DataD2Q9()
    for k in range(9):
        setattr(d, "f%d" % k, _ptr(f[k]))
    d.ux, d.uy, d.rho = [_ptr(m) for m in mom]
    d.psi, d.ueq_x, d.ueq_y = [_ptr(m) for m in sc]
    d.solid, d.solid_bound = _ptr(solid), _ptr(sb)
    d.width, d.height = W, H
    d.deviceCount, d.dev = 1, 0
    return d


def random_state(rng, Q, N, w):
    # positive populations near equilibrium with noise
    return (np.asarray(w, np.float32)[:, None] * (1.0 + 0.2 * rng.standard_normal((Q, N)))
            ).astype(np.float32)


def blob_solid(rng, W, H, D=1, frac=0.15):
    s = (rng.random((D, H, W)) < frac).astype(np.uint8)
    s[:, :, 8:16] = 1  # a thick block so that solid_bound is non-trivial
    return np.ascontiguousarray(s.reshape(-1))


@pytest.mark.parametrize("steps", [1, 5])
def test_d3q19_bitexact_vs_reference(ref, oracle, steps):
    abi = load_package().abi
    W, H, D = 32, 8, 8
    N = W * H * D
    rng = np.random.default_rng(7)
    f_ref = random_state(rng, 19, N, oracle.D3_W)
    f_orc = f_ref.copy()
    solid = blob_solid(rng, W, H, D)
    sb = oracle.d3q19_solid_bound(solid, W, H, D)
    mom_r = [np.zeros(N, np.float32) for _ in range(4)]
    mom_o = [np.zeros(N, np.float32) for _ in range(4)]
    plot_r = np.zeros(4 * N, np.float32)
    plot_o = np.zeros(4 * N, np.float32)
    d = make_d3q19(abi, W, H, D, f_ref, solid, sb, mom_r)
    g, b = abi.dim3(W // 32, H // 4, D), abi.dim3(32, 4, 1)
    w0, w1, w7 = np.float32(12. / 36.), np.float32(2. / 36.), np.float32(1. / 36.)
    tau_inv = np.float32(1. / (3. * 0.03 + 0.5))
    F = ctypes.c_float
    for _ in range(steps):
        ref.streaming_d3q19(ctypes.byref(d), g, b)
        ref.collision_d3q19(plot_r.ctypes.data_as(ctypes.c_void_p), ctypes.byref(d), F(w0), F(w1),
                            F(w7), F(tau_inv), F(0.05), F(0), F(0), F(1.0), F(0), F(0.15), F(0.98),
                            F(1.02), g, b)
        oracle.d3q19_stream(f_orc, sb, W, H, D)
        oracle.d3q19_collide(f_orc, solid, mom_o, W, H, D, w0, w1, w7, tau_inv, 0.05, 0, 0, 1.0,
                             plot=plot_o)
    assert np.array_equal(f_ref.view(np.uint32), f_orc.view(np.uint32))
    for a, b_ in zip(mom_r, mom_o):
        assert np.array_equal(a.view(np.uint32), b_.view(np.uint32))
    assert np.array_equal(plot_r.view(np.uint32), plot_o.view(np.uint32))


@pytest.mark.parametrize("G,Gads,Fy", [(0.0, 0.0, 0.0), (0.0, 0.0, 1e-4), (-120.0, 0.0, 0.0),
                                       (-120.0, -50.0, 1e-4), (5.0, 0.0, 0.0)])
def test_d2q9_bitexact_vs_reference(ref, oracle, G, Gads, Fy):
    abi = load_package().abi
    W, H = 64, 16
    N = W * H
    rng = np.random.default_rng(11)
    solid = blob_solid(rng, W, H, 1, frac=0.1)
    sb = oracle.d2q9_solid_bound(solid, W, H)
    if G != 0:
        # Shan-Chen around rho ~ 200 (the phase-separation sample's density)
        rho0 = (200.0 * (1 + 0.01 * rng.standard_normal(N))).astype(np.float32)
        f_ref = (oracle.D2_W[:, None] * rho0[None, :]).astype(np.float32)
    else:
        f_ref = random_state(rng, 9, N, oracle.D2_W)
    f_orc = f_ref.copy()
    mom_r = [np.zeros(N, np.float32) for _ in range(3)]
    mom_o = [np.zeros(N, np.float32) for _ in range(3)]
    sc_r = [np.zeros(N, np.float32) for _ in range(3)]
    sc_o = [np.zeros(N, np.float32) for _ in range(3)]
    # the reference's D2Q9 solid branch writes one float past W*H float4s
    plot_r = np.zeros(8 * N, np.float32)
    plot_o = np.zeros(4 * N, np.float32)
    d = make_d2q9(abi, W, H, f_ref, solid, sb, mom_r, sc_r)
    g, b = abi.dim3(W // 32, H // 4, 1), abi.dim3(32, 4, 1)
    w0, w1, w5 = np.float32(16. / 36.), np.float32(4. / 36.), np.float32(1. / 36.)
    tau_inv = np.float32(1. / (3. * 0.16667 + 0.5))
    F = ctypes.c_float
    for _ in range(4):
        ref.streaming_d2q9(ctypes.byref(d), g, b)
        ref.collision_d2q9(plot_r.ctypes.data_as(ctypes.c_void_p), ctypes.byref(d), F(w0), F(w1),
                           F(w5), F(tau_inv), F(0.01), F(0), F(1.0), F(0), F(0.015), F(0.98),
                           F(1.02), g, b, F(2e-6), F(Fy), F(G), F(Gads))
        oracle.d2q9_stream(f_orc, sb, W, H)
        oracle.d2q9_collide(f_orc, solid, mom_o, sc_o, W, H, w0, w1, w5, tau_inv, 0.01, 0, 1.0,
                            2e-6, Fy, G, Gads, plot=plot_o)
    assert np.array_equal(f_ref.view(np.uint32), f_orc.view(np.uint32))
    for a, b_ in zip(mom_r + sc_r, mom_o + sc_o):
        assert np.array_equal(a.view(np.uint32), b_.view(np.uint32))
    assert np.array_equal(plot_r[:4 * N].view(np.uint32), plot_o.view(np.uint32))


def test_borders_and_probe_vs_reference(ref, oracle):
    abi = load_package().abi
    rng = np.random.default_rng(3)
    W, H, D = 32, 8, 4
    N = W * H * D
    f = rng.standard_normal((19, N)).astype(np.float32)
    bord = [np.zeros(H * D, np.float32) for _ in range(10)]
    nb = [rng.standard_normal(H * D).astype(np.float32) for _ in range(10)]
    mom = [np.zeros(N, np.float32) for _ in range(4)]
    solid = np.zeros(N, np.uint8)
    d = make_d3q19(abi, W, H, D, f, solid, solid, mom)
    for name, a in zip(abi.DataD3Q19.BORDER, bord):
        setattr(d, name, _ptr(a))
    for name, a in zip(abi.DataD3Q19.NB_BORDER, nb):
        setattr(d, name, _ptr(a))
    g, b = abi.dim3(W // 32, H // 4, D), abi.dim3(32, 4, 1)
    f_o = f.copy()
    ref.get_border_d3q19(ctypes.byref(d), g, b)
    exp = [np.zeros(H * D, np.float32) for _ in range(10)]
    arr = (ctypes.c_void_p * 10)(*[_ptr(a) for a in exp])
    oracle.lib().lbo_d3q19_get_border(f_o.ctypes.data_as(ctypes.c_void_p), arr, W, H, D)
    for a, e in zip(bord, exp):
        assert np.array_equal(a, e)
    ref.apply_border_d3q19(ctypes.byref(d), g, b)
    arr = (ctypes.c_void_p * 10)(*[_ptr(a) for a in nb])
    oracle.lib().lbo_d3q19_apply_border(f_o.ctypes.data_as(ctypes.c_void_p), arr, W, H, D)
    assert np.array_equal(f, f_o)
    plot = rng.standard_normal(4 * N).astype(np.float32)
    val = np.zeros(4, np.float32)
    d.valueCur = _ptr(val)
    ref.read_value_3d(plot.ctypes.data_as(ctypes.c_void_p), ctypes.byref(d), 5, 3, 2)
    o = 5 + 3 * W + 2 * W * H
    assert np.array_equal(val, plot[4 * o:4 * o + 4])
