"""GPU parity: the CUDA path, called through the C ABI, against the golden
fixtures (outputs of the reference's own kernels) and against the oracle.

The bar is bit-exact: the library computes in float with the reference's
operation order and no FP contraction, so populations, moments and the plot
buffer must match to the last bit.  The one exception is psi = 1-exp(-rho)
(CUDA's expf and the host libm may differ by an ulp), where the tolerance is
stated in the test.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_package
from golden_io import bits, load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    p = load_package()
    lib = p.lib()
    n = ctypes.c_int(0)
    assert lib.lb_device_count(ctypes.byref(n)) == 0 and n.value >= 1, "no CUDA device"
    return p


def dim(*a):
    return load_package().abi.dim3(*a)


def beq(a, b):
    return np.array_equal(bits(a), bits(b))


# --------------------------------------------------------------------- drop-in ABI

@pytest.mark.parametrize("mode", [0, 1], ids=["standalone", "fused"])
def test_abi_d3q19_golden(pkg, mode):
    g = load("d3q19_ref")
    W, H, D = int(g["W"]), int(g["H"]), int(g["D"])
    L = pkg.lib()
    assert L.lb_abi_set_mode(mode) == 0
    try:
        dd = pkg.DeviceData(19, W, H, D)
        dd.upload(g["f_in"])
        dd.set_solid(g["solid"], g["solid_bound"])
        w = g["w"]
        F = ctypes.c_float
        for _ in range(int(g["steps"])):
            L.streaming_d3q19(dd.ptr(), dim(1, 1, 1), dim(32, 4, 1))
            L.collision_d3q19(ctypes.c_void_p(dd.plot), dd.ptr(), F(w[0]), F(w[1]), F(w[2]),
                              F(g["tau_inv"]), F(g["ux_in"]), F(0), F(0), F(g["rho_out"]),
                              F(0), F(0.15), F(0.98), F(1.02), dim(1, 1, 1), dim(32, 4, 1))
        assert L.lb_abi_last_error() == b""
        assert beq(dd.download(), g["f_out"])
        for k in ["ux", "uy", "uz", "rho"]:
            assert beq(dd.field(k), g[k]), k
        assert beq(dd.plot_data(), g["plot"])
        # fused mode moved the populations to the library's set (odd step count);
        # release copies them back into the caller's buffers
        assert L.lb_abi_release_d3q19(dd.ptr()) == 0
        assert [getattr(dd.s, n) for n in dd.s.POP] == dd.orig
        assert beq(dd.download(), g["f_out"])
        dd.close()
    finally:
        L.lb_abi_set_mode(0)


def test_abi_d3q19_stream_golden(pkg):
    g = load("d3q19_stream")
    W, H, D = int(g["W"]), int(g["H"]), int(g["D"])
    L = pkg.lib()
    dd = pkg.DeviceData(19, W, H, D)
    dd.upload(g["f_in"])
    L.streaming_d3q19(dd.ptr(), dim(1, 1, 1), dim(32, 4, 1))
    assert beq(dd.download(), g["f_out"])
    dd.close()


@pytest.mark.parametrize("name", ["d2q9_ref", "d2q9_sc"])
@pytest.mark.parametrize("mode", [0, 1], ids=["standalone", "fused"])
def test_abi_d2q9_golden(pkg, name, mode):
    g = load(name)
    W, H = int(g["W"]), int(g["H"])
    L = pkg.lib()
    assert L.lb_abi_set_mode(mode) == 0
    try:
        dd = pkg.DeviceData(9, W, H)
        dd.upload(g["f_in"])
        dd.set_solid(g["solid"], g["solid_bound"])
        w = g["w"]
        F = ctypes.c_float
        for _ in range(int(g["steps"])):
            L.streaming_d2q9(dd.ptr(), dim(1, 1, 1), dim(32, 4, 1))
            L.collision_d2q9(ctypes.c_void_p(dd.plot), dd.ptr(), F(w[0]), F(w[1]), F(w[2]),
                             F(g["tau_inv"]), F(g["ux_in"]), F(0), F(g["rho_out"]), F(0),
                             F(0.015), F(0.98), F(1.02), dim(1, 1, 1), dim(32, 4, 1),
                             F(g["Fx"]), F(g["Fy"]), F(g["G"]), F(g["Gads"]))
        assert L.lb_abi_last_error() == b""
        assert beq(dd.download(), g["f_out"])
        for k in ["ux", "uy", "rho"]:
            assert beq(dd.field(k), g[k]), k
        if "psi" in g:
            for k in ["psi", "ueq_x", "ueq_y"]:
                assert beq(dd.field(k), g[k]), k
        assert beq(dd.plot_data(), g["plot"])
        assert L.lb_abi_release_d2q9(dd.ptr()) == 0
        assert beq(dd.download(), g["f_out"])
        dd.close()
    finally:
        L.lb_abi_set_mode(0)


def test_abi_borders_and_probe(pkg, oracle):
    L = pkg.lib()
    rng = np.random.default_rng(21)
    W, H, D = 40, 6, 5
    N = W * H * D
    dd = pkg.DeviceData(19, W, H, D)
    f = rng.standard_normal((19, N)).astype(np.float32)
    dd.upload(f)
    L.get_border_d3q19(dd.ptr(), dim(1, 1, 1), dim(32, 4, 1))
    exp = [np.zeros(H * D, np.float32) for _ in range(10)]
    arr = (ctypes.c_void_p * 10)(*[a.ctypes.data for a in exp])
    oracle.lib().lbo_d3q19_get_border(f.ctypes.data_as(ctypes.c_void_p), arr, W, H, D)
    for name, e in zip(dd.s.BORDER, exp):
        assert beq(dd.d2h(getattr(dd.s, name), H * D), e), name
    nb = [rng.standard_normal(H * D).astype(np.float32) for _ in range(10)]
    for name, a in zip(dd.s.NB_BORDER, nb):
        dd.h2d(getattr(dd.s, name), a)
    L.apply_border_d3q19(dd.ptr(), dim(1, 1, 1), dim(32, 4, 1))
    arr = (ctypes.c_void_p * 10)(*[a.ctypes.data for a in nb])
    oracle.lib().lbo_d3q19_apply_border(f.ctypes.data_as(ctypes.c_void_p), arr, W, H, D)
    assert beq(dd.download(), f)
    plot = rng.standard_normal(4 * N).astype(np.float32)
    dd.h2d(dd.plot, plot)
    L.read_value_3d(ctypes.c_void_p(dd.plot), dd.ptr(), 7, 4, 3)
    o = 7 + 4 * W + 3 * W * H
    assert beq(dd.d2h(dd.s.valueCur, 4), plot[4 * o:4 * o + 4])
    L.read_value_3d(ctypes.c_void_p(dd.plot), dd.ptr(), W, 0, 0)
    assert b"outside" in L.lb_abi_last_error()
    L.lb_abi_clear_error()
    # D2Q9 faces
    dd2 = pkg.DeviceData(9, 64, 12)
    f2 = rng.standard_normal((9, 64 * 12)).astype(np.float32)
    dd2.upload(f2)
    L.get_border_d2q9(dd2.ptr(), dim(1, 1, 1), dim(32, 4, 1))
    exp = [np.zeros(12, np.float32) for _ in range(6)]
    arr = (ctypes.c_void_p * 6)(*[a.ctypes.data for a in exp])
    oracle.lib().lbo_d2q9_get_border(f2.ctypes.data_as(ctypes.c_void_p), arr, 64, 12)
    for name, e in zip(dd2.s.BORDER, exp):
        assert beq(dd2.d2h(getattr(dd2.s, name), 12), e), name
    dd.close()
    dd2.close()


def test_abi_reduce(pkg, oracle):
    L = pkg.lib()
    rng = np.random.default_rng(8)
    W, H, D = 64, 16, 8
    N = W * H * D
    dd = pkg.DeviceData(19, W, H, D)
    fields = {k: rng.random(N).astype(np.float32) for k in ["ux", "uy", "uz", "rho"]}
    solid = (rng.random(N) < 0.2).astype(np.uint8)
    for k, v in fields.items():
        dd.h2d(getattr(dd.s, k), v)
    dd.set_solid(solid, np.zeros(N, np.uint8))
    out = (ctypes.c_double * 7)()
    assert L.lb_reduce_d3q19(dd.ptr(), out) == 0
    exp = oracle.reduce_f32(fields["rho"], fields["ux"], fields["uy"], fields["uz"], solid)
    np.testing.assert_allclose(np.array(out[:]), exp, rtol=1e-12)
    dd.close()


# --------------------------------------------------------------------- context API

def _channel_flags(W, H, D, sphere=None, lid=False):
    fl = np.zeros((D, H, W), np.uint8)
    fl[:, 0, :] = fl[:, -1, :] = 1
    fl[0, :, :] = fl[-1, :, :] = 1
    if lid:
        fl[-1, 1:-1, :] = 3
    if sphere is not None:
        cx, cy, cz, r = sphere
        z, y, x = np.mgrid[0:D, 0:H, 0:W]
        fl[(x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2 <= r * r] = 1
    return fl.reshape(-1)


@pytest.mark.parametrize("tuning", [0x100, 0x101], ids=["forward", "alternating"])
def test_context_native_d3q19_vs_oracle(pkg, oracle, tuning):
    """The channel's physics on a small box: x-periodic channel, half-way bounce-back
    walls in y/z, a sphere, body force, a moving wall, 40 steps, bit-exact
    (with and without the alternating sweep order)."""
    W, H, D = 64, 24, 20
    N = W * H * D
    flags = _channel_flags(W, H, D, sphere=(20, 12, 10, 5), lid=True)
    rng = np.random.default_rng(2)
    rho = (1 + 0.01 * rng.standard_normal(N)).astype(np.float32)
    ux = (0.03 * rng.standard_normal(N)).astype(np.float32)
    uy = (0.01 * rng.standard_normal(N)).astype(np.float32)
    z = np.zeros(N, np.float32)
    w = pkg.W3
    tau_inv = np.float32(1 / 0.55)
    F = (np.float32(1e-6), np.float32(2e-7), np.float32(0))
    lat = pkg.Lattice(19, W, H, D, tau_inv=tau_inv, force=F, wall_u=(0.04, 0.0, 0.01),
                      graph_steps=8, tuning=tuning)
    lat.set_flags(flags)
    f0 = oracle.d3q19_equilibrium(rho, ux, uy, z, *w)
    lat.set_populations(f0)
    corr = oracle.wall_correction(19, (0.04, 0.0, 0.01))
    assert beq(lat.wall_correction(), corr)
    lat.step(40)
    f = f0.copy()
    mom = [np.zeros(N, np.float32) for _ in range(4)]
    for _ in range(40):
        oracle.d3q19_stream_native(f, flags, corr, W, H, D)
        oracle.d3q19_collide_native(f, flags, mom, W, H, D, *w, tau_inv, F)
    fluid = (flags & 1) == 0
    assert beq(lat.populations()[:, fluid], f[:, fluid])
    rho_g, ux_g, uy_g, uz_g = lat.moments()
    for a, b in zip((ux_g, uy_g, uz_g, rho_g), mom):
        assert beq(a, b)
    assert lat.launches() >= 40
    lat.close()


def test_context_reference_d3q19_vs_oracle(pkg, oracle):
    """Reference semantics (full-way walls stored in solid nodes, Zou-He in /
    out) through the fused context kernel, 30 steps, bit-exact everywhere."""
    W, H, D = 48, 16, 12
    N = W * H * D
    rng = np.random.default_rng(4)
    solid = (rng.random((D, H, W)) < 0.1).astype(np.uint8)
    solid[:, :, 20:26] = 1
    solid[:, 0, :] = 1
    solid = solid.reshape(-1)
    f0 = (oracle.D3_W[:, None] * (1 + 0.1 * rng.standard_normal((19, N)))).astype(np.float32)
    tau_inv = np.float32(1 / (3 * 0.03 + 0.5))
    lat = pkg.Lattice(19, W, H, D, mode=pkg.abi.LB_MODE_REFERENCE, tau_inv=tau_inv,
                      u_in=(0.05, 0, 0), rho_out=1.0, graph_steps=4)
    lat.set_flags(solid)
    lat.set_populations(f0)
    lat.step(30)
    f = f0.copy()
    sb = oracle.d3q19_solid_bound(solid, W, H, D)
    mom = [np.zeros(N, np.float32) for _ in range(4)]
    for _ in range(30):
        oracle.d3q19_stream(f, sb, W, H, D)
        oracle.d3q19_collide(f, solid, mom, W, H, D, *pkg.W3, tau_inv, 0.05, 0, 0, 1.0)
    assert beq(lat.populations(), f)
    rho_g, ux_g, uy_g, uz_g = lat.moments()
    for a, b in zip((ux_g, uy_g, uz_g, rho_g), mom):
        assert beq(a, b)
    lat.close()


def test_context_lid_cavity_d2q9_vs_oracle(pkg, oracle):
    """The lid-driven cavity's physics on 64x64: closed box, top row a moving lid."""
    W = H = 64
    N = W * H
    fl = np.zeros((H, W), np.uint8)
    fl[:, 0] = fl[:, -1] = fl[-1, :] = 1
    fl[0, :] = 3  # row 0 is the top (physical +y = row-1)
    fl = fl.reshape(-1)
    tau_inv = np.float32(1 / 0.6)
    lat = pkg.Lattice(9, W, H, tau_inv=tau_inv, wall_u=(0.1, 0, 0), graph_steps=16,
                      tuning=0x101)
    lat.set_flags(fl)
    lat.init_equilibrium()
    f = oracle.d2q9_equilibrium(np.ones(N, np.float32), np.zeros(N, np.float32),
                                np.zeros(N, np.float32), *pkg.W2)
    lat.step(150)
    corr = oracle.wall_correction(9, (0.1, 0, 0))
    mom = [np.zeros(N, np.float32) for _ in range(3)]
    for _ in range(150):
        oracle.d2q9_stream_native(f, fl, corr, W, H)
        oracle.d2q9_collide_native(f, fl, mom, W, H, *pkg.W2, tau_inv)
    fluid = (fl & 1) == 0
    assert beq(lat.populations()[:, fluid], f[:, fluid])
    rho_g, ux_g, uy_g, _ = lat.moments()
    assert beq(ux_g, mom[0]) and beq(uy_g, mom[1]) and beq(rho_g, mom[2])
    assert ux_g.reshape(H, W)[1, W // 2] > 0.01  # the lid drags the fluid along +x
    lat.close()


def test_context_reference_d2q9_shan_chen_vs_oracle(pkg, oracle):
    """Reference D2Q9 Shan-Chen (psi = 4 exp(-200/rho), FP64 like the reference)
    through the context API: bit-exact."""
    W, H = 64, 32
    N = W * H
    rng = np.random.default_rng(9)
    rho0 = (200 * (1 + 0.01 * rng.standard_normal(N))).astype(np.float32)
    f0 = (oracle.D2_W[:, None] * rho0[None, :]).astype(np.float32)
    solid = np.zeros(N, np.uint8)
    tau_inv = np.float32(1 / (3 * 0.16667 + 0.5))
    lat = pkg.Lattice(9, W, H, mode=pkg.abi.LB_MODE_REFERENCE, tau_inv=tau_inv, G=-120.0,
                      rho_out=200.0, psi_form=pkg.abi.LB_PSI_REF, graph_steps=4)
    lat.set_flags(solid)
    lat.set_populations(f0)
    lat.step(20)
    f = f0.copy()
    sb = np.zeros(N, np.uint8)
    mom = [np.zeros(N, np.float32) for _ in range(3)]
    sc = [np.zeros(N, np.float32) for _ in range(3)]
    for _ in range(20):
        oracle.d2q9_stream(f, sb, W, H)
        oracle.d2q9_collide(f, solid, mom, sc, W, H, *pkg.W2, tau_inv, 0.0, 0, 200.0, 0, 0,
                            -120.0, 0.0)
    assert beq(lat.populations(), f)
    lat.close()


def test_context_native_d2q9_shan_chen(pkg, oracle):
    """Native D2Q9 Shan-Chen with psi = 1-exp(-rho) (exp evaluated by the
    library's own float function on both sides), 50 steps, bit-exact."""
    W, H = 64, 64
    N = W * H
    rng = np.random.default_rng(10)
    rho = (0.693 * (1 + 0.02 * rng.uniform(-1, 1, N))).astype(np.float32)
    z = np.zeros(N, np.float32)
    lat = pkg.Lattice(9, W, H, tau_inv=1.0, G=-5.0, psi_form=pkg.abi.LB_PSI_EXP1)
    lat.set_flags(np.zeros(N, np.uint8))
    f0 = oracle.d2q9_equilibrium(rho, z, z, *pkg.W2)
    lat.set_populations(f0)
    lat.step(50)
    f = f0.copy()
    mom = [np.zeros(N, np.float32) for _ in range(3)]
    for _ in range(50):
        oracle.d2q9_stream_native(f, np.zeros(N, np.uint8), np.zeros(9, np.float32), W, H)
        oracle.d2q9_collide_native(f, np.zeros(N, np.uint8), mom, W, H, *pkg.W2, 1.0, G=-5.0,
                                   psi_form=oracle.PSI_EXP1)
    rho_g, ux_g, uy_g, _ = lat.moments()
    assert beq(rho_g, mom[2]) and beq(ux_g, mom[0]) and beq(uy_g, mom[1])
    assert beq(lat.populations(), f)
    lat.close()


def test_context_reduce_and_conservation(pkg, oracle):
    """Periodic native D3Q19 without walls or force conserves mass and momentum;
    the FP64 GPU sums match the oracle's sums of the same moments."""
    W, H, D = 64, 32, 32
    N = W * H * D
    rng = np.random.default_rng(12)
    rho = (1 + 0.05 * rng.standard_normal(N)).astype(np.float32)
    ux = (0.02 * rng.standard_normal(N)).astype(np.float32)
    z = np.zeros(N, np.float32)
    lat = pkg.Lattice(19, W, H, D, tau_inv=1 / 0.8)
    lat.set_flags(np.zeros(N, np.uint8))
    lat.init_equilibrium(rho, ux, z, z)
    lat.step(1)
    r0 = lat.reduce()
    rho_g, ux_g, uy_g, uz_g = lat.moments()
    exp = oracle.reduce_f32(rho_g, ux_g, uy_g, uz_g, np.zeros(N, np.uint8))
    np.testing.assert_allclose(r0, exp, rtol=1e-12, atol=1e-12)
    lat.step(200)
    r1 = lat.reduce()
    # FP32 rounding of the BGK update is not exactly conservative: about 2e-8
    # relative mass drift per step at this size, so 200 steps stay below 1e-5
    assert abs(r1[0] - r0[0]) / r0[0] < 1e-5       # mass
    assert abs(r1[1] - r0[1]) < 1e-5 * r0[0]        # x momentum
    assert r1[4] < r0[4]                            # kinetic energy decays
    lat.close()


def test_full_size_channel_steps_vs_oracle(pkg, oracle):
    """The bench workload itself (256x128x128, walls, sphere r=16, gx=1e-6,
    tau=0.55), started from a perturbed state (rho = 1 + 0.01 noise, u of
    0.02 noise, seeded) so that every node changes every step: 65 steps (one
    captured graph of 64 steps, as the bench replays them, and the eager last
    step) compared bit for bit with the oracle, populations and the last
    step's moments."""
    W, H, D = 256, 128, 128
    N = W * H * D
    steps = 65
    flags = _channel_flags(W, H, D, sphere=(64, 64, 64, 16))
    tau_inv = np.float32(1 / 0.55)
    F = (np.float32(1e-6), np.float32(0), np.float32(0))
    rng = np.random.default_rng(2026)
    rho = (1 + 0.01 * rng.standard_normal(N)).astype(np.float32)
    u = [(0.02 * rng.standard_normal(N)).astype(np.float32) for _ in range(3)]
    lat = pkg.Lattice(19, W, H, D, tau_inv=tau_inv, force=F)
    lat.set_flags(flags)
    lat.init_equilibrium(rho, *u)
    lat.step(steps)
    f = oracle.d3q19_equilibrium(rho, *u, *pkg.W3)
    mom = [np.zeros(N, np.float32) for _ in range(4)]
    for _ in range(steps):
        oracle.d3q19_stream_native(f, flags, np.zeros(19, np.float32), W, H, D)
        oracle.d3q19_collide_native(f, flags, mom, W, H, D, *pkg.W3, tau_inv, F)
    fluid = (flags & 1) == 0
    assert beq(lat.populations()[:, fluid], f[:, fluid])
    rho_g, ux_g, uy_g, uz_g = lat.moments()
    assert beq(rho_g, mom[3]) and beq(ux_g, mom[0]) and beq(uy_g, mom[1]) and beq(uz_g, mom[2])
    lat.close()


@pytest.mark.parametrize("storage", [1, 2], ids=["f16", "bf16"])
def test_full_size_channel_16bit_vs_oracle(pkg, oracle, storage):
    """The same 65 steps of the bench lattice in 16-bit deviation storage
    (rho_ref 1): the library's default 16-bit step at this size -- its L2
    prefetch of the rows 912 blocks ahead reaches real rows only on a lattice
    this large -- against the oracle with the storage emulated, every bit of
    every fluid node and the last step's moments."""
    from storage_emul import Emulated
    W, H, D = 256, 128, 128
    N = W * H * D
    steps = 65
    flags = _channel_flags(W, H, D, sphere=(64, 64, 64, 16))
    tau_inv = np.float32(1 / 0.55)
    F = (np.float32(1e-6), np.float32(0), np.float32(0))
    rng = np.random.default_rng(2027 + storage)
    rho = (1 + 0.01 * rng.standard_normal(N)).astype(np.float32)
    u = [(0.02 * rng.standard_normal(N)).astype(np.float32) for _ in range(3)]
    f0 = oracle.d3q19_equilibrium(rho, *u, *pkg.W3)
    lat = pkg.Lattice(19, W, H, D, tau_inv=tau_inv, force=F, storage=storage, rho_ref=1.0)
    lat.set_flags(flags)
    lat.set_populations(f0)
    lat.step(steps)
    em = Emulated(oracle, f0, storage, 1.0)
    mom = [np.zeros(N, np.float32) for _ in range(4)]
    for _ in range(steps):
        em.step(flags, np.zeros(19, np.float32), W, H, D, mom, pkg.W3, tau_inv, F)
    fluid = (flags & 1) == 0
    assert beq(lat.populations()[:, fluid], em.populations()[:, fluid])
    rho_g, ux_g, uy_g, uz_g = lat.moments()
    assert beq(rho_g, mom[3]) and beq(ux_g, mom[0]) and beq(uy_g, mom[1]) and beq(uz_g, mom[2])
    lat.close()
