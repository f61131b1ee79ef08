"""The oracle's binary16 / bfloat16 conversions (used to emulate the 16-bit
deviation storage) round to nearest even like numpy's float16 cast and like
an integer-arithmetic bfloat16 reference."""
import numpy as np


def _bf16_reference(a):
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16).astype(np.uint32) << 16
    out = r.astype(np.uint32).view(np.float32)
    nan = np.isnan(a)
    out[nan] = np.nan
    return out


def test_f16_roundtrip_matches_numpy(oracle):
    rng = np.random.default_rng(1)
    a = np.concatenate([
        rng.standard_normal(200000).astype(np.float32) * 1e-3,
        rng.standard_normal(200000).astype(np.float32) * 10,
        (rng.random(50000).astype(np.float32) * 2 - 1) * 7e-5,   # subnormal range of binary16
        np.array([0.0, -0.0, 65504.0, 65519.99, 65520.0, 1e9, -1e9, 2.0 ** -25, 2.0 ** -24,
                  3 * 2.0 ** -26, np.inf, -np.inf], np.float32)])
    got = oracle.f16_roundtrip(a)
    exp = a.astype(np.float16).astype(np.float32)
    assert np.array_equal(got.view(np.uint32), exp.view(np.uint32))


def test_bf16_roundtrip_matches_integer_reference(oracle):
    rng = np.random.default_rng(2)
    a = np.concatenate([rng.standard_normal(300000).astype(np.float32) * s
                        for s in (1e-30, 1e-3, 1.0, 1e30)])
    got = oracle.bf16_roundtrip(a)
    exp = _bf16_reference(a)
    assert np.array_equal(got.view(np.uint32), exp.view(np.uint32))


def test_expf_accuracy(oracle):
    """The float exp shared by the kernels and the oracle (Cody-Waite + Taylor)
    stays within 1.5 ulp of exp on [-20, 0] and [-87, 88] (1.12 measured)."""
    import ctypes
    fn = oracle.lib().lbo_expf
    fn.restype = ctypes.c_float
    fn.argtypes = [ctypes.c_float]
    for lo, hi, tol in [(-20.0, 0.0, 1.5), (-87.0, 88.0, 1.5)]:
        xs = np.linspace(lo, hi, 20001).astype(np.float32)
        got = np.array([fn(float(x)) for x in xs], np.float64)
        exact = np.exp(xs.astype(np.float64))
        ulp = np.spacing(exact.astype(np.float32)).astype(np.float64)
        assert np.max(np.abs(got - exact) / ulp) <= tol
    assert fn(-200.0) == 0.0 and fn(100.0) == float("inf")


def test_quantize_dev_keeps_walls(oracle):
    rng = np.random.default_rng(3)
    f = rng.random((19, 1000)).astype(np.float32)
    flags = (rng.random(1000) < 0.3).astype(np.uint8)
    wr = oracle.storage_offsets(19, 0.693)
    g = f.copy()
    oracle.quantize_dev(g, wr, flags, kind=1)
    assert np.array_equal(g[:, flags == 1], f[:, flags == 1])
    d = (f[:, flags == 0] - wr[:, None]).astype(np.float32)
    exp = (wr[:, None] + d.astype(np.float16).astype(np.float32)).astype(np.float32)
    assert np.array_equal(g[:, flags == 0], exp)


def test_deviation_step_tracks_the_float_step(oracle):
    """The deviation form of the native collision (16-bit storage's
    arithmetic, no narrowing here) gives the float step's populations,
    moments and psi to FP32 rounding: the offsets carry rho_ref exactly."""
    W, H, D = 12, 10, 8
    N = W * H * D
    rng = np.random.default_rng(3)
    rho = (0.693 * (1 + 0.01 * rng.uniform(-1, 1, N))).astype(np.float32)
    u = [(0.02 * rng.standard_normal(N)).astype(np.float32) for _ in range(3)]
    w = (np.float32(1 / 3), np.float32(1 / 18), np.float32(1 / 36))
    f = oracle.d3q19_equilibrium(rho, *u, *w)
    wr = oracle.storage_offsets(19, 0.693)
    d = np.ascontiguousarray(f - wr[:, None])
    flags = np.zeros(N, np.uint8)
    zc = np.zeros(19, np.float32)
    F = (np.float32(1e-5), np.float32(0), np.float32(0))
    m_f = [np.zeros(N, np.float32) for _ in range(4)]
    m_d = [np.zeros(N, np.float32) for _ in range(4)]
    psi_f, psi_d = np.zeros(N, np.float32), np.zeros(N, np.float32)
    for tau_inv in (np.float32(1.0), np.float32(1 / 0.7)):
        for _ in range(5):
            oracle.d3q19_stream_native(f, flags, zc, W, H, D)
            oracle.d3q19_collide_native(f, flags, m_f, W, H, D, *w, tau_inv, F, G=-5.0, psi=psi_f)
            oracle.d3q19_stream_native(d, flags, zc, W, H, D)
            oracle.d3q19_collide_native_dev(d, flags, m_d, W, H, D, *w, tau_inv, wr, F, G=-5.0,
                                            psi=psi_d)
        np.testing.assert_allclose(oracle.from_dev(d, wr), f, rtol=0, atol=2e-7)
        for a, b in zip(m_d, m_f):
            np.testing.assert_allclose(a, b, rtol=0, atol=2e-6)
        np.testing.assert_allclose(psi_d, psi_f, rtol=0, atol=1e-6)
    assert oracle.rho_offset(wr) == np.float32(np.sum(wr.astype(np.float64)))
