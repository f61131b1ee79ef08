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
