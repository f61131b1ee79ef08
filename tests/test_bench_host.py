"""Host logic of bench.py that feeds the GPU runs (CPU only): the reference's
solid_bound rule used by the drop-in end-to-end leg, and the channel flags of
the z-slab workload."""
import numpy as np

import bench


def test_solid_bound_matches_oracle(oracle):
    rng = np.random.default_rng(2)
    nx, ny, nz = 12, 9, 7
    for frac in (0.5, 0.9, 0.97, 1.0):
        s = (rng.random(nx * ny * nz) < frac).astype(np.uint8)
        assert np.array_equal(bench.solid_bound_d3q19(s, nx, ny, nz),
                              oracle.d3q19_solid_bound(s, nx, ny, nz))


def test_channel_flags_one_sphere_is_the_channel():
    wl = bench.WORKLOADS["channel"]
    nx, ny, nz = 64, 32, 128
    wl_small = bench.Workload("channel", 19, (nx, ny, nz), 0.55, 10, 153)
    a = bench.channel_flags(nx, ny, nz, 1)
    b = wl_small.flags()
    assert np.array_equal(a, b)
    two = bench.channel_flags(nx, ny, 256, 2).reshape(256, ny, nx)
    assert np.array_equal(two[:128][1:-1], two[128:][1:-1])  # the same section twice
    assert wl.size == (256, 128, 128)
