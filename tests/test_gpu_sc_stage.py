"""GPU parity of the single-pass D3Q19 Shan-Chen step whose populations reach
shared memory by bulk asynchronous copies (tuning LB_TUNE_SC_STAGED), on
lattices without wall nodes.

* Bit-exact against the two-pass step (density pass + fused step) for FP32,
  FP16 and BF16 storage, on lattices where a row wraps in x inside one tile
  (nx = 32: a staged row is copied in three pieces), the ring rows wrap in y
  (ny = 8), and the march runs over several z chunks (the chunk length is
  the shortest that divides nz when the lattice is small), with a body force
  and graph-replayed batches whose last step writes the moments.
* Tiles away from the lattice's edges get their stages by TMA tensor copies,
  edge tiles (periodic wrap) by cp.async chunks: the same lattices with every
  stage copied by cp.async give the same bits, and so do lattices of 3 x 3
  and 5 x 5 tiles per plane against the two-pass step.
* Bit-exact against the float oracle on its own.
* A lattice with a wall node takes the two-pass step whatever the tuning
  says (two launches per step), and returns to the staged step when the
  walls are removed.
"""
import ctypes

import numpy as np
import pytest

from storage_emul import Emulated

from conftest import load_package
from golden_io import bits

pytestmark = pytest.mark.gpu

STAGED = 0x100 | 0x040   # LB_TUNE_EXPLICIT | LB_TUNE_SC_STAGED
NO_TMA = 0x080           # LB_TUNE_SC_NO_TMA: every stage by cp.async chunks
TWO_PASS = 0x100         # LB_TUNE_EXPLICIT


@pytest.fixture(scope="module")
def pkg():
    p = load_package()
    n = ctypes.c_int(0)
    assert p.lib().lb_device_count(ctypes.byref(n)) == 0 and n.value >= 1, "no CUDA device"
    return p


def beq(a, b):
    return np.array_equal(bits(a), bits(b))


def spinodal(N, seed):
    rng = np.random.default_rng(seed)
    return (0.693 * (1 + rng.uniform(-0.01, 0.01, N))).astype(np.float32)


def run(pkg, shape, storage, tuning, steps, flags=None, seed=3, graph_steps=4):
    W, H, D = shape
    N = W * H * D
    rho = spinodal(N, seed)
    z = np.zeros(N, np.float32)
    F = (np.float32(2e-6), np.float32(0), np.float32(-1e-6))
    lat = pkg.Lattice(19, W, H, D, tau_inv=1.0, G=-5.0, psi_form=pkg.abi.LB_PSI_EXP1,
                      force=F, storage=storage, rho_ref=0.693, tuning=tuning,
                      graph_steps=graph_steps)
    lat.set_flags(np.zeros(N, np.uint8) if flags is None else flags)
    lat.init_equilibrium(rho, z, z, z)
    before = lat.launches()
    lat.step(steps)
    launches = lat.launches() - before
    out = (lat.populations(), lat.moments(), launches)
    lat.close()
    return out


@pytest.mark.parametrize("shape", [(32, 8, 8), (64, 16, 48), (96, 24, 20), (160, 40, 16)],
                         ids=["32x8x8", "64x16x48", "96x24x20", "160x40x16"])
@pytest.mark.parametrize("storage", [0, 1, 2], ids=["f32", "f16", "bf16"])
def test_staged_matches_two_pass(pkg, shape, storage):
    steps = 14
    f_s, m_s, l_s = run(pkg, shape, storage, STAGED, steps)
    f_t, m_t, l_t = run(pkg, shape, storage, TWO_PASS, steps)
    assert l_s == steps and l_t == 2 * steps, (l_s, l_t)
    assert np.isfinite(f_s).all()
    assert beq(f_s, f_t)
    for a, b in zip(m_s, m_t):
        assert beq(a, b)


@pytest.mark.parametrize("shape", [(96, 24, 20), (160, 40, 16), (256, 64, 8)],
                         ids=["3x3_tiles", "5x5_tiles", "8x8_tiles"])
@pytest.mark.parametrize("storage", [0, 1, 2], ids=["f32", "f16", "bf16"])
def test_tma_tiles_match_cp_async_tiles(pkg, shape, storage):
    f_t, m_t, l_t = run(pkg, shape, storage, STAGED, 11)
    f_c, m_c, l_c = run(pkg, shape, storage, STAGED | NO_TMA, 11)
    assert l_t == l_c == 11
    assert np.isfinite(f_t).all()
    assert beq(f_t, f_c)
    for a, b in zip(m_t, m_c):
        assert beq(a, b)


@pytest.mark.parametrize("storage", [0, 2], ids=["f32", "bf16"])
def test_staged_vs_oracle(pkg, oracle, storage):
    W, H, D = 128, 32, 12   # 4 x 4 tiles per plane: the middle four by TMA
    N = W * H * D
    steps = 10
    F = (np.float32(2e-6), np.float32(0), np.float32(-1e-6))
    f_g, m_g, _ = run(pkg, (W, H, D), storage, STAGED, steps, seed=11)
    rho = spinodal(N, 11)
    z = np.zeros(N, np.float32)
    flags = np.zeros(N, np.uint8)
    em = Emulated(oracle, oracle.d3q19_equilibrium(rho, z, z, z, *pkg.W3), storage, 0.693)
    mom = [np.zeros(N, np.float32) for _ in range(4)]
    psi = np.zeros(N, np.float32)
    zc = np.zeros(19, np.float32)
    for _ in range(steps):
        em.step(flags, zc, W, H, D, mom, pkg.W3, np.float32(1.0), F, G=-5.0, psi=psi)
    assert beq(f_g, em.populations())
    rho_g, ux_g, uy_g, uz_g = m_g
    assert beq(rho_g, mom[3]) and beq(ux_g, mom[0]) and beq(uy_g, mom[1]) and beq(uz_g, mom[2])


@pytest.mark.parametrize("storage", [0, 1], ids=["f32", "f16"])
def test_staged_reference_psi_matches_two_pass(pkg, storage):
    """The reference's pseudo-potential psi = 4 exp(-200/rho) (rho near 200,
    G = -120, as in the reference's Shan-Chen samples) through the staged
    step, bit-exact against the two-pass step."""
    W, H, D = 64, 16, 12
    N = W * H * D
    rng = np.random.default_rng(9)
    rho = (200.0 * (1 + rng.uniform(-0.01, 0.01, N))).astype(np.float32)
    z = np.zeros(N, np.float32)
    out = []
    for tuning in (STAGED, TWO_PASS):
        lat = pkg.Lattice(19, W, H, D, tau_inv=1.0, G=-120.0, psi_form=pkg.abi.LB_PSI_REF,
                          storage=storage, rho_ref=200.0, tuning=tuning, graph_steps=4)
        lat.set_flags(np.zeros(N, np.uint8))
        lat.init_equilibrium(rho, z, z, z)
        b = lat.launches()
        lat.step(10)
        n = lat.launches() - b  # before populations(): 16-bit reads launch conversions
        out.append((lat.populations(), lat.moments(), n))
        lat.close()
    (f_s, m_s, l_s), (f_t, m_t, l_t) = out
    assert l_s == 10 and l_t == 20
    assert np.isfinite(f_s).all()
    assert beq(f_s, f_t)
    for a, b in zip(m_s, m_t):
        assert beq(a, b)


def test_walls_take_the_two_pass_step(pkg):
    W, H, D = 64, 16, 16
    N = W * H * D
    flags = np.zeros(N, np.uint8)
    flags[5 + W * (3 + H * 7)] = 1  # one wall node
    f_s, m_s, l_s = run(pkg, (W, H, D), 0, STAGED, 6, flags=flags)
    f_t, m_t, l_t = run(pkg, (W, H, D), 0, TWO_PASS, 6, flags=flags)
    assert l_s == l_t == 12
    assert beq(f_s, f_t)
    # the same context switches back to the staged step once the wall is gone
    rho = spinodal(N, 5)
    z = np.zeros(N, np.float32)
    lat = pkg.Lattice(19, W, H, D, tau_inv=1.0, G=-5.0, psi_form=pkg.abi.LB_PSI_EXP1,
                      tuning=STAGED, graph_steps=4)
    lat.set_flags(flags)
    lat.init_equilibrium(rho, z, z, z)
    b = lat.launches()
    lat.step(4)
    assert lat.launches() - b == 8
    lat.set_flags(np.zeros(N, np.uint8))
    b = lat.launches()
    lat.step(4)
    assert lat.launches() - b == 4
    lat.close()
