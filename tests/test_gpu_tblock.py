"""GPU: D2Q9 temporal blocking (LB_TUNE_TBLOCK: one launch advances several
steps of a tile and its halo in shared memory) gives the bits of the per-step
path and of the oracle, for every block shape, for lattices smaller than a
tile and its halo (wrapped duplicates), for ragged tiles, for step counts that
leave a remainder, and for the in-kernel cursor probe."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EXPLICIT, PDL, TBLOCK = 0x100, 0x008, 0x020
PLAIN = EXPLICIT | PDL
SHAPE_STEPS = {1: 4, 2: 4, 3: 3, 4: 2, 5: 5, 6: 4, 7: 3, 8: 8, 9: 6, 10: 4}


def tb(shape):
    return EXPLICIT | TBLOCK | (shape << 12)


def beq(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def cavity_flags(W, H):
    fl = np.zeros((H, W), np.uint8)
    fl[:, 0] = fl[:, -1] = fl[-1, :] = 1
    fl[0, :] = 3
    return fl.reshape(-1)


def obstacle_flags(W, H, seed):
    """periodic in x, walls at the first and last row, random solid blocks"""
    rng = np.random.default_rng(seed)
    fl = (rng.random((H, W)) < 0.06).astype(np.uint8)
    fl[0, :] = fl[-1, :] = 1
    return fl.reshape(-1)


def run(pkg, W, H, tuning, steps, flags, rho=None, ux=None, **kw):
    lat = pkg.Lattice(9, W, H, tuning=tuning, graph_steps=16, **kw)
    lat.set_flags(flags)
    lat.init_equilibrium(rho, ux, None, None)
    for n in steps:
        lat.step(n)
    out = (lat.populations(), lat.moments()[:3], lat.launches(), lat.steps_done())
    lat.close()
    return out


def same(pkg, W, H, shape, steps, flags, **kw):
    f_t, m_t, _, done_t = run(pkg, W, H, tb(shape), steps, flags, **kw)
    f_p, m_p, _, done_p = run(pkg, W, H, PLAIN, steps, flags, **kw)
    assert done_t == done_p == sum(steps)
    assert beq(f_t, f_p)
    for a, b in zip(m_t, m_p):
        assert beq(a, b)


@pytest.mark.parametrize("shape", sorted(SHAPE_STEPS))
def test_cavity_every_shape(pkg, shape):
    W = H = 256
    same(pkg, W, H, shape, [1, 7, 37, 130], cavity_flags(W, H),
         tau_inv=np.float32(1 / 0.6), wall_u=(0.1, 0, 0))


@pytest.mark.parametrize("W,H", [(100, 37), (12, 10), (5, 70), (300, 3)])
@pytest.mark.parametrize("shape", [1, 3, 5, 8, 10])
def test_ragged_and_small_lattices_with_force(pkg, W, H, shape):
    """ragged tiles, and lattices narrower than a tile and its halo, where a
    block holds several wrapped copies of the same node"""
    rng = np.random.default_rng(W * H + shape)
    fl = obstacle_flags(W, H, W + H) if H > 4 else np.zeros(W * H, np.uint8)
    rho = (1 + 0.02 * rng.standard_normal(W * H)).astype(np.float32)
    ux = (0.03 * rng.standard_normal(W * H)).astype(np.float32)
    same(pkg, W, H, shape, [3, 16, 41], fl, rho=rho, ux=ux,
         tau_inv=np.float32(1 / 0.7), force=(2e-5, -1e-5, 0), wall_u=(0.02, 0, 0))


def test_moving_walls_everywhere(pkg):
    """moving walls on all four sides and inside, so near-wall nodes of every
    direction take the moving-wall term from shared memory"""
    W, H = 90, 66
    rng = np.random.default_rng(8)
    fl = np.where(rng.random((H, W)) < 0.08, 3, 0).astype(np.uint8)
    fl[0, :] = fl[-1, :] = 3
    fl[:, 0] = fl[:, -1] = 3
    same(pkg, W, H, 2, [64, 9], fl.reshape(-1), tau_inv=np.float32(1 / 0.55),
         wall_u=(0.05, -0.03, 0))


def test_cavity_vs_oracle(pkg, oracle):
    W, H = 96, 80
    N = W * H
    fl = cavity_flags(W, H)
    tau_inv = np.float32(1 / 0.6)
    f_t, (rho, ux, uy), _, _ = run(pkg, W, H, tb(1), [33, 90], fl, tau_inv=tau_inv,
                                   wall_u=(0.1, 0, 0))
    f = oracle.d2q9_equilibrium(np.ones(N, np.float32), np.zeros(N, np.float32),
                                np.zeros(N, np.float32), *pkg.W2)
    corr = oracle.wall_correction(9, (0.1, 0, 0))
    mom = [np.zeros(N, np.float32) for _ in range(3)]
    for _ in range(123):
        oracle.d2q9_stream_native(f, fl, corr, W, H)
        oracle.d2q9_collide_native(f, fl, mom, W, H, *pkg.W2, tau_inv)
    fluid = (fl & 1) == 0
    assert beq(f_t[:, fluid], f[:, fluid])
    assert beq(ux, mom[0]) and beq(uy, mom[1]) and beq(rho, mom[2])


def test_launch_count(pkg):
    """a 4-step block per launch: 64 steps are 16 launches (in graphs of 4)"""
    W = H = 64
    lat = pkg.Lattice(9, W, H, tuning=tb(1), graph_steps=16)
    lat.set_flags(cavity_flags(W, H))
    lat.init_equilibrium()
    before = lat.launches()
    lat.step(64)
    assert lat.launches() - before == 16
    before = lat.launches()
    lat.step(6)  # one block of 4 + two single steps
    assert lat.launches() - before == 3
    assert lat.steps_done() == 70
    lat.close()


@pytest.mark.parametrize("kw,per_step", [
    (dict(G=-5.0, tau_inv=1.0), 2),                       # Shan-Chen: two passes per step
    (dict(mode=0, u_in=(0.05, 0, 0), tau_inv=1.25), 1),   # reference mode: Zou-He columns
])
def test_ignored_where_it_does_not_apply(pkg, kw, per_step):
    W, H = 64, 32
    lat = pkg.Lattice(9, W, H, tuning=tb(1), graph_steps=8, **kw)
    lat.init_equilibrium(np.full(W * H, 0.7, np.float32), None, None, None)
    before = lat.launches()
    lat.step(5)
    assert lat.launches() - before == 5 * per_step
    lat.close()


def test_run_probe(pkg):
    """lb_run_probe through temporal blocks: the cursor node's moments of the
    last step, as on the per-step path"""
    L = pkg.lib()
    W, H = 128, 72
    fl = cavity_flags(W, H)
    vals = []
    for tuning in (tb(2), PLAIN):
        lat = pkg.Lattice(9, W, H, tuning=tuning, graph_steps=16, tau_inv=np.float32(1 / 0.6),
                          wall_u=(0.1, 0, 0))
        lat.set_flags(fl)
        lat.init_equilibrium()
        v = np.full(4, np.nan, np.float32)
        for n, x, y in [(43, 17, 5), (8, 100, 60), (5, 0, 0)]:
            assert L.lb_run_probe(lat.h, n, x, y, 0, v.ctypes.data_as(ctypes.c_void_p)) == 0
            vals.append(v.copy())
        lat.close()
    for a, b in zip(vals[:3], vals[3:]):
        assert beq(a, b)


@pytest.mark.parametrize("W,H,per_launch", [(256, 256, 5), (128, 64, 5), (1024, 1024, 1)])
def test_default_tuning(pkg, W, H, per_launch):
    """by default D2Q9 native mode without Shan-Chen runs temporal blocks of
    5 steps up to 2^19 nodes and one launch per step above"""
    lat = pkg.Lattice(9, W, H, graph_steps=20, tau_inv=np.float32(1 / 0.6), wall_u=(0.1, 0, 0))
    lat.set_flags(cavity_flags(W, H))
    lat.init_equilibrium()
    before = lat.launches()
    lat.step(100)
    assert lat.launches() - before == 100 // per_launch
    lat.close()
