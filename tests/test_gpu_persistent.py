"""GPU: the D2Q9 persistent step loop (LB_TUNE_PERSISTENT, one cooperative
launch per lb_step) gives the same bits as the per-step graph path and the
oracle, for band layouts of one and several rows per block."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PERSIST = 0x100 | 0x004   # LB_TUNE_EXPLICIT | LB_TUNE_PERSISTENT
PLAIN = 0x100


def beq(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def cavity_flags(W, H):
    fl = np.zeros((H, W), np.uint8)
    fl[:, 0] = fl[:, -1] = fl[-1, :] = 1
    fl[0, :] = 3
    return fl.reshape(-1)


def run(pkg, W, H, tuning, steps, mode=1, flags=None, **kw):
    lat = pkg.Lattice(9, W, H, mode=mode, tuning=tuning, graph_steps=8, **kw)
    if flags is not None:
        lat.set_flags(flags)
    lat.init_equilibrium()
    for n in steps:
        lat.step(n)
    out = (lat.populations(), lat.moments()[:3], lat.launches(), lat.steps_done())
    lat.close()
    return out


@pytest.mark.parametrize("W,H", [(64, 64), (100, 37), (512, 1024)])
def test_persistent_cavity_matches_graph_path(pkg, W, H):
    fl = cavity_flags(W, H)
    kw = dict(tau_inv=np.float32(1 / 0.6), wall_u=(0.1, 0, 0), flags=fl)
    steps = [1, 7, 40] if W * H < 100000 else [3, 9]
    f_p, m_p, launches_p, done_p = run(pkg, W, H, PERSIST, steps, **kw)
    f_g, m_g, _, done_g = run(pkg, W, H, PLAIN, steps, **kw)
    assert done_p == done_g == sum(steps)
    assert launches_p <= len(steps) + 2  # one launch per lb_step (plus the initialisation)
    assert beq(f_p, f_g)
    for a, b in zip(m_p, m_g):
        assert beq(a, b)


def test_persistent_cavity_vs_oracle(pkg, oracle):
    W, H = 96, 80
    N = W * H
    fl = cavity_flags(W, H)
    tau_inv = np.float32(1 / 0.6)
    f_p, (rho, ux, uy), _, _ = run(pkg, W, H, PERSIST, [33, 90], flags=fl, tau_inv=tau_inv,
                                   wall_u=(0.1, 0, 0))
    f = oracle.d2q9_equilibrium(np.ones(N, np.float32), np.zeros(N, np.float32),
                                np.zeros(N, np.float32), *pkg.W2)
    corr = oracle.wall_correction(9, (0.1, 0, 0))
    mom = [np.zeros(N, np.float32) for _ in range(3)]
    for _ in range(123):
        oracle.d2q9_stream_native(f, fl, corr, W, H)
        oracle.d2q9_collide_native(f, fl, mom, W, H, *pkg.W2, tau_inv)
    fluid = (fl & 1) == 0
    assert beq(f_p[:, fluid], f[:, fluid])
    assert beq(ux, mom[0]) and beq(uy, mom[1]) and beq(rho, mom[2])


def test_persistent_reference_mode_with_solids(pkg):
    """The reference's semantics (Zou-He inlet/outlet, full-way bounce-back
    solids) through the persistent loop: the same bits as the graph path."""
    W, H = 160, 48
    rng = np.random.default_rng(4)
    sol = (rng.random((H, W)) < 0.1).astype(np.uint8)
    sol[0, :] = sol[-1, :] = 1
    kw = dict(mode=0, flags=sol.reshape(-1), tau_inv=np.float32(1 / 0.8),
              u_in=(0.05, 0, 0), rho_out=1.0, force=(1e-5, 0, 0))
    f_p, m_p, _, _ = run(pkg, W, H, PERSIST, [5, 50], **kw)
    f_g, m_g, _, _ = run(pkg, W, H, PLAIN, [5, 50], **kw)
    assert beq(f_p, f_g)
    for a, b in zip(m_p, m_g):
        assert beq(a, b)


def test_persistent_is_skipped_for_shan_chen(pkg):
    """With a Shan-Chen pass the flag is ignored (two launches per step)."""
    W, H = 64, 32
    lat = pkg.Lattice(9, W, H, tuning=PERSIST, G=-5.0, tau_inv=1.0, graph_steps=8)
    lat.init_equilibrium(rho=np.full(W * H, 0.7, np.float32))
    before = lat.launches()
    lat.step(3)
    assert lat.launches() - before == 6
    lat.close()


PDL = 0x100 | 0x008       # LB_TUNE_EXPLICIT | LB_TUNE_PDL


@pytest.mark.parametrize("mode", [0, 1], ids=["reference", "native"])
def test_programmatic_dependent_launch_same_bits(pkg, mode):
    """LB_TUNE_PDL (each step a programmatic dependent launch, captured in
    the step graphs) gives the graph path's bits."""
    W, H = 200, 72
    rng = np.random.default_rng(6)
    if mode == 0:
        fl = (rng.random((H, W)) < 0.1).astype(np.uint8).reshape(-1)
        kw = dict(mode=0, u_in=(0.05, 0, 0), tau_inv=np.float32(1 / 0.8))
    else:
        fl = cavity_flags(W, H)
        kw = dict(mode=1, wall_u=(0.1, 0, 0), tau_inv=np.float32(1 / 0.6))
    f_p, m_p, _, _ = run(pkg, W, H, PDL, [1, 5, 37], flags=fl, **kw)
    f_g, m_g, _, _ = run(pkg, W, H, PLAIN, [1, 5, 37], flags=fl, **kw)
    assert beq(f_p, f_g)
    for a, b in zip(m_p, m_g):
        assert beq(a, b)
