"""z-slab decomposition on the GPU, through the C ABI: slabs stepped with
lb_slab_group_step, or with lb_slab_step / lb_slab_unpack and face buffers
moved by the caller, give the same populations and moments as one context
over the whole lattice, bit for bit (walls, a moving wall, a solid block
crossing slab boundaries, a body force, periodic z; FP32 and BF16 storage;
slabs of one and two planes, where the boundary planes are all there is)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W, H, D = 40, 12, 18


def setup(pkg, oracle, seed=3):
    fl = np.zeros((D, H, W), np.uint8)
    fl[:, 0, :] = 1
    fl[:, H - 1, :] = 3
    fl[3:9, 4:8, 10:17] = 1
    fl = fl.reshape(-1)
    rng = np.random.default_rng(seed)
    N = W * H * D
    rho = (1 + 0.02 * rng.standard_normal(N)).astype(np.float32)
    u = [(0.03 * rng.standard_normal(N)).astype(np.float32) for _ in range(3)]
    f = oracle.d3q19_equilibrium(rho, *u, *pkg.W3)
    return fl, f


PHYS = dict(tau_inv=np.float32(1 / 0.6), force=(np.float32(2e-5), np.float32(0), np.float32(-1e-5)),
            wall_u=(0.04, 0, 0.01))


def whole(pkg, fl, f, steps, storage=0):
    lat = pkg.Lattice(19, W, H, D, graph_steps=4, storage=storage,
                      rho_ref=1.0 if storage else 0.0, **PHYS)
    lat.set_flags(fl)
    lat.set_populations(f)
    lat.step(steps)
    out = lat.populations(), lat.moments(), lat.reduce()
    lat.close()
    return out


def make_slabs(pkg, fl, f, bounds, storage=0, graph_steps=64):
    S = pkg.slab
    P = W * H
    slabs = []
    for z0, nz in bounds:
        s = S.Slab(W, H, D, z0, nz, storage=storage, rho_ref=1.0 if storage else 0.0,
                   graph_steps=graph_steps, **PHYS)
        planes = s.planes()
        s.set_flags(np.ascontiguousarray(fl.reshape(D, P)[planes].reshape(-1)))
        s.set_populations(np.ascontiguousarray(f.reshape(19, D, P)[:, planes].reshape(19, -1)))
        slabs.append(s)
    return slabs


def gather(slabs):
    P = W * H
    f = np.zeros((19, D * P), np.float32)
    mom = [np.zeros(D * P, np.float32) for _ in range(4)]
    for s in slabs:
        a, b = s.z0 * P, (s.z0 + s.nz) * P
        f[:, a:b] = s.own(s.populations())
        for i, m in enumerate(s.moments()):
            mom[i][a:b] = s.own(m)
    return f, mom


@pytest.mark.parametrize("bounds", [[(0, 18)], [(0, 9), (9, 9)], [(0, 7), (7, 4), (11, 7)],
                                    [(0, 1), (1, 2), (3, 15)]],
                         ids=["one", "two", "three", "thin"])
def test_slab_group_bit_exact(pkg, oracle, bounds):
    fl, f = setup(pkg, oracle)
    steps = 9
    f_ref, mom_ref, red_ref = whole(pkg, fl, f, steps)
    slabs = make_slabs(pkg, fl, f, bounds)
    grp = pkg.slab.SlabGroup(slabs)
    grp.step(steps - 4)
    grp.step(4)
    grp.synchronize()
    got, mom = gather(slabs)
    assert np.array_equal(got.view(np.uint32), f_ref.view(np.uint32))
    for a, b in zip(mom, mom_ref):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    # conservation sums over the own planes of every slab add up to the whole
    # lattice's (FP64, summed in another order)
    reds = np.array([s.reduce() for s in slabs])
    np.testing.assert_allclose(reds[:, :5].sum(axis=0), red_ref[:5], rtol=1e-12, atol=1e-15)
    assert reds[:, 5].max() == red_ref[5] and reds[:, 6].sum() == red_ref[6]
    for s in slabs:
        s.close()


@pytest.mark.parametrize("bounds", [[(0, 18)], [(0, 7), (7, 4), (11, 7)]], ids=["one", "three"])
def test_slab_group_graphs(pkg, oracle, bounds):
    """Batches replayed from captured graphs (4 steps each, on every slab's
    two streams), then eager steps: the same bits as one context, and the
    step counts and moments of the last step follow."""
    fl, f = setup(pkg, oracle, seed=9)
    steps = 23
    f_ref, mom_ref, _ = whole(pkg, fl, f, steps)
    slabs = make_slabs(pkg, fl, f, bounds, graph_steps=4)
    grp = pkg.slab.SlabGroup(slabs)
    grp.step(13)   # three graphs of 4, one eager step
    grp.step(10)   # the graphs again (same set and parity), then one eager step
    grp.synchronize()
    got, mom = gather(slabs)
    assert np.array_equal(got.view(np.uint32), f_ref.view(np.uint32))
    for a, b in zip(mom, mom_ref):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert all(s.steps_done() == steps for s in slabs)
    ms = grp.time_steps(9)
    assert ms > 0 and all(s.steps_done() == steps + 9 for s in slabs)
    for s in slabs:
        s.close()


def test_slab_group_bf16(pkg, oracle):
    fl, f = setup(pkg, oracle, seed=4)
    steps = 6
    f_ref, mom_ref, _ = whole(pkg, fl, f, steps, storage=2)
    slabs = make_slabs(pkg, fl, f, pkg.slab.slab_bounds(D, 2), storage=2)
    pkg.slab.SlabGroup(slabs).step(steps)
    got, mom = gather(slabs)
    assert np.array_equal(got.view(np.uint32), f_ref.view(np.uint32))
    assert np.array_equal(mom[0].view(np.uint32), mom_ref[0].view(np.uint32))
    for s in slabs:
        s.close()


def test_slab_caller_transport(pkg, oracle):
    """The external-transport protocol: lb_slab_step packs each slab's new
    faces into the caller's device buffers, the caller moves them (here a
    device copy per face, as a transport between processes would), and
    lb_slab_unpack writes the received faces into the ghost planes."""
    L = pkg.lib()
    fl, f = setup(pkg, oracle, seed=5)
    steps = 5
    f_ref, _, _ = whole(pkg, fl, f, steps)
    slabs = make_slabs(pkg, fl, f, pkg.slab.slab_bounds(D, 3))
    fb = slabs[0].face_bytes
    assert fb == 5 * W * H * 4

    def dev(n):
        p = ctypes.c_void_p()
        assert L.lb_malloc(ctypes.byref(p), n) == 0
        return p

    send = [[dev(fb), dev(fb)] for _ in slabs]
    recv = [[dev(fb), dev(fb)] for _ in slabs]
    n = len(slabs)
    for t in range(steps):
        for i, s in enumerate(slabs):
            s.step_slab(t == steps - 1, send[i][0], send[i][1])
        for s in slabs:
            s.synchronize()
        for i in range(n):
            lo, hi = (i - 1) % n, (i + 1) % n
            # my from_below is the lower slab's to_above, my from_above the upper's to_below
            hbuf = np.empty(fb, np.uint8)
            assert L.lb_memcpy_d2h(hbuf.ctypes.data_as(ctypes.c_void_p), send[lo][1], fb) == 0
            assert L.lb_memcpy_h2d(recv[i][0], hbuf.ctypes.data_as(ctypes.c_void_p), fb) == 0
            assert L.lb_memcpy_d2h(hbuf.ctypes.data_as(ctypes.c_void_p), send[hi][0], fb) == 0
            assert L.lb_memcpy_h2d(recv[i][1], hbuf.ctypes.data_as(ctypes.c_void_p), fb) == 0
        for i, s in enumerate(slabs):
            s.unpack(recv[i][0], recv[i][1])
    got, _ = gather(slabs)
    assert np.array_equal(got.view(np.uint32), f_ref.view(np.uint32))
    for pair in send + recv:
        for p in pair:
            L.lb_free(p)
    for s in slabs:
        s.close()


def test_slab_faces_match_host_restatement(pkg, oracle):
    """lb_slab_pack writes exactly the planes the host restatement names."""
    L = pkg.lib()
    fl, f = setup(pkg, oracle, seed=6)
    S = pkg.slab
    s = make_slabs(pkg, fl, f, [(4, 6)])[0]
    fb = s.face_bytes
    bufs = []
    for _ in range(2):
        p = ctypes.c_void_p()
        assert L.lb_malloc(ctypes.byref(p), fb) == 0
        bufs.append(p)
    s.pack(bufs[0], bufs[1])
    s.synchronize()
    host = [np.empty((5, W * H), np.float32) for _ in range(2)]
    for h, p in zip(host, bufs):
        assert L.lb_memcpy_d2h(h.ctypes.data_as(ctypes.c_void_p), p, fb) == 0
    lo, hi = S.face_arrays(s.populations(), W, H, 1, 6)
    assert np.array_equal(host[0], lo) and np.array_equal(host[1], hi)
    for p in bufs:
        L.lb_free(p)
    s.close()


def test_slab_refuses_what_it_cannot_do(pkg):
    L = pkg.lib()
    s = pkg.slab.Slab(W, H, D, 0, 4)
    assert L.lb_step(s.h, 1) == pkg.abi.LB_ERR_STATE
    s.close()
    with pytest.raises(pkg.LBError):
        pkg.slab.Slab(W, H, D, 10, 9)  # past the global lattice


def test_slab_rank_torch_transport_single_rank(pkg, oracle):
    """The multi-process driver (SlabRank: faces in torch CUDA tensors, moved
    on the slab's own stream wrapped as a torch ExternalStream) with one rank,
    whose slab is its own z-neighbour: the exchange is then a local tensor
    copy, and everything else -- the library stream seen by torch, torch
    device buffers handed to lb_slab_step / lb_slab_unpack -- is the path the
    NCCL ranks take."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA")
    fl, f = setup(pkg, oracle, seed=12)
    steps = 7
    f_ref, mom_ref, _ = whole(pkg, fl, f, steps)
    (s,) = make_slabs(pkg, fl, f, [(0, D)])
    S = pkg.slab
    sr = S.SlabRank(s, S.SlabExchange(None, 0, 1))
    sr.refresh_ghosts()
    sr.step(steps)
    s.synchronize()
    got, mom = gather([s])
    assert np.array_equal(got.view(np.uint32), f_ref.view(np.uint32))
    assert np.array_equal(mom[0].view(np.uint32), mom_ref[0].view(np.uint32))
    s.close()
