"""Host logic of the multi-process z-slab exchange on CPU (gloo, world sizes 2
and 3), with the oracle standing in for each rank's slab step.

Each rank holds planes z0 .. z0+nz-1 of a D3Q19 lattice (walls, a moving
wall, a solid block that crosses slab boundaries, a body force; periodic in
z, so the last rank's upper neighbour is rank 0) plus one ghost plane on each
side.  Per step it runs the oracle's native stream + collide on its nz + 2
planes, packs the c_z = -1 populations of its first plane and the c_z = +1
populations of its last one (the faces lb_slab_step packs), moves them with
SlabExchange over gloo and writes the received faces into its ghost planes
(what lb_slab_unpack does).  The own planes gathered from all ranks must
equal the oracle's run over the whole lattice bit for bit.
"""
import os
import socket
import sys

import numpy as np
import pytest

from conftest import ROOT, load_package

W, H, D = 12, 10, 9
STEPS = 6


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def lattice_setup():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import lb_oracle as orc
    fl = np.zeros((D, H, W), np.uint8)
    fl[:, 0, :] = 1
    fl[:, H - 1, :] = 3  # moving wall
    fl[2:6, 4:7, 3:6] = 1  # a block crossing the slab boundaries
    fl = fl.reshape(-1)
    rng = np.random.default_rng(11)
    N = W * H * D
    rho = (1 + 0.02 * rng.standard_normal(N)).astype(np.float32)
    ux = (0.03 * rng.standard_normal(N)).astype(np.float32)
    uy = (0.03 * rng.standard_normal(N)).astype(np.float32)
    uz = (0.03 * rng.standard_normal(N)).astype(np.float32)
    w = tuple(np.float32(v) for v in (12 / 36, 2 / 36, 1 / 36))
    f = orc.d3q19_equilibrium(rho, ux, uy, uz, *w)
    corr = orc.wall_correction(19, (0.04, 0, 0.01))
    phys = dict(w=w, tau_inv=np.float32(1 / 0.6),
                F=(np.float32(2e-5), np.float32(0), np.float32(-1e-5)))
    return orc, fl, f, corr, phys


def oracle_step(orc, f, fl, corr, phys, d):
    orc.d3q19_stream_native(f, fl, corr, W, H, d)
    orc.d3q19_collide_native(f, fl, None, W, H, d, *phys["w"], phys["tau_inv"], phys["F"])


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch
    import torch.distributed as dist
    from conftest import load_package as lp
    S = lp().slab
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    orc, fl, f0, corr, phys = lattice_setup()
    P = W * H
    z0, nz = S.slab_bounds(D, ws)[rank]
    planes = S.slab_planes(z0, nz, D)
    f = np.ascontiguousarray(f0.reshape(19, D, P)[:, planes].reshape(19, -1))
    sfl = np.ascontiguousarray(fl.reshape(D, P)[planes].reshape(-1))
    ex = S.SlabExchange(dist, rank, ws)
    for _ in range(STEPS):
        oracle_step(orc, f, sfl, corr, phys, nz + 2)
        lo, hi = S.face_arrays(f, W, H, 1, nz)
        to_below, to_above = torch.from_numpy(lo.copy()), torch.from_numpy(hi.copy())
        from_below, from_above = torch.empty_like(to_above), torch.empty_like(to_below)
        ex.exchange(to_below, to_above, from_below, from_above)
        S.write_ghosts(f, W, H, nz, from_below.numpy(), from_above.numpy())
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, z0, nz, f[:, P:P * (nz + 1)].copy()))


@pytest.mark.parametrize("ws", [2, 3])
def test_slab_exchange_gloo_matches_whole_lattice(ws, oracle):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    parts = [q.get(timeout=300) for _ in range(ws)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    orc, fl, f, corr, phys = lattice_setup()
    for _ in range(STEPS):
        oracle_step(orc, f, fl, corr, phys, D)
    P = W * H
    got = np.zeros_like(f)
    covered = np.zeros(D, bool)
    for rank, z0, nz, own in parts:
        got[:, z0 * P:(z0 + nz) * P] = own
        covered[z0:z0 + nz] = True
    assert covered.all()
    assert np.array_equal(got.view(np.uint32), f.view(np.uint32))


def test_slab_exchange_single_rank_wraps_onto_itself(oracle):
    """World size 1: the slab is its own z-neighbour; the exchange is a local
    copy and the slab run equals the whole-lattice run."""
    torch = pytest.importorskip("torch")
    S = load_package().slab
    orc, fl, f0, corr, phys = lattice_setup()
    P = W * H
    planes = S.slab_planes(0, D, D)
    f = np.ascontiguousarray(f0.reshape(19, D, P)[:, planes].reshape(19, -1))
    sfl = np.ascontiguousarray(fl.reshape(D, P)[planes].reshape(-1))
    ex = S.SlabExchange(None, 0, 1)
    ref = f0.copy()
    for _ in range(STEPS):
        oracle_step(orc, f, sfl, corr, phys, D + 2)
        lo, hi = S.face_arrays(f, W, H, 1, D)
        fb, fa = torch.empty(hi.shape, dtype=torch.float32), torch.empty(lo.shape, dtype=torch.float32)
        ex.exchange(torch.from_numpy(lo.copy()), torch.from_numpy(hi.copy()), fb, fa)
        S.write_ghosts(f, W, H, D, fb.numpy(), fa.numpy())
        oracle_step(orc, ref, fl, corr, phys, D)
    assert np.array_equal(f[:, P:P * (D + 1)].view(np.uint32), ref.view(np.uint32))


def test_slab_bounds_cover_the_lattice():
    S = load_package().slab
    for nzg in (1, 5, 9, 128):
        for parts in range(1, min(nzg, 8) + 1):
            b = S.slab_bounds(nzg, parts)
            assert b[0][0] == 0 and sum(n for _, n in b) == nzg
            assert all(b[i][0] + b[i][1] == b[i + 1][0] for i in range(parts - 1))
            assert max(n for _, n in b) - min(n for _, n in b) <= 1
    assert S.slab_planes(0, 3, 9) == [8, 0, 1, 2, 3]
    assert S.slab_planes(6, 3, 9) == [5, 6, 7, 8, 0]
