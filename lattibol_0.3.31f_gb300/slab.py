"""z-slab decomposition of one D3Q19 lattice (include/lbgb300.h, part 7).

The reference splits its lattice into x-slabs, one per device, and exchanges
the faces every step with get_border -> copy_border -> apply_border
(reference src/get_border.cu:59-98, src/copy_border.cu:49-81,
src/apply_border.cu:58-97, driven from src/simulation_d3q19.cu:363-406).
Here the cut is along z, so each of the 5 populations crossing a face is one
contiguous plane:

* ``Slab`` -- one slab context (lb_slab_create): own planes z0 .. z0+nz-1
  plus a ghost plane on each side; every per-node array covers nz + 2 planes.
* ``SlabGroup`` -- all slabs of a lattice held by this process on one
  device, stepped with lb_slab_group_step (faces moved by device copies).
* ``SlabExchange`` -- the host logic of the multi-process form: each rank
  holds one slab and moves its two faces to its z-neighbours with
  torch.distributed point-to-point operations (NCCL between GPUs; gloo on
  CPU tensors for the tests of this logic).

Every slab step is bit-identical to the same step of one context over the
whole lattice.
"""
import ctypes

import numpy as np

from . import abi
from .lattice import LBError, Lattice, _lib


def slab_bounds(nz_global, parts):
    """(z0, nz) of `parts` slabs covering nz_global planes, sizes differing by
    at most one plane (the larger ones first)."""
    if not 1 <= parts <= nz_global:
        raise ValueError("need 1 <= parts <= nz_global")
    base, extra = divmod(nz_global, parts)
    out, z0 = [], 0
    for i in range(parts):
        nz = base + (1 if i < extra else 0)
        out.append((z0, nz))
        z0 += nz
    return out


def slab_planes(z0, nz, nz_global):
    """Global plane indices of a slab's nz + 2 planes (ghosts included),
    periodic in z."""
    return [(z0 - 1 + i) % nz_global for i in range(nz + 2)]


class Slab(Lattice):
    """One z-slab of a D3Q19 native-mode lattice (no Shan-Chen).  Arrays given
    to or taken from it (flags, populations, moments) cover its nz + 2 planes:
    the ghost plane below, the own planes, the ghost plane above."""

    def __init__(self, nx, ny, nz_global, z0, nz, tau_inv=1.0, force=(0, 0, 0),
                 wall_u=(0, 0, 0), storage=abi.LB_STORE_F32, rho_ref=0.0, graph_steps=64):
        L = _lib()
        cfg = abi.lb_config()
        L.lb_config_default(ctypes.byref(cfg), 19, nx, ny, nz_global)
        cfg.mode, cfg.tau_inv, cfg.storage, cfg.rho_ref = abi.LB_MODE_NATIVE, tau_inv, storage, rho_ref
        cfg.graph_steps = graph_steps  # lb_slab_group_step: steps per captured graph
        for i in range(3):
            cfg.force[i], cfg.wall_u[i] = force[i], wall_u[i]
        h = ctypes.c_void_p()
        rc = L.lb_slab_create(ctypes.byref(cfg), int(z0), int(nz), ctypes.byref(h))
        if rc != abi.LB_OK:
            raise LBError("lb_slab_create failed (%d): %s" % (rc, L.lb_abi_last_error().decode()))
        self.h = h
        self.cfg = cfg
        self.Q = 19
        self.z0, self.nz, self.nz_global = int(z0), int(nz), int(nz_global)
        self.shape = (nx, ny, nz + 2)
        self.N = nx * ny * (nz + 2)
        fb = ctypes.c_size_t()
        self._check(L.lb_slab_info(h, None, None, None, ctypes.byref(fb)), "lb_slab_info")
        self.face_bytes = fb.value

    def planes(self):
        return slab_planes(self.z0, self.nz, self.nz_global)

    def own(self, a):
        """The own planes of a per-node array of this slab (..., nz+2 planes)."""
        plane = self.shape[0] * self.shape[1]
        return a[..., plane:plane * (self.nz + 1)]

    def stream(self):
        """The context's CUDA stream (cudaStream_t as an int) for an external
        transport."""
        return _lib().lb_stream(self.h) or 0

    def pack(self, to_below, to_above):
        self._check(_lib().lb_slab_pack(self.h, to_below, to_above), "lb_slab_pack")

    def step_slab(self, moments, to_below, to_above):
        self._check(_lib().lb_slab_step(self.h, int(moments), to_below, to_above), "lb_slab_step")

    def unpack(self, from_below, from_above):
        self._check(_lib().lb_slab_unpack(self.h, from_below, from_above), "lb_slab_unpack")


class SlabGroup:
    """All slabs of one lattice in this process, on the current device, in z
    order (periodic)."""

    def __init__(self, slabs):
        self.slabs = list(slabs)
        self._arr = (ctypes.c_void_p * len(self.slabs))(*[s.h.value for s in self.slabs])

    def step(self, n=1):
        rc = _lib().lb_slab_group_step(self._arr, len(self.slabs), int(n))
        if rc != abi.LB_OK:
            raise LBError("lb_slab_group_step failed (%d): %s"
                          % (rc, _lib().lb_abi_last_error().decode()))

    def time_steps(self, n):
        """n steps timed on the device (ms)."""
        ms = ctypes.c_float()
        rc = _lib().lb_slab_group_time(self._arr, len(self.slabs), int(n), ctypes.byref(ms))
        if rc != abi.LB_OK:
            raise LBError("lb_slab_group_time failed (%d): %s"
                          % (rc, _lib().lb_abi_last_error().decode()))
        return ms.value

    def launches(self):
        return sum(s.launches() for s in self.slabs)

    def synchronize(self):
        for s in self.slabs:
            s.synchronize()


class SlabExchange:
    """Moves a slab's two faces to its z-neighbours, one slab per rank,
    periodic in z (rank r's lower neighbour is r - 1, its upper r + 1).

    Each rank posts, in this order: send to_below -> lower rank, send to_above
    -> upper rank, receive from_above <- upper rank, receive from_below <-
    lower rank.  With two ranks both neighbours are the same rank and the two
    messages between them are told apart by their order (NCCL matches
    point-to-point operations between a pair of ranks in order) and by their
    tags (gloo): tag 0 for faces moving down, 1 for faces moving up.  With one
    rank the slab is its own neighbour and the faces are copied locally."""

    DOWN, UP = 0, 1

    def __init__(self, dist, rank, world):
        self.dist, self.rank, self.world = dist, rank, world
        self.lower = (rank - 1) % world
        self.upper = (rank + 1) % world

    def ops(self, to_below, to_above, from_below, from_above):
        """The point-to-point operations of one exchange, in posting order."""
        d = self.dist
        return [d.P2POp(d.isend, to_below, self.lower, tag=self.DOWN),
                d.P2POp(d.isend, to_above, self.upper, tag=self.UP),
                d.P2POp(d.irecv, from_above, self.upper, tag=self.DOWN),
                d.P2POp(d.irecv, from_below, self.lower, tag=self.UP)]

    def exchange(self, to_below, to_above, from_below, from_above):
        """Blocking for gloo; for NCCL the operations are queued on the
        current CUDA stream (wrap the slab's stream with
        torch.cuda.ExternalStream and make it current first)."""
        if self.world == 1:
            from_below.copy_(to_above)
            from_above.copy_(to_below)
            return
        for w in self.dist.batch_isend_irecv(self.ops(to_below, to_above, from_below, from_above)):
            w.wait()


class SlabRank:
    """One rank's slab of a lattice stepped with SlabExchange over NCCL: the
    faces travel in torch CUDA tensors on the slab's own stream."""

    def __init__(self, slab, exchange):
        import torch
        self.torch = torch
        self.slab, self.ex = slab, exchange
        n = slab.face_bytes
        dev = torch.device("cuda", torch.cuda.current_device())
        self.buf = [torch.empty(n, dtype=torch.uint8, device=dev) for _ in range(4)]
        self.stream = torch.cuda.ExternalStream(slab.stream(), device=dev)

    def _ptrs(self):
        return [ctypes.c_void_p(b.data_ptr()) for b in self.buf]

    def refresh_ghosts(self):
        """Ghost planes from the neighbours' current faces (before the first
        step when the state was set slab by slab)."""
        tb, ta, fb, fa = self._ptrs()
        self.slab.pack(tb, ta)
        self._move()
        self.slab.unpack(fb, fa)

    def _move(self):
        with self.torch.cuda.stream(self.stream):
            self.ex.exchange(self.buf[0], self.buf[1], self.buf[2], self.buf[3])

    def step(self, n=1, moments_last=True):
        tb, ta, fb, fa = self._ptrs()
        for i in range(n):
            self.slab.step_slab(moments_last and i == n - 1, tb, ta)
            self._move()
            self.slab.unpack(fb, fa)


def face_arrays(f, nx, ny, plane_lo, plane_hi):
    """Host restatement of the packed faces of a population array f[19, nodes]
    (used by the tests): the c_z = -1 populations of plane plane_lo and the
    c_z = +1 populations of plane plane_hi, each [5, nx*ny]."""
    P = nx * ny
    down = [6, 10, 14, 16, 18]
    up = [5, 9, 13, 15, 17]
    lo = np.stack([f[k, plane_lo * P:(plane_lo + 1) * P] for k in down])
    hi = np.stack([f[k, plane_hi * P:(plane_hi + 1) * P] for k in up])
    return lo, hi


def write_ghosts(f, nx, ny, nz_own, from_below, from_above):
    """Host restatement of lb_slab_unpack on f[19, (nz_own + 2) * nx * ny]."""
    P = nx * ny
    down = [6, 10, 14, 16, 18]
    up = [5, 9, 13, 15, 17]
    for i, k in enumerate(up):
        f[k, 0:P] = from_below[i]
    top = (nz_own + 1) * P
    for i, k in enumerate(down):
        f[k, top:top + P] = from_above[i]

