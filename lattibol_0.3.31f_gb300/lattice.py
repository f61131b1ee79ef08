"""Python mirror of the library's host interfaces.

``Lattice`` wraps the context API (lb_create / lb_step / ...) with numpy
arrays.  ``DeviceData`` allocates the reference's per-device struct
(DataD2Q9 / DataD3Q19) on the GPU the way the reference's Simulation
constructors do (reference src/simulation_d3q19.cu:206-289,
src/simulation_d2q9.cu:336-390), so that the drop-in entry points can be
driven exactly like the reference's runLBM drives them.
"""
import ctypes
import os

import numpy as np

from . import abi

W3 = (np.float32(12. / 36.), np.float32(2. / 36.), np.float32(1. / 36.))
W2 = (np.float32(16. / 36.), np.float32(4. / 36.), np.float32(1. / 36.))


class LBError(RuntimeError):
    pass


def _lib():
    from . import lib
    return lib()


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Lattice:
    """One lattice on the GPU (context API).  Populations are exchanged as
    float32 arrays of shape (Q, N), node = x + nx*(y + ny*z)."""

    def __init__(self, lattice, nx, ny, nz=1, mode=abi.LB_MODE_NATIVE, tau_inv=1.0,
                 force=(0, 0, 0), u_in=(0, 0, 0), rho_out=1.0, wall_u=(0, 0, 0), G=0.0,
                 G_ads=0.0, psi_form=abi.LB_PSI_EXP1, graph_steps=64,
                 storage=abi.LB_STORE_F32, tuning=abi.LB_TUNE_DEFAULT, rho_ref=0.0):
        L = _lib()
        cfg = abi.lb_config()
        L.lb_config_default(ctypes.byref(cfg), lattice, nx, ny, nz)
        cfg.mode, cfg.tau_inv, cfg.rho_out = mode, tau_inv, rho_out
        cfg.storage = storage
        for i in range(3):
            cfg.force[i], cfg.u_in[i], cfg.wall_u[i] = force[i], u_in[i], wall_u[i]
        cfg.G, cfg.G_ads, cfg.psi_form, cfg.graph_steps = G, G_ads, psi_form, graph_steps
        cfg.tuning = tuning
        cfg.rho_ref = rho_ref
        self.cfg = cfg
        self.Q = lattice
        self.shape = (nx, ny, nz if lattice == 19 else 1)
        self.N = nx * ny * self.shape[2]
        h = ctypes.c_void_p()
        rc = L.lb_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != abi.LB_OK:
            raise LBError("lb_create failed: %d" % rc)
        self.h = h

    def _check(self, rc, what):
        if rc != abi.LB_OK:
            raise LBError("%s: %d %s" % (what, rc, _lib().lb_error(self.h).decode()))

    def close(self):
        if self.h:
            _lib().lb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_flags(self, flags):
        f = np.ascontiguousarray(flags, np.uint8).reshape(-1)
        assert f.size == self.N
        self._check(_lib().lb_set_flags(self.h, _ptr(f)), "lb_set_flags")

    def set_populations(self, f):
        f = np.ascontiguousarray(f, np.float32)
        assert f.size == self.Q * self.N
        self._check(_lib().lb_set_populations(self.h, _ptr(f)), "lb_set_populations")

    def populations(self):
        f = np.empty((self.Q, self.N), np.float32)
        self._check(_lib().lb_get_populations(self.h, _ptr(f)), "lb_get_populations")
        return f

    def init_equilibrium(self, rho=None, ux=None, uy=None, uz=None):
        args = [None if a is None else np.ascontiguousarray(a, np.float32).reshape(-1)
                for a in (rho, ux, uy, uz)]
        self._keep = args
        self._check(_lib().lb_init_equilibrium(self.h, *[None if a is None else _ptr(a)
                                                         for a in args]), "lb_init_equilibrium")

    def step(self, n=1):
        self._check(_lib().lb_step(self.h, int(n)), "lb_step")

    def synchronize(self):
        self._check(_lib().lb_synchronize(self.h), "lb_synchronize")

    def time_steps(self, n):
        ms = ctypes.c_float()
        self._check(_lib().lb_time_steps(self.h, int(n), ctypes.byref(ms)), "lb_time_steps")
        return ms.value

    def moments(self):
        """(rho, ux, uy, uz) of the last step (uz is None for D2Q9)."""
        out = [np.empty(self.N, np.float32) for _ in range(4 if self.Q == 19 else 3)]
        ptrs = [_ptr(a) for a in out] + ([None] if self.Q == 9 else [])
        self._check(_lib().lb_get_moments(self.h, *ptrs), "lb_get_moments")
        return tuple(out) + ((None,) if self.Q == 9 else ())

    def reduce(self):
        out = (ctypes.c_double * 7)()
        self._check(_lib().lb_reduce(self.h, out), "lb_reduce")
        return np.array(out[:])

    def launches(self):
        return _lib().lb_launch_count(self.h)

    def wall_correction(self):
        c = np.zeros(self.Q, np.float32)
        self._check(_lib().lb_wall_correction(self.h, _ptr(c)), "lb_wall_correction")
        return c

    def steps_done(self):
        return _lib().lb_steps_done(self.h)

    def save_checkpoint(self, path):
        self._check(_lib().lb_checkpoint_save(self.h, os.fsencode(path)), "lb_checkpoint_save")

    def load_checkpoint(self, path):
        """Restore a checkpoint; returns the library status (LB_ERR_ARG for a
        checkpoint of another lattice, LB_ERR_IO for a damaged file)."""
        return _lib().lb_checkpoint_load(self.h, os.fsencode(path))

    def save_vtk(self, directory, vtk_id):
        self._check(_lib().lb_vtk_save_ctx(self.h, os.fsencode(directory), int(vtk_id)),
                    "lb_vtk_save_ctx")

    @classmethod
    def from_checkpoint(cls, path):
        """A new lattice with the configuration and state of a checkpoint."""
        L = _lib()
        h = ctypes.c_void_p()
        rc = L.lb_checkpoint_create(os.fsencode(path), ctypes.byref(h))
        if rc != abi.LB_OK:
            raise LBError("lb_checkpoint_create failed (%d): %s"
                          % (rc, L.lb_abi_last_error().decode()))
        self = cls.__new__(cls)
        cfg = abi.lb_config()
        L.lb_checkpoint_info(os.fsencode(path), ctypes.byref(cfg), None)
        self.cfg = cfg
        self.Q = cfg.lattice
        self.shape = (cfg.nx, cfg.ny, cfg.nz if cfg.lattice == 19 else 1)
        self.N = cfg.nx * cfg.ny * self.shape[2]
        self.h = h
        return self


def sc_coexistence(G, n=4000):
    """Liquid and vapour densities of the Shan-Chen fluid with psi = 1-exp(-rho)
    (pressure p = rho/3 + G psi^2 / 6) at coexistence, from the mechanical
    stability condition of Shan & Chen: p(rho_v) = p(rho_l) = p0 and
    integral_{rho_v}^{rho_l} (p0 - p) psi'/psi^2 drho = 0, solved for p0 by
    bisection between the spinodal pressures."""
    G = float(G)
    rho = np.linspace(1e-3, 6.0, 24001)
    psi = 1 - np.exp(-rho)
    p = rho / 3 + G * psi ** 2 / 6
    dp = np.gradient(p, rho)
    neg = np.where(dp < 0)[0]
    if len(neg) == 0:
        raise ValueError("G = %g is above the critical coupling (no coexistence)" % G)
    i_max, i_min = neg[0], neg[-1]  # local maximum and minimum of p(rho)
    p_hi, p_lo = p[i_max], p[i_min]

    def roots(p0):
        rv = np.interp(p0, p[:i_max + 1], rho[:i_max + 1])            # p rising on [0, i_max]
        rl = np.interp(p0, p[i_min:], rho[i_min:])                     # p rising after i_min
        return rv, rl

    def excess(p0):
        rv, rl = roots(p0)
        r = np.linspace(rv, rl, n)
        s = 1 - np.exp(-r)
        integrand = (p0 - (r / 3 + G * s ** 2 / 6)) * np.exp(-r) / s ** 2
        return float(np.sum((integrand[1:] + integrand[:-1]) * np.diff(r)) / 2)

    # excess grows with p0: a positive excess means p0 is above coexistence
    lo, hi = max(p_lo, p[0]), p_hi
    for _ in range(80):
        mid = 0.5 * (lo + hi)
        if excess(mid) > 0:
            hi = mid
        else:
            lo = mid
    return roots(0.5 * (lo + hi))[::-1]  # (rho_liquid, rho_vapour)


def droplet_ensemble(ndomains, seed=4, side_choices=None, width=2.0, densities="coexistence"):
    """Seeded droplet ensemble: side lengths uniform over the multiples of 32
    in [64, 512], G ~ U[-5.5, -4.5], one centred droplet of radius
    U[0.1, 0.3]*side (interface smoothed by tanh over `width` nodes).
    densities = (rho_liquid, rho_vapour) for every domain, or "coexistence":
    each domain starts at the coexistence pair of its own G (sc_coexistence).
    Returns (nx, ny, G, packed rho)."""
    rng = np.random.default_rng(seed)
    sides = np.asarray(side_choices if side_choices is not None else np.arange(64, 513, 32))
    nx = rng.choice(sides, ndomains).astype(np.int32)
    ny = nx.copy()
    G = rng.uniform(-5.5, -4.5, ndomains).astype(np.float32)
    frac = rng.uniform(0.1, 0.3, ndomains)
    rhos = []
    for d in range(ndomains):
        n = int(nx[d])
        rl, rv = sc_coexistence(G[d]) if densities == "coexistence" else densities
        y, x = np.mgrid[0:n, 0:n]
        r = np.sqrt((x - (n - 1) / 2.0) ** 2 + (y - (n - 1) / 2.0) ** 2)
        R = frac[d] * n
        rho = 0.5 * (rl + rv) - 0.5 * (rl - rv) * np.tanh((r - R) / width)
        rhos.append(rho.astype(np.float32).reshape(-1))
    return nx, ny, G, np.concatenate(rhos)


class Ensemble:
    """Independent periodic D2Q9 Shan-Chen domains advanced together
    (lb_ensemble_* of the C ABI)."""

    def __init__(self, nx, ny, G, tau_inv=None, psi_form=abi.LB_PSI_EXP1):
        L = _lib()
        self.nx = np.ascontiguousarray(nx, np.int32)
        self.ny = np.ascontiguousarray(ny, np.int32)
        self.G = np.ascontiguousarray(G, np.float32)
        nd = len(self.nx)
        self.tau_inv = np.ascontiguousarray(np.ones(nd) if tau_inv is None else tau_inv,
                                            np.float32)
        h = ctypes.c_void_p()
        rc = L.lb_ensemble_create(nd, _ptr(self.nx), _ptr(self.ny), _ptr(self.G),
                                  _ptr(self.tau_inv), psi_form, ctypes.byref(h))
        if rc != abi.LB_OK:
            raise LBError("lb_ensemble_create failed: %d" % rc)
        self.h = h
        self.NT = L.lb_ensemble_nodes(h)
        self.offsets = [L.lb_ensemble_offset(h, d) for d in range(nd)]

    def _check(self, rc, what):
        if rc != abi.LB_OK:
            raise LBError("%s: %d %s" % (what, rc, _lib().lb_ensemble_error(self.h).decode()))

    def close(self):
        if self.h:
            _lib().lb_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_equilibrium(self, rho):
        rho = np.ascontiguousarray(rho, np.float32)
        self._check(_lib().lb_ensemble_init_equilibrium(self.h, _ptr(rho)), "init")

    def set_populations(self, f):
        f = np.ascontiguousarray(f, np.float32)
        self._check(_lib().lb_ensemble_set_populations(self.h, _ptr(f)), "set_populations")

    def populations(self):
        f = np.empty((9, self.NT), np.float32)
        self._check(_lib().lb_ensemble_get_populations(self.h, _ptr(f)), "get_populations")
        return f

    def step(self, n):
        self._check(_lib().lb_ensemble_step(self.h, int(n)), "step")

    def time_steps(self, n):
        ms = ctypes.c_float()
        self._check(_lib().lb_ensemble_time_steps(self.h, int(n), ctypes.byref(ms)), "time")
        return ms.value

    def moments(self):
        out = [np.empty(self.NT, np.float32) for _ in range(3)]
        self._check(_lib().lb_ensemble_get_moments(self.h, *[_ptr(a) for a in out]), "moments")
        return tuple(out)

    def set_launch(self, threads_x, rows, blocks_per_sm):
        self._check(_lib().lb_ensemble_set_launch(self.h, threads_x, rows, blocks_per_sm),
                    "set_launch")

    def autotune(self, trial_steps=3):
        out = np.zeros(3, np.int32)
        self._check(_lib().lb_ensemble_autotune(self.h, trial_steps, _ptr(out)), "autotune")
        return tuple(int(v) for v in out)

    def launches(self):
        return _lib().lb_ensemble_launch_count(self.h)

    def domain(self, arr, d):
        """The slice of a packed per-node array belonging to domain d."""
        o = self.offsets[d]
        return arr[..., o:o + int(self.nx[d]) * int(self.ny[d])]


class DeviceData:
    """The reference's per-device struct with every array on the GPU.

    lattice = 9 or 19; arrays are allocated with lb_malloc and freed by
    close().  ``upload``/``download`` move (Q, N) population arrays."""

    def __init__(self, lattice, W, H, D=1, plot=True):
        self.L = _lib()
        self.Q = lattice
        self.W, self.H, self.D = W, H, (D if lattice == 19 else 1)
        self.N = W * H * self.D
        self.s = abi.DataD3Q19() if lattice == 19 else abi.DataD2Q9()
        self._bufs = []
        N = self.N
        face = H * self.D
        names_f = self.s.POP
        for n in names_f:
            setattr(self.s, n, self._alloc(4 * N))
        mom = ["ux", "uy", "uz", "rho"] if lattice == 19 else ["ux", "uy", "rho", "psi", "ueq_x",
                                                               "ueq_y"]
        for n in mom:
            setattr(self.s, n, self._alloc(4 * N))
        self.s.solid = self._alloc(N)
        self.s.solid_bound = self._alloc(N)
        for n in self.s.BORDER + self.s.NB_BORDER:
            setattr(self.s, n, self._alloc(4 * face))
        self.s.valueCur = self._alloc(16)
        self.s.width, self.s.height = W, H
        if lattice == 19:
            self.s.depth = self.D
        self.s.deviceCount, self.s.dev = 1, 0
        self.plot = self._alloc(16 * N) if plot else None
        self.orig = [getattr(self.s, n) for n in names_f]

    def _alloc(self, nbytes):
        p = ctypes.c_void_p()
        if self.L.lb_malloc(ctypes.byref(p), nbytes) != abi.LB_OK:
            raise LBError("lb_malloc(%d) failed" % nbytes)
        self.L.lb_memset(p, 0, nbytes)
        self._bufs.append(p.value)
        return p.value

    def close(self):
        if getattr(self, "_bufs", None) is not None:
            if self.Q == 19:
                self.L.lb_abi_release_d3q19(ctypes.byref(self.s))
            else:
                self.L.lb_abi_release_d2q9(ctypes.byref(self.s))
            for p in self._bufs:
                self.L.lb_free(ctypes.c_void_p(p))
            self._bufs = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def h2d(self, dev_ptr, arr):
        arr = np.ascontiguousarray(arr)
        rc = self.L.lb_memcpy_h2d(ctypes.c_void_p(dev_ptr), _ptr(arr), arr.nbytes)
        if rc != abi.LB_OK:
            raise LBError("lb_memcpy_h2d failed")

    def d2h(self, dev_ptr, shape, dtype=np.float32):
        out = np.empty(shape, dtype)
        rc = self.L.lb_memcpy_d2h(_ptr(out), ctypes.c_void_p(dev_ptr), out.nbytes)
        if rc != abi.LB_OK:
            raise LBError("lb_memcpy_d2h failed")
        return out

    def upload(self, f):
        for k, n in enumerate(self.s.POP):
            self.h2d(getattr(self.s, n), np.asarray(f[k], np.float32))

    def download(self):
        return np.stack([self.d2h(getattr(self.s, n), self.N) for n in self.s.POP])

    def set_solid(self, solid, solid_bound):
        self.h2d(self.s.solid, np.ascontiguousarray(solid, np.uint8))
        self.h2d(self.s.solid_bound, np.ascontiguousarray(solid_bound, np.uint8))

    def field(self, name):
        return self.d2h(getattr(self.s, name), self.N)

    def plot_data(self):
        return self.d2h(self.plot, 4 * self.N)

    def ptr(self):
        return ctypes.byref(self.s)
