"""Learned sub-grid closure for under-resolved D3Q19 flow (host side).

Taylor-Green vortex u = U0 sin x cos y cos z, v = -U0 cos x sin y cos z,
w = 0 on a periodic box of N nodes (x = (i + 1/2) 2 pi / N), Re = U0 L / nu
with L = N / (2 pi).  A fine run (N_f) is box-filtered by `factor` onto the
coarse grid (N_c = N_f / factor): its filtered fields give the training data
of the closure network (features and eddy-viscosity targets, built on the GPU
by lb_closure_sample) and the reference kinetic-energy decay.  Coarse runs
at the same Re compare plain BGK (the fallback) with the trained closure.

Everything runs on the GPU through the C ABI; numpy only moves arrays.
"""
import ctypes
import time

import numpy as np

from . import abi
from .lattice import LBError, Lattice, _lib, _ptr


class DeviceArray:
    """A float32 device buffer (lb_malloc)."""

    def __init__(self, n):
        self.n = int(n)
        p = ctypes.c_void_p()
        if _lib().lb_malloc(ctypes.byref(p), 4 * max(self.n, 1)) != abi.LB_OK:
            raise LBError("lb_malloc(%d floats) failed" % self.n)
        self.ptr = p

    def upload(self, a):
        a = np.ascontiguousarray(a, np.float32).reshape(-1)
        assert a.size <= self.n
        _lib().lb_memcpy_h2d(self.ptr, _ptr(a), a.nbytes)

    def download(self, n=None):
        out = np.empty(self.n if n is None else n, np.float32)
        _lib().lb_memcpy_d2h(_ptr(out), self.ptr, out.nbytes)
        return out

    def offset(self, i):
        return ctypes.c_void_p(self.ptr.value + 4 * int(i))

    def free(self):
        if self.ptr:
            _lib().lb_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Mlp:
    """The closure network on the GPU (lb_mlp_*)."""

    N_IN = 19

    def __init__(self, seed=1):
        h = ctypes.c_void_p()
        rc = _lib().lb_mlp_create(seed, ctypes.byref(h))
        if rc != abi.LB_OK:
            raise LBError("lb_mlp_create: %d" % rc)
        self.h = h
        self.nparam = _lib().lb_mlp_num_params()

    def _check(self, rc, what):
        if rc != abi.LB_OK:
            raise LBError("%s: %d %s" % (what, rc, _lib().lb_mlp_error(self.h).decode()))

    def params(self):
        p = np.empty(self.nparam, np.float32)
        self._check(_lib().lb_mlp_get_params(self.h, _ptr(p)), "get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        self._check(_lib().lb_mlp_set_params(self.h, _ptr(p)), "set_params")

    def forward(self, X):
        X = np.ascontiguousarray(X, np.float32)
        n = len(X)
        dx, dy = DeviceArray(n * self.N_IN), DeviceArray(n)
        dx.upload(X)
        self._check(_lib().lb_mlp_forward(self.h, dx.ptr, dy.ptr, n), "forward")
        return dy.download()

    def grad(self, X, Z):
        X = np.ascontiguousarray(X, np.float32)
        n = len(X)
        dx, dz = DeviceArray(n * self.N_IN), DeviceArray(n)
        dx.upload(X)
        dz.upload(Z)
        g = np.empty(self.nparam, np.float32)
        loss = ctypes.c_double()
        self._check(_lib().lb_mlp_grad(self.h, dx.ptr, dz.ptr, n, _ptr(g), ctypes.byref(loss)),
                    "grad")
        return g, loss.value

    def train_device(self, dx, dz, n, steps, batch, lr, seed=7):
        log = np.zeros(steps, np.float32)
        self._check(_lib().lb_mlp_train(self.h, dx.ptr, dz.ptr, n, steps, batch, lr, seed,
                                        _ptr(log)), "train")
        return log

    def close(self):
        if self.h:
            _lib().lb_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tgv_fields(n, U0):
    """Taylor-Green initial velocity and density (pressure) fields, nodes at
    (i + 1/2) 2 pi / n, flattened x-fastest."""
    x = (np.arange(n) + 0.5) * 2 * np.pi / n
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    ux = U0 * np.sin(X) * np.cos(Y) * np.cos(Z)
    uy = -U0 * np.cos(X) * np.sin(Y) * np.cos(Z)
    p = (U0 ** 2 / 16) * (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2)
    rho = 1 + 3 * p
    f = lambda a: np.ascontiguousarray(a.reshape(-1), np.float32)  # noqa: E731
    return f(rho), f(ux), f(uy), f(np.zeros_like(ux))


def viscosity(n, U0, Re):
    return U0 * (n / (2 * np.pi)) / Re


def ke_mean(lat):
    rho, ux, uy, uz = lat.moments()
    return float(np.mean(0.5 * rho.astype(np.float64) * (ux.astype(np.float64) ** 2 + uy ** 2
                                                          + uz ** 2)))


class FineRun:
    """The fine Taylor-Green run: filtered kinetic energy at every sample and
    training data at the requested samples (device arrays)."""

    def __init__(self, n_fine, factor, U0, Re, z_max=200.0):
        self.nf, self.fac, self.U0, self.Re = n_fine, factor, U0, Re
        self.nc = n_fine // factor
        self.nu_f = viscosity(n_fine, U0, Re)
        self.nu_c = viscosity(self.nc, U0, Re)
        self.s_ref = U0 * 2 * np.pi / self.nc
        self.z_max = z_max
        self.lat = Lattice(19, n_fine, n_fine, n_fine,
                           tau_inv=np.float32(1 / (0.5 + 3 * self.nu_f)))
        self.lat.set_flags(np.zeros(n_fine ** 3, np.uint8))
        rho, ux, uy, uz = tgv_fields(n_fine, U0)
        self.lat.init_equilibrium(rho, ux, uy, uz)
        self.steps = 0
        self.seconds = 0.0

    def advance(self, fine_steps):
        if fine_steps > 0:
            t0 = time.perf_counter()
            self.lat.step(fine_steps)
            self.lat.synchronize()
            self.seconds += time.perf_counter() - t0
            self.steps += fine_steps

    def sample(self, feat=None, targ=None, offset=0):
        """Filtered resolved KE (mean per coarse cell); with device arrays,
        writes features/targets of all coarse cells starting at row offset."""
        ke = ctypes.c_double()
        f = feat.offset(offset * 19) if feat is not None else None
        t = targ.offset(offset) if targ is not None else None
        rc = _lib().lb_closure_sample(self.lat.h, self.fac, np.float32(self.nu_c),
                                      np.float32(self.s_ref), np.float32(self.z_max), f, t,
                                      ctypes.byref(ke))
        if rc != abi.LB_OK:
            raise LBError("lb_closure_sample: %d" % rc)
        return ke.value

    def close(self):
        self.lat.close()


def coarse_run(nc, U0, Re, steps, sample_every, mlp=None, z_max=200.0, graph_steps=64,
               tuning=abi.LB_TUNE_DEFAULT):
    """Coarse Taylor-Green run (plain BGK or with the closure): mean KE at
    every sample (step 0 included) and the wall time.  A run that produces
    non-finite values stops there (returned as NaN from then on)."""
    nu = viscosity(nc, U0, Re)
    lat = Lattice(19, nc, nc, nc, tau_inv=np.float32(1 / (0.5 + 3 * nu)),
                  graph_steps=graph_steps, tuning=tuning)
    lat.set_flags(np.zeros(nc ** 3, np.uint8))
    rho, ux, uy, uz = tgv_fields(nc, U0)
    lat.init_equilibrium(rho, ux, uy, uz)
    if mlp is not None:
        rc = _lib().lb_closure_enable(lat.h, mlp.h, np.float32(nu),
                                      np.float32(U0 * 2 * np.pi / nc), np.float32(z_max), None)
        if rc != abi.LB_OK:
            raise LBError("lb_closure_enable: %d" % rc)
    ke = [float(np.mean(0.5 * rho * (ux.astype(np.float64) ** 2 + uy ** 2)))]
    seconds = 0.0
    done = 0
    while done < steps:
        k = min(sample_every, steps - done)
        t0 = time.perf_counter()
        lat.step(k)
        lat.synchronize()
        seconds += time.perf_counter() - t0
        done += k
        e = ke_mean(lat)
        ke.append(e if np.isfinite(e) else float("nan"))
        if not np.isfinite(e):
            ke += [float("nan")] * ((steps - done + sample_every - 1) // sample_every)
            break
    lat.close()
    return np.array(ke), seconds


def ke_error(coarse, reference):
    """RMS of E/E0 differences over the samples (inf if the coarse run blew up)."""
    a = np.asarray(coarse) / coarse[0]
    b = np.asarray(reference) / reference[0]
    if not np.all(np.isfinite(a)):
        return float("inf")
    return float(np.sqrt(np.mean((a - b) ** 2)))
