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

    def sample(self, feat=None, targ=None, offset=0, factor=None, avg_radius=0):
        """Filtered resolved KE (mean per coarse cell); with device arrays,
        writes features/targets of all coarse cells starting at row offset.
        factor: another filter width than the run's own (coarse grid
        n_fine / factor); avg_radius: the target's neighbourhood averaging
        (lb_closure_sample_avg)."""
        fac = self.fac if factor is None else int(factor)
        nc = self.nf // fac
        ke = ctypes.c_double()
        f = feat.offset(offset * 19) if feat is not None else None
        t = targ.offset(offset) if targ is not None else None
        rc = _lib().lb_closure_sample_avg(self.lat.h, fac, np.float32(viscosity(nc, self.U0, self.Re)),
                                          np.float32(self.U0 * 2 * np.pi / nc),
                                          np.float32(self.z_max), int(avg_radius), f, t,
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


def active_inputs(feat, n_rows, rows_per_snapshot, probe=20000):
    """Which of the 19 inputs are non-zero somewhere in the training rows
    (a probe of every snapshot's first rows).  The stress features and |S|
    are; the higher non-equilibrium moments are zero in filtered fine data
    (they vanish at first order), so their first-layer weights would get no
    gradient and keep their random initial values."""
    active = np.zeros(Mlp.N_IN, bool)
    for off in range(0, n_rows, rows_per_snapshot):
        m = min(rows_per_snapshot, probe, n_rows - off)
        rows = feat.download((off + m) * Mlp.N_IN).reshape(-1, Mlp.N_IN)[off:off + m]
        active |= np.abs(rows).max(axis=0) > 0
    return active


def zero_inputs(net, active):
    """First-layer weights of the inactive inputs set to zero (they then get
    zero gradients and stay zero: the network ignores inputs it never saw)."""
    p = net.params()
    p[:64 * Mlp.N_IN].reshape(64, Mlp.N_IN)[:, ~np.asarray(active)] = 0
    net.set_params(p)


def scale_output(net, c, base=None):
    """The network's output scaled by c (output layer w3, b3; the eddy
    viscosity nu0 * clamp(y, 0, z_max) then scales with it)."""
    p = (net.params() if base is None else base).copy()
    p[-65:] *= np.float32(c)
    net.set_params(p)


CALIBRATION_SCALES = (1.0, 0.7, 0.5, 0.35, 0.25, 0.18, 0.12)


def calibrate(net, nc, U0, Re, ke_ref, every, steps, scales=CALIBRATION_SCALES, window=0.5):
    """A posteriori fit of one scalar: the output scale c (from `scales`) whose
    coarse run best tracks the reference kinetic energy over the first
    `window` of the trajectory.  The coarse LBM dissipates by itself (its
    truncation error acts as an implicit sub-grid model), so the sub-grid
    dissipation fitted a priori from the filtered stress is too much for it;
    c takes out that double count.  The remaining part of the trajectory is
    not seen by the fit.  Returns (c, {c: window error})."""
    base = net.params()
    nwin = max(1, int(round(len(ke_ref) * window)) - 1)
    errs = {}
    for c in scales:
        scale_output(net, c, base)
        ke, _ = coarse_run(nc, U0, Re, nwin * every, every, mlp=net)
        errs[c] = ke_error(ke, ke_ref[:nwin + 1])
    best = min(errs, key=lambda c: errs[c])
    scale_output(net, best, base)
    return best, errs


def resolution_sweep(n_fine, factors, U0=0.05, Re=1600.0, t_end=10.0, fine_every=256,
                     train_snapshots=16, train_steps=3000, batch=16384, lr=2e-3, avg_radius=1,
                     plain_only=(), seed=2, log=None):
    """Plain coarse BGK against the learned closure over several coarse grids.

    One fine run (n_fine^3) is box-filtered by every factor at every sample
    (each fine_every fine steps): the reference kinetic energy of each coarse
    grid and, at train_snapshots samples, its training data (features and
    neighbourhood-averaged targets).  For each factor not in plain_only a
    network is trained on that grid's data (inputs never excited in the data
    masked), its output scale calibrated on the first half of the
    trajectory, and run over the whole trajectory; every factor also gets a
    plain BGK run.  Returns a dict with the fine run's time and one entry per
    run (grid, kind, KE error, wall time of the steps, steps)."""
    fr = FineRun(n_fine, factors[0], U0, Re)
    steps_f = int(round(t_end * (n_fine / (2 * np.pi)) / U0))
    nsamp = steps_f // fine_every
    train_at = set(np.linspace(0, nsamp, train_snapshots).astype(int).tolist())
    learned = [f for f in factors if f not in plain_only]
    data = {}
    for f in learned:
        nc3 = (n_fine // f) ** 3
        data[f] = (DeviceArray(len(train_at) * nc3 * 19), DeviceArray(len(train_at) * nc3))
    ke = {f: [] for f in factors}
    slot = 0
    for i in range(nsamp + 1):
        if i:
            fr.advance(fine_every)
        for f in factors:
            if f in data and i in train_at:
                nc3 = (n_fine // f) ** 3
                ke[f].append(fr.sample(data[f][0], data[f][1], slot * nc3, factor=f,
                                       avg_radius=avg_radius))
            else:
                ke[f].append(fr.sample(factor=f))
        if i in train_at:
            slot += 1
    out = {"fine_seconds": fr.seconds, "fine_steps": fr.steps, "fine_n": n_fine, "runs": [],
           "samples": nsamp + 1}
    fr.close()
    for f in factors:
        nc = n_fine // f
        every = fine_every // f
        ke_p, t_p = coarse_run(nc, U0, Re, nsamp * every, every)
        e_p = ke_error(ke_p, ke[f])
        out["runs"].append({"n": nc, "kind": "plain", "ke_error": e_p, "seconds": t_p,
                            "steps": nsamp * every})
        if log:
            log("plain %d^3: KE error %.5g, %.4f s" % (nc, e_p, t_p))
        if f not in data:
            continue
        feat, targ = data.pop(f)
        nc3 = nc ** 3
        net = Mlp(seed=seed)
        active = active_inputs(feat, slot * nc3, nc3)
        zero_inputs(net, active)
        t0 = time.perf_counter()
        tlog = net.train_device(feat, targ, slot * nc3, steps=train_steps, batch=batch, lr=lr)
        train_s = time.perf_counter() - t0
        feat.free()
        targ.free()
        c, cal = calibrate(net, nc, U0, Re, ke[f], every, nsamp * every)
        ke_l, t_l = coarse_run(nc, U0, Re, nsamp * every, every, mlp=net)
        e_l = ke_error(ke_l, ke[f])
        net.close()
        out["runs"].append({"n": nc, "kind": "closure", "ke_error": e_l, "seconds": t_l,
                            "steps": nsamp * every, "train_seconds": train_s,
                            "final_loss": float(np.mean(tlog[-20:])), "output_scale": c,
                            "calibration_errors": {str(k): v for k, v in cal.items()},
                            "active_inputs": np.nonzero(active)[0].tolist(),
                            "ke_curve": [round(float(v / ke_l[0]), 5) for v in ke_l[::4]]})
        if log:
            log("closure %d^3: KE error %.5g, %.4f s (scale %g)" % (nc, e_l, t_l, c))
    out["ke_ref"] = {str(n_fine // f): [round(v / ke[f][0], 5) for v in ke[f][::4]]
                     for f in factors}
    return out


def headline(pairs, max_error=0.01):
    """The largest speed-up among the closure runs whose KE error is at most
    max_error (None if there is none)."""
    ok = [p for p in pairs if p["speedup"] and p["closure_ke_error"] <= max_error]
    return max(ok, key=lambda p: p["speedup"], default=None)


def speedup_at_equal_error(runs):
    """For every closure run: the cheapest plain run whose KE error is at most
    the closure's (finite), and the ratio of their wall times."""
    plain = sorted([r for r in runs if r["kind"] == "plain" and np.isfinite(r["ke_error"])],
                   key=lambda r: r["seconds"])
    res = []
    for r in runs:
        if r["kind"] != "closure" or not np.isfinite(r["ke_error"]):
            continue
        match = next((p for p in plain if p["ke_error"] <= r["ke_error"]), None)
        res.append({"closure_n": r["n"], "closure_ke_error": r["ke_error"],
                    "closure_seconds": r["seconds"],
                    "plain_n": match["n"] if match else None,
                    "plain_ke_error": match["ke_error"] if match else None,
                    "plain_seconds": match["seconds"] if match else None,
                    "speedup": match["seconds"] / r["seconds"] if match else None})
    return res
