"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` to verify results against; the GPU library never imports it.  The oracle is
a C restatement of lattibol's per-step update (see lb_oracle.h); ``build()``
compiles it with the recipe in oracle/Makefile.

Arrays are numpy, SoA ``f[k, node]`` with node = x + y*W + z*W*H.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liblboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "liblbref.so")


def ref_dir():
    """Location of the reference tree: the environment variable
    LATTIBOL_REF_DIR, else the default of the build recipe (oracle/Makefile,
    ``make ref-dir``).  Callers check that it exists: it does not where only
    this repository was copied."""
    d = os.environ.get("LATTIBOL_REF_DIR")
    if d:
        return d
    try:
        r = subprocess.run(["make", "-s", "-C", HERE, "ref-dir"], capture_output=True, text=True,
                           check=True)
        return r.stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return ""


def ref_src():
    return os.path.join(ref_dir(), "src")

PSI_REF = 0
PSI_EXP1 = 1
SOLID = 0x01
MOVING = 0x02

# lattice tables (same order as lb_oracle.c)
D3_C = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                 [1, 1, 0], [1, -1, 0], [1, 0, 1], [1, 0, -1], [-1, 1, 0], [-1, -1, 0],
                 [-1, 0, 1], [-1, 0, -1], [0, 1, 1], [0, 1, -1], [0, -1, 1], [0, -1, -1]])
D3_OPP = [0, 2, 1, 4, 3, 6, 5, 12, 11, 14, 13, 8, 7, 10, 9, 18, 17, 16, 15]
D3_W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
# D2Q9: (x offset, row offset); physical y = -row
D2_CXR = np.array([[0, 0], [1, 0], [0, -1], [-1, 0], [0, 1], [1, -1], [-1, -1], [-1, 1], [1, 1]])
D2_OPP = [0, 3, 4, 1, 2, 7, 8, 5, 6]
D2_W = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)


def build(ref=None):
    """Compile the oracle (and, where the reference sources exist, the
    reference's own kernels for the host into oracle/_ref)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref is None:
        ref = os.path.isdir(ref_src())
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        _lib = ctypes.CDLL(LIB_PATH)
    return _lib


def ref_lib():
    """The reference's kernels compiled for the host, or None where the
    reference sources are absent."""
    if not os.path.exists(REF_PATH):
        if not os.path.isdir(ref_src()):
            return None
        build(ref=True)
    return ctypes.CDLL(REF_PATH)


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _real(dtype):
    return (ctypes.c_float, "f32") if np.dtype(dtype) == np.float32 else (ctypes.c_double, "f64")


def _check(a, dtype, n=None):
    assert a.dtype == dtype and a.flags.c_contiguous, (a.dtype, dtype)
    if n is not None:
        assert a.size == n


# ---------------------------------------------------------------- reference semantics

def d3q19_solid_bound(solid, W, H, D):
    sb = np.zeros(W * H * D, np.uint8)
    lib().lbo_d3q19_solid_bound(_p(np.ascontiguousarray(solid, np.uint8)), _p(sb), W, H, D)
    return sb


def d2q9_solid_bound(solid, W, H):
    sb = np.zeros(W * H, np.uint8)
    lib().lbo_d2q9_solid_bound(_p(np.ascontiguousarray(solid, np.uint8)), _p(sb), W, H)
    return sb


def d3q19_stream(f, solid_bound, W, H, D):
    c, s = _real(f.dtype)
    getattr(lib(), "lbo_d3q19_stream_" + s)(_p(f), _p(solid_bound), W, H, D)


def d3q19_collide(f, solid, mom, W, H, D, w0, w1, w7, tau_inv, ux_in, uy_in, uz_in, rho_out,
                  plot=None, dev=0, ndev=1):
    """mom = (ux, uy, uz, rho) arrays of f.dtype."""
    c, s = _real(f.dtype)
    ux, uy, uz, rho = mom
    getattr(lib(), "lbo_d3q19_collide_" + s)(
        _p(plot), _p(f), _p(solid), _p(ux), _p(uy), _p(uz), _p(rho), W, H, D, dev, ndev,
        c(w0), c(w1), c(w7), c(tau_inv), c(ux_in), c(uy_in), c(uz_in), c(rho_out))


def d2q9_stream(f, solid_bound, W, H):
    c, s = _real(f.dtype)
    getattr(lib(), "lbo_d2q9_stream_" + s)(_p(f), _p(solid_bound), W, H)


def d2q9_collide(f, solid, mom, sc, W, H, w0, w1, w5, tau_inv, ux_in, uy_in, rho_out, Fx, Fy,
                 G, Gads, plot=None, dev=0, ndev=1):
    """mom = (ux, uy, rho); sc = (psi, ueq_x, ueq_y)."""
    c, s = _real(f.dtype)
    ux, uy, rho = mom
    psi, ueq_x, ueq_y = sc
    getattr(lib(), "lbo_d2q9_collide_" + s)(
        _p(plot), _p(f), _p(solid), _p(ux), _p(uy), _p(rho), _p(psi), _p(ueq_x), _p(ueq_y),
        W, H, dev, ndev, c(w0), c(w1), c(w5), c(tau_inv), c(ux_in), c(uy_in), c(rho_out),
        c(Fx), c(Fy), c(G), c(Gads))


# ---------------------------------------------------------------- native mode

def d3q19_stream_native(f, flags, corr, W, H, D):
    c, s = _real(f.dtype)
    corr = np.ascontiguousarray(corr, f.dtype)
    getattr(lib(), "lbo_d3q19_stream_native_" + s)(_p(f), _p(flags), _p(corr), W, H, D)


def d3q19_collide_native(f, flags, mom, W, H, D, w0, w1, w7, tau_inv, F=(0, 0, 0), G=0.0,
                         psi=None, psi_form=PSI_EXP1):
    c, s = _real(f.dtype)
    ux, uy, uz, rho = mom if mom is not None else (None,) * 4
    getattr(lib(), "lbo_d3q19_collide_native_" + s)(
        _p(f), _p(flags), _p(ux), _p(uy), _p(uz), _p(rho), _p(psi), W, H, D, c(w0), c(w1),
        c(w7), c(tau_inv), c(F[0]), c(F[1]), c(F[2]), c(G), psi_form)


def d2q9_stream_native(f, flags, corr, W, H):
    c, s = _real(f.dtype)
    corr = np.ascontiguousarray(corr, f.dtype)
    getattr(lib(), "lbo_d2q9_stream_native_" + s)(_p(f), _p(flags), _p(corr), W, H)


def d2q9_collide_native(f, flags, mom, W, H, w0, w1, w5, tau_inv, F=(0, 0), G=0.0, Gads=0.0,
                        psi=None, psi_form=PSI_EXP1):
    c, s = _real(f.dtype)
    ux, uy, rho = mom if mom is not None else (None,) * 3
    if G != 0 and psi is None:
        psi = np.zeros(W * H, f.dtype)
    getattr(lib(), "lbo_d2q9_collide_native_" + s)(
        _p(f), _p(flags), _p(ux), _p(uy), _p(rho), _p(psi), W, H, c(w0), c(w1), c(w5),
        c(tau_inv), c(F[0]), c(F[1]), c(G), c(Gads), psi_form)


def d3q19_equilibrium(rho, ux, uy, uz, w0, w1, w7):
    dt = rho.dtype
    c, s = _real(dt)
    n = rho.size
    f = np.empty((19, n), dt)
    getattr(lib(), "lbo_d3q19_equilibrium_" + s)(_p(f), _p(rho), _p(ux), _p(uy), _p(uz),
                                                 ctypes.c_long(n), c(w0), c(w1), c(w7))
    return f


def d2q9_equilibrium(rho, ux, uy, w0, w1, w5):
    dt = rho.dtype
    c, s = _real(dt)
    n = rho.size
    f = np.empty((9, n), dt)
    getattr(lib(), "lbo_d2q9_equilibrium_" + s)(_p(f), _p(rho), _p(ux), _p(uy),
                                                ctypes.c_long(n), c(w0), c(w1), c(w5))
    return f


def wall_correction(lattice, wall_u):
    """6 w_k (c_k . u_wall) per direction, evaluated in double and rounded to
    float (physical velocity components; D2Q9 physical c_y = -row offset)."""
    if lattice == 19:
        c, w = D3_C.astype(np.float64), D3_W
        u = np.array(wall_u[:3], np.float64)
    else:
        c = np.stack([D2_CXR[:, 0], -D2_CXR[:, 1]], 1).astype(np.float64)
        w = D2_W
        u = np.array(wall_u[:2], np.float64)
    out = np.empty(len(w), np.float32)
    for k in range(len(w)):
        dot = 0.0
        for a in range(len(u)):
            dot = dot + c[k, a] * float(np.float32(u[a]))
        out[k] = np.float32(6.0 * w[k] * dot)
    return out


def reduce_f32(rho, ux, uy, uz, solid):
    out = (ctypes.c_double * 7)()
    lib().lbo_reduce_f32(_p(rho), _p(ux), _p(uy), _p(uz), _p(solid), ctypes.c_long(rho.size), out)
    return np.array(out[:])


def num_threads():
    return lib().lbo_num_threads()


def set_threads(n):
    lib().lbo_set_threads(int(n))


def storage_offsets(lattice, rho_ref=1.0):
    """wr_k = w_k * rho_ref, evaluated in double and rounded to float."""
    w = D3_W if lattice == 19 else D2_W
    r = float(np.float32(rho_ref))
    return np.array([np.float32(wk * r) for wk in w], np.float32)


# ---- 16-bit storage as the library's step kernels keep it: the deviations
# d_k = f_k - wr_k themselves (the step's arithmetic works on d, lb_common.cuh
# d3q19_*_dev), narrowed and widened on every store and load

def rho_offset(wr):
    """The density the offsets carry, sum_k wr_k in double rounded to float."""
    return np.float32(np.sum(np.asarray(wr, np.float64)))


def to_dev(f, wr, kind):
    """The stored deviations of a float population state: widen(narrow(f -
    wr)) for every node (lb_set_populations)."""
    d = np.ascontiguousarray(np.asarray(f, np.float32) - np.asarray(wr, np.float32)[:, None])
    lib().lbo_round_storage(_p(d), ctypes.c_long(d.size), kind)
    return d


def from_dev(d, wr):
    """Float populations wr + d (lb_get_populations)."""
    return np.asarray(wr, np.float32)[:, None] + d


def quantize(d, kind, flags=None):
    """In place: d = widen(narrow(d)) on non-wall nodes (a step's stores)."""
    assert d.dtype == np.float32 and d.flags.c_contiguous
    if flags is None:
        lib().lbo_round_storage(_p(d), ctypes.c_long(d.size), kind)
        return
    fluid = (np.asarray(flags) & SOLID) == 0
    q = np.ascontiguousarray(d[:, fluid])
    lib().lbo_round_storage(_p(q), ctypes.c_long(q.size), kind)
    d[:, fluid] = q


def d3q19_collide_native_dev(d, flags, mom, W, H, D, w0, w1, w7, tau_inv, wr, F=(0, 0, 0),
                             G=0.0, psi=None, psi_form=PSI_EXP1):
    """The native collision on the deviation state d of 16-bit storage (float)."""
    assert d.dtype == np.float32
    c = ctypes.c_float
    wr = np.ascontiguousarray(wr, np.float32)
    ux, uy, uz, rho = mom if mom is not None else (None,) * 4
    lib().lbo_d3q19_collide_native_dev_f32(
        _p(d), _p(flags), _p(ux), _p(uy), _p(uz), _p(rho), _p(psi), W, H, D, c(w0), c(w1),
        c(w7), c(tau_inv), c(F[0]), c(F[1]), c(F[2]), c(G), psi_form, c(rho_offset(wr)), _p(wr))


def quantize_dev(f, wr, flags=None, kind=1):
    """In place: f[k] = wr[k] + widen(narrow(f[k] - wr[k])) on non-wall nodes
    (kind 1 = binary16, 2 = bfloat16)."""
    assert f.dtype == np.float32 and f.flags.c_contiguous
    Q, N = f.shape
    wr = np.ascontiguousarray(wr, np.float32)
    lib().lbo_quantize_dev(_p(f), Q, ctypes.c_long(N), _p(wr),
                           _p(None if flags is None else np.ascontiguousarray(flags, np.uint8)),
                           kind)


def f16_roundtrip(a):
    a = np.ascontiguousarray(a, np.float32).copy()
    lib().lbo_round_storage(_p(a), ctypes.c_long(a.size), 1)
    return a


def bf16_roundtrip(a):
    a = np.ascontiguousarray(a, np.float32).copy()
    lib().lbo_round_storage(_p(a), ctypes.c_long(a.size), 2)
    return a
