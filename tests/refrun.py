"""Drive the reference's own kernels (compiled for the host into oracle/_ref)
through their extern "C" entry points with numpy host buffers.  Used by the
oracle pin test and by tests/golden/make_golden.py; needs the reference
sources, so it only runs where they exist."""
import ctypes

import numpy as np

F = ctypes.c_float


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p).value


def d3q19_struct(abi, W, H, D, f, solid, sb, mom):
    d = abi.DataD3Q19()
    for k in range(19):
        setattr(d, "f%d" % k, ptr(f[k]))
    d.ux, d.uy, d.uz, d.rho = [ptr(m) for m in mom]
    d.solid, d.solid_bound = ptr(solid), ptr(sb)
    d.width, d.height, d.depth = W, H, D
    d.deviceCount, d.dev = 1, 0
    return d


def d2q9_struct(abi, W, H, f, solid, sb, mom, sc):
    d = abi.DataD2Q9()
    for k in range(9):
        setattr(d, "f%d" % k, ptr(f[k]))
    d.ux, d.uy, d.rho = [ptr(m) for m in mom]
    d.psi, d.ueq_x, d.ueq_y = [ptr(m) for m in sc]
    d.solid, d.solid_bound = ptr(solid), ptr(sb)
    d.width, d.height = W, H
    d.deviceCount, d.dev = 1, 0
    return d


def run_d3q19(ref, abi, W, H, D, f, solid, sb, steps, w, tau_inv, ux_in, rho_out, plot):
    """Advance f (in place) by `steps` reference steps; returns (ux,uy,uz,rho)."""
    N = W * H * D
    mom = [np.zeros(N, np.float32) for _ in range(4)]
    d = d3q19_struct(abi, W, H, D, f, solid, sb, mom)
    g, b = abi.dim3(W // 32, H // 4, D), abi.dim3(32, 4, 1)
    for _ in range(steps):
        ref.streaming_d3q19(ctypes.byref(d), g, b)
        ref.collision_d3q19(ctypes.c_void_p(ptr(plot)), ctypes.byref(d), F(w[0]), F(w[1]),
                            F(w[2]), F(tau_inv), F(ux_in), F(0), F(0), F(rho_out), F(0),
                            F(0.15), F(0.98), F(1.02), g, b)
    return mom


def run_d2q9(ref, abi, W, H, f, solid, sb, steps, w, tau_inv, ux_in, rho_out, Fx, Fy, G, Gads,
             plot, sc=None):
    """Advance f (in place); plot must hold 8*W*H floats (the reference's solid
    branch writes one float past the first W*H float4s).  Returns (mom, sc)."""
    N = W * H
    mom = [np.zeros(N, np.float32) for _ in range(3)]
    if sc is None:
        sc = [np.zeros(N, np.float32) for _ in range(3)]
    d = d2q9_struct(abi, W, H, f, solid, sb, mom, sc)
    g, b = abi.dim3(W // 32, H // 4, 1), abi.dim3(32, 4, 1)
    for _ in range(steps):
        ref.streaming_d2q9(ctypes.byref(d), g, b)
        ref.collision_d2q9(ctypes.c_void_p(ptr(plot)), ctypes.byref(d), F(w[0]), F(w[1]),
                           F(w[2]), F(tau_inv), F(ux_in), F(0), F(rho_out), F(0), F(0.015),
                           F(0.98), F(1.02), g, b, F(Fx), F(Fy), F(G), F(Gads))
    return mom, sc
