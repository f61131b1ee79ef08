"""Generate the golden fixtures of tests/golden/ from the reference's own
kernels (src/streaming.cu, src/collision.cu, src/get_border.cu,
src/apply_border.cu), compiled for the host by `make -C oracle ref`.

Run from the repository root where the reference sources exist:
    python tests/golden/make_golden.py
Inputs are seeded; every fixture stores its inputs and the reference's
outputs, so the tests need neither the reference nor this script.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import lb_oracle  # noqa: E402
import refrun  # noqa: E402
from conftest import load_package  # noqa: E402

W3 = np.array([12. / 36., 2. / 36., 1. / 36.], np.float32)
W2 = np.array([16. / 36., 4. / 36., 1. / 36.], np.float32)


def noisy(rng, w, N, amp=0.2):
    return (np.asarray(w, np.float32)[:, None] * (1.0 + amp * rng.standard_normal((len(w), N)))
            ).astype(np.float32)


def solid_field(rng, shape, frac, block):
    s = (rng.random(shape) < frac).astype(np.uint8)
    s[..., block[0]:block[1]] = 1
    return np.ascontiguousarray(s.reshape(-1))


def main():
    ref = lb_oracle.ref_lib()
    assert ref is not None, "reference sources not found"
    abi = load_package().abi
    out = {}

    # D3Q19: solids (incl. a block thick enough for solid_bound), Zou-He in/out
    W, H, D = 32, 4, 4
    N = W * H * D
    rng = np.random.default_rng(1001)
    f0 = noisy(rng, lb_oracle.D3_W, N)
    solid = solid_field(rng, (D, H, W), 0.12, (10, 16))
    sb = lb_oracle.d3q19_solid_bound(solid, W, H, D)
    f = f0.copy()
    plot = np.zeros(4 * N, np.float32)
    tau_inv = np.float32(1. / (3. * 0.03 + 0.5))
    mom = refrun.run_d3q19(ref, abi, W, H, D, f, solid, sb, 3, W3, tau_inv, 0.05, 1.0, plot)
    out["d3q19_ref"] = dict(W=W, H=H, D=D, steps=3, w=W3, tau_inv=tau_inv, ux_in=np.float32(0.05),
                            rho_out=np.float32(1.0), f_in=f0, solid=solid, solid_bound=sb,
                            f_out=f, ux=mom[0], uy=mom[1], uz=mom[2], rho=mom[3], plot=plot)

    # D3Q19 streaming alone (a permutation): all-fluid, random populations
    rng = np.random.default_rng(1002)
    f0 = rng.standard_normal((19, N)).astype(np.float32)
    f = f0.copy()
    zero = np.zeros(N, np.uint8)
    d = refrun.d3q19_struct(abi, W, H, D, f, zero, zero, [np.zeros(N, np.float32)] * 4)
    ref.streaming_d3q19(ctypes.byref(d), abi.dim3(W // 32, H // 4, D), abi.dim3(32, 4, 1))
    out["d3q19_stream"] = dict(W=W, H=H, D=D, f_in=f0, f_out=f)

    # D2Q9 BGK with body force, solids, Zou-He
    W, H = 64, 8
    N = W * H
    rng = np.random.default_rng(1003)
    f0 = noisy(rng, lb_oracle.D2_W, N)
    solid = solid_field(rng, (H, W), 0.1, (20, 26))
    sb = lb_oracle.d2q9_solid_bound(solid, W, H)
    f = f0.copy()
    plot = np.zeros(8 * N, np.float32)
    tau_inv = np.float32(1.0)
    (mom, sc) = refrun.run_d2q9(ref, abi, W, H, f, solid, sb, 3, W2, tau_inv, 0.01, 1.0,
                                2.035e-6, 1e-5, 0.0, 0.0, plot)
    out["d2q9_ref"] = dict(W=W, H=H, steps=3, w=W2, tau_inv=tau_inv, ux_in=np.float32(0.01),
                           rho_out=np.float32(1.0), Fx=np.float32(2.035e-6), Fy=np.float32(1e-5),
                           G=np.float32(0), Gads=np.float32(0), f_in=f0, solid=solid,
                           solid_bound=sb, f_out=f, ux=mom[0], uy=mom[1], rho=mom[2],
                           plot=plot[:4 * N])

    # D2Q9 Shan-Chen with adhesion and gravity (psi = 4 exp(-200/rho)), rho ~ 200
    W, H = 32, 8
    N = W * H
    rng = np.random.default_rng(1004)
    solid = np.zeros((H, W), np.uint8)
    solid[H - 1, :] = 1
    solid = np.ascontiguousarray(solid.reshape(-1))
    sb = lb_oracle.d2q9_solid_bound(solid, W, H)
    rho0 = (200.0 * (1 + 0.02 * rng.standard_normal(N))).astype(np.float32)
    f0 = (lb_oracle.D2_W[:, None] * rho0[None, :]).astype(np.float32)
    f = f0.copy()
    plot = np.zeros(8 * N, np.float32)
    tau_inv = np.float32(1. / (3. * 0.16667 + 0.5))
    (mom, sc) = refrun.run_d2q9(ref, abi, W, H, f, solid, sb, 3, W2, tau_inv, 0.0, 200.0,
                                0.0, -1e-4, -120.0, -50.0, plot)
    out["d2q9_sc"] = dict(W=W, H=H, steps=3, w=W2, tau_inv=tau_inv, ux_in=np.float32(0.0),
                          rho_out=np.float32(200.0), Fx=np.float32(0), Fy=np.float32(-1e-4),
                          G=np.float32(-120.0), Gads=np.float32(-50.0), f_in=f0, solid=solid,
                          solid_bound=sb, f_out=f, ux=mom[0], uy=mom[1], rho=mom[2], psi=sc[0],
                          ueq_x=sc[1], ueq_y=sc[2], plot=plot[:4 * N])

    for name, d in out.items():
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **{k: np.asarray(v) for k, v in d.items()})
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
