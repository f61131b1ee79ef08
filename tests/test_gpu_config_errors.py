"""Error statements at the configurations' own sizes and lengths.

* Lid-driven cavity (D2Q9, 256 x 256, tau 0.6, lid 0.1, half-way bounce-back
  walls, equilibrium start), 10 000 steps on the library's default path
  (temporal blocks): bit-identical to the oracle's float run of the same
  arithmetic, and its error against the FP64 oracle.
* Spinodal decomposition (D3Q19 Shan-Chen, 256^3 periodic, tau 1, G -5,
  psi = 1 - exp(-rho), rho = 0.693 (1 + eps), eps ~ U[-0.01, 0.01], seed
  2024): FP32 bit-identical to the float oracle over 50 steps on the full
  lattice; rho against the FP64 oracle after 50 steps for FP32 / FP16 / BF16
  storage; mass drift (FP64 sum on the GPU) after 10 000 steps.

The figures are printed (CONFIG_ERRORS lines) and recorded with the
configurations' results; the bounds below are loose guards around them.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def beq(a, b):
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


def cavity_flags(W, H):
    fl = np.zeros((H, W), np.uint8)
    fl[:, 0] = fl[:, -1] = fl[-1, :] = 1
    fl[0, :] = 3  # row 0 is the top wall (physical +y is row - 1), moving with the lid
    return fl.reshape(-1)


def test_cavity_256_10000_steps(pkg, oracle):
    W = H = 256
    N = W * H
    steps = 10000
    fl = cavity_flags(W, H)
    tau_inv = np.float32(1 / 0.6)
    lat = pkg.Lattice(9, W, H, tau_inv=tau_inv, wall_u=(0.1, 0, 0))
    lat.set_flags(fl)
    lat.init_equilibrium()
    lat.step(steps)
    f_gpu = lat.populations()
    rho, ux, uy, _ = lat.moments()
    lat.close()
    corr = oracle.wall_correction(9, (0.1, 0, 0))
    # the oracle's float run of the same arithmetic: every bit
    f = oracle.d2q9_equilibrium(np.ones(N, np.float32), np.zeros(N, np.float32),
                                np.zeros(N, np.float32), *pkg.W2)
    mom = [np.zeros(N, np.float32) for _ in range(3)]
    for _ in range(steps):
        oracle.d2q9_stream_native(f, fl, corr, W, H)
        oracle.d2q9_collide_native(f, fl, mom, W, H, *pkg.W2, tau_inv)
    fluid = (fl & 1) == 0
    assert beq(f_gpu[:, fluid], f[:, fluid])
    assert beq(ux, mom[0]) and beq(uy, mom[1]) and beq(rho, mom[2])
    # the FP64 oracle (same algorithm in double)
    f64 = oracle.d2q9_equilibrium(np.ones(N), np.zeros(N), np.zeros(N), 4 / 9, 1 / 9, 1 / 36)
    m64 = [np.zeros(N) for _ in range(3)]
    for _ in range(steps):
        oracle.d2q9_stream_native(f64, fl, corr.astype(np.float64), W, H)
        oracle.d2q9_collide_native(f64, fl, m64, W, H, 4 / 9, 1 / 9, 1 / 36, 1 / 0.6)
    ux64, uy64, rho64 = (m[fluid] for m in m64)
    u = np.hypot(ux[fluid].astype(np.float64), uy[fluid])
    u64 = np.hypot(ux64, uy64)
    du = np.hypot(ux[fluid] - ux64, uy[fluid] - uy64)
    r = rho[fluid].astype(np.float64)
    ke, ke64 = np.sum(r * u ** 2), np.sum(rho64 * u64 ** 2)
    rep = {"max_abs_u_err": float(du.max()), "max_u": float(u64.max()),
           "u_rel_l2": float(np.linalg.norm(du) / np.linalg.norm(u64)),
           "rho_max_abs_err": float(np.abs(r - rho64).max()),
           "rho_rel_l2_of_fluctuation": float(np.linalg.norm(r - rho64) /
                                              np.linalg.norm(rho64 - rho64.mean())),
           "ke_rel_err": float(abs(ke - ke64) / ke64),
           "mass_rel_err": float(abs(r.sum() - rho64.sum()) / rho64.sum())}
    print("CONFIG_ERRORS cavity 256^2 10000 steps FP32 vs FP64 oracle: %s" % rep)
    # the density fluctuations of the cavity are ~1e-3, so the FP32 mass
    # drift (about 1e-4 after 10 000 steps: each collision's float rounding
    # does not conserve the sum exactly) shows as a sizeable fraction of them
    assert rep["u_rel_l2"] < 1e-3 and rep["ke_rel_err"] < 1e-3
    assert rep["rho_max_abs_err"] < 1e-3 and rep["mass_rel_err"] < 1e-3


def spinodal_init(n):
    rng = np.random.default_rng(2024)
    return (0.693 * (1 + rng.uniform(-0.01, 0.01, n ** 3))).astype(np.float32)


def test_spinodal_256_statement(pkg, oracle):
    n = 256
    N = n ** 3
    rho0 = spinodal_init(n)
    z32 = np.zeros(N, np.float32)
    flags = np.zeros(N, np.uint8)
    zc = np.zeros(19, np.float32)
    early = 50
    # float oracle, 50 steps: the FP32 GPU run must match every bit
    f = oracle.d3q19_equilibrium(rho0, z32, z32, z32, *pkg.W3)
    mom32 = [np.zeros(N, np.float32) for _ in range(4)]
    psi32 = np.zeros(N, np.float32)
    for _ in range(early):
        oracle.d3q19_stream_native(f, flags, zc, n, n, n)
        oracle.d3q19_collide_native(f, flags, mom32, n, n, n, *pkg.W3, np.float32(1.0),
                                    G=-5.0, psi=psi32, psi_form=oracle.PSI_EXP1)
    rho32_oracle = mom32[3].copy()
    del f, mom32, psi32
    # FP64 oracle, 50 steps
    f64 = oracle.d3q19_equilibrium(rho0.astype(np.float64), np.zeros(N), np.zeros(N),
                                   np.zeros(N), 1 / 3, 1 / 18, 1 / 36)
    mom64 = [np.zeros(N) for _ in range(4)]
    psi64 = np.zeros(N)
    for _ in range(early):
        oracle.d3q19_stream_native(f64, flags, zc.astype(np.float64), n, n, n)
        oracle.d3q19_collide_native(f64, flags, mom64, n, n, n, 1 / 3, 1 / 18, 1 / 36, 1.0,
                                    G=-5.0, psi=psi64, psi_form=oracle.PSI_EXP1)
    rho64 = mom64[3]
    del f64, mom64, psi64
    m0 = float(np.sum(rho0.astype(np.float64)))
    fluct = np.linalg.norm(rho64 - rho64.mean())
    rep = {}
    for storage, name in [(0, "f32"), (1, "f16"), (2, "bf16")]:
        lat = pkg.Lattice(19, n, n, n, tau_inv=1.0, G=-5.0, psi_form=pkg.abi.LB_PSI_EXP1,
                          storage=storage, rho_ref=0.693)
        lat.set_flags(flags)
        lat.init_equilibrium(rho0, z32, z32, z32)
        lat.step(early)
        rho = lat.moments()[0]
        if storage == 0:
            assert beq(rho, rho32_oracle), "FP32 staged step differs from the float oracle"
        r = {"rho_rel_l2_of_fluctuation@50": float(np.linalg.norm(rho - rho64) / fluct),
             "mass_drift@50": abs(lat.reduce()[0] - m0) / m0}
        lat.step(1000 - early)
        r["mass_drift@1000"] = abs(lat.reduce()[0] - m0) / m0
        lat.step(10000 - 1000)
        red = lat.reduce()
        r["mass_drift@10000"] = abs(red[0] - m0) / m0
        r["finite@10000"] = bool(np.isfinite(red[0]))
        rep[name] = r
        lat.close()
    print("CONFIG_ERRORS spinodal 256^3 vs FP64 oracle (rho @50) and FP64 GPU sums (mass): %s"
          % rep)
    assert rep["f32"]["rho_rel_l2_of_fluctuation@50"] < 1e-3
    for name, b in [("f32", 1e-3), ("f16", 5e-2), ("bf16", 3e-1)]:
        assert rep[name]["finite@10000"] and rep[name]["mass_drift@10000"] < b, (name, rep[name])
