"""The oracle reproduces the golden fixtures (outputs of the reference's own
kernels) bit for bit.  Needs no reference sources, so it also runs where only
the fixtures travel."""
import numpy as np

from golden_io import bits, load


def test_golden_d3q19(oracle):
    g = load("d3q19_ref")
    W, H, D = int(g["W"]), int(g["H"]), int(g["D"])
    N = W * H * D
    f = g["f_in"].copy()
    mom = [np.zeros(N, np.float32) for _ in range(4)]
    plot = np.zeros(4 * N, np.float32)
    w = g["w"]
    for _ in range(int(g["steps"])):
        oracle.d3q19_stream(f, g["solid_bound"], W, H, D)
        oracle.d3q19_collide(f, g["solid"], mom, W, H, D, w[0], w[1], w[2], g["tau_inv"],
                             g["ux_in"], 0, 0, g["rho_out"], plot=plot)
    assert np.array_equal(bits(f), bits(g["f_out"]))
    for a, k in zip(mom, ["ux", "uy", "uz", "rho"]):
        assert np.array_equal(bits(a), bits(g[k])), k
    assert np.array_equal(bits(plot), bits(g["plot"]))


def test_golden_d3q19_stream(oracle):
    g = load("d3q19_stream")
    W, H, D = int(g["W"]), int(g["H"]), int(g["D"])
    f = g["f_in"].copy()
    oracle.d3q19_stream(f, np.zeros(W * H * D, np.uint8), W, H, D)
    assert np.array_equal(bits(f), bits(g["f_out"]))


def _d2q9(oracle, name):
    g = load(name)
    W, H = int(g["W"]), int(g["H"])
    N = W * H
    f = g["f_in"].copy()
    mom = [np.zeros(N, np.float32) for _ in range(3)]
    sc = [np.zeros(N, np.float32) for _ in range(3)]
    plot = np.zeros(4 * N, np.float32)
    w = g["w"]
    for _ in range(int(g["steps"])):
        oracle.d2q9_stream(f, g["solid_bound"], W, H)
        oracle.d2q9_collide(f, g["solid"], mom, sc, W, H, w[0], w[1], w[2], g["tau_inv"],
                            g["ux_in"], 0, g["rho_out"], g["Fx"], g["Fy"], g["G"], g["Gads"],
                            plot=plot)
    assert np.array_equal(bits(f), bits(g["f_out"]))
    for a, k in zip(mom, ["ux", "uy", "rho"]):
        assert np.array_equal(bits(a), bits(g[k])), k
    if "psi" in g:
        for a, k in zip(sc, ["psi", "ueq_x", "ueq_y"]):
            assert np.array_equal(bits(a), bits(g[k])), k
    assert np.array_equal(bits(plot), bits(g["plot"]))


def test_golden_d2q9(oracle):
    _d2q9(oracle, "d2q9_ref")


def test_golden_d2q9_shan_chen(oracle):
    _d2q9(oracle, "d2q9_sc")
