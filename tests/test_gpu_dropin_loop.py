"""GPU: lb_run_lbm_d3q19, the reference's per-step host sequence run inside
the library (streaming_d3q19, collision_d3q19 into the plot buffer,
read_value_3d, a 16-byte copy of the cursor value), gives the same bits as
the same entry points called one by one from the host, in both drop-in
modes, and leaves the last step's cursor value in the caller's buffer."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu

NX, NY, NZ, STEPS = 40, 16, 12, 9
CURSOR = (NX // 2, NY // 3, NZ // 2)
TAU_INV = np.float32(1 / 0.8)


@pytest.fixture(scope="module")
def pkg():
    p = load_package()
    n = C.c_int(0)
    assert p.lib().lb_device_count(C.byref(n)) == 0 and n.value >= 1, "no CUDA device"
    return p


def _case(pkg):
    """Walls at z = 0 and nz-1 and a sphere of radius 3 (full-way bounce-back
    solids), solid_bound by the reference's rule, a perturbed rest state."""
    z, y, x = np.meshgrid(np.arange(NZ), np.arange(NY), np.arange(NX), indexing="ij")
    s = (z == 0) | (z == NZ - 1) | ((x - 12) ** 2 + (y - 8) ** 2 + (z - 6) ** 2 <= 9)
    sb = s.copy()
    for cz in (-1, 0, 1):
        for cy in (-1, 0, 1):
            for cx in (-1, 0, 1):
                if abs(cx) + abs(cy) + abs(cz) in (1, 2):
                    sb &= np.roll(s, (-cz, -cy, -cx), (0, 1, 2))
    sb[:, :, 0] = sb[:, :, -1] = False
    w = np.array([pkg.W3[0]] + [pkg.W3[1]] * 6 + [pkg.W3[2]] * 12, np.float32)
    rng = np.random.default_rng(5)
    f0 = (w[:, None] * (1 + 0.01 * rng.standard_normal((19, NX * NY * NZ)))).astype(np.float32)
    return s.reshape(-1).astype(np.uint8), sb.reshape(-1).astype(np.uint8), f0


def _params(pkg):
    prm = pkg.abi.lb_run_params_d3q19()
    prm.w0, prm.w1, prm.w7 = (float(v) for v in pkg.W3)
    prm.tau_inv, prm.ux_in, prm.uy_in, prm.uz_in, prm.rho_out = TAU_INV, 0.01, 0.0, 0.0, 1.0
    prm.cursor[0], prm.cursor[1], prm.cursor[2] = CURSOR
    return prm


def _run(pkg, mode, in_library, pinned=False):
    L, a = pkg.lib(), pkg.abi
    solid, sb, f0 = _case(pkg)
    dd = pkg.DeviceData(19, NX, NY, NZ, plot=True)
    L.lb_abi_set_mode(mode)
    vp = C.c_void_p()
    try:
        dd.set_solid(solid, sb)
        dd.upload(f0)
        prm = _params(pkg)
        if pinned:  # page-locked: the fused pass writes the cursor value into it directly
            assert L.lb_malloc_host(C.byref(vp), 16) == 0
            value = (C.c_float * 4).from_address(vp.value)
        else:
            value = (C.c_float * 4)()
        value[:] = [-1.0] * 4
        if in_library:
            rc = L.lb_run_lbm_d3q19(dd.ptr(), C.c_void_p(dd.plot), C.byref(prm), STEPS, value)
            assert rc == 0, L.lb_abi_last_error()
        else:
            g, b = a.dim3(NX // 32 or 1, NY // 4, NZ), a.dim3(32, 4, 1)
            F = np.float32
            for _ in range(STEPS):
                L.streaming_d3q19(dd.ptr(), g, b)
                L.collision_d3q19(C.c_void_p(dd.plot), dd.ptr(), F(prm.w0), F(prm.w1), F(prm.w7),
                                  F(prm.tau_inv), F(prm.ux_in), F(prm.uy_in), F(prm.uz_in),
                                  F(prm.rho_out), F(0), F(0), F(0), F(0), g, b)
                L.read_value_3d(C.c_void_p(dd.plot), dd.ptr(), *CURSOR)
            v = dd.d2h(dd.s.valueCur, 4)
            value[:] = [float(t) for t in v]
        assert L.lb_abi_release_d3q19(dd.ptr()) == 0
        out = (dd.download(), [dd.field(k) for k in ("rho", "ux", "uy", "uz")], dd.plot_data(),
               np.array(value[:], np.float32), dd.d2h(dd.s.valueCur, 4))
    finally:
        L.lb_abi_set_mode(a.LB_ABI_STANDALONE)
        if vp.value:
            L.lb_free_host(vp)
        dd.close()
    return out


@pytest.mark.parametrize("value_buf", ["pageable", "pinned"])
@pytest.mark.parametrize("mode", ["standalone", "fused"])
def test_run_lbm_matches_per_step_entry_points(pkg, mode, value_buf):
    m = pkg.abi.LB_ABI_FUSED if mode == "fused" else pkg.abi.LB_ABI_STANDALONE
    f_a, mom_a, plot_a, val_a, cur_a = _run(pkg, m, True, value_buf == "pinned")
    f_b, mom_b, plot_b, val_b, cur_b = _run(pkg, m, False)
    assert np.isfinite(f_a).all()
    # data->valueCur holds the last step's value too, as after read_value_3d
    assert np.array_equal(cur_a.view(np.uint32), cur_b.view(np.uint32))
    assert np.array_equal(f_a.view(np.uint32), f_b.view(np.uint32))
    for x, y in zip(mom_a, mom_b):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    assert np.array_equal(plot_a.view(np.uint32), plot_b.view(np.uint32))
    assert np.array_equal(val_a.view(np.uint32), val_b.view(np.uint32))
    # the value is the last step's plot-buffer entry at the cursor
    o = CURSOR[0] + NX * (CURSOR[1] + NY * CURSOR[2])
    assert np.array_equal(val_a.view(np.uint32), plot_a.reshape(-1, 4)[o].view(np.uint32))


def test_run_lbm_rejects_a_cursor_outside_the_lattice(pkg):
    L = pkg.lib()
    dd = pkg.DeviceData(19, NX, NY, NZ, plot=True)
    try:
        prm = _params(pkg)
        prm.cursor[2] = NZ
        value = (C.c_float * 4)()
        assert L.lb_run_lbm_d3q19(dd.ptr(), C.c_void_p(dd.plot), C.byref(prm), 2, value) != 0
        assert b"cursor" in L.lb_abi_last_error()
    finally:
        L.lb_abi_clear_error()
        dd.close()
