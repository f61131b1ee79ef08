"""GPU: the reference's sample cases run headless through the drop-in entry
points (Input -> SimulationD2Q9/D3Q19 -> runLBM; 3-D solids voxelised from
the cases' STL surfaces on the GPU), bit-exact against the oracle;
checkpoint/resume bit-identity; VTK output of a context."""
import json
import os

import numpy as np
import pytest

import case_oracle as co
from test_case_files import fixture_mask, fixture_params, fixtures

pytestmark = pytest.mark.gpu

STEPS = 16


def beq(a, b):
    """bit-identical, except that a NaN matches any NaN: the bit pattern of a
    NaN made by an invalid operation differs between the GPU and the host CPU
    (two sample cases, the 0 and 90 degree contact angles, go non-finite
    within 16 steps in the reference's own semantics)"""
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype != np.float32:
        return np.array_equal(a.view(np.uint8), b.view(np.uint8))
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint32),
                                                     b[~nb].view(np.uint32))


def distinct_2d_cases():
    cases, masks = fixtures()
    seen, out = set(), []
    for e in cases:
        if "width" not in e:
            continue
        key = (e["mask"], json.dumps(e["params"], sort_keys=True))
        if key not in seen:
            seen.add(key)
            out.append(e)
    return out, masks


def make_input(pkg, p, mask):
    inp = pkg.Input()
    for k, v in p.items():
        if k == "ext_f":
            for i in range(3):
                inp.p.ext_f[i] = float(v[i])
        else:
            setattr(inp.p, k, v if isinstance(v, int) else float(v))
    inp.setSolids(mask)
    return inp


def oracle_run(oracle, pkg, p, mask, steps):
    """the reference loop (stream, collide) on the oracle from the case's
    initial state"""
    H, W = mask.shape
    init = co.init_d2q9(p, mask)
    f = init["f"].copy()
    mom = [init[k].copy() for k in ("ux", "uy", "rho")]
    sc = [init[k].copy() for k in ("psi", "ueq_x", "ueq_y")]
    solid = np.ascontiguousarray(mask.reshape(-1), np.uint8)
    plot = np.zeros(4 * W * H, np.float32)
    for _ in range(steps):
        oracle.d2q9_stream(f, init["solid_bound"], W, H)
        oracle.d2q9_collide(f, solid, mom, sc, W, H, *pkg.W2, p["tau_inv"], p["ux"], p["uy"],
                            p["rho"], p["ext_f"][0], p["ext_f"][1], p["G"], p["G_ads"],
                            plot=plot)
    return f, mom, sc, plot


@pytest.mark.parametrize("mode", [0, 1], ids=["standalone", "fused"])
def test_sample_cases_vs_oracle(pkg, oracle, mode):
    """Every distinct 2-D sample case of the reference (its .dat parameters
    and .bmp solids) for 16 steps of the reference's own loop: populations,
    moments, Shan-Chen fields and the plot buffer bit-identical."""
    L = pkg.lib()
    cases, masks = distinct_2d_cases()
    assert len(cases) >= 15
    assert L.lb_abi_set_mode(mode) == 0
    try:
        for e in cases:
            p, mask = fixture_params(e), fixture_mask(e, masks)
            sim = pkg.SimulationD2Q9(make_input(pkg, p, mask))
            sim.runLBM(STEPS)
            assert sim.getSteps() == STEPS
            f, mom, sc, plot = oracle_run(oracle, pkg, p, mask, STEPS)
            assert L.lb_abi_release_d2q9(sim.data.ptr()) == 0
            assert beq(sim.populations(), f), e["name"]
            for k, a in zip(("ux", "uy", "rho"), mom):
                assert beq(sim.field(k), a), (e["name"], k)
            if p["G"] < 0:
                for k, a in zip(("psi", "ueq_x", "ueq_y"), sc):
                    assert beq(sim.field(k), a), (e["name"], k)
            assert beq(sim.data.plot_data(), plot), e["name"]
            sim.close()
    finally:
        L.lb_abi_set_mode(0)


def test_sample_case_vtk_output(pkg, tmp_path):
    """SimulationD2Q9.saveVTK writes the reference's file pair from the
    device moments."""
    cases, masks = distinct_2d_cases()
    e = min(cases, key=lambda c: c["width"] * c["height"])
    p, mask = fixture_params(e), fixture_mask(e, masks)
    sim = pkg.SimulationD2Q9(make_input(pkg, p, mask))
    sim.runLBM(3)
    sim.saveVTK(str(tmp_path))
    H, W = mask.shape
    text = (tmp_path / "r0000p00.vti").read_text()
    assert text == co.vtk_text(0, W, H, 1, sim.field("rho"), sim.field("ux"), sim.field("uy"))
    assert (tmp_path / "r0000.pvti").read_text() == co.pvti_text(0, 1, W, H, 1)
    sim.close()


# ----------------------------------------------------------------- checkpoints

def lattice_cases(pkg):
    a = pkg.abi
    rng = np.random.default_rng(21)
    out = []
    # D3Q19 channel: walls in y, a moving wall, body force
    W, H, D = 40, 20, 12
    fl = np.zeros((D, H, W), np.uint8)
    fl[:, 0, :] = a.LB_CELL_WALL
    fl[:, H - 1, :] = a.LB_CELL_WALL | a.LB_CELL_MOVING
    out.append(("d3q19_native_f32", dict(lattice=19, nx=W, ny=H, nz=D, tau_inv=1 / 0.6,
                                         force=(1e-5, 0, 0), wall_u=(0.05, 0, 0)),
                fl.reshape(-1), None))
    # D3Q19 Shan-Chen with bf16 storage
    n = 24 ** 3
    rho = (0.693 * (1 + 0.01 * (2 * rng.random(n) - 1))).astype(np.float32)
    out.append(("d3q19_sc_bf16", dict(lattice=19, nx=24, ny=24, nz=24, tau_inv=1.0, G=-5.0,
                                      storage=a.LB_STORE_BF16, rho_ref=0.693),
                np.zeros(n, np.uint8), rho))
    # D3Q19 Shan-Chen FP32 on a wall-free lattice the staged single-pass step tiles
    n3 = 32 * 16 * 12
    rho3 = (0.693 * (1 + 0.01 * (2 * rng.random(n3) - 1))).astype(np.float32)
    out.append(("d3q19_sc_staged_f32", dict(lattice=19, nx=32, ny=16, nz=12, tau_inv=1.0,
                                            G=-5.0, force=(1e-6, 0, 0)),
                np.zeros(n3, np.uint8), rho3))
    # D2Q9 in the reference's semantics: Zou-He, solids, Shan-Chen
    W2, H2 = 48, 32
    sol = (rng.random((H2, W2)) < 0.08).astype(np.uint8)
    out.append(("d2q9_reference_sc", dict(lattice=9, nx=W2, ny=H2, mode=a.LB_MODE_REFERENCE,
                                          tau_inv=1 / (3 * 0.16667 + 0.5), G=-120.0,
                                          rho_out=200.0, psi_form=a.LB_PSI_REF),
                sol.reshape(-1), np.full(W2 * H2, 200.0, np.float32)))
    return out


def build(pkg, kw, flags, rho):
    kw = dict(kw)
    lat = pkg.Lattice(kw.pop("lattice"), kw.pop("nx"), kw.pop("ny"), kw.pop("nz", 1),
                      graph_steps=4, **kw)
    lat.set_flags(flags)
    lat.init_equilibrium(rho=rho)
    return lat


@pytest.mark.parametrize("idx", [0, 1, 2, 3], ids=["d3q19_native_f32", "d3q19_sc_bf16",
                                                   "d3q19_sc_staged_f32", "d2q9_reference_sc"])
def test_checkpoint_resume_is_bit_identical(pkg, tmp_path, idx):
    name, kw, flags, rho = lattice_cases(pkg)[idx]
    K = 9
    a = build(pkg, kw, flags, rho)
    a.step(2 * K)
    ref_f, ref_m = a.populations(), a.moments()
    a.close()

    b = build(pkg, kw, flags, rho)
    b.step(K)
    path = tmp_path / (name + ".ckpt")
    b.save_checkpoint(path)
    mid_f = b.populations()
    b.close()
    assert not os.path.exists(str(path) + ".tmp")

    c = pkg.Lattice.from_checkpoint(path)
    assert c.steps_done() == K
    assert beq(c.populations(), mid_f)
    c.step(K)
    assert c.steps_done() == 2 * K
    assert beq(c.populations(), ref_f)
    for x, y in zip(c.moments(), ref_m):
        if x is not None:
            assert beq(x, y)
    c.close()

    # into an existing context of the same lattice; a damaged copy and a
    # lattice of another size are refused and leave the context as it was
    d = build(pkg, kw, flags, rho)
    before = d.populations()
    bad = tmp_path / "damaged.ckpt"
    raw = bytearray(path.read_bytes())
    raw[256 + d.N + 7] ^= 0x10
    bad.write_bytes(bytes(raw))
    assert d.load_checkpoint(bad) == pkg.abi.LB_ERR_IO
    assert beq(d.populations(), before)
    assert d.load_checkpoint(path) == pkg.abi.LB_OK
    assert beq(d.populations(), mid_f) and d.steps_done() == K
    d.close()
    kw2 = dict(kw, nx=kw["nx"] + 1)
    e = pkg.Lattice(kw2.pop("lattice"), kw2.pop("nx"), kw2.pop("ny"), kw2.pop("nz", 1), **kw2)
    assert e.load_checkpoint(path) == pkg.abi.LB_ERR_ARG
    e.close()


def test_context_vtk_matches_oracle(pkg, tmp_path):
    name, kw, flags, rho = lattice_cases(pkg)[0]
    lat = build(pkg, kw, flags, rho)
    lat.step(5)
    lat.save_vtk(str(tmp_path), 7)
    r, ux, uy, uz = lat.moments()
    text = (tmp_path / "r0007p00.vti").read_text()
    assert text == co.vtk_text(0, kw["nx"], kw["ny"], kw["nz"], r, ux, uy, uz)
    lat.close()


# ----------------------------------------------------------------- 3-D cases

def gpu_voxelize(pkg, tri, max_dim):
    import ctypes
    L = pkg.lib()
    tri = np.ascontiguousarray(tri, np.float32)
    P = tri.ctypes.data_as(ctypes.c_void_p)
    dims = (ctypes.c_int * 3)()
    assert L.lb_voxelize(P, len(tri), max_dim, dims, None, 0, None) == 0
    W, H, D = dims
    m = np.zeros(W * H * D, np.uint8)
    opn = ctypes.c_int(-1)
    assert L.lb_voxelize(P, len(tri), max_dim, dims, m.ctypes.data_as(ctypes.c_void_p),
                         m.nbytes, ctypes.byref(opn)) == 0, L.lb_abi_last_error()
    return m.reshape(D, H, W), opn.value


def box(lo, hi):
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], np.float32)
    f = [(0, 2, 1), (0, 3, 2), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4),
         (2, 3, 7), (2, 7, 6), (1, 2, 6), (1, 6, 5), (3, 0, 4), (3, 4, 7)]
    return v[np.array(f)]


def test_voxelize_boxes_and_random_surfaces_vs_oracle(pkg):
    m, opn = gpu_voxelize(pkg, box((0, 0, 0), (20, 10, 6)), 20)
    assert m.shape == (6, 10, 20) and m.all() and opn == 0
    # a hole whose faces pass through voxel centres, and a rotated box: the
    # tie rule and the fixed-point depths must give the oracle's voxels
    rng = np.random.default_rng(12)
    rot = np.linalg.qr(rng.standard_normal((3, 3)))[0].astype(np.float32)
    shapes = [np.concatenate([box((0, 0, 0), (20, 10, 6)), box((5.5, 2.5, 1.5), (14.5, 7.5, 4.5))]),
              (box((-3, -2, -1), (3, 2, 1)) @ rot.T).astype(np.float32)]
    for tri, md in zip(shapes, (20, 48)):
        m, opn = gpu_voxelize(pkg, tri, md)
        assert opn == 0
        assert np.array_equal(m, co.voxelize(tri, md))


def test_voxelize_sample_surfaces_like_the_fixtures(pkg):
    import hashlib
    cases, _ = fixtures()
    surf = np.load(os.path.join(os.path.dirname(__file__), "golden", "case_stl.npz"))
    n = 0
    for e in cases:
        if "stl" not in e:
            continue
        m, _ = gpu_voxelize(pkg, surf[e["stl"]], e["params"]["max_dim"])
        assert list(m.shape[::-1]) == e["stl_dims"], e["name"]
        assert hashlib.sha256(m.tobytes()).hexdigest() == e["stl_sha256"], e["name"]
        n += 1
    assert n >= 6


STEPS3 = 8


@pytest.mark.parametrize("mode", [0, 1], ids=["standalone", "fused"])
def test_3d_sample_cases_vs_oracle(pkg, oracle, mode):
    """The reference's 3-D sample cases (the .dat parameters, the STL surface
    voxelised on the GPU) for 8 steps of SimulationD3Q19.runLBM through the
    drop-in, bit-exact against the oracle from the same initial state."""
    cases, _ = fixtures()
    surf = np.load(os.path.join(os.path.dirname(__file__), "golden", "case_stl.npz"))
    L = pkg.lib()
    seen = set()
    assert L.lb_abi_set_mode(mode) == 0
    try:
        for e in cases:
            if "stl" not in e:
                continue
            key = (e["stl"], json.dumps(e["params"], sort_keys=True))
            if key in seen:
                continue
            seen.add(key)
            p = fixture_params(e)
            mask, _ = gpu_voxelize(pkg, surf[e["stl"]], p["max_dim"])
            D, H, W = mask.shape
            sim = pkg.SimulationD3Q19(make_input(pkg, p, mask))
            sim.runLBM(STEPS3)
            init = co.init_d3q19(p, mask)
            f = init["f"].copy()
            mom = [init[k].copy() for k in ("ux", "uy", "uz", "rho")]
            solid = np.ascontiguousarray(mask.reshape(-1), np.uint8)
            plot = np.zeros(4 * W * H * D, np.float32)
            for _ in range(STEPS3):
                oracle.d3q19_stream(f, init["solid_bound"], W, H, D)
                oracle.d3q19_collide(f, solid, mom, W, H, D, *pkg.W3, p["tau_inv"], p["ux"],
                                     p["uy"], p["uz"], p["rho"], plot=plot)
            assert L.lb_abi_release_d3q19(sim.data.ptr()) == 0
            assert beq(sim.populations(), f), e["name"]
            for k, a in zip(("ux", "uy", "uz", "rho"), mom):
                assert beq(sim.field(k), a), (e["name"], k)
            assert beq(sim.data.plot_data(), plot), e["name"]
            sim.close()
        assert len(seen) >= 6
    finally:
        L.lb_abi_set_mode(0)
