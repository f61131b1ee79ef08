"""Case files on the CPU: the library's parameter and bitmap readers, initial
states and VTK writer (host code in liblbgb300.so) against the case-file
oracle, on synthetic files covering the formats and on the reference's own
sample cases (fixtures in tests/golden/cases.json and case_masks.npz)."""
import ctypes
import hashlib
import json
import os
import struct

import numpy as np
import pytest

import case_oracle as co
import lb_oracle

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
# the reference's sample cases: present only where the reference tree is (its
# location: LATTIBOL_REF_DIR, else the oracle recipe's default)
SAMPLES = os.path.join(lb_oracle.ref_dir() or "/nonexistent", "samples")


def lib(pkg):
    return pkg.lib()


def load_params(pkg, path):
    p = pkg.abi.lb_case_params()
    rc = lib(pkg).lb_case_load_parameters(os.fsencode(path), ctypes.byref(p))
    return rc, p


def load_mask(pkg, path):
    L = lib(pkg)
    w, h = ctypes.c_int(), ctypes.c_int()
    rc = L.lb_case_load_solids_bmp(os.fsencode(path), ctypes.byref(w), ctypes.byref(h), None, 0)
    if rc != 0:
        return rc, None
    m = np.zeros(w.value * h.value, np.uint8)
    rc = L.lb_case_load_solids_bmp(os.fsencode(path), ctypes.byref(w), ctypes.byref(h),
                                   m.ctypes.data_as(ctypes.c_void_p), m.nbytes)
    return rc, m.reshape(h.value, w.value)


def bits(v):
    return int(np.float32(v).view(np.uint32))


def params_equal(p, o):
    """library struct p vs oracle dict o, floats compared bit for bit"""
    for k in ("device_count", "max_dim", "update_steps"):
        assert getattr(p, k) == o[k], k
    for k in ("ux", "uy", "uz", "rho", "viscosity", "G", "G_ads", "tau_inv", "min_u", "max_u",
              "min_rho", "max_rho"):
        a, b = np.float32(getattr(p, k)), np.float32(o[k])
        assert (np.isnan(a) and np.isnan(b)) or bits(a) == bits(b), (k, a, b)
    for i in range(3):
        assert bits(p.ext_f[i]) == bits(o["ext_f"][i]), ("ext_f", i)


# ------------------------------------------------------------ parameter files

DAT_CASES = {
    "plain": "1\n1\n0.10\n0.00\n0.00\n1.00\n0.03\n1\n",
    "full_crlf": "1\r\n1\r\n0.01\r\n0\r\n0\r\n1.00\r\n0.166667\r\n100\r\n0.000002035\r\n0\r\n"
                 "0\r\n-120\r\n-187.16\r\n",
    "extra_lines": "1\n1\n0\n0\n0\n200\n0.16667\n1\n0\n0\n0\n-120\n0\n0.03333\n1.2\n0\n",
    "int_as_float": "2\n200.00\n 5e-2 \n+0.5\n-.25\n1.\n1e-2\n3.0\n1E-7\n",
    "garbage": "x\n1\nabc\n0x10\n1e\n--1\n1e400\n99999999999\n\n",
    "specials": "-7\n-3\ninf\n-inf\nnan\n3.4e38\n3.5e38\n+12\n1e-46\n1e-40\n",
    "empty": "",
    "no_newline_end": "1\n1\n0.02\n0\n0\n1\n0.035\n10",
    "tabs": "\t1\t\n 1 \n\t0.1 \n",
}


@pytest.mark.parametrize("name", sorted(DAT_CASES))
def test_parameter_reader_vs_oracle(pkg, tmp_path, name):
    path = tmp_path / (name + ".dat")
    path.write_bytes(DAT_CASES[name].encode())
    rc, p = load_params(pkg, path)
    assert rc == 0
    params_equal(p, co.load_parameters(str(path)))


def test_parameter_reader_known_values(pkg, tmp_path):
    path = tmp_path / "k.dat"
    path.write_bytes(DAT_CASES["int_as_float"].encode())
    rc, p = load_params(pkg, path)
    assert rc == 0
    assert p.device_count == 2 and p.max_dim == 1  # "200.00" is not an int: 0 -> 1
    assert p.ux == np.float32(0.05) and p.uy == np.float32(0.5) and p.uz == np.float32(-0.25)
    assert p.update_steps == 0                      # "3.0" is not an int
    assert p.tau_inv == np.float32(1.0 / (3.0 * float(np.float32(0.01)) + 0.5))
    path.write_bytes(DAT_CASES["garbage"].encode())
    rc, p = load_params(pkg, path)
    assert (p.device_count, p.ux, p.uy, p.uz, p.rho, p.viscosity, p.update_steps) == \
        (0, 0, 0, 0, 0, 0, 0)


def test_parameter_reader_missing_file(pkg, tmp_path):
    rc, _ = load_params(pkg, tmp_path / "none.dat")
    assert rc == pkg.abi.LB_ERR_IO
    assert b"cannot open" in lib(pkg).lb_abi_last_error()
    lib(pkg).lb_abi_clear_error()


# --------------------------------------------------------------------- bitmaps

def write_bmp(path, rows, bpp, *, top_down=False, comp=0, masks=None, hsize=40, palette=None):
    """rows: (h, w) array of pixel values (palette indices or packed colours)"""
    h, w = rows.shape
    stride = (w * bpp + 31) // 32 * 4
    data = bytearray()
    order = range(h) if top_down else range(h - 1, -1, -1)
    for y in order:
        r = rows[y]
        line = bytearray()
        if bpp < 8:
            acc, nbit = 0, 0
            for v in r:
                acc = (acc << bpp) | int(v)
                nbit += bpp
                if nbit == 8:
                    line.append(acc)
                    acc, nbit = 0, 0
            if nbit:
                line.append(acc << (8 - nbit))
        else:
            nb = bpp // 8
            for v in r:
                line += int(v).to_bytes(nb, "little")
        line += bytes(stride - len(line))
        data += line
    pal = b""
    if palette is not None:
        pal = b"".join(bytes([bb, gg, rr, 0]) for rr, gg, bb in palette)
    extra = b""
    if comp == 3 and hsize == 40:
        extra = struct.pack("<III", *masks[:3])
    info = struct.pack("<IiiHHIIiiII", hsize, w, -h if top_down else h, 1, bpp, comp,
                       len(data), 2835, 2835, len(palette) if palette else 0, 0)
    if hsize > 40:
        tail = bytearray(hsize - 40)
        if comp == 3:
            tail[0:16] = struct.pack("<IIII", *(list(masks) + [0])[:4])
        info += bytes(tail)
    off = 14 + len(info) + len(extra) + len(pal)
    head = b"BM" + struct.pack("<IHHI", off + len(data), 0, 0, off)
    path.write_bytes(head + info + extra + pal + bytes(data))


def pixel_rows(rng, mask, kind):
    """pixel values that make `mask` the black set for each bitmap kind"""
    h, w = mask.shape
    if kind in ("p1", "p4", "p8"):
        bpp = int(kind[1:])
        n = 1 << bpp
        pal = [tuple(int(c) for c in rng.integers(1, 256, 3)) for _ in range(n)]
        pal[int(rng.integers(0, n))] = (0, 0, 0)
        if n > 2:
            pal[(pal.index((0, 0, 0)) + 1) % n] = (0, 0, 1)  # near-black is fluid
        black = [i for i, c in enumerate(pal) if c == (0, 0, 0)]
        other = [i for i, c in enumerate(pal) if c != (0, 0, 0)]
        rows = np.where(mask, rng.choice(black, mask.shape), rng.choice(other, mask.shape))
        return rows, bpp, dict(palette=pal)
    if kind == "rgb24":
        col = rng.integers(1, 1 << 24, mask.shape)
        return np.where(mask, 0, col), 24, {}
    if kind == "rgb16":
        col = rng.integers(1, 1 << 15, mask.shape)
        return np.where(mask, rng.choice([0, 0x8000], mask.shape), col), 16, {}
    if kind == "rgb32":
        col = rng.integers(1, 1 << 24, mask.shape) | (rng.integers(0, 256, mask.shape) << 24)
        return np.where(mask, rng.integers(0, 256, mask.shape) << 24, col), 32, {}
    if kind == "bf16_565":
        col = rng.integers(1, 1 << 16, mask.shape)
        return (np.where(mask, 0, col), 16,
                dict(comp=3, masks=(0xF800, 0x07E0, 0x001F)))
    if kind == "bf32_alpha":
        # opaque black is solid; transparent black and colours are fluid
        col = rng.integers(1, 1 << 24, mask.shape) | (0xFF << 24)
        transparent = rng.integers(0, 255, mask.shape) << 24
        fluid = np.where(rng.random(mask.shape) < 0.3, transparent, col)
        return (np.where(mask, 0xFF << 24, fluid), 32,
                dict(comp=3, masks=(0xFF0000, 0xFF00, 0xFF, 0xFF000000), hsize=108))
    raise ValueError(kind)


KINDS = ["p1", "p4", "p8", "rgb16", "rgb24", "rgb32", "bf16_565", "bf32_alpha"]


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("top_down", [False, True], ids=["bottom_up", "top_down"])
def test_bmp_reader_vs_oracle(pkg, tmp_path, kind, top_down):
    rng = np.random.default_rng(hash((kind, top_down)) % 2**32)
    for (h, w) in [(7, 13), (20, 33), (1, 1), (64, 40)]:
        mask = (rng.random((h, w)) < 0.4).astype(np.uint8)
        rows, bpp, kw = pixel_rows(rng, mask, kind)
        path = tmp_path / ("%s_%d_%d.bmp" % (kind, h, w))
        write_bmp(path, rows, bpp, top_down=top_down, **kw)
        rc, m = load_mask(pkg, path)
        assert rc == 0, lib(pkg).lb_abi_last_error()
        ow, oh, om = co.load_solids_bmp(str(path))
        assert (ow, oh) == (w, h)
        assert np.array_equal(om, mask)
        assert np.array_equal(m, mask)


def test_bmp_reader_errors(pkg, tmp_path):
    L = lib(pkg)
    w, h = ctypes.c_int(), ctypes.c_int()

    def rc_of(data):
        p = tmp_path / "e.bmp"
        p.write_bytes(data)
        return L.lb_case_load_solids_bmp(os.fsencode(p), ctypes.byref(w), ctypes.byref(h),
                                         None, 0)

    good = tmp_path / "g.bmp"
    write_bmp(good, np.zeros((4, 8), np.int64), 24)
    b = good.read_bytes()
    assert rc_of(b) == 0 and (w.value, h.value) == (8, 4)
    assert rc_of(b"GIF89a" + b[6:]) == pkg.abi.LB_ERR_IO
    assert rc_of(b[:-5]) == pkg.abi.LB_ERR_IO                      # truncated pixels
    rle = bytearray(b)
    rle[30:34] = struct.pack("<I", 1)                               # BI_RLE8
    assert rc_of(bytes(rle)) == pkg.abi.LB_ERR_IO
    assert b"compression" in L.lb_abi_last_error()
    assert L.lb_case_load_solids_bmp(os.fsencode(tmp_path / "none.bmp"), ctypes.byref(w),
                                     ctypes.byref(h), None, 0) == pkg.abi.LB_ERR_IO
    # a buffer smaller than the image is an argument error
    m = np.zeros(8, np.uint8)
    assert L.lb_case_load_solids_bmp(os.fsencode(good), ctypes.byref(w), ctypes.byref(h),
                                     m.ctypes.data_as(ctypes.c_void_p), 8) == pkg.abi.LB_ERR_ARG
    L.lb_abi_clear_error()


# -------------------------------------------------------- the sample fixtures

def fixtures():
    with open(os.path.join(GOLDEN, "cases.json")) as fh:
        cases = json.load(fh)
    masks = np.load(os.path.join(GOLDEN, "case_masks.npz"))
    return cases, masks


def fixture_params(entry):
    out = {}
    for k, v in entry["params"].items():
        if isinstance(v, list):
            out[k] = [np.uint32(int(x, 16)).view(np.float32) for x in v]
        elif isinstance(v, str):
            out[k] = np.uint32(int(v, 16)).view(np.float32)
        else:
            out[k] = v
    return out


def fixture_mask(entry, masks):
    w, h = entry["width"], entry["height"]
    m = np.unpackbits(masks["m_" + entry["mask"]])[:w * h].reshape(h, w)
    assert hashlib.sha256(m.tobytes()).hexdigest() == entry["sha256"]
    return m


def params_struct(pkg, p):
    s = pkg.abi.lb_case_params()
    for k, v in p.items():
        if k == "ext_f":
            for i in range(3):
                s.ext_f[i] = float(v[i])
        else:
            setattr(s, k, v if isinstance(v, int) else float(v))
    return s


def test_fixtures_self_consistent():
    cases, masks = fixtures()
    n2d = 0
    for e in cases:
        if "width" in e:
            m = fixture_mask(e, masks)
            assert int(m.sum()) == e["solids"]
            n2d += 1
    assert n2d >= 20 and len(cases) >= 30


@pytest.mark.skipif(not os.path.isdir(SAMPLES), reason="reference samples not present")
def test_library_reads_every_sample_like_the_fixtures(pkg):
    cases, masks = fixtures()
    for e in cases:
        rc, p = load_params(pkg, os.path.join(SAMPLES, e["name"]))
        assert rc == 0
        params_equal(p, fixture_params(e))
        if "width" in e:
            rc, m = load_mask(pkg, os.path.join(SAMPLES, e["name"][:-3] + "bmp"))
            assert rc == 0
            assert hashlib.sha256(m.tobytes()).hexdigest() == e["sha256"], e["name"]


# ------------------------------------------------------------ initial states

def lib_init_d2q9(pkg, p, mask):
    H, W = mask.shape
    N = W * H
    out = dict(f=np.zeros((9, N), np.float32), solid_bound=np.zeros(N, np.uint8))
    for k in ("ux", "uy", "rho", "psi", "ueq_x", "ueq_y"):
        out[k] = np.zeros(N, np.float32)
    m = np.ascontiguousarray(mask.reshape(-1), np.uint8)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    s = params_struct(pkg, p)
    rc = lib(pkg).lb_case_init_d2q9(ctypes.byref(s), W, H, P(m), P(out["f"]), P(out["ux"]),
                                    P(out["uy"]), P(out["rho"]), P(out["psi"]),
                                    P(out["ueq_x"]), P(out["ueq_y"]), P(out["solid_bound"]))
    assert rc == 0
    return out


def same(a, b):
    return np.array_equal(np.asarray(a).view(np.uint8), np.asarray(b).view(np.uint8))


def check_init_d2q9(pkg, p, mask):
    got = lib_init_d2q9(pkg, p, mask)
    exp = co.init_d2q9(p, mask)
    for k in exp:
        assert same(got[k], exp[k]), k
    return got


def test_init_d2q9_every_sample_vs_oracle(pkg):
    cases, masks = fixtures()
    seen = set()
    for e in cases:
        if "width" not in e:
            continue
        key = (e["mask"], json.dumps(e["params"], sort_keys=True))
        if key in seen:
            continue
        seen.add(key)
        check_init_d2q9(pkg, fixture_params(e), fixture_mask(e, masks))


def synthetic_params(**kw):
    p = dict(device_count=1, max_dim=1, ux=np.float32(0.01), uy=np.float32(-0.003),
             uz=np.float32(0), rho=np.float32(200), viscosity=np.float32(0.16667),
             update_steps=1, ext_f=[np.float32(2e-6), np.float32(-1e-6), np.float32(0)],
             G=np.float32(-120), G_ads=np.float32(-187.16), min_u=np.float32(0),
             max_u=np.float32(0), min_rho=np.float32(0), max_rho=np.float32(0))
    p.update(kw)
    p["tau_inv"] = np.float32(1.0 / (3.0 * float(p["viscosity"]) + 0.5))
    return p


@pytest.mark.parametrize("node0", ["fluid_near_wall", "solid", "fluid_free"])
@pytest.mark.parametrize("G", [-120.0, 0.0])
def test_init_d2q9_synthetic_vs_oracle(pkg, node0, G):
    rng = np.random.default_rng(3)
    H, W = 24, 40
    mask = (rng.random((H, W)) < 0.15).astype(np.uint8)
    mask[0, :] = 0
    mask[:, 0] = 0
    if node0 == "fluid_near_wall":
        mask[0, 1] = 1       # node 0 fluid with a solid neighbour: adhesion moves the base
        mask[1, 1] = 1
    elif node0 == "solid":
        mask[0, 0] = 1
    else:
        mask[1, :3] = 0
        mask[H - 1, :3] = 0
        mask[:3, W - 1] = 0
    got = check_init_d2q9(pkg, synthetic_params(G=np.float32(G)), mask)
    if G != 0 and node0 == "fluid_near_wall":
        # the base u_eq carries node 0's adhesion shift to every fluid node
        free = co.init_d2q9(synthetic_params(G=np.float32(G)), np.zeros_like(mask))
        assert got["ueq_x"][5 * W + 20] != free["ueq_x"][5 * W + 20] or \
            got["ueq_y"][5 * W + 20] != free["ueq_y"][5 * W + 20]


def test_init_d3q19_vs_oracle(pkg):
    rng = np.random.default_rng(5)
    D, H, W = 6, 7, 9
    mask = (rng.random((D, H, W)) < 0.5).astype(np.uint8)
    mask[:, :, 3:6] = 1
    p = synthetic_params(ux=np.float32(0.05), uy=np.float32(-0.02), uz=np.float32(0.013),
                         rho=np.float32(1.02), G=np.float32(0))
    N = W * H * D
    out = dict(f=np.zeros((19, N), np.float32), solid_bound=np.zeros(N, np.uint8))
    for k in ("ux", "uy", "uz", "rho"):
        out[k] = np.zeros(N, np.float32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    m = np.ascontiguousarray(mask.reshape(-1))
    s = params_struct(pkg, p)
    assert lib(pkg).lb_case_init_d3q19(ctypes.byref(s), W, H, D, P(m), P(out["f"]),
                                       P(out["ux"]), P(out["uy"]), P(out["uz"]), P(out["rho"]),
                                       P(out["solid_bound"])) == 0
    exp = co.init_d3q19(p, mask)
    for k in exp:
        assert same(out[k], exp[k]), k
    assert out["solid_bound"].sum() > 0


# ------------------------------------------------------------------------ VTK

@pytest.mark.parametrize("dims", [(5, 3, 1), (4, 3, 2)], ids=["2d", "3d"])
def test_vtk_writer_vs_oracle(pkg, tmp_path, dims):
    W, H, Lz = dims
    rng = np.random.default_rng(8)
    n = W * H * Lz
    f = [(rng.standard_normal(n) * 10.0 ** rng.integers(-8, 4, n)).astype(np.float32)
         for _ in range(4)]
    f[2][:2] = [0.0, -0.0]
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    L = lib(pkg)
    for dev in (0, 3):
        uz = P(f[3]) if Lz > 1 else None
        assert L.lb_vtk_save(os.fsencode(tmp_path), 42, dev, W, H, Lz, P(f[0]), P(f[1]),
                             P(f[2]), uz) == 0
        text = (tmp_path / ("r0042p%02d.vti" % dev)).read_text()
        assert text == co.vtk_text(dev, W, H, Lz, f[0], f[1], f[2], f[3] if Lz > 1 else None)
    assert L.lb_vtk_save_parallel(os.fsencode(tmp_path), 42, 4, W, H, Lz) == 0
    assert (tmp_path / "r0042.pvti").read_text() == co.pvti_text(42, 4, W, H, Lz)
    assert L.lb_vtk_save(os.fsencode(tmp_path), 10000, 0, W, H, Lz, P(f[0]), P(f[1]),
                         P(f[2]), P(f[3])) == pkg.abi.LB_ERR_ARG
    assert L.lb_vtk_save(os.fsencode(tmp_path / "missing_dir"), 1, 0, W, H, Lz, P(f[0]),
                         P(f[1]), P(f[2]), P(f[3])) == pkg.abi.LB_ERR_IO
    L.lb_abi_clear_error()


def test_output_mirror_names_files_like_the_reference(pkg, tmp_path):
    inp = pkg.Input()
    inp.setSolids(np.zeros((3, 4), np.uint8))
    out = pkg.Output(inp)
    z = np.zeros(12, np.float32)
    out.saveParVTK(str(tmp_path))
    out.saveVTK(0, z, z, z, directory=str(tmp_path))
    out.saveVTK(0, z, z, z, directory=str(tmp_path))
    assert sorted(os.listdir(tmp_path)) == ["r0000.pvti", "r0000p00.vti", "r0001p00.vti"]


# ------------------------------------------------------- the Input mirror

def test_input_mirror_loads_a_case(pkg, tmp_path):
    rng = np.random.default_rng(1)
    mask = (rng.random((10, 16)) < 0.3).astype(np.uint8)
    rows, bpp, kw = pixel_rows(rng, mask, "p1")
    write_bmp(tmp_path / "c.bmp", rows, bpp, **kw)
    (tmp_path / "c.dat").write_bytes(DAT_CASES["full_crlf"].encode())
    inp = pkg.Input().loadFile(str(tmp_path / "c.dat"))
    assert (inp.getWidth(), inp.getHeight(), inp.getLength()) == (16, 10, 1)
    assert np.array_equal(inp.getSolids()[0], mask)
    assert inp.getG() == np.float32(-120) and inp.getUpdateSteps() == 100
    assert inp.getExtFx() == np.float32(0.000002035)
    inp.setViscosity(0.1)
    assert inp.getTauInv() == np.float32(1.0 / (3.0 * float(np.float32(0.1)) + 0.5))
    assert not pkg.Input().loadParameters(str(tmp_path / "none.dat"))
    assert not pkg.Input().loadSolids(str(tmp_path / "c.dat"))


def test_checkpoint_info_rejects_non_checkpoints(pkg, tmp_path):
    L = lib(pkg)
    cfg = pkg.abi.lb_config()
    steps = ctypes.c_int64()
    p = tmp_path / "x.ckpt"
    p.write_bytes(b"LBGBCKPT" + bytes(100))
    assert L.lb_checkpoint_info(os.fsencode(p), ctypes.byref(cfg), ctypes.byref(steps)) == \
        pkg.abi.LB_ERR_IO
    assert L.lb_checkpoint_info(os.fsencode(tmp_path / "none"), ctypes.byref(cfg),
                                ctypes.byref(steps)) == pkg.abi.LB_ERR_IO
    L.lb_abi_clear_error()


# ------------------------------------------------------------------ STL files

def stl_fixtures():
    return np.load(os.path.join(GOLDEN, "case_stl.npz"))


def lib_read_stl(pkg, path):
    L = lib(pkg)
    n = ctypes.c_int64()
    assert L.lb_stl_read(os.fsencode(path), ctypes.byref(n), None, 0) == 0
    tri = np.zeros(9 * n.value, np.float32)
    assert L.lb_stl_read(os.fsencode(path), ctypes.byref(n),
                         tri.ctypes.data_as(ctypes.c_void_p), tri.size) == 0
    return tri.reshape(-1, 3, 3)


def write_binary_stl(path, tri, header=b"binary"):
    tri = np.asarray(tri, np.float32).reshape(-1, 3, 3)
    rec = np.zeros(len(tri), np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")]))
    rec["v"] = tri
    path.write_bytes(header.ljust(80, b" ") + struct.pack("<I", len(tri)) + rec.tobytes())


def write_ascii_stl(path, tri):
    lines = ["solid test"]
    for t in np.asarray(tri, np.float32).reshape(-1, 3, 3):
        lines += ["  facet normal 0 0 0", "    outer loop"]
        lines += ["      vertex %.9g %.9g %.9g" % tuple(float(c) for c in v) for v in t]
        lines += ["    endloop", "  endfacet"]
    path.write_text("\n".join(lines + ["endsolid test", ""]))


def test_stl_reader_binary_ascii_and_solid_header(pkg, tmp_path):
    rng = np.random.default_rng(2)
    tri = rng.standard_normal((37, 3, 3)).astype(np.float32) * 10
    write_binary_stl(tmp_path / "b.stl", tri)
    write_binary_stl(tmp_path / "s.stl", tri, header=b"solid but binary")
    write_ascii_stl(tmp_path / "a.stl", tri)
    for name in ("b.stl", "s.stl", "a.stl"):
        got = lib_read_stl(pkg, tmp_path / name)
        assert np.array_equal(got, co.read_stl(str(tmp_path / name))), name
        assert np.array_equal(got, tri), name
    n = ctypes.c_int64()
    assert lib(pkg).lb_stl_read(os.fsencode(tmp_path / "none.stl"), ctypes.byref(n), None, 0) \
        == pkg.abi.LB_ERR_IO
    lib(pkg).lb_abi_clear_error()


@pytest.mark.skipif(not os.path.isdir(SAMPLES), reason="reference samples not present")
def test_library_reads_every_sample_stl_like_the_fixtures(pkg):
    cases, _ = fixtures()
    surf = stl_fixtures()
    for e in cases:
        if "stl" in e:
            got = lib_read_stl(pkg, os.path.join(SAMPLES, e["name"][:-3] + "stl"))
            assert np.array_equal(got, surf[e["stl"]]), e["name"]


def test_voxel_grid_dims_vs_oracle(pkg):
    """lb_voxelize with no output buffer computes the grid on the host."""
    cases, _ = fixtures()
    surf = stl_fixtures()
    n3d = 0
    for e in cases:
        if "stl" not in e:
            continue
        tri = np.ascontiguousarray(surf[e["stl"]], np.float32)
        dims = (ctypes.c_int * 3)()
        assert lib(pkg).lb_voxelize(tri.ctypes.data_as(ctypes.c_void_p), len(tri),
                                    e["params"]["max_dim"], dims, None, 0, None) == 0
        _, _, want = co.voxel_grid(tri, e["params"]["max_dim"])
        assert list(dims) == want == e["stl_dims"], e["name"]
        n3d += 1
    assert n3d >= 6


def test_oracle_voxeliser_on_closed_shapes():
    """The oracle voxeliser on shapes whose solid voxels are known: an
    axis-aligned box, and a box with a box-shaped hole (two closed surfaces),
    faces between voxel centres."""
    def box(lo, hi):
        x0, y0, z0 = lo
        x1, y1, z1 = hi
        v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                      [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], np.float32)
        f = [(0, 2, 1), (0, 3, 2), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4),
             (2, 3, 7), (2, 7, 6), (1, 2, 6), (1, 6, 5), (3, 0, 4), (3, 4, 7)]
        return v[np.array(f)]
    # the bounding box is the box itself: 20 x 10 x 6 units, max_dim 20 -> 1 unit voxels
    m = co.voxelize(box((0, 0, 0), (20, 10, 6)), 20)
    assert m.shape == (6, 10, 20) and m.all()
    # a box inside a larger frame box (two closed surfaces): the inner one is a hole
    tri = np.concatenate([box((0, 0, 0), (20, 10, 6)), box((5, 2, 1), (15, 8, 5))])
    m = co.voxelize(tri, 20)
    hole = np.zeros((6, 10, 20), bool)
    hole[1:5, 2:8, 5:15] = True
    assert np.array_equal(m.astype(bool), ~hole)
