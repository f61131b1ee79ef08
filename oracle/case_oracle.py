"""Oracle for the case files and output files (TEST INFRASTRUCTURE ONLY).

A CPU restatement, in numpy, of the reference's host-side case handling:

* the parameter file reader, reference src/input.cpp:51-94
  (Input::loadParameters; Qt's QString::toInt / toFloat rules as of the Qt 5
  the reference was written against: surrounding white space is ignored, a
  line that is not a number or is missing reads as 0, a finite value beyond
  the float range reads as 0);
* the bitmap solid mask, reference src/input.cpp:96-116 (Input::loadSolids: a
  node is solid where the pixel equals opaque black, y = 0 the top row);
* the initial states of reference src/simulation_d2q9.cu:100-334 and
  src/simulation_d3q19.cu:99-204 (one device, the whole width), with every
  float and double operation in the reference's order and type;
* the VTK text of reference src/output.cpp:52-155 (saveParVTK, saveVTK).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline may use this
module, and only to verify results against.
"""
import math
import re
import struct

import numpy as np

F32 = np.float32
F64 = np.float64
FLT_MAX = float(np.finfo(np.float32).max)

_INT = re.compile(r"^[+-]?[0-9]+$")
_FLOAT = re.compile(r"^[+-]?([0-9]+\.?[0-9]*|\.[0-9]+)([eE][+-]?[0-9]+)?$")
_WS = " \t\n\v\f\r"


def q_to_int(text):
    """QString::toInt (base 10): 0 unless the trimmed text is a decimal int."""
    t = text.strip(_WS)
    if not _INT.match(t):
        return 0
    v = int(t)
    return v if -2**31 <= v < 2**31 else 0


def q_to_float(text):
    """QString::toFloat: the C-locale number, via double, to float; 0 when the
    text is not a number or the value is finite and beyond the float range."""
    t = text.strip(_WS)
    low = t.lower()
    body = low[1:] if low[:1] in "+-" else low
    if body in ("inf", "infinity"):
        return F32(-np.inf) if low.startswith("-") else F32(np.inf)
    if body == "nan":
        return F32(np.nan)
    if not _FLOAT.match(t):
        return F32(0)
    d = float(t)
    if math.isinf(d) or abs(d) > FLT_MAX:
        return F32(0)
    return F32(d)


def read_lines(path):
    """The lines as a Qt text stream returns them (no "\\n" / "\\r\\n")."""
    with open(path, "rb") as fh:
        raw = fh.read().decode("latin-1")
    lines = raw.split("\n")
    return [ln[:-1] if ln.endswith("\r") else ln for ln in lines]


def load_parameters(path):
    """Input::loadParameters, reference src/input.cpp:51-94."""
    lines = read_lines(path)

    def line(i):
        return lines[i] if i < len(lines) else ""

    p = {}
    p["device_count"] = q_to_int(line(0))
    md = q_to_int(line(1))
    p["max_dim"] = md if md > 1 else 1               # src/input.cpp:149-152
    p["ux"], p["uy"], p["uz"] = (q_to_float(line(i)) for i in (2, 3, 4))
    p["rho"] = q_to_float(line(5))
    p["viscosity"] = q_to_float(line(6))
    p["tau_inv"] = F32(1.0 / (3.0 * float(p["viscosity"]) + 0.5))  # src/input.cpp:168-171
    p["update_steps"] = q_to_int(line(7))
    p["ext_f"] = [q_to_float(line(i)) for i in (8, 9, 10)]
    p["G"] = q_to_float(line(11))
    p["G_ads"] = q_to_float(line(12))
    p["min_u"] = F32(0.0)
    with np.errstate(over="ignore"):        # beyond float: inf, as the C cast gives
        p["max_u"] = F32(float(p["ux"]) * 1.5)
        p["min_rho"] = F32(float(p["rho"]) * 0.98)
        p["max_rho"] = F32(float(p["rho"]) * 1.02)
    return p


# ------------------------------------------------------------------ bitmaps

def load_solids_bmp(path):
    """(width, height, mask) with mask[y, x] = 1 where the pixel is opaque
    black; y = 0 is the image's top row.  Uncompressed 1/4/8/16/24/32 bpp and
    BI_BITFIELDS 16/32."""
    with open(path, "rb") as fh:
        b = fh.read()
    if len(b) < 26 or b[:2] != b"BM":
        raise ValueError("not a Windows bitmap")
    off_bits, hsize = struct.unpack_from("<II", b, 10)
    comp, clr_used, entry = 0, 0, 4
    if hsize == 12:
        w, h, _planes, bpp = struct.unpack_from("<HhHH", b, 18)
        entry = 3
    elif 40 <= hsize <= 124:
        w, h, _planes, bpp, comp = struct.unpack_from("<iiHHI", b, 18)
        clr_used = struct.unpack_from("<I", b, 46)[0]
    else:
        raise ValueError("unsupported header size")
    if w <= 0 or h == 0:
        raise ValueError("bad size")
    top_down = h < 0
    h = abs(h)
    if bpp not in (1, 4, 8, 16, 24, 32):
        raise ValueError("unsupported depth")
    masks = None
    if comp == 3:
        if bpp not in (16, 32):
            raise ValueError("bitfields need 16/32 bpp")
        rm, gm, bm = struct.unpack_from("<III", b, 54)
        am = struct.unpack_from("<I", b, 66)[0] if hsize >= 56 else 0
        masks = (rm, gm, bm, am)
    elif comp == 0:
        if bpp == 16:
            masks = (0x7C00, 0x03E0, 0x001F, 0)
        elif bpp == 32:
            masks = (0xFF0000, 0xFF00, 0xFF, 0)
    else:
        raise ValueError("unsupported compression")
    stride = (w * bpp + 31) // 32 * 4
    if off_bits + stride * h > len(b):
        raise ValueError("truncated")
    rows = np.frombuffer(b, np.uint8, count=stride * h, offset=off_bits).reshape(h, stride)
    if not top_down:
        rows = rows[::-1]                      # file order is bottom-up
    if bpp <= 8:
        ncol = clr_used if clr_used else (1 << bpp)
        po = 14 + hsize
        pal = np.frombuffer(b, np.uint8, count=ncol * entry, offset=po).reshape(ncol, entry)
        black = np.all(pal[:, :3] == 0, axis=1)
        bits = np.unpackbits(rows, axis=1)     # MSB first
        idx = np.zeros((h, w), np.int64)
        for j in range(bpp):
            idx = (idx << 1) | bits[:, j:w * bpp:bpp][:, :w]
        black_ext = np.concatenate([black, np.zeros(256, bool)])
        mask = black_ext[idx]                  # an index past the table is not black
    elif bpp == 24:
        px = rows[:, :3 * w].reshape(h, w, 3)
        mask = np.all(px == 0, axis=2)
    else:
        nb = bpp // 8
        raw = rows[:, :nb * w].reshape(h, w, nb).astype(np.uint32)
        v = np.zeros((h, w), np.uint32)
        for j in range(nb):
            v |= raw[:, :, j] << np.uint32(8 * j)
        rm, gm, bm, am = (np.uint32(m) for m in masks)
        mask = ((v & rm) == 0) & ((v & gm) == 0) & ((v & bm) == 0)
        if am:
            mask &= (v & am) == am
    return w, h, mask.astype(np.uint8)


# ------------------------------------------------------------ initial state

def _feq(w, rho, s, usq):
    """w*rho in float, the bracket in double, the product rounded to float."""
    wr = (F32(w) * rho).astype(F64)
    s = s.astype(F64)
    br = ((1.0 + 3.0 * s) + (4.5 * s) * s) - 1.5 * usq.astype(F64)
    return (wr * br).astype(F32)


def _feq0(w, rho, usq):
    wr = (F32(w) * rho).astype(F64)
    return (wr * (1.0 - 1.5 * usq.astype(F64))).astype(F32)


def d2q9_solid_bound(solid2d):
    """reference src/simulation_d2q9.cu:318-334 (x in 1..W-2, periodic y)."""
    s = solid2d.astype(bool)
    H, W = s.shape
    allsolid = s.copy()
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            allsolid &= np.roll(np.roll(s, -dy, axis=0), -dx, axis=1)
    sb = np.zeros_like(s)
    sb[:, 1:W - 1] = allsolid[:, 1:W - 1]
    return sb.astype(np.uint8)


def init_d2q9(p, solid2d):
    """The initial state of reference src/simulation_d2q9.cu:100-334 for one
    device.  Returns f (9, N) and ux, uy, rho, psi, ueq_x, ueq_y, solid_bound
    (N each); solid nodes of a Shan-Chen case are 0 (unset in the reference)."""
    solid2d = np.asarray(solid2d, np.uint8)
    H, W = solid2d.shape
    N = W * H
    solid = solid2d.reshape(N).astype(bool)
    w0, w1, w2 = F32(16.0 / 36.0), F32(4.0 / 36.0), F32(1.0 / 36.0)
    ux = np.zeros(N, F32); uy = np.zeros(N, F32); rho = np.zeros(N, F32)
    psi = np.zeros(N, F32); ueq_x = np.zeros(N, F32); ueq_y = np.zeros(N, F32)
    f = np.zeros((9, N), F32)
    ux0, uy0, rho0 = F32(p["ux"]), F32(p["uy"]), F32(p["rho"])
    bx, by = ux0, uy0                        # ueq_x[0], ueq_y[0]
    ti = F32(0)
    if F32(p["ext_f"][0]) != 0:
        ti = F32(p["tau_inv"])
        bx = ux0 + F32(p["ext_f"][0]) / (ti * rho0)
    if F32(p["ext_f"][1]) != 0:
        ti = F32(p["tau_inv"])
        by = uy0 + F32(p["ext_f"][1]) / (ti * rho0)
    ux[0], uy[0], rho[0] = ux0, uy0, rho0

    def fill(idx, r, ex, ey):
        usq = ex * ex + ey * ey
        f[0, idx] = _feq0(w0, r, usq)
        for k, (w, s) in enumerate([(w1, ex), (w1, ey), (w1, -ex), (w1, -ey), (w2, ex + ey),
                                    (w2, -ex + ey), (w2, -ex - ey), (w2, ex - ey)], start=1):
            f[k, idx] = _feq(w, r, s, usq)

    G = F32(p["G"])
    if G != 0:
        Gads = F32(p["G_ads"])
        ti = F32(p["tau_inv"])
        fl = ~solid
        rho[fl] = rho0
        psi_val = F32(4.0 * math.exp(-200.0 / float(rho0)))
        psi[fl] = psi_val
        ux[fl] = ux0
        uy[fl] = uy0
        P = psi.reshape(H, W)
        S = solid.reshape(H, W)

        def nb(a, dy, dx):                   # a[(y+dy) % H, (x+dx) % W]
            return np.roll(np.roll(a, -dy, axis=0), -dx, axis=1).reshape(N)

        # neighbour order of the reference's init: 1 (x+1), 2 (y+1), 3 (x-1),
        # 4 (y-1), 5 (x+1,y+1), 6 (x-1,y+1), 7 (x-1,y-1), 8 (x+1,y-1)
        d = [None, (0, 1), (1, 0), (0, -1), (-1, 0), (1, 1), (1, -1), (-1, -1), (-1, 1)]
        p_ = [None] + [nb(P, *d[k]) for k in range(1, 9)]
        s_ = [None] + [nb(S, *d[k]) for k in range(1, 9)]
        IFx = np.zeros(N, F32); IFy = np.zeros(N, F32)
        IFx = IFx + w1 * p_[1]; IFx = IFx - w1 * p_[3]; IFx = IFx + w2 * p_[5]
        IFx = IFx - w2 * p_[6]; IFx = IFx - w2 * p_[7]; IFx = IFx + w2 * p_[8]
        IFy = IFy + w1 * p_[2]; IFy = IFy - w1 * p_[4]; IFy = IFy + w2 * p_[5]
        IFy = IFy + w2 * p_[6]; IFy = IFy - w2 * p_[7]; IFy = IFy - w2 * p_[8]
        IFx = (-G * psi) * IFx
        IFy = (-G * psi) * IFy
        Fsx = np.zeros(N, F32); Fsy = np.zeros(N, F32)
        Fsx = np.where(s_[1], Fsx + w1, Fsx)
        Fsy = np.where(s_[2], Fsy - w1, Fsy)
        Fsx = np.where(s_[3], Fsx - w1, Fsx)
        Fsy = np.where(s_[4], Fsy + w1, Fsy)
        Fsx = np.where(s_[5], Fsx + w2, Fsx); Fsy = np.where(s_[5], Fsy - w2, Fsy)
        Fsx = np.where(s_[6], Fsx - w2, Fsx); Fsy = np.where(s_[6], Fsy - w2, Fsy)
        Fsx = np.where(s_[7], Fsx - w2, Fsx); Fsy = np.where(s_[7], Fsy + w2, Fsy)
        Fsx = np.where(s_[8], Fsx + w2, Fsx); Fsy = np.where(s_[8], Fsy + w2, Fsy)
        Fsx = (-Gads * psi) * Fsx
        Fsy = (-Gads * psi) * Fsy
        den = ti * rho
        # node 0, when fluid, is visited first and its u_eq becomes the base of
        # every later node (the reference reads ueq_x[0] while it loops)
        if fl[0]:
            bx = (bx + IFx[0] / den[0]) + Fsx[0] / den[0]
            by = (by + IFy[0] / den[0]) + Fsy[0] / den[0]
        ueq_x[fl] = (bx + IFx[fl] / den[fl]) + Fsx[fl] / den[fl]
        ueq_y[fl] = (by + IFy[fl] / den[fl]) + Fsy[fl] / den[fl]
        if fl[0]:
            ueq_x[0], ueq_y[0] = bx, by
        else:
            ueq_x[0], ueq_y[0] = bx, by      # set before the loop, never overwritten
        idx = np.nonzero(fl)[0]
        fill(idx, rho[idx], ueq_x[idx], ueq_y[idx])
    else:
        ueq_x[0], ueq_y[0] = bx, by
        one = np.array([0])
        fill(one, np.array([rho0], F32), np.array([bx], F32), np.array([by], F32))
        f[:, :] = f[:, :1]
        ux[:] = ux0; uy[:] = uy0; rho[:] = rho0
    sb = d2q9_solid_bound(solid2d).reshape(N)
    return dict(f=f, ux=ux, uy=uy, rho=rho, psi=psi, ueq_x=ueq_x, ueq_y=ueq_y, solid_bound=sb)


def d3q19_solid_bound(solid3d):
    """reference src/simulation_d3q19.cu:167-204 (x in 1..W-2, periodic y, z)."""
    s = solid3d.astype(bool)
    D, H, W = s.shape
    offs = [(0, 0, 0), (0, 0, 1), (0, 0, -1), (0, 1, 0), (0, -1, 0), (1, 0, 0), (-1, 0, 0),
            (0, 1, 1), (0, -1, 1), (1, 0, 1), (-1, 0, 1), (0, 1, -1), (0, -1, -1), (1, 0, -1),
            (-1, 0, -1), (1, 1, 0), (-1, 1, 0), (1, -1, 0), (-1, -1, 0)]
    allsolid = np.ones_like(s)
    for dz, dy, dx in offs:
        allsolid &= np.roll(s, (-dz, -dy, -dx), axis=(0, 1, 2))
    sb = np.zeros_like(s)
    sb[:, :, 1:W - 1] = allsolid[:, :, 1:W - 1]
    return sb.astype(np.uint8)


def init_d3q19(p, solid3d):
    """reference src/simulation_d3q19.cu:99-204 (one device): uniform
    equilibrium, uz set only at node 0, the 19-point solid_bound rule."""
    solid3d = np.asarray(solid3d, np.uint8)
    D, H, W = solid3d.shape
    N = W * H * D
    w0, w1, w2 = F32(12.0 / 36.0), F32(2.0 / 36.0), F32(1.0 / 36.0)
    x, y, z, r = (np.array([F32(p[k])], F32) for k in ("ux", "uy", "uz", "rho"))
    usq = x * x + y * y + z * z
    dirs = [(w1, x), (w1, -x), (w1, y), (w1, -y), (w1, z), (w1, -z),
            (w2, x + y), (w2, x - y), (w2, x + z), (w2, x - z), (w2, -x + y), (w2, -x - y),
            (w2, -x + z), (w2, -x - z), (w2, y + z), (w2, y - z), (w2, -y + z), (w2, -y - z)]
    f0 = [_feq0(w0, r, usq)[0]] + [_feq(w, r, s, usq)[0] for w, s in dirs]
    f = np.empty((19, N), F32)
    for k in range(19):
        f[k] = f0[k]
    uz = np.zeros(N, F32)
    uz[0] = z[0]
    return dict(f=f, ux=np.full(N, x[0], F32), uy=np.full(N, y[0], F32), uz=uz,
                rho=np.full(N, r[0], F32), solid_bound=d3q19_solid_bound(solid3d).reshape(N))


# ---------------------------------------------------------------------- VTK

def _g(v):
    return "%g" % float(v)


def vtk_text(device_id, width, height, length, rho, ux, uy, uz=None):
    """Output::saveVTK, reference src/output.cpp:96-155."""
    ext = "%d %d 0 %d 0 %d" % (device_id * width, (device_id + 1) * width, height - 1, length - 1)
    out = ['<VTKFile type="ImageData" version="0.1" byte_order="LittleEndian">\n',
           '  <ImageData WholeExtent="%s" Origin="0 0 0" Spacing="1 1 1">\n' % ext,
           '  <Piece Extent="%s">\n' % ext,
           '    <PointData Scalars="Pressure" Vectors="Velocity">\n',
           '      <DataArray type="Float32" Name="Pressure" format="ascii" >\n      ']
    n = width * height * length
    rho = np.asarray(rho, F32); ux = np.asarray(ux, F32); uy = np.asarray(uy, F32)
    for i in range(n):
        out.append(_g(rho[i]) + " ")
        if (i + 1) % width == 0:
            out.append("0\n      ")
    out.append('</DataArray>\n      <DataArray type="Float32" Name="Velocity" '
               'NumberOfComponents="3" format="ascii">\n      ')
    for i in range(n):
        out.append(_g(ux[i]) + " ")
        if length > 1:
            out.append(_g(uy[i]) + " " + _g(np.asarray(uz, F32)[i]) + "   ")
        else:
            out.append(_g(-uy[i]) + " 0   ")
        if (i + 1) % width == 0:
            out.append("0 0 0\n      ")
    out.append("</DataArray>\n    </PointData>\n    <CellData>\n    </CellData>\n  </Piece>\n"
               "  </ImageData>\n</VTKFile>\n")
    return "".join(out)


def pvti_text(vtk_id, device_count, width, height, length):
    """Output::saveParVTK, reference src/output.cpp:52-94."""
    out = ['<VTKFile type="PImageData" version="0.1" byte_order="LittleEndian">\n',
           '  <PImageData WholeExtent="0 %d 0 %d 0 %d" GhostLevel="#" Origin="0 0 0" '
           'Spacing="1 1 1">\n' % (width * device_count - 1, height - 1, length - 1),
           '    <PPointData Scalars="Pressure" Vectors="Velocity">\n',
           '      <DataArray type="Float32" Name="Pressure" format="ascii"/>\n',
           '      <DataArray type="Float32" Name="Velocity" NumberOfComponents="3" '
           'format="ascii"/>\n    </PPointData>\n    <PCellData>\n    </PCellData>\n']
    for i in range(device_count):
        out.append('    <Piece Extent="%d %d 0 %d 0 %d" Source="r%04dp%02d.vti"/>\n'
                   % (i * width, (i + 1) * width, height - 1, length - 1, vtk_id, i))
    out.append("  </PImageData>\n</VTKFile>\n")
    return "".join(out)


# ---------------------------------------------------------------- STL solids

def read_stl(path):
    """Triangles (n, 3, 3) float32 of a binary or ASCII STL file."""
    with open(path, "rb") as fh:
        b = fh.read()
    ascii_ = True
    if len(b) >= 84:
        n = struct.unpack_from("<I", b, 80)[0]
        ascii_ = b[:5] == b"solid" and 84 + 50 * n != len(b)
    if ascii_:
        toks = b.decode("latin-1").split()
        vals = []
        for i, t in enumerate(toks):
            if t == "vertex":
                vals += [np.float32(float(toks[i + 1])), np.float32(float(toks[i + 2])),
                         np.float32(float(toks[i + 3]))]
        return np.array(vals, np.float32).reshape(-1, 3, 3)
    dt = np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")])
    return np.frombuffer(b, dt, count=n, offset=84)["v"].astype(np.float32)


def voxel_grid(tri, max_dim):
    """(lo[3], h, dims[3]) of the voxel grid: the longest bounding-box side
    spans max_dim voxels, each axis ceil(extent / h) voxels."""
    v = np.asarray(tri, np.float32).reshape(-1, 3).astype(np.float64)
    lo, hi = v.min(0), v.max(0)
    ext = max(hi - lo)
    h = ext / max_dim
    dims = [max(1, int(math.ceil((hi[a] - lo[a]) / h - 1e-9))) for a in range(3)]
    return lo, h, dims


def _round_half_away(v):
    f = np.floor(v)
    return np.where(v - f >= 0.5, f + 1, f).astype(np.int64)


def voxelize(tri, max_dim):
    """Solid mask (D, H, W) of a closed triangle surface: voxel centres with
    an odd number of surface crossings below them in their z column, the
    crossings found with fixed-point (2^-16 voxel) edge functions and a
    consistent tie rule (the library's lb_voxelize, restated)."""
    FRAC = 16
    tri = np.asarray(tri, np.float32).reshape(-1, 3, 3)
    lo, h, (W, H, D) = voxel_grid(tri, max_dim)
    sc = float(1 << FRAC) / h
    q = _round_half_away((tri.astype(np.float64) - lo[None, None, :]) * sc)  # (n, 3 vertices, 3)
    cols, zs = [], []
    inv = 1.0 / float(1 << FRAC)
    for t in range(len(q)):
        (x0, y0, z0), (x1, y1, z1), (x2, y2, z2) = [tuple(int(c) for c in q[t, v]) for v in range(3)]
        area = (x1 - x0) * (y2 - y0) - (y1 - y0) * (x2 - x0)
        if area == 0:
            continue
        if area < 0:
            x1, y1, z1, x2, y2, z2 = x2, y2, z2, x1, y1, z1
        bx0 = int(math.floor(min(x0, x1, x2) * inv - 0.5))
        bx1 = int(math.ceil(max(x0, x1, x2) * inv - 0.5))
        by0 = int(math.floor(min(y0, y1, y2) * inv - 0.5))
        by1 = int(math.ceil(max(y0, y1, y2) * inv - 0.5))
        xs = np.arange(max(bx0, 0), min(bx1, W - 1) + 1, dtype=np.int64)
        ys = np.arange(max(by0, 0), min(by1, H - 1) + 1, dtype=np.int64)
        if len(xs) == 0 or len(ys) == 0:
            continue
        X, Y = np.meshgrid(xs, ys)
        px = (2 * X + 1) << (FRAC - 1)
        py = (2 * Y + 1) << (FRAC - 1)

        def ef(ax, ay, bx, by):
            e = (bx - ax) * (py - ay) - (by - ay) * (px - ax)
            dx, dy = bx - ax, by - ay
            tie = (dy > 0) or (dy == 0 and dx < 0)
            return e, (e > 0) | ((e == 0) & tie)

        e0, k0 = ef(x1, y1, x2, y2)
        e1, k1 = ef(x2, y2, x0, y0)
        e2, k2 = ef(x0, y0, x1, y1)
        m = k0 & k1 & k2
        if not m.any():
            continue
        e0, e1, e2 = (e[m].astype(np.float64) for e in (e0, e1, e2))
        a = e0 + e1 + e2
        z = (e0 * float(z0) + e1 * float(z1) + e2 * float(z2)) / a
        cols.append((Y[m] * W + X[m]).astype(np.int64))
        zs.append(z)
    solid = np.zeros((D, H * W), np.uint8)
    if cols:
        c = np.concatenate(cols)
        z = np.concatenate(zs)
        order = np.lexsort((z, c))
        c, z = c[order], z[order]
        centres = np.array([float((2 * k + 1) << (FRAC - 1)) for k in range(D)])
        starts = np.flatnonzero(np.r_[True, c[1:] != c[:-1]])
        ends = np.r_[starts[1:], len(c)]
        for s, e in zip(starts, ends):
            below = np.searchsorted(z[s:e], centres, side="left")
            solid[:, c[s]] = (below & 1).astype(np.uint8)
    return solid.reshape(D, H, W)
