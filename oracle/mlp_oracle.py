"""numpy restatement of the learned closure (TEST INFRASTRUCTURE ONLY).

The closure network 19 -> 64 -> 64 -> 1 (ReLU), its mean-squared-error
gradient, the Favre box filter of a fine lattice and the features / targets
built from the filtered fields -- computed in float64 with the GPU kernels'
rounding points (inputs, W1, W2 and the first hidden layer rounded to
bfloat16 in the forward pass; the operands of the gradient contractions
rounded to bfloat16 in the backward pass).  Used only by the tests, to
verify lb_closure.cu against.
"""
import numpy as np

IN, H = 19, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * IN
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
NPARAM = OFF_B3 + 1

D3_C = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                 [1, 1, 0], [1, -1, 0], [1, 0, 1], [1, 0, -1], [-1, 1, 0], [-1, -1, 0],
                 [-1, 0, 1], [-1, 0, -1], [0, 1, 1], [0, 1, -1], [0, -1, 1], [0, -1, -1]], float)
D3_W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


def bf16(a):
    """Round to bfloat16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[OFF_W1:OFF_B1].reshape(H, IN), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(H, H),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3], p[OFF_B3])


def forward(p, X):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    W1b = bf16(W1).astype(np.float64)
    W2b = bf16(W2).astype(np.float64)
    xb = bf16(X).astype(np.float64)
    a1 = xb @ W1b.T + b1
    h1 = bf16(np.maximum(a1, 0.0)).astype(np.float64)
    a2 = h1 @ W2b.T + b2
    h2 = np.maximum(a2, 0.0)
    y = h2 @ w3 + b3
    return {"xb": xb, "h1": h1, "h2": h2, "y": y, "W2b": W2b}


def grad(p, X, Z, backward_bf16=True):
    """Gradient of mean((y - z)^2) over the rows, with the rounding treated as
    the identity in the backward pass except where the GPU backward rounds:
    every contraction over the samples runs on the tensor cores, so dH2
    enters dH1 = dH2 W2, dW2 = dH2^T H1 and db2 = dH2^T 1, dH1 enters
    dW1 = dH1^T X and db1 = dH1^T 1, and h2 and dy enter dw3 = H2^T dy and
    db3 = dy^T 1, as bfloat16 (lb_closure.cu, mlp_tc_kernel).  With
    backward_bf16=False the backward pass rounds nothing: the exact gradient
    of the forward pass for the parameters behind its last rounding point."""
    rb = bf16 if backward_bf16 else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, w3, b3 = unpack(p)
    f = forward(p, X)
    n = len(X)
    dy = 2.0 * (f["y"] - Z) / n
    dyb = rb(dy).astype(np.float64)
    g = np.zeros(NPARAM)
    g[OFF_W3:OFF_B3] = rb(f["h2"]).astype(np.float64).T @ dyb
    g[OFF_B3] = dyb.sum()
    dh2 = (dy[:, None] * w3[None, :]) * (f["h2"] > 0)
    dh2b = rb(dh2).astype(np.float64)
    g[OFF_W2:OFF_B2] = (dh2b.T @ f["h1"]).reshape(-1)
    g[OFF_B2:OFF_W3] = dh2b.sum(0)
    dh1 = (dh2b @ f["W2b"]) * (f["h1"] > 0)
    dh1b = rb(dh1).astype(np.float64)
    g[OFF_W1:OFF_B1] = (dh1b.T @ f["xb"]).reshape(-1)
    g[OFF_B1:OFF_W2] = dh1b.sum(0)
    loss = float(np.mean((f["y"] - Z) ** 2))
    return g, loss


def box_filter(rho, ux, uy, uz, W, H, D, fac):
    """Favre box filter: rho_bar, u_bar (3), T (xx, yy, zz, xy, xz, yz)."""
    sh = (D // fac, fac, H // fac, fac, W // fac, fac)

    def m(a):
        return a.astype(np.float64).reshape(sh).sum(axis=(1, 3, 5))
    r = rho.reshape(D, H, W)
    u = [a.reshape(D, H, W).astype(np.float64) for a in (ux, uy, uz)]
    sr = m(r)
    su = [m(r * a) for a in u]
    ub = [s / sr for s in su]
    pairs = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    T = [m(r * u[a] * u[b]) / sr - ub[a] * ub[b] for a, b in pairs]
    return sr / fac ** 3, ub, T


def features_targets(ub, T, nu0, s_ref, z_max, avg_radius=0):
    """The closure's training features [Nc][19] and targets z = nu_t/nu0 from
    filtered fields on a periodic coarse grid (axes z, y, x).  avg_radius > 0:
    T_dev : S and S : S summed over the (2 r + 1)^3 cells around each cell
    before nu_t is formed (the target of lb_closure_sample_avg)."""
    def d(a, axis):  # derivative along lattice axis (0 = x, 1 = y, 2 = z)
        ax = {0: 2, 1: 1, 2: 0}[axis]
        return 0.5 * (np.roll(a, -1, ax) - np.roll(a, 1, ax))
    du = [[d(ub[b], a) for b in range(3)] for a in range(3)]
    S = [[0.5 * (du[a][b] + du[b][a]) for b in range(3)] for a in range(3)]
    tr = (T[0] + T[1] + T[2]) / 3
    TS = ((T[0] - tr) * S[0][0] + (T[1] - tr) * S[1][1] + (T[2] - tr) * S[2][2]
          + 2 * (T[3] * S[0][1] + T[4] * S[0][2] + T[5] * S[1][2]))
    SS = (S[0][0] ** 2 + S[1][1] ** 2 + S[2][2] ** 2
          + 2 * (S[0][1] ** 2 + S[0][2] ** 2 + S[1][2] ** 2))
    TSa, SSa = TS, SS
    if avg_radius > 0:
        rr = range(-avg_radius, avg_radius + 1)
        TSa = sum(np.roll(TS, (k, j, i), (0, 1, 2)) for k in rr for j in rr for i in rr)
        SSa = sum(np.roll(SS, (k, j, i), (0, 1, 2)) for k in rr for j in rr for i in rr)
    nut = np.maximum(0.0, -TSa / (2 * SSa + 1e-30))
    z = np.minimum(nut / nu0, z_max).reshape(-1)
    n = z.size
    F = np.zeros((n, IN))
    q = -2.0 / s_ref
    for i, (a, b) in enumerate([(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]):
        F[:, 3 + i] = (q * S[a][b]).reshape(-1)
    F[:, 18] = (np.sqrt(2 * SS) / s_ref).reshape(-1)
    return F, z


def cell_features(g, tau0, s_ref):
    """Features of cells from their pre-collision populations g[19][n]."""
    g = np.asarray(g, np.float64)
    rho = g.sum(0)
    u = (D3_C.T @ g) / rho
    cu = D3_C @ u
    usq = (u ** 2).sum(0)
    feq = D3_W[:, None] * rho * (1 + 3 * cu + 4.5 * cu ** 2 - 1.5 * usq)
    fn = g - feq
    cx, cy, cz = D3_C.T
    polys = [cx, cy, cz, cx * cx, cy * cy, cz * cz, cx * cy, cx * cz, cy * cz,
             cx * cy * cy, cx * cz * cz, cy * cx * cx, cy * cz * cz, cz * cx * cx, cz * cy * cy,
             cx * cx * cy * cy, cx * cx * cz * cz, cy * cy * cz * cz]
    m = np.stack([pl @ fn for pl in polys])
    scale = 1.0 / (rho * (1 / 3) * tau0 * s_ref)
    F = np.zeros((g.shape[1], IN))
    F[:, :18] = (m * scale).T
    h = -0.5 * scale
    s = [h * m[i] for i in range(3, 9)]
    F[:, 18] = np.sqrt(2 * (s[0] ** 2 + s[1] ** 2 + s[2] ** 2 + 2 * (s[3] ** 2 + s[4] ** 2
                                                                    + s[5] ** 2)))
    return F
