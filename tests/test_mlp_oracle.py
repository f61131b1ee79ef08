"""CPU checks of the closure network's numpy oracle: its analytic gradient
agrees with central finite differences for the parameters behind the last
rounding point (b2, w3, b3, where the loss is smooth), the gradient with the
GPU's bfloat16 backward operands stays within bfloat16 rounding of the exact
one, and the filter/feature restatement recovers a known linear shear."""
import sys

import numpy as np

from conftest import ORACLE_DIR

sys.path.insert(0, ORACLE_DIR)
import mlp_oracle as M  # noqa: E402


def test_gradient_vs_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.standard_normal(M.NPARAM) * 0.3
    X = rng.standard_normal((64, 19)).astype(np.float32)
    Z = rng.standard_normal(64)
    g, _ = M.grad(p, X, Z, backward_bf16=False)
    for idx in list(range(M.OFF_B2, M.OFF_B2 + 8)) + list(range(M.OFF_W3, M.OFF_W3 + 8)) + \
            [M.OFF_B3]:
        e = 1e-6
        q = p.copy()
        q[idx] += e
        lp = M.grad(q, X, Z)[1]
        q[idx] -= 2 * e
        lm = M.grad(q, X, Z)[1]
        assert abs(g[idx] - (lp - lm) / (2 * e)) <= 1e-6 + 1e-5 * abs(g[idx])


def test_bf16_backward_operands_stay_near_the_exact_gradient():
    """Rounding the gradient contractions' operands to bfloat16 (8 significant
    bits) moves each parameter group by a few parts in 10^3."""
    rng = np.random.default_rng(3)
    p = rng.standard_normal(M.NPARAM) * 0.3
    X = rng.standard_normal((512, 19)).astype(np.float32)
    Z = rng.standard_normal(512)
    g, loss = M.grad(p, X, Z)
    e, loss_e = M.grad(p, X, Z, backward_bf16=False)
    assert loss == loss_e
    for a, b in [(M.OFF_W1, M.OFF_B1), (M.OFF_B1, M.OFF_W2), (M.OFF_W2, M.OFF_B2),
                 (M.OFF_B2, M.OFF_W3), (M.OFF_W3, M.OFF_B3)]:
        assert np.linalg.norm(g[a:b] - e[a:b]) <= 4e-3 * np.linalg.norm(e[a:b])
    assert abs(g[M.OFF_B3] - e[M.OFF_B3]) <= 4e-3 * np.abs(e[M.OFF_B3])


def test_features_of_uniform_shear():
    """u_x = a * y on a periodic-compatible sine shear: the stress features
    recover -2 S / s_ref = -du/dy / s_ref at the nodes where sin is linear."""
    n, fac = 16, 1
    y = np.arange(n)
    a = 1e-3
    ux = np.tile((a * n / (2 * np.pi) * np.sin(2 * np.pi * y / n))[None, :, None], (n, 1, n))
    z = np.zeros_like(ux)
    r, ub, T = M.box_filter(np.ones(n ** 3), ux.reshape(-1), z.reshape(-1), z.reshape(-1),
                            n, n, n, fac)
    F, zt = M.features_targets(ub, T, 1e-3, 1.0, 100.0)
    F = F.reshape(n, n, n, 19)
    # at y = 0 the discrete derivative is a * n/(2 pi) * sin(2 pi/n): S_xy = half of it
    d = a * n / (2 * np.pi) * np.sin(2 * np.pi / n)
    assert np.allclose(F[:, 0, :, 6], -d)
    assert np.allclose(zt, 0.0)  # no sub-grid stress without filtering
