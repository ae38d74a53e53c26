"""The CPU oracle of the learned-grid network, pinned by finite differences of
its own loss (the network has no counterpart in the reference), and its BF16
rounding against known bit patterns."""
import numpy as np

from oracle import mlp_oracle as mo


def test_bf16_rounding_known_values():
    vals = np.array([1.0, 1.00390625, 1.001953125, 1.005859375, -2.5, 3.0e38, 1.0e-40], dtype=np.float32)
    r = mo.bf16_round(vals)
    # 7 mantissa bits: 1 + 2^-8 is a tie -> even (1.0); 1 + 2^-9 -> 1.0; 1 + 3*2^-9 -> 1 + 2^-7
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 and r[3] == np.float32(1.0078125)
    assert r[4] == -2.5
    assert (r.view(np.uint32) & 0xFFFF).max() == 0


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = mo.init_params(11).astype(np.float64)
    x = rng.normal(size=(64, mo.F))
    y = (rng.random(64) < 0.3).astype(np.float64)
    _, g = mo.loss_and_grad(p, x, y, 4.0, round_weights=False)
    eps = 1e-6
    idx = np.concatenate([rng.choice(np.arange(mo.OFF_B1), 20, replace=False), np.arange(mo.OFF_B1, mo.OFF_B1 + 5),
                          rng.choice(np.arange(mo.OFF_W2, mo.OFF_B2), 30, replace=False), np.arange(mo.OFF_W3, mo.NPARAM)])
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        lp, _ = mo.loss_and_grad(pp, x, y, 4.0, round_weights=False)
        lm, _ = mo.loss_and_grad(pm, x, y, 4.0, round_weights=False)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])
