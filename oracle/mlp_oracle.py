"""CPU oracle of the learned-grid network (test infrastructure only: the tests
use it to check the GPU forward pass and gradients; nothing in the product
imports it).

The network has no counterpart in the reference, so there is nothing to pin
against there; this restatement is pinned instead by central finite
differences of its own loss (tests/test_mlp_oracle.py).

Network: x (8) -> h1 = relu(W1 x + b1) (64) -> h2 = relu(W2 h1 + b2) (64)
-> z = W3 . h2 + b3; loss = sum_s w_s [max(z,0) - z y + log(1 + exp(-|z|))] /
sum_s w_s with w_s = pos_weight for y = 1, else 1.  The forward pass uses the
BF16-rounded weights (round to nearest even), the arithmetic is float64 here.
"""
import numpy as np

F, H = 8, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * F
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
NPARAM = OFF_B3 + 1


def bf16_round(a):
    """float32 -> nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounded = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return rounded.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[OFF_W1:OFF_B1].reshape(H, F), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(H, H), p[OFF_B2:OFF_W3],
            p[OFF_W3:OFF_B3], p[OFF_B3])


def init_params(seed):
    """He-style initialisation used by the training script (weights), zero biases."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, dtype=np.float32)
    p[OFF_W1:OFF_B1] = rng.normal(0.0, np.sqrt(2.0 / F), H * F)
    p[OFF_W2:OFF_B2] = rng.normal(0.0, np.sqrt(2.0 / H), H * H)
    p[OFF_W3:OFF_B3] = rng.normal(0.0, np.sqrt(1.0 / H), H)
    return p


def forward(p, x, round_weights=True):
    w = bf16_round(p).astype(np.float64) if round_weights else np.asarray(p, dtype=np.float64)
    W1, b1, W2, b2, W3, b3 = unpack(w)
    x = np.asarray(x, dtype=np.float64)
    a1 = x @ W1.T + b1
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0.0)
    z = h2 @ W3 + b3
    return z, (x, h1, h2, w)


def prob(p, x):
    z, _ = forward(p, x)
    return 1.0 / (1.0 + np.exp(-z))


def loss_and_grad(p, x, y, pos_weight, round_weights=True):
    """Weighted BCE and its gradient with respect to the (rounded) weights."""
    z, (x, h1, h2, w) = forward(p, x, round_weights)
    _, _, W2, _, W3, _ = unpack(w)
    y = np.asarray(y, dtype=np.float64)
    ws = np.where(y > 0.5, pos_weight, 1.0)
    ws = ws / ws.sum()
    loss = float(np.sum(ws * (np.maximum(z, 0.0) - z * y + np.log1p(np.exp(-np.abs(z))))))
    g = ws * (1.0 / (1.0 + np.exp(-z)) - y)
    d2 = np.where(h2 > 0.0, g[:, None] * W3[None, :], 0.0)
    d1 = np.where(h1 > 0.0, d2 @ W2, 0.0)
    grad = np.zeros(NPARAM)
    grad[OFF_W1:OFF_B1] = (d1.T @ x).ravel()
    grad[OFF_B1:OFF_W2] = d1.sum(0)
    grad[OFF_W2:OFF_B2] = (d2.T @ h1).ravel()
    grad[OFF_B2:OFF_W3] = d2.sum(0)
    grad[OFF_W3:OFF_B3] = g @ h2
    grad[OFF_B3] = g.sum()
    return loss, grad
