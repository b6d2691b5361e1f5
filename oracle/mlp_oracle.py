"""CPU restatement of the learned flip proposal's MLP (test infrastructure:
only tests, smoke checks and the benchmark's baseline leg use it).

The network scores one candidate flip from its 192 input features:
    h1 = relu(W1 x + b1)      W1 [256][192]
    h2 = relu(W2 h1 + b2)     W2 [256][256]
    s  = w3 . h2 + b3         w3 [256]
with bf16 weights and activations between layers, fp32 accumulation, and the
binary cross-entropy of sigmoid(s) against "the rank dropped within the next
1000 flips".  The reference has no learned component; this file is the
oracle the GPU kernels are checked against (forward values and gradients).
"""
import numpy as np

D_IN, HIDDEN = 192, 256


def bf16_bits(x):
    """float32 -> bf16 bit patterns, round to nearest even."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32)
    return ((b + np.uint32(0x7FFF) + ((b >> np.uint32(16)) & np.uint32(1))) >> np.uint32(16)).astype(np.uint16)


def bf16_value(bits):
    return (np.asarray(bits, np.uint16).astype(np.uint32) << np.uint32(16)).view(np.float32)


def bf16_round(x):
    return bf16_value(bf16_bits(x))


def forward(x, W1, b1, W2, b2, w3, b3):
    """x [B][192] (0/1 features); weights fp32 masters (rounded to bf16 for the products)."""
    xb = bf16_round(x)
    h1 = bf16_round(np.maximum(xb @ bf16_round(W1).T + b1, 0.0))
    h2 = bf16_round(np.maximum(h1 @ bf16_round(W2).T + b2, 0.0))
    s = h2 @ w3.astype(np.float32) + np.float32(b3)
    return h1, h2, s.astype(np.float32)


def loss_and_grads(x, y, W1, b1, W2, b2, w3, b3):
    """Mean binary cross-entropy of sigmoid(s) vs y and its gradients, following the
    GPU step: dZ2, dH1 and dZ1 are rounded to bf16 where the GPU stores them in bf16."""
    B = x.shape[0]
    xb = bf16_round(x)
    h1, h2, s = forward(x, W1, b1, W2, b2, w3, b3)
    p = 1.0 / (1.0 + np.exp(-s.astype(np.float64)))
    loss = float(np.mean(np.logaddexp(0.0, s) - y * s))
    ds = ((p - y) / B).astype(np.float32)                     # dL/ds
    gw3 = h2.T @ ds
    gb3 = np.float32(ds.sum())
    dz2 = bf16_round(np.where(h2 > 0, ds[:, None] * w3[None, :], 0.0).astype(np.float32))
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(axis=0)
    dh1 = dz2 @ bf16_round(W2)
    dz1 = bf16_round(np.where(h1 > 0, dh1, 0.0).astype(np.float32))
    gW1 = dz1.T @ xb
    gb1 = dz1.sum(axis=0)
    return loss, {"W1": gW1, "b1": gb1, "W2": gW2, "b2": gb2, "w3": gw3, "b3": gb3}


def init_params(seed):
    """He-uniform initialisation (the GPU trainer uses the same formula and this generator's values)."""
    rng = np.random.default_rng(seed)
    W1 = (rng.uniform(-1, 1, (HIDDEN, D_IN)) * np.sqrt(6.0 / D_IN)).astype(np.float32)
    W2 = (rng.uniform(-1, 1, (HIDDEN, HIDDEN)) * np.sqrt(6.0 / HIDDEN)).astype(np.float32)
    w3 = (rng.uniform(-1, 1, HIDDEN) * np.sqrt(3.0 / HIDDEN)).astype(np.float32)
    return {"W1": W1, "b1": np.zeros(HIDDEN, np.float32), "W2": W2, "b2": np.zeros(HIDDEN, np.float32),
            "w3": w3, "b3": np.float32(0.0)}
