"""Tensor-core (tcgen05) GEMM and the learned proposal's MLP against the CPU oracle."""
import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu
fg = pytest.importorskip("flipgraphgpu_gb300")


def rand_bf16(rng, shape, scale=1.0):
    return M.bf16_bits(rng.standard_normal(shape).astype(np.float32) * scale)


@pytest.mark.parametrize("m,n,k", [(128, 64, 64), (128, 128, 192), (256, 256, 256), (384, 256, 448), (128, 192, 1024)])
def test_gemm_f32(m, n, k):
    rng = np.random.default_rng(m + n + k)
    a, b = rand_bf16(rng, (m, k)), rand_bf16(rng, (n, k))
    want = M.bf16_value(a).astype(np.float64) @ M.bf16_value(b).astype(np.float64).T
    got = fg.gemm_bf16(a, b, mode=0)
    assert np.allclose(got, want, rtol=1e-4, atol=1e-3 * np.sqrt(k))
    acc = rng.standard_normal((m, n)).astype(np.float32)
    got2 = fg.gemm_bf16(a, b, mode=0, accumulate=acc.copy())
    assert np.allclose(got2, want + acc, rtol=1e-4, atol=1e-3 * np.sqrt(k))


def test_gemm_bias_relu_and_mask():
    rng = np.random.default_rng(5)
    m, n, k = 256, 256, 192
    a, b = rand_bf16(rng, (m, k)), rand_bf16(rng, (n, k), 0.1)
    bias = rng.standard_normal(n).astype(np.float32)
    z = (M.bf16_value(a).astype(np.float64) @ M.bf16_value(b).astype(np.float64).T) + bias
    got = M.bf16_value(fg.gemm_bf16(a, b, mode=1, bias=bias))
    want = M.bf16_round(np.maximum(z, 0).astype(np.float32))
    assert np.allclose(got, want, rtol=1e-2, atol=1e-3)
    assert np.array_equal(got > 0, want > 0) or np.mean((got > 0) != (want > 0)) < 1e-3
    mask = M.bf16_bits(rng.standard_normal((m, n)).astype(np.float32))
    got = M.bf16_value(fg.gemm_bf16(a, b, mode=2, mask=mask))
    zz = z - bias
    want = M.bf16_round(np.where(M.bf16_value(mask) > 0, zz, 0).astype(np.float32))
    assert np.allclose(got, want, rtol=1e-2, atol=1e-3)
    assert np.array_equal(got == 0, want == 0)


def pack(p):
    return np.concatenate([p["W1"].ravel(), p["b1"], p["W2"].ravel(), p["b2"], p["w3"], [p["b3"]]]).astype(np.float32)


def unpack(v):
    H, D = M.HIDDEN, M.D_IN
    o = [0]

    def take(n, shape=None):
        a = v[o[0]:o[0] + n]
        o[0] += n
        return a.reshape(shape) if shape else a
    return {"W1": take(H * D, (H, D)), "b1": take(H), "W2": take(H * H, (H, H)), "b2": take(H), "w3": take(H),
            "b3": np.float32(take(1)[0])}


def random_features(rng, rows, density=0.15):
    bits = rng.random((rows, 192)) < density
    words = np.zeros((rows, 3), np.uint64)
    for w in range(3):
        for q in range(64):
            words[:, w] |= bits[:, 64 * w + q].astype(np.uint64) << np.uint64(q)
    return words, bits.astype(np.float32)


def rel_err(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12))


@pytest.mark.parametrize("rows", [512, 300])
def test_mlp_gradients_match_oracle(rows):
    rng = np.random.default_rng(rows)
    p = M.init_params(11)
    p["b1"] = rng.standard_normal(M.HIDDEN).astype(np.float32) * 0.1
    p["b2"] = rng.standard_normal(M.HIDDEN).astype(np.float32) * 0.1
    p["b3"] = np.float32(0.2)
    words, x = random_features(rng, rows)
    y = (rng.random(rows) < 0.3).astype(np.float32)
    with fg.Mlp(seed=1) as net:
        net.set_params(pack(p))
        assert np.array_equal(net.params(), pack(p))
        loss, g = net.gradients(words, y)
        s = net.score(words)
    want_loss, want = M.loss_and_grads(x, y, **p)
    _, _, want_s = M.forward(x, **p)
    assert abs(loss - want_loss) < 1e-3 * max(1.0, abs(want_loss))
    assert np.allclose(s, want_s, rtol=1e-2, atol=1e-2)
    got = unpack(g)
    for k in ("W1", "b1", "W2", "b2", "w3"):
        assert rel_err(got[k], want[k]) < 2e-2, (k, rel_err(got[k], want[k]))
    assert abs(float(got["b3"]) - float(want["b3"])) < 1e-4 + 1e-2 * abs(float(want["b3"]))


def test_mlp_trains_on_a_learnable_rule():
    """The label is a conjunction of feature bits; after a few epochs the network's scores
    separate the classes (AUC), which a uniform scorer cannot (AUC 0.5)."""
    rng = np.random.default_rng(3)
    n = 32768
    words, x = random_features(rng, n, density=0.3)
    y = ((x[:, 3] > 0) & (x[:, 70] > 0) | (x[:, 150] > 0) & (x[:, 10] == 0)).astype(np.float32)
    with fg.Mlp(seed=2) as net:
        before = net.gradients(words[:4096], y[:4096])[0]
        last = net.train(words[:n - 4096], y[:n - 4096], batch=1024, epochs=4, lr=2e-3, seed=5)
        s = net.score(words[n - 4096:])
    yt = y[n - 4096:]
    order = np.argsort(s)
    ranks = np.empty(len(s))
    ranks[order] = np.arange(len(s))
    pos = yt > 0
    auc = (ranks[pos].mean() - (pos.sum() - 1) / 2) / (~pos).sum()
    assert last < before * 0.5
    assert auc > 0.95
