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
