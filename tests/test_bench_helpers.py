"""Host helpers of bench.py that need no GPU: the committed 4x4x4 scheme the reducer and
minimizer legs start from parses into coefficient rows and is an exact Z2 scheme."""
import numpy as np

import bench
from oracle import oracle as O


def test_reducer_scheme_parses_and_is_exact():
    n, m, coef = bench.read_reducer_scheme()
    assert list(n) == [4, 4, 4] and m == 47
    assert coef.shape == (1, 3, m, 64)
    assert set(np.unique(coef).tolist()) <= {0, 1}
    b = O.WalkBatch(1, m, "z2")
    b.n[0] = n
    b.m[0] = m
    for c in range(3):
        bits = (coef[0, c, :, :16] != 0).astype(np.uint64) << np.arange(16, dtype=np.uint64)
        b.fac[0, c, :m] = bits.sum(axis=1, dtype=np.uint64)
    assert O.validate(b).all()
