"""The bounded-integer ring (ZB, |c| <= 2) in the CPU oracle: walks keep every
scheme exact over the integers (Brent equations), use coefficients of
magnitude 2, stay within the bound, and find rank drops (2x2x2 reaches 7)."""
import numpy as np

from oracle import oracle as O


def run(shape, S, iters, plus, seed, launches=1, expand_p=0.01, reduce_p=0.0):
    cap = int(np.prod(shape)) + 4
    b = O.WalkBatch(S, cap, "zb")
    O.init_naive(b, *shape)
    assert O.validate(b).all()
    assert O.walk(b, b.cfg("fast", iterations=iters, plus_iterations=plus, launches=launches, expand_p=expand_p,
                           reduce_p=reduce_p, seed=seed)) == 0
    return b


def test_walks_stay_exact_and_bounded():
    for shape in [(2, 2, 2), (2, 3, 4), (3, 3, 3)]:
        b = run(shape, 16, 3000, 300, 5, launches=2, expand_p=5.0, reduce_p=5.0)
        assert O.validate(b).all() and O.validate(b, best=True).all()
        coef = O.zb_coefficients(b.fac, b.sgn, b.fac2)
        assert np.abs(coef).max() == 2
        # sign canonical form: first nonzero of u and of v positive
        for w in range(b.S):
            for t in range(b.m[w]):
                for c in (0, 1):
                    nz = coef[w, c, t][coef[w, c, t] != 0]
                    assert nz.size and nz[0] > 0


def test_2x2x2_reaches_rank_7():
    b = run((2, 2, 2), 32, 30000, 3000, 9)
    assert b.best_rank.min() == 7
    assert O.validate(b, best=True).all()


def test_rejects_list_modes():
    b = O.WalkBatch(2, 12, "zb")
    O.init_naive(b, 2, 2, 2)
    assert O.walk(b, b.cfg("philox", iterations=10, seed=1)) == -1
