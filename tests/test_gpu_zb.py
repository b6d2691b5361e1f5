"""Bounded-integer ring (ZB, coefficients in [-2, 2]) on the GPU against the
CPU oracle's restatement of the same walk (no reference counterpart: the
reference's integer ring is {-1, 0, 1}).

Same seed, same starting records: after every launch the library's warp-per-
walk kernel and the oracle agree on every field (sizes, rank, factors as
sign-magnitude masks, flips counter, best rank and scheme, stream position),
and every scheme passes the exact integer Brent check on the device and in
the oracle.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
fg = pytest.importorskip("flipgraphgpu_gb300")

FIELDS = ["n", "m", "fac", "sgn", "fac2", "flips", "best_rank", "best_m", "best_fac", "best_sgn", "best_fac2",
          "rng_pos", "status"]


def oracle_batch(rec):
    b = O.WalkBatch(rec.walks, rec.cap, "zb")
    for f in ["n", "m", "fac", "sgn", "fac2", "flips", "best_rank", "best_m", "best_fac", "best_sgn", "best_fac2",
              "rng_pos"]:
        getattr(b, f)[...] = getattr(rec, f)
    return b


@pytest.mark.parametrize("shapes,per,iters,plus,expand_p,reduce_p,launches", [
    ([(2, 2, 2)], 64, 2000, 300, 0.01, 0.0, 2),
    ([(3, 3, 3)], 64, 1000, 200, 0.01, 0.0, 2),
    ([(4, 4, 4)], 32, 500, 100, 0.01, 0.0, 2),
    ([(2, 3, 4)], 48, 1000, 100, 40.0, 0.0, 2),
    ([(3, 3, 3)], 48, 800, 150, 0.01, 60.0, 2),
    ([(2, 2, 2), (2, 2, 3), (3, 3, 4), (4, 4, 4)], 24, 400, 100, 5.0, 5.0, 2),
    ([(4, 4, 8)], 8, 300, 100, 10.0, 0.0, 1),
])
def test_zb_walk_matches_oracle(shapes, per, iters, plus, expand_p, reduce_p, launches):
    S = per * len(shapes)
    cap = max(a * b * c for a, b, c in shapes) + 4
    seed = 900 + S
    sh = np.array([shapes[w // per] for w in range(S)], np.int32)
    with fg.Engine(S, cap, "zb", "fast", seed, iters, plus, expand_p, reduce_p) as eng:
        eng.init_naive_shapes(sh)
        rec0 = eng.records()
        stats = [eng.run(1) for _ in range(launches)]
        rec = eng.records()
        valid, valid_best = eng.validate(), eng.validate(best=True)
    assert valid.all() and valid_best.all()
    assert all(s["walks_failed"] == 0 and s["flips"] > 0 for s in stats)
    b = oracle_batch(rec0)
    assert O.walk(b, b.cfg("fast", iterations=iters, plus_iterations=plus, launches=launches, expand_p=expand_p,
                           reduce_p=reduce_p, seed=seed)) == 0
    for f in FIELDS:
        a, o = getattr(rec, f), getattr(b, f)
        if not np.array_equal(a, o):
            bad = np.argwhere(a != o)
            raise AssertionError(f"field {f} differs at {bad[:5].tolist()} (of {len(bad)})")
    assert O.validate(b).all() and O.validate(b, best=True).all()
    coef = rec.coefficients()
    assert np.abs(coef).max() == 2  # the wider bound is used


def test_zb_rejects_other_modes():
    with pytest.raises(fg.FlipGraphError):
        fg.Engine(4, 27, "zb", "reference", 1, 100, 100)
    with pytest.raises(fg.FlipGraphError):
        fg.Engine(4, 27, "zb", "fast", 1, 100, 100, resize_p=0.5)
