"""The oracle's bounds on the loops the reference leaves unbounded (CPU).

The reference's tryPlus redraws its two terms until they share no factor
(scheme_z2.cu:1036-1039, scheme_integer.cu:984-987); on a scheme where every
pair of terms shares a factor it never returns.  The oracle, like the
library, stops after `retry_cap` redraws and marks the walk (status bit 2);
a record with fewer slots than a plus transition needs stops with status
bit 4.  The GPU twins of these cases are in test_gpu_failures.py.
"""
import numpy as np
import pytest

from oracle import oracle as O

RETRY, OVERFLOW = 2, 4
STUCK = [(1, 1, 1), (1, 2, 2)]


def batch(ring, cap, S, terms, lists):
    b = O.WalkBatch(S, cap, ring)
    b.n[:] = (2, 2, 2)
    m = len(terms)
    b.m[:] = m
    for t, uvw in enumerate(terms):
        for c in range(3):
            b.fac[:, c, t] = uvw[c]
    if ring == "zt":
        b.valid[:, :, :m] = 1
    b.best_fac[:] = b.fac
    if ring == "zt":
        b.best_valid[:] = b.valid
    b.best_rank[:] = m
    b.best_m[:] = m
    if lists:  # the only equal pair: terms 0 and 1 in the first component
        b.list_size[:, 0] = 1
        b.list_pairs[:, 0, 0] = (0 << 16) | 1
    return b


@pytest.mark.parametrize("ring,rng", [("z2", "fast"), ("z2", "philox"), ("zt", "philox")])
@pytest.mark.parametrize("cap_retry", [10, 200])
def test_retry_bound_stops_every_walk(ring, rng, cap_retry):
    S = 16
    b = batch(ring, 8, S, STUCK, lists=rng != "fast")
    O.walk(b, b.cfg(rng, iterations=50, plus_iterations=1, expand_p=0.0, seed=11, retry_cap=cap_retry))
    assert (b.status & RETRY).all()
    assert (b.m == 2).all()
    # the first plus transition spent its 2 draws and 2 per redraw, cap_retry redraws, then stopped
    assert (b.rng_pos >= 2 * (cap_retry + 1)).all()
    assert (b.rng_pos < 2 * (cap_retry + 1) + 64).all()


def test_default_bound_keeps_a_feasible_walk_running():
    b = O.WalkBatch(8, 8, "z2")
    O.init_naive(b, 2, 2, 2)
    O.walk(b, b.cfg("fast", iterations=400, plus_iterations=1, expand_p=0.0, seed=3))
    assert not b.status.any()
    assert O.validate(b).all()


@pytest.mark.parametrize("rng", ["fast", "philox"])
def test_slot_overflow_stops_the_walk(rng):
    terms = [(1, 1, 1), (1, 2, 2), (2, 4, 4), (4, 8, 8)]
    b = batch("z2", 4, 16, terms, lists=rng != "fast")
    O.walk(b, b.cfg(rng, iterations=50, plus_iterations=1, expand_p=0.0, seed=5))
    assert (b.status & OVERFLOW).all()
    assert (b.m == 4).all()
