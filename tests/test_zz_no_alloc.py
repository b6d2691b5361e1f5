"""fg_reducer_run_noalloc (no device allocation, static scratch) against the
allocating entry point (fg_reducer_create + fg_reducer_run) on two calls in a
row with different inputs: the second call must not see anything the first
left in the shared scratch.  Named to be collected last."""
import gzip

import numpy as np
import pytest

from helpers import golden, read_scheme_text

pytestmark = pytest.mark.gpu
fg = pytest.importorskip("flipgraphgpu_gb300")

KEYS = ("additions", "fresh", "naive", "mode", "draws", "scale")


def load_input(ring):
    with gzip.open(golden(f"input_{ring}_333.txt.gz"), "rt") as f:
        return read_scheme_text(f.read())


def allocating(n, m, coef, count, seed, best_fresh=None, best_vars=None):
    red = fg.Reducer(n, m, coef[None], count=count, schemes=1, seed=seed)
    try:
        return red.run(independent=True, best_fresh=best_fresh, best_vars=best_vars)
    finally:
        red.close()


def test_noalloc_matches_allocating_entry_point_twice_in_a_row():
    n, m, coef = load_input("zt")
    # call 1: fresh reducers
    want1 = allocating(n, m, coef, 24, 41)
    got1 = fg.reducer_run_noalloc(n, m, coef[None], count=24, schemes=1, seed=41)
    for k in KEYS:
        assert np.array_equal(got1[k], want1[k]), ("first", k)
    assert (got1["additions"] > 0).all()
    # call 2, straight after: other seed and count, partial initialisation from
    # the first call's reducer 0 (the same scheme)
    bf, bv = want1["fresh"][0].copy(), want1["vars"][0].copy()
    want2 = allocating(n, m, coef, 12, 7, bf, bv)
    got2 = fg.reducer_run_noalloc(n, m, coef[None], count=12, schemes=1, seed=7, best_fresh=bf, best_vars=bv)
    for k in KEYS:
        assert np.array_equal(got2[k], want2[k]), ("second", k)


def test_noalloc_other_scheme_after_a_larger_call():
    n, m, coef = load_input("z2")
    want = allocating(n, m, coef, 8, 5)
    got = fg.reducer_run_noalloc(n, m, coef[None], count=8, schemes=1, seed=5)
    for k in KEYS:
        assert np.array_equal(got[k], want[k]), k


def test_noalloc_rejects_oversize_inputs():
    n, m, coef = load_input("zt")
    with pytest.raises(RuntimeError):
        fg.reducer_run_noalloc(n, m, coef[None], count=1025, schemes=1, seed=1)
    with pytest.raises(RuntimeError):
        fg.reducer_run_noalloc(n, m, np.repeat(coef[None], 1200, axis=0), count=8, schemes=1200, seed=1)


def test_noalloc_rejects_pair_tables_beyond_shared_memory():
    """A dense 4x4x4 scheme of rank 64: each of the 16 W expressions holds 64 variables,
    2,016 pair occurrences each, far beyond one block's shared memory.  The allocating
    path moves such tables to global memory; the no-allocation one reports capacity."""
    n, m = (4, 4, 4), 64
    coef = np.zeros((1, 3, m, 64), np.int8)
    coef[0, :, :, :16] = 1
    with pytest.raises(fg.FlipGraphError) as e:
        fg.reducer_run_noalloc(n, m, coef, count=4, schemes=1, seed=1)
    assert e.value.status == 3  # FG_ERR_CAPACITY
    assert "shared-memory" in str(e.value)
