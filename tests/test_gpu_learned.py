"""Learned-proposal walk (FG_MODE_LEARNED) on the GPU.

* One candidate per step is the plain walk: the lockstep kernels reproduce the
  fast kernels (and so the oracle) bit for bit, records and stream position.
* Several candidates, scored by the network or chosen uniformly, keep every
  scheme exactly valid (Brent equations verified on the device).
* Training records from plain walks carry consistent features and labels, and a
  network trained on them ranks rank-dropping flips above the others on
  held-out records, which the uniform proposal cannot (AUC 0.5).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
fg = pytest.importorskip("flipgraphgpu_gb300")

FIELDS = ("n", "m", "fac", "flips", "best_rank", "best_m", "best_fac", "rng_pos", "status")


def run(mode, shapes, per, iters, plus, expand_p, reduce_p, seed, launches, proposal=None):
    S = per * len(shapes)
    cap = max(a * b * c for a, b, c in shapes)
    sh = np.array([shapes[w // per] for w in range(S)], np.int32)
    with fg.Engine(S, cap, "z2", mode, seed, iters, plus, expand_p, reduce_p) as eng:
        if proposal is not None:
            eng.set_proposal(**proposal)
        eng.init_naive_shapes(sh)
        stats = [eng.run(1) for _ in range(launches)]
        rec = eng.records()
        valid = eng.validate(), eng.validate(best=True)
    return rec, stats, valid


@pytest.mark.parametrize("shapes,iters,plus,expand_p,reduce_p", [
    ([(3, 3, 3)], 3000, 300, 0.01, 0.0),
    ([(2, 2, 2)], 1500, 50, 2.0, 0.0),
    ([(2, 3, 4)], 1500, 300, 0.01, 20.0),
    ([(4, 4, 4)], 1500, 500, 0.01, 0.0),
    ([(2, 2, 3), (3, 3, 4), (3, 4, 5), (4, 4, 4)], 1000, 400, 0.5, 0.0),
])
def test_one_candidate_reproduces_fast_mode(shapes, iters, plus, expand_p, reduce_p):
    args = (shapes, 48, iters, plus, expand_p, reduce_p, 4242, 2)
    want, wst, _ = run("fast", *args)
    got, gst, valid = run("learned", *args)
    for f in FIELDS:
        assert np.array_equal(getattr(got, f), getattr(want, f)), f
    assert [s["flips"] for s in gst] == [s["flips"] for s in wst]
    assert valid[0].all() and valid[1].all()


@pytest.mark.parametrize("scored", [False, True])
def test_candidates_keep_schemes_valid(scored):
    mlp = fg.Mlp(seed=9) if scored else None
    try:
        rec, stats, valid = run("learned", [(3, 3, 3), (4, 4, 4)], 256, 300, 5000, 0.01, 0.0, 77, 2,
                                proposal=dict(mlp=mlp, candidates=8, temperature=1.0, min_entropy=0.0))
    finally:
        if mlp is not None:
            mlp.close()
    assert valid[0].all() and valid[1].all()
    assert all(s["flips"] > 0 and s["walks_failed"] == 0 for s in stats)
    assert (rec.best_rank <= rec.n.prod(axis=1)).all()


def collect(shapes, per, seed, launches, iters=2000, every=8):
    S = per * len(shapes)
    cap = max(a * b * c for a, b, c in shapes)
    sh = np.array([shapes[w // per] for w in range(S)], np.int32)
    with fg.Engine(S, cap, "z2", "learned", seed, iters, 50000, 0.01, 0.0) as eng:
        eng.init_naive_shapes(sh)
        return eng.collect_records(every=every, horizon=1000, launches=launches, capacity=1 << 21)


def auc(scores, y):
    order = np.argsort(scores, kind="stable")
    ranks = np.empty(len(scores))
    ranks[order] = np.arange(len(scores))
    pos = y > 0
    return (ranks[pos].mean() - (pos.sum() - 1) / 2) / (~pos).sum()


def test_records_are_consistent():
    f, y = collect([(3, 3, 3), (4, 4, 4)], 512, 5, 2)
    assert len(y) > 10000
    assert set(np.unique(y)) <= {0.0, 1.0}
    assert 0.01 < y.mean() < 0.99
    ctx = f[:, 2]
    comp = (ctx & np.uint64(7)).astype(np.int64)
    assert np.isin(comp, [1, 2, 4]).all()          # one-hot component
    assert (f[:, 0] != 0).all() and (f[:, 1] != 0).all()


def test_trained_network_ranks_rank_drops_above_uniform():
    f, y = collect([(3, 3, 3), (3, 4, 5), (4, 4, 4)], 1024, 11, 3)
    n = len(y)
    perm = np.random.default_rng(0).permutation(n)
    f, y = f[perm], y[perm]
    split = int(n * 0.8)
    with fg.Mlp(seed=3) as net:
        net.train(f[:split], y[:split], batch=4096, epochs=3, lr=1e-3, seed=1)
        s = net.score(f[split:])
    a = auc(s, y[split:])
    assert a > 0.6, a
