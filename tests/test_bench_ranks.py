"""The benchmark's multi-rank bookkeeping on CPU (gloo, two ranks): the job's time is the
slowest rank's, its units the sum over ranks; rank 0 of the reference arm runs alone."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seconds, units = bench.reduce_over_ranks(1.0 + rank, 100 * (rank + 1), dist)
    out[rank] = (seconds, units, bench.dist_env())
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_reduce_to_max_time_and_total_units():
    world = 2
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        seconds, units, env = res[rank]
        assert seconds == 2.0 and units == 300.0
        assert env == (world, rank)


def test_single_rank_passes_through():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(1.5, 7) == (1.5, 7.0)


def test_reference_arm_runs_on_rank_0_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    assert bench.reference_arm(None) == 0  # returns before touching its arguments
    assert capsys.readouterr().out == ""
