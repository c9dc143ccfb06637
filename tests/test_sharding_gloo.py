"""The multi-GPU path of bench.py on CPU: q sharded across ranks with no
data-path collective, and the timed region reduced with MAX (gloo,
world_size 2)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from brille_gb300.sharding import shard_range  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    a, b = shard_range(n, rank, world)
    # each rank "processes" its shard; a slower rank dominates the timing
    t = torch.tensor([0.010 * (rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    counts = torch.tensor([b - a])
    dist.all_reduce(counts, op=dist.ReduceOp.SUM)
    out[rank] = (a, b, float(t.item()), int(counts.item()))
    dist.destroy_process_group()


def test_shards_cover_all_q_and_time_is_max_over_ranks():
    world, n = 2, 1_000_003
    port = _free_port()
    manager = mp.Manager()
    out = manager.dict()
    mp.spawn(_worker, args=(world, port, n, out), nprocs=world, join=True)
    spans = sorted(out[r][:2] for r in range(world))
    assert spans[0][0] == 0 and spans[-1][1] == n
    assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
    assert all(out[r][2] == pytest.approx(0.020) for r in range(world))
    assert all(out[r][3] == n for r in range(world))


def test_shard_range_edges():
    assert shard_range(0, 0, 4) == (0, 0)
    parts = [shard_range(10, r, 3) for r in range(3)]
    assert parts == [(0, 4), (4, 7), (7, 10)]
    assert np.diff([p[0] for p in parts]).min() >= 3
