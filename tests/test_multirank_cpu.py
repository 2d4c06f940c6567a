"""Multi-rank host logic on CPU (gloo, world size 2): instance sharding has no
collective in the data path; ranks only agree on timing (max) and counts (sum)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    import __graft_entry__ as ge
    pkg = ge.load()
    templates, itpl, par, off, probes = bench.workload(pkg, 256, 7)
    mine = bench.shard(itpl, templates, rank, world)
    # every rank reports its shard; the timing reduction is a max, counts a sum
    t = bench.reduce_max(dist, float(rank + 1))
    s = bench.reduce_sum(dist, float(len(mine)))
    sizes = sum(templates[itpl[i]].n for i in mine)
    out[rank] = (mine.tolist(), t, s, sizes)
    dist.destroy_process_group()


def test_shards_are_disjoint_covering_and_balanced():
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    shards = [out[r][0] for r in range(world)]
    allidx = sorted(shards[0] + shards[1])
    assert allidx == list(range(256))
    assert not set(shards[0]) & set(shards[1])
    assert out[0][1] == out[1][1] == 2.0          # max over ranks
    assert out[0][2] == out[1][2] == 256.0        # sum over ranks
    s0, s1 = out[0][3], out[1][3]
    assert abs(s0 - s1) / max(s0, s1) < 0.05      # work balanced by size
