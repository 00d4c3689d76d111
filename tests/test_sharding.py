"""Multi-rank path of bench.py on CPU (gloo, world size 2): disjoint window
shards per rank, no collective on the data path, max-over-ranks timing."""
import os
import socket

import torch.distributed as dist
import torch.multiprocessing as mp

import bench
from spoa_gb300 import synth


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    n = 6
    start = bench.shard_start(n, rank)
    ids = list(range(start, start + n))
    wins = synth.batch_windows(n, start=start)
    # the same window id gives the same window on every rank
    assert wins[0].reads == synth.batch_window(start).reads
    step = 1.0 + rank  # rank 1 is the slow one
    mx = bench.max_over_ranks(step, dist, "cpu")
    gathered = [None] * world
    dist.all_gather_object(gathered, ids)
    out[rank] = (mx, gathered)
    dist.destroy_process_group()


def test_two_ranks_shard_windows_and_take_the_max_time():
    port = _free_port()
    world = 2
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        mx, gathered = res[rank]
        assert mx == 2.0
        flat = [w for ids in gathered for w in ids]
        assert len(flat) == len(set(flat)) == 12  # disjoint, complete
