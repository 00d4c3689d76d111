"""Multi-rank path of bench.py on CPU (gloo, world size 2): disjoint window
shards per rank, no collective on the data path, max-over-ranks timing, and
each rank's POA work (the oracle on its own shard, standing in for the GPU
path that needs one device per rank) gathering to the single-rank result."""
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
    # the shard's windows on this rank
    from oracle import pyoracle as po
    params = synth.SCORING["batch_10k"][1]
    cons, _ = po.batch_run(2, *params, [w.reads for w in wins], n_threads=2)
    all_cons = [None] * world
    dist.all_gather_object(all_cons, cons)
    out[rank] = (mx, gathered, all_cons)
    dist.destroy_process_group()


def test_two_ranks_shard_windows_and_take_the_max_time():
    port = _free_port()
    world = 2
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    from oracle import pyoracle as po
    params = synth.SCORING["batch_10k"][1]
    single, _ = po.batch_run(2, *params, [w.reads for w in synth.batch_windows(12)],
                             n_threads=2)
    for rank in range(world):
        mx, gathered, all_cons = res[rank]
        assert mx == 2.0
        flat = [w for ids in gathered for w in ids]
        assert len(flat) == len(set(flat)) == 12  # disjoint, complete
        assert [c for cs in all_cons for c in cs] == single  # same as one rank
