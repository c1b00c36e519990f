"""Multi-GPU runs are independent replicas ("replicas only": no exchange step
on the data path).  The host logic of the benchmark's N>1 path -- the
max-over-ranks timing and the per-replica seeds -- runs here over gloo with
two CPU ranks."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    t = bench.max_over_ranks(1.0 + 2.5 * rank, world)
    seeds = [None] * world
    dist.all_gather_object(seeds, bench.replica_seed(1234, rank))
    out[rank] = (t, tuple(seeds))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_max_timing_and_distinct_seeds():
    world = 2
    port = _free_port()
    ctx = mp.get_context('spawn')
    mgr = ctx.Manager()
    out = mgr.dict()
    procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    assert out[0][0] == out[1][0] == pytest.approx(3.5)
    seeds = out[0][1]
    assert len(set(seeds)) == world


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(2.0, 1) == 2.0
    assert bench.replica_seed(5, 0) == 5
