"""bench.py's multi-GPU mode runs one replica per rank (the path needs no collective): the
job time is the slowest rank's and the value counts every rank's images. Checked here with
two gloo ranks on the CPU."""
import os
import socket

import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.dist_info()
    t, v = bench.aggregate_over_ranks(dist, [5.0, 7.0][rank], w, 1000)
    dist.barrier()
    out.put((r, w, local, t, v))
    dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, world, local, t, v) in enumerate(res):
        assert (rank, world, local) == (r, 2, r)
        assert t == 7.0  # the slowest replica
        assert abs(v - 2 * 1000 / 0.007) < 1e-6
