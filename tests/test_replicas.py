"""Multi-GPU paths, checked with gloo ranks on the CPU.

bench.py's multi-GPU mode runs one replica per rank (the path needs no collective): the job
time is the slowest rank's and the value counts every rank's images. A database can also be
row-sharded (shard_rows / merge_shard_hits): each rank scans its slice with the whole query
batch and rank 0 gathers the hit lists with their row offsets; the merged list must be the
scan of the whole database."""
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


def _shard_rank(rank, world, port, out):
    import sys
    import numpy as np
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import __graft_entry__ as g
    import oracle
    yp = g.load_package()
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rows = yp.synth.rows_128(30011, seed=61)  # every rank builds the same database
    q = yp.synth.rows_128(24, seed=62)
    yp.synth.plant(rows, q, 300, 0, 40, seed=63)
    lo, hi = yp.shard_rows(rows.shape[0], world, rank)
    # this rank's scan of its slice (the oracle's matcher stands in for the GPU scan)
    local = oracle.find_all(rows[lo:hi], q, 31)
    gathered = [None] * world
    dist.all_gather_object(gathered, (local, lo))
    if rank == 0:
        merged = yp.merge_shard_hits(gathered)
        full = oracle.find_all(rows, q, 31)
        out.put(bool(len(full) > 0 and np.array_equal(merged, full)))
    dist.barrier()
    dist.destroy_process_group()


def test_row_sharded_scan_three_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_rank, args=(r, 3, port, q)) for r in range(3)]
    for p in procs:
        p.start()
    ok = q.get(timeout=180)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert ok



def test_shard_rows_partition_and_merge():
    """shard_rows tiles [0, n_rows) in rank order with slice sizes differing by at most one,
    also with more ranks than rows; merge_shard_hits restores global indices in
    (index, query) order and accepts empty shards."""
    import sys
    import numpy as np
    sys.path.insert(0, ROOT)
    import __graft_entry__ as g
    yp = g.load_package()
    for n_rows in (0, 1, 2, 7, 1000, 10_000_019):
        for world in (1, 2, 3, 8):
            parts = [yp.shard_rows(n_rows, world, r) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == n_rows
            assert all(parts[r][1] == parts[r + 1][0] for r in range(world - 1))
            sizes = [hi - lo for lo, hi in parts]
            assert max(sizes) - min(sizes) <= 1
    rng = np.random.default_rng(3)
    full = np.zeros(50, yp.HIT_DTYPE)
    full["index"] = np.sort(rng.choice(1000, 50, replace=False))
    full["query"] = rng.integers(0, 9, 50)
    full["distance"] = rng.integers(0, 32, 50)
    full = full[np.lexsort((full["query"], full["index"]))]
    shards = []
    for lo, hi in [yp.shard_rows(1000, 4, r) for r in range(4)] + [(1000, 1000)]:
        local = full[(full["index"] >= lo) & (full["index"] < hi)].copy()
        local["index"] -= np.uint64(lo)
        shards.append((local[::-1], lo))  # any order within a shard
    merged = yp.merge_shard_hits(shards)
    assert np.array_equal(merged, full)
    try:
        yp.shard_rows(10, 2, 2)
        raise AssertionError("rank out of range accepted")
    except ValueError:
        pass


def test_bench_gpus_flag_starts_n_ranks():
    """`bench.py --gpus 2` outside torchrun starts two replica processes that join one gloo
    group (world 2, local ranks 0 and 1) and agree on the slowest rank's time."""
    import json
    import subprocess
    import sys
    env = {k: v for k, v in os.environ.items()
           if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT")}
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2",
                        "--ranks-only"], capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert sorted((d["rank"], d["local_rank"]) for d in lines) == [(0, 0), (1, 1)]
    assert all(d["world"] == 2 and d["max_ms"] == 2.0 for d in lines)


def test_bench_rejects_rank_count_mismatch():
    """A run whose WORLD_SIZE differs from --gpus fails instead of reporting the wrong N."""
    import subprocess
    import sys
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2",
                        "--ranks-only"], capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode != 0 and "--gpus 2" in r.stderr
