"""Parity at the benchmark's own sizes, through the C ABI.

The screening step that bench.py times: 1,024 seeded blob images (seed 2025) hashed on the
GPU with their 8 dihedral hashes (8,192 queries, numbered image * 8 + slot), scanned at
t = 31 against 10,000,000 rows of exactly 128 set bits (ypdq_synth_rows, seed 2025) in
which 10,000 rows are replaced by copies of the queries at distances 0..31. At 8,192
queries YPDQ_SCAN_AUTO runs one tensor-core launch of 32 passes of 256 queries on the
128-bit prefix bound. The GPU's sorted hit list must equal the oracle scalar matcher's over
all 8,192 x 10M pairs (CpuMatcher::find, src/matching/mod.rs:336-362), and the hashes the
oracle's f32 pipeline. The scan-only configuration's batches of 256 and 1,024 queries are
checked the same way through every scan kernel.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_IMAGES, N_ROWS, N_PLANTED, SEED, T = 1024, 10_000_000, 10_000, 2025, 31


def as_tuples(h):
    return np.stack([h["index"].astype(np.int64), h["query"].astype(np.int64),
                     h["distance"].astype(np.int64)], axis=1) if len(h) else np.zeros((0, 3), np.int64)


@pytest.fixture(scope="module")
def workload(ctx, yp, oracle):
    imgs = yp.synth.blob_images(N_IMAGES, seed=SEED)
    d_img = ctx.to_device(imgs)
    d_hash = ctx.alloc(N_IMAGES * 256)
    yp.core.hash_batch_device(ctx, d_img, N_IMAGES, yp._lib.INPUT_F32, d_hash)
    d_rows = ctx.alloc(N_ROWS * 32)
    yp._lib.check(ctx.lib.ypdq_synth_rows(ctx.handle, d_rows.ptr, N_ROWS, 0, SEED, None))
    ctx.sync()
    d_img.free()
    hashes = d_hash.download((N_IMAGES, 8, 32), np.uint8)
    rows = d_rows.download((N_ROWS, 32), np.uint8)
    yp.synth.plant_near_duplicates(rows, hashes, N_PLANTED, SEED + 99)
    d_rows.upload(rows)
    yield imgs, hashes, rows, d_hash, d_rows
    d_rows.free()
    d_hash.free()


def gpu_hits(ctx, yp, d_rows, d_q, nq, algo, cap):
    d_hits, d_cnt = ctx.alloc(cap * 16), ctx.alloc(8)
    yp.core.scan_device(ctx, d_rows, N_ROWS, d_q, nq, T, d_hits, cap, d_cnt, algo)
    ctx.sync()
    total = int(d_cnt.download((1,), np.uint64)[0])
    assert total <= cap, (total, cap)
    yp.core.sort_hits_device(ctx, d_hits, total)
    got = d_hits.download((total,), yp.HIT_DTYPE)
    d_hits.free()
    d_cnt.free()
    return got


def test_bench_step_hashes_and_hits(ctx, yp, oracle, workload):
    imgs, hashes, rows, d_hash, d_rows = workload
    want_h, _, _, _ = oracle.hash_batch(imgs)
    assert np.array_equal(hashes, want_h)
    queries = want_h.reshape(-1, 32)
    want = oracle.find_all(rows, queries, T)
    # every planted row is a hit of the hash it was copied from; with those of its siblings
    assert len(want) >= N_PLANTED
    assert oracle.count_all(rows, queries, T) == len(want)
    got = gpu_hits(ctx, yp, d_rows, d_hash, queries.shape[0], yp._lib.SCAN_AUTO, 1 << 20)
    assert np.array_equal(as_tuples(got), as_tuples(want))


@pytest.mark.parametrize("nq", [256, 1024])
def test_scan_only_batches(ctx, yp, oracle, workload, nq):
    _, hashes, rows, d_hash, d_rows = workload
    queries = hashes.reshape(-1, 32)[:nq]
    want = oracle.find_all(rows, queries, T)
    assert len(want) > 0
    for algo in (yp._lib.SCAN_AUTO, yp._lib.SCAN_SIMT, yp._lib.SCAN_TC):
        got = gpu_hits(ctx, yp, d_rows, d_hash, nq, algo, 1 << 16)
        assert np.array_equal(as_tuples(got), as_tuples(want)), algo
