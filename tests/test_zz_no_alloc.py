"""ypdq_screen_noalloc: screening for callers that cannot allocate device memory.

Callers that own all device memory through their own pool, or that screen on a path where
an allocation is not allowed, call ypdq_screen_noalloc with buffers they already hold. The
library keeps the intermediate hashes in a fixed 1 MiB device array. This test calls the
entry point twice in a row through the C ABI and checks each result against the existing
screening entry point (ypdq_screen_host), exactly: the same (index, query, distance) hits.
The second call is smaller than the first, so stale contents of the shared array would
show up as wrong hits. This file sorts last so a failure here comes after every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def sorted_tuples(h):
    t = np.stack([h["index"].astype(np.int64), h["query"].astype(np.int64),
                  h["distance"].astype(np.int64)], axis=1)
    return t[np.lexsort((t[:, 1], t[:, 0]))]


def test_screen_noalloc_matches_screen_host(ctx, yp):
    lib = ctx.lib
    rows = yp.synth.rows_128(200_000, seed=901)
    batches = [yp.synth.blob_images(5, seed=902), yp.synth.blob_images(3, seed=903)]
    # plant near-duplicates of both batches' hashes so each call has hits
    for i, imgs in enumerate(batches):
        h = yp.hash_batch(ctx, imgs)["hashes"].reshape(-1, 32)
        yp.synth.plant(rows, h, 300, 0, 31, seed=904 + i)
    db = yp.Database(ctx, rows)
    d_rows, n_rows = db.device_rows()
    cap = 4096
    d_hits = ctx.alloc(cap * 16)
    d_count = ctx.alloc(8)
    for imgs in batches:
        want = yp.screen_host(ctx, db, imgs, threshold=31)
        assert len(want) > 0
        d_img = ctx.to_device(imgs)
        st = lib.ypdq_screen_noalloc(d_img.ptr, len(imgs), 0, 0, d_rows, n_rows, 31, d_hits.ptr,
                                     cap, d_count.ptr, None)
        assert st == 0, lib.ypdq_last_error()
        ctx.sync()
        total = int(d_count.download((1,), np.uint64)[0])
        assert total == len(want)
        got = d_hits.download((total,), yp.HIT_DTYPE)
        assert np.array_equal(sorted_tuples(got), sorted_tuples(want))


def test_screen_noalloc_rejects_oversized_batch(ctx, yp):
    lib = ctx.lib
    d = ctx.alloc(64)
    st = lib.ypdq_screen_noalloc(d.ptr, 4097, 0, 0, d.ptr, 1, 31, d.ptr, 1, d.ptr, None)
    assert st == yp._lib.ERR_INVALID
    assert b"4096" in lib.ypdq_last_error()
