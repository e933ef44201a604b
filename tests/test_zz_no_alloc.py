"""ypdq_screen_noalloc: screening for callers that cannot allocate device memory.

Callers that own all device memory through their own pool, or that screen on a path where
an allocation is not allowed, call ypdq_screen_noalloc with buffers they already hold. The
library keeps the intermediate hashes in a fixed 1 MiB device array. These tests call the
entry point through the C ABI, two calls in a row for each input kind and dihedral sign
convention, and check each result against the existing screening entry point
(ypdq_screen_host) exactly: the same (index, query, distance) hits. They also check that
the calls leave the device's free memory unchanged, that a zero-image call reports zero
hits, that a call after one whose scan timed out starts from a clear error word, and that
the set-up is redone after cudaDeviceReset. This file sorts last so a failure here comes
after every other test.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

KINDS = {"f32": 0, "u8": 1}
SEMS = {"exact": 0, "avx2": 1, "scalar": 2}


def sorted_tuples(h):
    t = np.stack([h["index"].astype(np.int64), h["query"].astype(np.int64),
                  h["distance"].astype(np.int64)], axis=1) if len(h) else np.zeros((0, 3), np.int64)
    return t[np.lexsort((t[:, 1], t[:, 0]))]


def cudart():
    """The CUDA runtime the library loaded (for cudaMemGetInfo / cudaDeviceReset)."""
    for line in open("/proc/self/maps"):
        if "libcudart.so" in line:
            lib = ctypes.CDLL(line.split()[-1])
            lib.cudaMemGetInfo.argtypes = [ctypes.POINTER(ctypes.c_size_t)] * 2
            return lib
    raise RuntimeError("libcudart not loaded")


def free_bytes(rt):
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


@pytest.fixture(scope="module")
def planted(ctx, yp):
    """Rows with near-duplicates of every batch's hashes under every convention."""
    rows = yp.synth.rows_128(200_000, seed=901)
    batches = [yp.synth.blob_images(5, seed=902), yp.synth.blob_images(5, seed=903),
               yp.synth.blob_images(40, seed=904)]
    for i, imgs in enumerate(batches):
        for sem in SEMS:
            for k, data in enumerate((imgs, yp.synth.to_u8(imgs))):
                h = yp.hash_batch(ctx, data, semantics=sem)["hashes"].reshape(-1, 32)
                yp.synth.plant(rows, h, 100, 0, 31, seed=910 + 6 * i + 2 * SEMS[sem] + k)
    db = yp.Database(ctx, rows)
    return batches, db


def screen_noalloc(ctx, yp, d_img, n, kind, sem, db, d_hits, cap, d_count):
    d_rows, n_rows = db.device_rows()
    st = ctx.lib.ypdq_screen_noalloc(d_img.ptr if d_img is not None else None, n, kind, sem,
                                     d_rows, n_rows, 31, d_hits.ptr, cap, d_count.ptr, None)
    assert st == 0, ctx.lib.ypdq_last_error()
    ctx.sync()
    return int(d_count.download((1,), np.uint64)[0])


@pytest.mark.parametrize("kind", list(KINDS))
@pytest.mark.parametrize("sem", list(SEMS))
def test_screen_noalloc_matches_screen_host(ctx, yp, planted, kind, sem):
    """Two calls in a row on different images (5 then 5, then 40 images: passes of each scan
    kernel), each equal to ypdq_screen_host's hits for the same input and convention."""
    batches, db = planted
    cap = 1 << 14
    d_hits, d_count = ctx.alloc(cap * 16), ctx.alloc(8)
    for imgs in batches:
        data = yp.synth.to_u8(imgs) if kind == "u8" else imgs
        want = yp.screen_host(ctx, db, data, threshold=31, semantics=sem)
        assert len(want) > 0
        d_img = ctx.to_device(data)
        total = screen_noalloc(ctx, yp, d_img, len(imgs), KINDS[kind], SEMS[sem], db, d_hits,
                               cap, d_count)
        assert total == len(want)
        got = d_hits.download((total,), yp.HIT_DTYPE)
        assert np.array_equal(sorted_tuples(got), sorted_tuples(want))


def test_screen_noalloc_allocates_nothing(ctx, yp, planted):
    """The device's free memory is the same before and after two calls (after one warm-up
    call of the same sizes, which loads the kernels)."""
    batches, db = planted
    rt = cudart()
    cap = 1 << 14
    d_hits, d_count = ctx.alloc(cap * 16), ctx.alloc(8)
    d_imgs = [ctx.to_device(b) for b in batches]
    for d_img, imgs in zip(d_imgs, batches):
        screen_noalloc(ctx, yp, d_img, len(imgs), 0, 0, db, d_hits, cap, d_count)
    before = free_bytes(rt)
    for d_img, imgs in zip(d_imgs, batches):
        screen_noalloc(ctx, yp, d_img, len(imgs), 0, 0, db, d_hits, cap, d_count)
        screen_noalloc(ctx, yp, d_img, len(imgs), 0, 0, db, d_hits, cap, d_count)
    assert free_bytes(rt) == before


def test_screen_noalloc_zero_images_and_timeout_recovery(ctx, yp, planted):
    """n = 0 sets the count to 0. A call whose scan times out (a stalled producer under a
    1 ms wait limit) reports UINT64_MAX; the next call starts from a clear error word and
    returns the exact hits."""
    batches, db = planted
    lib = ctx.lib
    cap = 1 << 14
    d_hits, d_count = ctx.alloc(cap * 16), ctx.alloc(8)
    d_count.upload(np.array([12345], np.uint64))
    assert screen_noalloc(ctx, yp, None, 0, 0, 0, db, d_hits, cap, d_count) == 0
    imgs = batches[2]
    want = yp.screen_host(ctx, db, imgs, threshold=31)
    d_img = ctx.to_device(imgs)
    assert lib.ypdq_set_scan_wait_limit(1_000_000) == 0
    try:
        assert lib.ypdq_debug_stall_scans(1) == 0
        assert screen_noalloc(ctx, yp, d_img, len(imgs), 0, 0, db, d_hits, cap,
                              d_count) == 2 ** 64 - 1
    finally:
        lib.ypdq_debug_stall_scans(0)
        lib.ypdq_set_scan_wait_limit(0)
    total = screen_noalloc(ctx, yp, d_img, len(imgs), 0, 0, db, d_hits, cap, d_count)
    assert total == len(want)
    got = d_hits.download((total,), yp.HIT_DTYPE)
    assert np.array_equal(sorted_tuples(got), sorted_tuples(want))


def test_screen_noalloc_rejects_oversized_batch_and_misalignment(ctx, yp):
    lib = ctx.lib
    d = ctx.alloc(256)
    st = lib.ypdq_screen_noalloc(d.ptr, 4097, 0, 0, d.ptr, 1, 31, d.ptr, 1, d.ptr, None)
    assert st == yp._lib.ERR_INVALID
    assert b"4096" in lib.ypdq_last_error()
    odd = ctypes.c_void_p(d.address + 4)
    assert lib.ypdq_screen_noalloc(d.ptr, 1, 0, 0, d.ptr, 1, 31, d.ptr, 1, odd, None) == yp._lib.ERR_ALIGN
    assert lib.ypdq_screen_noalloc(d.ptr, 1, 0, 0, d.ptr, 1, 31, odd, 1, d.ptr, None) == yp._lib.ERR_ALIGN


RESET_SCRIPT = r"""
import ctypes, sys
import numpy as np
sys.path.insert(0, %(root)r)
import __graft_entry__ as g
yp = g.load_package()
imgs = yp.synth.blob_images(4, seed=61)
rows = yp.synth.rows_128(20_000, seed=62)
results = []
for round_ in range(2):
    ctx = yp.Context(0)
    h = yp.hash_batch(ctx, imgs)["hashes"].reshape(-1, 32)
    yp.synth.plant(rows, h, 50, 0, 31, seed=63)
    db = yp.Database(ctx, rows)
    want = yp.screen_host(ctx, db, imgs, threshold=31)
    d_img, d_hits, d_count = ctx.to_device(imgs), ctx.alloc(1 << 16), ctx.alloc(8)
    d_rows, n_rows = db.device_rows()
    st = ctx.lib.ypdq_screen_noalloc(d_img.ptr, 4, 0, 0, d_rows, n_rows, 31, d_hits.ptr, 4096,
                                     d_count.ptr, None)
    assert st == 0, ctx.lib.ypdq_last_error()
    ctx.sync()
    n = int(d_count.download((1,), np.uint64)[0])
    got = d_hits.download((n,), yp.HIT_DTYPE)
    got = got[np.lexsort((got["query"], got["index"]))]
    results.append(n == len(want) and np.array_equal(got, want))
    del d_img, d_hits, d_count
    db.close()
    ctx.close()
    if round_ == 0:
        for line in open("/proc/self/maps"):
            if "libcudart.so" in line:
                assert ctypes.CDLL(line.split()[-1]).cudaDeviceReset() == 0
                break
print("results", results)
"""


def test_screen_noalloc_after_device_reset():
    """In a fresh process: a call, cudaDeviceReset, a new context, another call. The second
    call redoes the per-context set-up and returns the exact hits again."""
    r = subprocess.run([sys.executable, "-c", RESET_SCRIPT % {"root": ROOT}], capture_output=True,
                       text=True, timeout=600, cwd=ROOT, env=dict(os.environ))
    assert r.returncode == 0, r.stderr[-3000:]
    assert "results [True, True]" in r.stdout, r.stdout + r.stderr[-2000:]
