"""Continuous-batching screening service over a device-resident database (ypdq_server_*).

Requests of 1..max_step_images images are queued by `submit`, packed oldest first into
device steps by the library's worker thread, hashed (8 dihedrals per image) and matched
exactly against the database. `poll` returns finished requests with their hits sorted by
(database index, query), query numbers local to the request (8 * image + slot): the same
hits the request gets when screened alone (`core.screen_host`).

The reference has no serving loop; its nearest relative is the CLI's two-thread `pipe`
loop (src/main.rs:391-836), which hashes one frame at a time.
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import HIT_DTYPE, YpdqError, check, ptr

_KINDS = {"f32": _lib.INPUT_F32, "u8": _lib.INPUT_U8, "rgb8": _lib.INPUT_RGB8,
          "rgba8": _lib.INPUT_RGBA8}
_SHAPES = {_lib.INPUT_F32: ((512, 512), np.float32), _lib.INPUT_U8: ((512, 512), np.uint8),
           _lib.INPUT_RGB8: ((512, 512, 3), np.uint8), _lib.INPUT_RGBA8: ((512, 512, 4), np.uint8)}


class PinnedArray:
    """A numpy array in page-locked host memory (ypdq_malloc_host); copies from it to the
    device run asynchronously at full link speed."""

    def __init__(self, ctx, shape, dtype):
        self.ctx = ctx
        dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dtype.itemsize
        self._p = ctypes.c_void_p()
        check(ctx.lib.ypdq_malloc_host(ctx.handle, max(nbytes, 1), ctypes.byref(self._p)))
        buf = (ctypes.c_uint8 * max(nbytes, 1)).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=np.uint8, count=nbytes).view(dtype).reshape(shape)

    def free(self):
        if self._p and self._p.value:
            self.array = None
            self.ctx.lib.ypdq_free_host(self.ctx.handle, self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


@dataclass
class Result:
    request_id: int
    tag: int
    status: int
    n_images: int
    n_hits: int
    hits: np.ndarray        # HIT_DTYPE, min(n_hits, hit_capacity) entries
    hashes: np.ndarray      # (n_images, 8, 32) u8 or None
    quality: np.ndarray     # (n_images, 8) f32 or None
    latency_us: float
    step: int

    @property
    def ok(self):
        return self.status == _lib.OK


class Server:
    """ypdq_server: see include/ypdq.h for the scheduling and admission rules."""

    def __init__(self, ctx, db, threshold=31, input_kind="f32", dct=_lib.DCT_FP32,
                 semantics="exact", max_step_images=1024, slots=3, step_hit_capacity=1 << 20,
                 device_bytes=0, max_queued_images=0, autotune=False, target_step_ms=0.0):
        self.ctx, self.db = ctx, db
        cfg = _lib.ServerConfig()
        check(ctx.lib.ypdq_server_config_default(ctypes.byref(cfg)))
        cfg.input_kind = _KINDS[input_kind] if isinstance(input_kind, str) else int(input_kind)
        cfg.dct_precision = int(dct)
        cfg.semantics = _lib.SEMANTICS[semantics] if isinstance(semantics, str) else int(semantics)
        cfg.threshold = int(threshold)
        cfg.max_step_images = int(max_step_images)
        cfg.slots = int(slots)
        cfg.step_hit_capacity = int(step_hit_capacity)
        cfg.device_bytes = int(device_bytes)
        cfg.max_queued_images = int(max_queued_images)
        cfg.autotune = 1 if autotune else 0
        cfg.target_step_ms = float(target_step_ms)
        self.input_kind = cfg.input_kind
        self.handle = ctypes.c_void_p()
        check(ctx.lib.ypdq_server_create(ctx.handle, db.handle, ctypes.byref(cfg),
                                         ctypes.byref(self.handle)))
        self._live = {}  # request id -> buffers the worker reads or writes
        self._comp = (_lib.Completion * 256)()

    def _check_images(self, images):
        shape, want = _SHAPES[self.input_kind]
        if images.dtype != want or images.shape[1:] != shape:
            raise ValueError("images must be (n, %s) %s"
                             % (", ".join(map(str, shape)), np.dtype(want).name))
        if not images.flags.c_contiguous:
            raise ValueError("images must be C-contiguous")

    def try_submit(self, images, hit_capacity=4096, want_hashes=False, tag=0):
        """Queue one request; returns its id, or None when the queue is full (BUSY).
        `images` must stay unchanged until the request is polled (it is kept alive here)."""
        self._check_images(images)
        n = images.shape[0]
        hits = np.zeros(max(int(hit_capacity), 1), HIT_DTYPE)
        hashes = np.zeros((n, 8, 32), np.uint8) if want_hashes else None
        quality = np.zeros((n, 8), np.float32) if want_hashes else None
        rid = ctypes.c_uint64()
        st = self.ctx.lib.ypdq_server_submit(self.handle, ptr(images), n, ptr(hits),
                                             int(hit_capacity), ptr(hashes), ptr(quality),
                                             int(tag), ctypes.byref(rid))
        if st == _lib.ERR_BUSY:
            return None
        check(st)
        self._live[rid.value] = (images, hits, hashes, quality)
        return rid.value

    def submit(self, images, hit_capacity=4096, want_hashes=False, tag=0):
        rid = self.try_submit(images, hit_capacity, want_hashes, tag)
        if rid is None:
            raise YpdqError(_lib.ERR_BUSY, "server queue is full")
        return rid

    def poll(self, timeout_us=0, max_results=256):
        """Finished requests (up to max_results), waiting up to timeout_us (-1: until one
        is done or nothing is outstanding)."""
        n = ctypes.c_uint32()
        m = min(max_results, len(self._comp))
        check(self.ctx.lib.ypdq_server_poll(self.handle, self._comp, m, ctypes.byref(n),
                                            int(timeout_us)))
        out = []
        for i in range(n.value):
            c = self._comp[i]
            _, hits, hashes, quality = self._live.pop(c.request_id)
            out.append(Result(c.request_id, c.user_tag, c.status, c.n_images, c.n_hits,
                              hits[: min(c.n_hits, len(hits))], hashes, quality, c.latency_us,
                              c.step))
        return out

    def replay(self, pool, first, n_images, arrival_ns=None, duration_s=1e9, hit_capacity=0):
        """ypdq_server_replay: requests of pool[first[i] : first[i] + n_images[i]] submitted
        from native code at arrival_ns[i] ns after the call starts (None: as soon as the
        queue has room) until duration_s; returns (submitted, rejected, n_hits) once all
        submitted requests have completed (n_hits[i]: request i's true hit count). With
        hit_capacity > 0 also the hit buffers, one row per request. No other request of this
        server may be in flight meanwhile."""
        self._check_images(pool)
        first = np.ascontiguousarray(first, np.uint32)
        n_images = np.ascontiguousarray(n_images, np.uint32)
        if first.shape != n_images.shape:
            raise ValueError("first and n_images differ in length")
        arr = None if arrival_ns is None else np.ascontiguousarray(arrival_ns, np.uint64)
        if arr is not None and arr.shape != first.shape:
            raise ValueError("arrival_ns and first differ in length")
        hits = (np.zeros((len(first), int(hit_capacity)), HIT_DTYPE) if hit_capacity
                else None)
        n_hits = np.zeros(len(first), np.uint64)
        sub, rej = ctypes.c_uint64(), ctypes.c_uint64()
        check(self.ctx.lib.ypdq_server_replay(
            self.handle, ptr(pool), pool.shape[0], ptr(first), ptr(n_images), ptr(arr),
            len(first), int(duration_s * 1e9), ptr(hits), int(hit_capacity), ptr(n_hits),
            ctypes.byref(sub), ctypes.byref(rej)))
        if hits is not None:
            return sub.value, rej.value, n_hits, hits
        return sub.value, rej.value, n_hits

    def drain(self, timeout_us=-1):
        """Poll until every submitted request has completed."""
        out = []
        while self._live:
            got = self.poll(timeout_us=timeout_us)
            if not got:  # timed out, or (timeout < 0) nothing is outstanding any more
                break
            out.extend(got)
        return out

    def stats(self, reset=False):
        s = _lib.ServerStats()
        check(self.ctx.lib.ypdq_server_get_stats(self.handle, ctypes.byref(s), 1 if reset else 0))
        d = {k: getattr(s, k) for k, _ in _lib.ServerStats._fields_ if not k.startswith("bucket")}
        nb = s.n_buckets
        d["buckets"] = [{"images": s.bucket_images[i],
                         "algo": ({1: "simt", 3: ("tc", "tc pairs", "tc rows", "tc fp4 triples",
                                                  "tc fp4 rows")[s.bucket_kernel[i]]}
                                  .get(s.bucket_algo[i], s.bucket_algo[i])),
                         "n_tile": s.bucket_n_tile[i], "ms": round(float(s.bucket_ms[i]), 4),
                         "steps": s.bucket_steps[i]} for i in range(nb)]
        return d

    def close(self):
        if self.handle:
            check(self.ctx.lib.ypdq_server_destroy(self.handle))
            self.handle = ctypes.c_void_p()
            self._live.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            if self.handle:
                self.close()
        except Exception:
            pass
