"""Host-side objects over the C ABI: context, device buffers, batched hash and scan."""
import ctypes
import os

import numpy as np

from . import _lib
from ._lib import check, ptr, HIT_DTYPE


class Context:
    """A CUDA context of the library on one device (ypdq_ctx)."""

    def __init__(self, device=0):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        check(self.lib.ypdq_ctx_create(device, ctypes.byref(h)))
        self.handle = h
        self.device = device
        sms, ctas = ctypes.c_int(), ctypes.c_int()
        check(self.lib.ypdq_device_info(h, ctypes.byref(sms), ctypes.byref(ctas)))
        self.num_sms = sms.value
        self.hash_ctas_per_sm = ctas.value

    def close(self):
        if self.handle:
            self.lib.ypdq_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- memory
    def alloc(self, nbytes):
        return DeviceBuffer(self, nbytes)

    def to_device(self, array, stream=None):
        a = np.ascontiguousarray(array)
        buf = DeviceBuffer(self, a.nbytes)
        buf.upload(a, stream)
        return buf

    def sync(self, stream=None):
        check(self.lib.ypdq_stream_sync(self.handle, stream))

    def check_device_errors(self):
        check(self.lib.ypdq_check_device_errors(self.handle))

    def stream(self):
        s = ctypes.c_void_p()
        check(self.lib.ypdq_stream_create(self.handle, ctypes.byref(s)))
        return s

    def event(self):
        e = ctypes.c_void_p()
        check(self.lib.ypdq_event_create(self.handle, ctypes.byref(e)))
        return e

    def record(self, event, stream=None):
        check(self.lib.ypdq_event_record(self.handle, event, stream))

    def elapsed_ms(self, start, end):
        ms = ctypes.c_float()
        check(self.lib.ypdq_event_elapsed_ms(self.handle, start, end, ctypes.byref(ms)))
        return ms.value


class DeviceBuffer:
    """Device memory from ypdq_malloc_device; freed with the object."""

    def __init__(self, ctx, nbytes):
        self.ctx = ctx
        self.nbytes = int(nbytes)
        p = ctypes.c_void_p()
        check(ctx.lib.ypdq_malloc_device(ctx.handle, max(self.nbytes, 1), ctypes.byref(p)))
        self.ptr = p

    @property
    def address(self):
        return self.ptr.value

    def at(self, offset):
        return ctypes.c_void_p(self.ptr.value + int(offset))

    def upload(self, array, stream=None, offset=0):
        a = np.ascontiguousarray(array)
        assert a.nbytes + offset <= self.nbytes
        check(self.ctx.lib.ypdq_memcpy(self.ctx.handle, self.at(offset), ptr(a), a.nbytes,
                                       _lib.H2D, stream))
        if stream is None:
            self.ctx.sync(None)

    def download(self, shape, dtype, stream=None, offset=0):
        out = np.empty(shape, dtype)
        assert out.nbytes + offset <= self.nbytes
        check(self.ctx.lib.ypdq_memcpy(self.ctx.handle, ptr(out), self.at(offset), out.nbytes,
                                       _lib.D2H, stream))
        self.ctx.sync(stream)
        return out

    def zero(self, stream=None):
        check(self.ctx.lib.ypdq_memset(self.ctx.handle, self.ptr, 0, self.nbytes, stream))

    def free(self):
        if self.ptr is not None and self.ptr.value:
            self.ctx.lib.ypdq_free_device(self.ctx.handle, self.ptr)
        self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _semantics(sem):
    return _lib.SEMANTICS[sem] if isinstance(sem, str) else int(sem)


def hash_batch_device(ctx, d_images, n, input_kind, d_hashes=None, d_quality=None,
                      d_thresholds=None, d_pdqf=None, pdqf_slots=1, d_buf1=None,
                      dct=_lib.DCT_FP32, semantics="exact", stream=None):
    """Launch ypdq_hash_batch on device buffers (asynchronous)."""
    def dp(b):
        return None if b is None else (b.ptr if isinstance(b, DeviceBuffer) else b)
    check(ctx.lib.ypdq_hash_batch(ctx.handle, dp(d_images), int(n), int(input_kind), int(dct),
                                  _semantics(semantics), dp(d_hashes), dp(d_quality),
                                  dp(d_thresholds), dp(d_pdqf), int(pdqf_slots), dp(d_buf1),
                                  stream))


def input_kind_of(images):
    """(contiguous images, ypdq_input_kind) for host images: [n, 512, 512] f32 or u8, or
    [n, 512, 512, 3 | 4] u8 (RGB8 / RGBA8)."""
    imgs = np.ascontiguousarray(images)
    if imgs.ndim == 4:
        if imgs.dtype != np.uint8 or imgs.shape[1:3] != (512, 512) or imgs.shape[3] not in (3, 4):
            raise ValueError("colour images must be [n, 512, 512, 3|4] u8, got %s %s"
                             % (imgs.dtype, imgs.shape))
        return imgs, (_lib.INPUT_RGB8 if imgs.shape[3] == 3 else _lib.INPUT_RGBA8)
    if imgs.ndim != 3 or imgs.shape[1:] != (512, 512):
        raise ValueError("images must be [n, 512, 512], got %s" % (imgs.shape,))
    if imgs.dtype == np.uint8:
        return imgs, _lib.INPUT_U8
    return imgs.astype(np.float32, copy=False), _lib.INPUT_F32


def hash_batch(ctx, images, semantics="exact", dct=_lib.DCT_FP32, want_pdqf=False,
               pdqf_slots=1, want_buf1=False):
    """Hash host images on the GPU: [n, 512, 512] f32 or u8, or [n, 512, 512, 3|4] u8
    (RGB8 / RGBA8, converted to BT.601 luma in the kernel).

    Returns a dict with hashes [n, 8, 32] u8, quality [n, 8], thresholds [n, 8] and,
    when asked, pdqf [n, slots, 16, 16] and buf1 [n, 127, 127].
    """
    imgs, kind = input_kind_of(images)
    n = imgs.shape[0]
    d_img = ctx.to_device(imgs)
    d_h = ctx.alloc(n * 256)
    d_q = ctx.alloc(n * 32)
    d_t = ctx.alloc(n * 32)
    d_p = ctx.alloc(n * pdqf_slots * 1024) if want_pdqf else None
    d_b = ctx.alloc(n * 127 * 128 * 4) if want_buf1 else None
    hash_batch_device(ctx, d_img, n, kind, d_h, d_q, d_t, d_p, pdqf_slots, d_b, dct, semantics)
    ctx.sync()
    out = {
        "hashes": d_h.download((n, 8, 32), np.uint8),
        "quality": d_q.download((n, 8), np.float32),
        "thresholds": d_t.download((n, 8), np.float32),
    }
    if want_pdqf:
        out["pdqf"] = d_p.download((n, pdqf_slots, 16, 16), np.float32)
    if want_buf1:
        out["buf1"] = d_b.download((n, 127, 128), np.float32)[:, :, :127]
    return out


def dihedrals_batch(ctx, pdqf, thresholds, semantics="exact"):
    """Derived dihedrals of given PDQF matrices [n, 16, 16] at thresholds [n] (8 slots each)."""
    p = np.ascontiguousarray(pdqf, np.float32).reshape(-1, 256)
    t = np.ascontiguousarray(thresholds, np.float32).reshape(-1)
    n = p.shape[0]
    d_p, d_t = ctx.to_device(p), ctx.to_device(t)
    d_h, d_q, d_to, d_po = ctx.alloc(n * 256), ctx.alloc(n * 32), ctx.alloc(n * 32), ctx.alloc(n * 8192)
    check(ctx.lib.ypdq_dihedrals_batch(ctx.handle, d_p.ptr, d_t.ptr, n, _semantics(semantics),
                                       d_h.ptr, d_q.ptr, d_to.ptr, d_po.ptr, None))
    ctx.sync()
    return {
        "hashes": d_h.download((n, 8, 32), np.uint8),
        "quality": d_q.download((n, 8), np.float32),
        "thresholds": d_to.download((n, 8), np.float32),
        "pdqf": d_po.download((n, 8, 16, 16), np.float32),
    }


def dct2d_batch(ctx, buffers):
    """Kernel::dct2d of n compressed buffers on the GPU (ypdq_dct2d_batch): [n, 127, w] f32
    with w >= 127 (127 or the reference's padded 128; the first 127 columns are read)
    -> PDQF [n, 16, 16]."""
    b = np.ascontiguousarray(buffers, np.float32)
    if b.ndim != 3 or b.shape[1] < 127 or b.shape[2] < 127:
        raise ValueError("buffers must be [n, 127+, 127+], got %s" % (b.shape,))
    b = np.ascontiguousarray(b[:, :127])
    n, w = b.shape[0], b.shape[2]
    if n == 0:
        return np.zeros((0, 16, 16), np.float32)
    d_b, d_p = ctx.to_device(b), ctx.alloc(n * 1024)
    check(ctx.lib.ypdq_dct2d_batch(ctx.handle, d_b.ptr, n, w, d_p.ptr, None))
    ctx.sync()
    return d_p.download((n, 16, 16), np.float32)


def sum_of_gradients_batch(ctx, pdqf):
    """Kernel::sum_of_gradients of n PDQF matrices [n, 16, 16] on the GPU -> [n] f32."""
    p = np.ascontiguousarray(pdqf, np.float32).reshape(-1, 256)
    n = p.shape[0]
    if n == 0:
        return np.zeros(0, np.float32)
    d_p, d_g = ctx.to_device(p), ctx.alloc(n * 4)
    check(ctx.lib.ypdq_sum_of_gradients_batch(ctx.handle, d_p.ptr, n, d_g.ptr, None))
    ctx.sync()
    return d_g.download((n,), np.float32)


def pdqf_transform_batch(ctx, pdqf, op, negate=False, semantics="exact"):
    """One Kernel PDQF transform (ypdq_pdqf_op: _lib.PDQF_T, PDQF_NEGATE_ALT_COLS,
    PDQF_NEGATE_ALT_ROWS, PDQF_NEGATE_OFF_DIAGONALS) of n matrices [n, 16, 16] on the GPU,
    as the kernel of `semantics` implements it; returns the transformed matrices."""
    p = np.ascontiguousarray(pdqf, np.float32).reshape(-1, 256)
    n = p.shape[0]
    if n == 0:
        return p.reshape(0, 16, 16).copy()
    d_p = ctx.to_device(p)
    check(ctx.lib.ypdq_pdqf_transform_batch(ctx.handle, d_p.ptr, n, int(op), int(bool(negate)),
                                            _semantics(semantics), None))
    ctx.sync()
    return d_p.download((n, 16, 16), np.float32)


BT601 = (0.299, 0.587, 0.114)  # src/kernel/constants.rs:23


def cvt_luma8f(ctx, pixels, coeffs=BT601):
    """Kernel::cvt_rgb8_to_luma8f / cvt_rgba8_to_luma8f on the GPU (ypdq_cvt_luma8f):
    pixels [..., 3 | 4] u8 -> f32 luma [...], (r_c r + g_c g) + b_c b rounded step by step."""
    px = np.ascontiguousarray(pixels, np.uint8)
    ch = px.shape[-1]
    if ch not in (3, 4):
        raise ValueError("pixels must end in 3 (RGB8) or 4 (RGBA8) channels")
    n = px.size // ch
    if n == 0:
        return np.zeros(px.shape[:-1], np.float32)
    d_px, d_out = ctx.to_device(px), ctx.alloc(n * 4)
    r, g, b = (float(np.float32(c)) for c in coeffs)
    check(ctx.lib.ypdq_cvt_luma8f(ctx.handle, d_px.ptr, n, ch, r, g, b, d_out.ptr, None))
    ctx.sync()
    return d_out.download(px.shape[:-1], np.float32)


def scan_device(ctx, d_rows, n_rows, d_queries, n_queries, threshold, d_hits, capacity, d_count,
                algo=_lib.SCAN_AUTO, stream=None):
    def dp(b):
        return b.ptr if isinstance(b, DeviceBuffer) else b
    check(ctx.lib.ypdq_scan(ctx.handle, dp(d_rows), int(n_rows), dp(d_queries), int(n_queries),
                            int(threshold), dp(d_hits), int(capacity), dp(d_count), int(algo),
                            stream))


def sort_hits_device(ctx, d_hits, n, stream=None):
    check(ctx.lib.ypdq_sort_hits(ctx.handle, d_hits.ptr if isinstance(d_hits, DeviceBuffer) else d_hits,
                                 int(n), stream))


def scan(ctx, db_rows, queries, threshold, algo=_lib.SCAN_AUTO, capacity=1 << 16, sort=True):
    """Exact scan of host rows [n, 32] u8 against host queries [q, 32] u8. Returns hits."""
    rows = np.ascontiguousarray(db_rows, np.uint8).reshape(-1, 32)
    q = np.ascontiguousarray(queries, np.uint8).reshape(-1, 32)
    d_rows = ctx.to_device(rows) if rows.shape[0] else ctx.alloc(32)
    d_q = ctx.to_device(q) if q.shape[0] else ctx.alloc(32)
    d_cnt = ctx.alloc(8)
    while True:
        d_hits = ctx.alloc(max(capacity, 1) * 16)
        scan_device(ctx, d_rows, rows.shape[0], d_q, q.shape[0], threshold, d_hits, capacity,
                    d_cnt, algo)
        ctx.sync()
        total = int(d_cnt.download((1,), np.uint64)[0])
        if total <= capacity:
            break
        capacity = total
    if sort and total > 1:
        sort_hits_device(ctx, d_hits, total)
        ctx.sync()
    return d_hits.download((total,), HIT_DTYPE) if total else np.zeros(0, HIT_DTYPE)


class Database:
    """Device-resident database of 256-bit rows (ypdq_db)."""

    def __init__(self, ctx, rows=None, device_buffer=None, n_rows=None):
        self.ctx = ctx
        h = ctypes.c_void_p()
        if device_buffer is not None:
            self._keep = device_buffer
            check(ctx.lib.ypdq_db_wrap(ctx.handle, device_buffer.ptr, int(n_rows), ctypes.byref(h)))
            self.n_rows = int(n_rows)
        else:
            r = np.ascontiguousarray(rows, np.uint8).reshape(-1, 32)
            check(ctx.lib.ypdq_db_create(ctx.handle, ptr(r), r.shape[0], ctypes.byref(h)))
            self.n_rows = r.shape[0]
        self.handle = h

    @classmethod
    def from_file(cls, ctx, path, chunk_bytes=0):
        """ypdq_db_load_file: a flat file of 32-byte rows onto the device."""
        self = cls.__new__(cls)
        self.ctx = ctx
        h = ctypes.c_void_p()
        check(ctx.lib.ypdq_db_load_file(ctx.handle, os.fsencode(path), int(chunk_bytes),
                                        ctypes.byref(h)))
        self.handle = h
        self.n_rows = self.device_rows()[1]
        return self

    def save(self, path, chunk_bytes=0):
        """ypdq_db_save_file: the device rows to a flat file."""
        check(self.ctx.lib.ypdq_db_save_file(self.handle, os.fsencode(path), int(chunk_bytes)))

    def device_rows(self):
        p = ctypes.c_void_p()
        n = ctypes.c_uint64()
        check(self.ctx.lib.ypdq_db_info(self.handle, ctypes.byref(p), ctypes.byref(n)))
        return p, n.value

    def close(self):
        if self.handle:
            self.ctx.lib.ypdq_db_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def shard_rows(n_rows, world, rank):
    """Row range [lo, hi) of shard `rank` when a database of n_rows is split over `world`
    GPUs in contiguous slices (sizes differ by at most one row). Each GPU scans its slice
    with the whole query batch; no collective is needed."""
    if not 0 <= rank < world:
        raise ValueError("rank %d of world %d" % (rank, world))
    return n_rows * rank // world, n_rows * (rank + 1) // world


def merge_shard_hits(parts):
    """One hit list from per-shard lists: `parts` holds (hits, row_offset) pairs, hits with
    shard-local indices; the result has global indices in the scalar matcher's
    (index, query) order, the list a single scan of the whole database returns."""
    arrs = []
    for hits, offset in parts:
        h = np.array(hits, dtype=HIT_DTYPE, copy=True)
        h["index"] += np.uint64(offset)
        arrs.append(h)
    out = np.concatenate(arrs) if arrs else np.zeros(0, HIT_DTYPE)
    return out[np.lexsort((out["query"], out["index"]))]


def screen_host(ctx, db, images, threshold=31, semantics="exact", dct=_lib.DCT_FP32,
                capacity=1 << 16, want_hashes=False):
    """ypdq_screen_host: hash + 8 dihedrals + scan, from host images to sorted host hits."""
    imgs, kind = input_kind_of(images)
    n = imgs.shape[0]
    while True:
        hits = np.zeros(max(capacity, 1), HIT_DTYPE)
        nh = ctypes.c_uint64()
        hashes = np.zeros((n, 8, 32), np.uint8) if want_hashes else None
        st = ctx.lib.ypdq_screen_host(ctx.handle, db.handle, ptr(imgs), n, kind, int(dct),
                                      _semantics(semantics), int(threshold), ptr(hits), capacity,
                                      ctypes.byref(nh), ptr(hashes), None)
        if st == _lib.ERR_OVERFLOW:
            capacity = int(nh.value)
            continue
        check(st)
        break
    out = hits[: nh.value]
    return (out, hashes) if want_hashes else out
