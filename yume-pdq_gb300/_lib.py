"""ctypes binding of libyumepdq_gb300.so (include/ypdq.h and include/yume_pdq.h).

No computation falls back to the CPU: if the library is missing or no CUDA device
exists, the calls raise.
"""
import ctypes
import os

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB_PATH

HIT_DTYPE = np.dtype([("index", "<u8"), ("query", "<u4"), ("distance", "<u4")])

(OK, ERR_INVALID, ERR_ALIGN, ERR_CUDA, ERR_NOMEM, ERR_OVERFLOW, ERR_TIMEOUT, ERR_UNSUPPORTED,
 ERR_BUSY) = range(9)
STATUS_NAMES = {
    0: "OK", 1: "INVALID", 2: "ALIGN", 3: "CUDA", 4: "NOMEM", 5: "OVERFLOW", 6: "TIMEOUT",
    7: "UNSUPPORTED", 8: "BUSY",
}

INPUT_F32, INPUT_U8, INPUT_RGB8, INPUT_RGBA8 = 0, 1, 2, 3
DCT_FP32, DCT_TF32, DCT_BF16X3 = 0, 1, 2
DIHEDRAL_EXACT, DIHEDRAL_AVX2, DIHEDRAL_SCALAR = 0, 1, 2
SEMANTICS = {"exact": DIHEDRAL_EXACT, "avx2": DIHEDRAL_AVX2, "scalar": DIHEDRAL_SCALAR}
SCAN_AUTO, SCAN_SIMT, SCAN_B1MMA, SCAN_TC, SCAN_TC_FP4, SCAN_TC_FP8 = 0, 1, 2, 3, 4, 5
PDQF_T, PDQF_NEGATE_ALT_COLS, PDQF_NEGATE_ALT_ROWS, PDQF_NEGATE_OFF_DIAGONALS = 0, 1, 2, 3
H2D, D2H, D2D = 0, 1, 2


class YpdqError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


SERVER_MAX_BUCKETS = 16


class ServerConfig(ctypes.Structure):
    """ypdq_server_config."""
    _fields_ = [("input_kind", ctypes.c_int), ("dct_precision", ctypes.c_int),
                ("semantics", ctypes.c_int), ("threshold", ctypes.c_uint32),
                ("max_step_images", ctypes.c_uint32), ("slots", ctypes.c_uint32),
                ("step_hit_capacity", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64),
                ("max_queued_images", ctypes.c_uint64), ("autotune", ctypes.c_int),
                ("target_step_ms", ctypes.c_double)]


class Completion(ctypes.Structure):
    """ypdq_completion."""
    _fields_ = [("request_id", ctypes.c_uint64), ("user_tag", ctypes.c_uint64),
                ("status", ctypes.c_int32), ("n_images", ctypes.c_uint32),
                ("n_hits", ctypes.c_uint64), ("step", ctypes.c_uint64),
                ("latency_us", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    """ypdq_server_stats."""
    _fields_ = [("submitted", ctypes.c_uint64), ("rejected", ctypes.c_uint64),
                ("completed", ctypes.c_uint64), ("images_completed", ctypes.c_uint64),
                ("hits_completed", ctypes.c_uint64), ("steps", ctypes.c_uint64),
                ("rescans", ctypes.c_uint64), ("queued_requests", ctypes.c_uint32),
                ("queued_images", ctypes.c_uint32), ("inflight_steps", ctypes.c_uint32),
                ("slots", ctypes.c_uint32), ("max_step_images", ctypes.c_uint32),
                ("p50_us", ctypes.c_double), ("p99_us", ctypes.c_double),
                ("mean_us", ctypes.c_double), ("max_us", ctypes.c_double),
                ("mean_step_images", ctypes.c_double), ("elapsed_s", ctypes.c_double),
                ("n_buckets", ctypes.c_uint32),
                ("bucket_images", ctypes.c_uint32 * SERVER_MAX_BUCKETS),
                ("bucket_algo", ctypes.c_int32 * SERVER_MAX_BUCKETS),
                ("bucket_n_tile", ctypes.c_uint32 * SERVER_MAX_BUCKETS),
                ("bucket_ms", ctypes.c_float * SERVER_MAX_BUCKETS),
                ("bucket_steps", ctypes.c_uint64 * SERVER_MAX_BUCKETS),
                ("bucket_kernel", ctypes.c_uint32 * SERVER_MAX_BUCKETS)]


# name -> (restype, argtypes); the exported surface of include/*.h
P = ctypes.c_void_p
i32, u32, i64, u64, f32, sz = (ctypes.c_int, ctypes.c_uint32, ctypes.c_int64, ctypes.c_uint64,
                               ctypes.c_float, ctypes.c_size_t)
PP = ctypes.POINTER(ctypes.c_void_p)
SIGNATURES = {
    "ypdq_ctx_create": (i32, [i32, PP]),
    "ypdq_ctx_destroy": (i32, [P]),
    "ypdq_last_error": (ctypes.c_char_p, []),
    "ypdq_check_device_errors": (i32, [P]),
    "ypdq_device_info": (i32, [P, P, P]),
    "ypdq_hash_occupancy": (i32, [P, i32, i32, ctypes.POINTER(ctypes.c_int)]),
    "ypdq_hash_batch": (i32, [P, P, i64, i32, i32, i32, P, P, P, P, i32, P, P]),
    "ypdq_dihedrals_batch": (i32, [P, P, P, i64, i32, P, P, P, P, P]),
    "ypdq_dct2d_batch": (i32, [P, P, i64, i32, P, P]),
    "ypdq_sum_of_gradients_batch": (i32, [P, P, i64, P, P]),
    "ypdq_pdqf_transform_batch": (i32, [P, P, i64, i32, i32, i32, P]),
    "ypdq_cvt_luma8f": (i32, [P, P, i64, i32, f32, f32, f32, P, P]),
    "ypdq_scan": (i32, [P, P, u64, P, u32, u32, P, u64, P, i32, P]),
    "ypdq_sort_hits": (i32, [P, P, u64, P]),
    "ypdq_db_create": (i32, [P, P, u64, PP]),
    "ypdq_db_wrap": (i32, [P, P, u64, PP]),
    "ypdq_db_destroy": (i32, [P]),
    "ypdq_db_info": (i32, [P, P, P]),
    "ypdq_db_load_file": (i32, [P, ctypes.c_char_p, u64, PP]),
    "ypdq_db_save_file": (i32, [P, ctypes.c_char_p, u64]),
    "ypdq_screen_host": (i32, [P, P, P, i64, i32, i32, i32, u32, P, u64, P, P, P]),
    "ypdq_screen_plan": (i32, [i64, i32, i32, u64, u32, P, ctypes.POINTER(ctypes.c_int)]),
    "ypdq_malloc_device": (i32, [P, sz, PP]),
    "ypdq_free_device": (i32, [P, P]),
    "ypdq_malloc_host": (i32, [P, sz, PP]),
    "ypdq_free_host": (i32, [P, P]),
    "ypdq_memcpy": (i32, [P, P, P, sz, i32, P]),
    "ypdq_memset": (i32, [P, P, i32, sz, P]),
    "ypdq_stream_create": (i32, [P, PP]),
    "ypdq_stream_destroy": (i32, [P, P]),
    "ypdq_stream_sync": (i32, [P, P]),
    "ypdq_event_create": (i32, [P, PP]),
    "ypdq_event_destroy": (i32, [P, P]),
    "ypdq_event_record": (i32, [P, P, P]),
    "ypdq_event_elapsed_ms": (i32, [P, P, P, ctypes.POINTER(ctypes.c_float)]),
    "ypdq_synth_rows": (i32, [P, P, u64, u64, u64, P]),
    "ypdq_synth_clustered_rows": (i32, [P, P, u64, u64, u64, u32, u64, P]),
    "ypdq_constants": (i32, [P, P]),
    "ypdq_dropin_semantics": (i32, [ctypes.POINTER(ctypes.c_int)]),
    "ypdq_set_scan_wait_limit": (i32, [u64]),
    "ypdq_debug_stall_scans": (i32, [i32]),
    "ypdq_screen_noalloc": (i32, [P, i64, i32, i32, P, u64, u32, P, u64, P, P]),
    "ypdq_server_config_default": (i32, [ctypes.POINTER(ServerConfig)]),
    "ypdq_server_create": (i32, [P, P, ctypes.POINTER(ServerConfig), PP]),
    "ypdq_server_submit": (i32, [P, P, u32, P, u64, P, P, u64, ctypes.POINTER(ctypes.c_uint64)]),
    "ypdq_server_replay": (i32, [P, P, u32, P, P, P, u32, u64, P, u64, P,
                                 ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
    "ypdq_server_poll": (i32, [P, ctypes.POINTER(Completion), u32, ctypes.POINTER(ctypes.c_uint32),
                               i64]),
    "ypdq_server_get_stats": (i32, [P, ctypes.POINTER(ServerStats), i32]),
    "ypdq_server_destroy": (i32, [P]),
    "yume_pdq_hash_smart_kernel": (f32, [P, P, P, P, P, P]),
    "yume_pdq_visit_dihedrals_smart_kernel": (ctypes.c_bool, [P, f32, P, P, P]),
}
DATA_SYMBOLS = [
    "YUME_PDQ_VERSION_MAJOR", "YUME_PDQ_VERSION_MINOR", "YUME_PDQ_VERSION_PATCH",
    "YUME_PDQ_VERSION_STRING", "YUME_PDQ_DIHEDRAL_NORMAL", "YUME_PDQ_DIHEDRAL_FLIPPED",
    "YUME_PDQ_DIHEDRAL_FLOPPED", "YUME_PDQ_DIHEDRAL_ROTATED_180", "YUME_PDQ_DIHEDRAL_ROTATED_90",
    "YUME_PDQ_DIHEDRAL_ROTATED_270", "YUME_PDQ_DIHEDRAL_ROTATED_90_FLOPPED",
    "YUME_PDQ_DIHEDRAL_FLOPPED_ROTATED_270",
]

DihedralCallback = ctypes.CFUNCTYPE(ctypes.c_bool, ctypes.c_void_p, ctypes.c_uint32,
                                    ctypes.c_float, ctypes.c_float)

_lib = None


def load(build_if_missing=True):
    """Load the shared library (building it first if it is absent). Raises on failure."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise OSError("libyumepdq_gb300.so is not built (%s)" % LIB_PATH)
        _build.build()
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status):
    if status != OK:
        msg = load().ypdq_last_error()
        raise YpdqError(status, msg.decode() if msg else "")
    return status


def ptr(a):
    """Host pointer of a numpy array (or None)."""
    if a is None:
        return None
    return ctypes.c_void_p(a.ctypes.data)
