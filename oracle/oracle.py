"""ctypes binding of the CPU oracle (``oracle/ypdq_oracle.c``).

TEST INFRASTRUCTURE ONLY. The tests, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` use it as the reference for results. The product never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libypdq_oracle.so")

# Sign conventions of pdqf_negate_alt_rows::<true> / pdqf_negate_alt_cols::<false>
# (bit i set = row/column i negated).
SEMANTICS = {
    "exact": (0x5555, 0x5555),   # Avx512F32Kernel: the true flip/flop sign pattern
    "avx2": (0x5555, 0x0055),    # Avx2F32Kernel: columns 8..15 are left untouched
    "scalar": (0xAAAA, 0x5555),  # trait default: DefaultKernel / ReferenceKernel
}

HIT_DTYPE = np.dtype([("index", "<u8"), ("query", "<u4"), ("distance", "<u4")])

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        f32, i64, u32, i32 = ctypes.c_float, ctypes.c_int64, ctypes.c_uint32, ctypes.c_int
        sig = {
            "ypdqo_init": (None, []),
            "ypdqo_dct_matrix_f32": (None, [P]),
            "ypdqo_dct_matrix_f64": (None, [P]),
            "ypdqo_tent_weights": (None, [P]),
            "ypdqo_compress": (None, [P, P]),
            "ypdqo_dct2d": (None, [P, P]),
            "ypdqo_dct2d_f64": (None, [P, P]),
            "ypdqo_sum_of_gradients": (f32, [P]),
            "ypdqo_adjust_quality": (f32, [f32]),
            "ypdqo_torben_median": (f32, [P]),
            "ypdqo_threshold_2d": (None, [P, P, f32]),
            "ypdqo_quantize": (None, [P, P, P]),
            "ypdqo_hash_get_threshold": (f32, [P, P, P, P, P]),
            "ypdqo_dihedrals": (None, [P, f32, u32, u32, P, P, P, P]),
            "ypdqo_hash_batch": (None, [P, i64, i32, u32, u32, P, P, P, P, i32]),
            "ypdqo_find_all": (i64, [P, i64, P, i32, u32, P, i64, i32]),
            "ypdqo_count_all": (i64, [P, i64, P, i32, u32, i32]),
            "ypdqo_fm_sine_image": (None, [P]),
            "ypdqo_synth_rows": (None, [P, i64, ctypes.c_uint64, ctypes.c_uint64, i32]),
            "ypdqo_luma": (None, [P, i64, i32, P]),
            "ypdqo_jarosz_compress": (None, [P, P]),
            "ypdqo_dct2d_reference": (None, [P, P]),
            "ypdqo_hash_batch_avx2": (None, [P, i64, i32, P, P, P, P, i32]),
            "ypdqo_dct2d_matrix": (None, [P, P, P]),
            "ypdqo_dct2d_avx2_matrix": (None, [P, P, P]),
            "ypdqo_hash_batch_reference": (None, [P, i64, i32, ctypes.c_uint32, ctypes.c_uint32,
                                                  P, P, P, P, P, i32]),
            "ypdqo_synth_clustered": (None, [P, i64, ctypes.c_uint64, ctypes.c_uint64,
                                             ctypes.c_uint32, ctypes.c_uint64, i32]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        L.ypdqo_init()
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def dct_matrix_f32():
    out = np.empty((16, 127), np.float32)
    lib().ypdqo_dct_matrix_f32(_p(out))
    return out


def dct_matrix_f64():
    out = np.empty((16, 127), np.float64)
    lib().ypdqo_dct_matrix_f64(_p(out))
    return out


def tent_weights():
    out = np.empty((7, 7), np.float32)
    lib().ypdqo_tent_weights(_p(out))
    return out


def compress(img):
    img = np.ascontiguousarray(img, np.float32)
    out = np.empty((127, 127), np.float32)
    lib().ypdqo_compress(_p(img), _p(out))
    return out


def dct2d(buf):
    buf = np.ascontiguousarray(buf, np.float32)
    out = np.empty((16, 16), np.float32)
    lib().ypdqo_dct2d(_p(buf), _p(out))
    return out


def dct2d_f64(buf):
    buf = np.ascontiguousarray(buf, np.float32)
    out = np.empty((16, 16), np.float64)
    lib().ypdqo_dct2d_f64(_p(buf), _p(out))
    return out


def sum_of_gradients(p):
    return lib().ypdqo_sum_of_gradients(_p(np.ascontiguousarray(p, np.float32)))


def adjust_quality(g):
    return lib().ypdqo_adjust_quality(g)


def torben_median(p):
    return lib().ypdqo_torben_median(_p(np.ascontiguousarray(p, np.float32)))


def threshold_2d(p, thr):
    out = np.zeros(32, np.uint8)
    lib().ypdqo_threshold_2d(_p(np.ascontiguousarray(p, np.float32)), _p(out), thr)
    return out


def quantize(p):
    out = np.zeros(32, np.uint8)
    thr = np.zeros(1, np.float32)
    lib().ypdqo_quantize(_p(np.ascontiguousarray(p, np.float32)), _p(thr), _p(out))
    return out, float(thr[0])


def hash_get_threshold(img):
    """(hash[32], threshold, quality, buf127x127, pdqf16x16) for one 512x512 f32 image."""
    img = np.ascontiguousarray(img, np.float32)
    out = np.zeros(32, np.uint8)
    thr = np.zeros(1, np.float32)
    buf = np.empty((127, 127), np.float32)
    pdqf = np.empty((16, 16), np.float32)
    q = lib().ypdqo_hash_get_threshold(_p(img), _p(thr), _p(out), _p(buf), _p(pdqf))
    return out, float(thr[0]), float(q), buf, pdqf


def dihedrals(pdqf, threshold, semantics="exact"):
    """Seven derived variants in visit order: (hashes[7,32], thr[7], quality[7], pdqf[7,16,16])."""
    rm, cm = SEMANTICS[semantics]
    p = np.ascontiguousarray(pdqf, np.float32)
    h = np.zeros((7, 32), np.uint8)
    t = np.zeros(7, np.float32)
    q = np.zeros(7, np.float32)
    pv = np.zeros((7, 16, 16), np.float32)
    lib().ypdqo_dihedrals(_p(p), threshold, rm, cm, _p(h), _p(t), _p(q), _p(pv))
    return h, t, q, pv


def hash_batch(imgs, semantics="exact", nthreads=None, want_pdqf=False):
    """Hash n images (f32 or u8, [n,512,512]); returns hashes[n,8,32], quality[n,8], thr[n,8], pdqf."""
    rm, cm = SEMANTICS[semantics]
    imgs = np.ascontiguousarray(imgs)
    is_u8 = imgs.dtype == np.uint8
    if not is_u8:
        imgs = imgs.astype(np.float32, copy=False)
    n = imgs.shape[0]
    h = np.zeros((n, 8, 32), np.uint8)
    q = np.zeros((n, 8), np.float32)
    t = np.zeros((n, 8), np.float32)
    p = np.zeros((n, 16, 16), np.float32) if want_pdqf else None
    nt = nthreads or os.cpu_count() or 1
    lib().ypdqo_hash_batch(_p(imgs), n, int(is_u8), rm, cm, _p(h), _p(q), _p(t),
                           _p(p) if p is not None else None, nt)
    return h, q, t, p


def find_all(db, needles, threshold, nthreads=None, cap=None):
    """All hits (index, query, distance) in scalar-matcher order; db [n,32] u8, needles [q,32] u8."""
    db = np.ascontiguousarray(db, np.uint8)
    needles = np.ascontiguousarray(needles, np.uint8)
    nt = nthreads or os.cpu_count() or 1
    if cap is None:
        cap = 1 << 16
    while True:
        out = np.zeros(cap, HIT_DTYPE)
        n = lib().ypdqo_find_all(_p(db), db.shape[0], _p(needles), needles.shape[0],
                                 threshold, _p(out), cap, nt)
        if n <= cap:
            return out[:n]
        cap = n


def count_all(db, needles, threshold, nthreads=None):
    db = np.ascontiguousarray(db, np.uint8)
    needles = np.ascontiguousarray(needles, np.uint8)
    nt = nthreads or os.cpu_count() or 1
    return lib().ypdqo_count_all(_p(db), db.shape[0], _p(needles), needles.shape[0],
                                 threshold, nt)


def fm_sine_image():
    out = np.empty((512, 512), np.float32)
    lib().ypdqo_fm_sine_image(_p(out))
    return out


def synth_rows(n, seed, first=0, nthreads=None):
    """CPU twin of the library's ypdq_synth_rows (identical rows for the same seed)."""
    out = np.empty((n, 32), np.uint8)
    lib().ypdqo_synth_rows(_p(out), n, first, seed, nthreads or os.cpu_count() or 1)
    return out


def synth_clustered(n, members, trials, seed, first=0, nthreads=None):
    """CPU twin of the library's ypdq_synth_clustered_rows (identical rows)."""
    out = np.empty((n, 32), np.uint8)
    lib().ypdqo_synth_clustered(_p(out), n, first, members, trials, seed,
                                nthreads or os.cpu_count() or 1)
    return out


def luma(px):
    """RGB8/RGBA8 pixels [..., 3 or 4] u8 -> f32 luma [...] in the reference's scalar order."""
    px = np.ascontiguousarray(px, np.uint8)
    out = np.empty(px.shape[:-1], np.float32)
    lib().ypdqo_luma(_p(px), out.size, px.shape[-1], _p(out))
    return out


def jarosz_compress(img):
    """ReferenceKernel<f32>::jarosz_compress: full Jarosz filter + sampling -> [127, 127]."""
    img = np.ascontiguousarray(img, np.float32)
    out = np.empty((127, 127), np.float32)
    lib().ypdqo_jarosz_compress(_p(img), _p(out))
    return out


def hash_batch_reference(imgs, semantics="scalar", nthreads=None):
    """ReferenceKernel<f32> over n images (f32 or u8 [n, 512, 512]) with dihedrals; returns
    hashes [n,8,32], quality [n,8], thresholds [n,8], pdqf [n,16,16], buf127 [n,127,127]."""
    rm, cm = SEMANTICS[semantics]
    imgs = np.ascontiguousarray(imgs)
    is_u8 = imgs.dtype == np.uint8
    if not is_u8:
        imgs = imgs.astype(np.float32, copy=False)
    n = imgs.shape[0]
    h = np.zeros((n, 8, 32), np.uint8)
    q = np.zeros((n, 8), np.float32)
    t = np.zeros((n, 8), np.float32)
    p = np.zeros((n, 16, 16), np.float32)
    b = np.zeros((n, 127, 127), np.float32)
    lib().ypdqo_hash_batch_reference(_p(imgs), n, int(is_u8), rm, cm, _p(h), _p(q), _p(t), _p(p),
                                     _p(b), nthreads or os.cpu_count() or 1)
    return h, q, t, p, b


def hash_batch_avx2(imgs, nthreads=None):
    """yume-pdq's Avx2F32Kernel (FMA compress and DCT, residual-mean quantizer, its own
    dihedral sign patterns) over n images (f32 or u8 [n, 512, 512]); returns hashes
    [n,8,32], quality [n,8], thresholds [n,8], pdqf [n,16,16]."""
    imgs = np.ascontiguousarray(imgs)
    is_u8 = imgs.dtype == np.uint8
    if not is_u8:
        imgs = imgs.astype(np.float32, copy=False)
    n = imgs.shape[0]
    h = np.zeros((n, 8, 32), np.uint8)
    q = np.zeros((n, 8), np.float32)
    t = np.zeros((n, 8), np.float32)
    p = np.zeros((n, 16, 16), np.float32)
    lib().ypdqo_hash_batch_avx2(_p(imgs), n, int(is_u8), _p(h), _p(q), _p(t), _p(p),
                                nthreads or os.cpu_count() or 1)
    return h, q, t, p


def dct2d_matrix(D, buf127):
    """The DefaultKernel DCT (four partial sums) of a 127x127 buffer with a given 16x127
    matrix."""
    D = np.ascontiguousarray(D, np.float32)
    b = np.ascontiguousarray(buf127, np.float32)
    out = np.zeros((16, 16), np.float32)
    lib().ypdqo_dct2d_matrix(_p(D), _p(b), _p(out))
    return out


def dct2d_avx2_matrix(D, buf128):
    """The Avx2F32Kernel DCT of a 128x128 zero-padded buffer with a given 16x127 matrix."""
    D = np.ascontiguousarray(D, np.float32)
    b = np.ascontiguousarray(buf128, np.float32)
    out = np.zeros((16, 16), np.float32)
    lib().ypdqo_dct2d_avx2_matrix(_p(D), _p(b), _p(out))
    return out


def pdqf_transform(pdqf, op, negate=False, semantics="scalar"):
    """The Kernel trait's PDQF transforms as each reference kernel implements them, on one
    16x16 matrix (a copy is returned). op: 0 pdqf_t (src/kernel/mod.rs:345-361), 1
    pdqf_negate_alt_cols::<NEGATE> (trait :368-383; Avx2F32Kernel src/kernel/x86.rs:330-378,
    one 8-wide multiply per row; Avx512F32Kernel :1026-1079), 2 pdqf_negate_alt_rows::<NEGATE>
    (trait :391-406; AVX2 :285-327 and AVX-512 :989-1024 start at the other row), 3
    pdqf_negate_off_diagonals (:413-427, the same in every kernel)."""
    q = np.array(pdqf, np.float32, copy=True).reshape(16, 16)
    if op == 0:
        for i in range(16):
            for j in range(16):
                if i < j:
                    q[i, j], q[j, i] = q[j, i], q[i, j]
    elif op == 1:
        if semantics == "avx2":
            coef = np.array(([1.0, -1.0] if negate else [-1.0, 1.0]) * 4, np.float32)
            for i in range(16):
                q[i, :8] = q[i, :8] * coef
        else:
            for i in range(16):
                for j in range(1 if negate else 0, 16, 2):
                    q[i, j] = -q[i, j]
    elif op == 2:
        start = (1 if negate else 0) if semantics == "scalar" else (0 if negate else 1)
        for i in range(start, 16, 2):
            q[i, :] = -q[i, :]
    elif op == 3:
        for i in range(16):
            for j in range(16):
                if (j - i) % 2 == 1:
                    q[i, j] = -q[i, j]
    else:
        raise ValueError(op)
    return q


def luma_with(px, coeffs):
    """cvt_rgb8_to_luma8f / cvt_rgba8_to_luma8f (src/kernel/mod.rs:303-340) with given
    coefficients: (r_c r + g_c g) + b_c b, every product and sum rounded to f32."""
    px = np.asarray(px, np.uint8)
    r, g, b = (px[..., c].astype(np.float32) for c in range(3))
    rc, gc, bc = (np.float32(c) for c in coeffs)
    return ((rc * r + gc * g) + bc * b).astype(np.float32)
