"""The reference's pipeline API and Kernel surface, backed by the CUDA library.

Mirrors yume-pdq's src/lib.rs (hash, hash_get_threshold, hash_float, visit_dihedrals,
Dihedrals) and the Kernel trait (src/kernel/mod.rs:268-497). Arguments have the same meaning
and order; Rust's `&mut` outputs become numpy arrays filled in place, and the functions
return what the Rust functions return. Per-image calls run a batch of one on the GPU. The
batched entry point `CudaKernel.hash_batch` is the fast path.
"""
import numpy as np

from . import _lib, core

QUALITY_ADJUST_DIVISOR = 180  # src/kernel/mod.rs:257


def _pack(xx, xy, yx, yy):
    return int.from_bytes(bytes([xx & 0xFF, xy & 0xFF, yx & 0xFF, yy & 0xFF]), "big")


class Dihedrals:
    """Packed dihedral transforms (src/lib.rs:85-134)."""

    NORMAL = _pack(1, 0, 0, 1)
    FLIPPED = _pack(1, 0, 0, -1)
    FLOPPED = _pack(-1, 0, 0, 1)
    ROTATED_180 = _pack(-1, 0, 0, -1)
    ROTATED_90 = _pack(0, 1, -1, 0)
    ROTATED_270 = _pack(0, 1, 1, 0)
    ROTATED_90_FLOPPED = _pack(0, -1, -1, 0)
    FLOPPED_ROTATED_270 = _pack(0, -1, 1, 0)

    @staticmethod
    def into_tuples(packed):
        b = [((packed >> s) & 0xFF) for s in (24, 16, 8, 0)]
        b = [x - 256 if x > 127 else x for x in b]
        return (b[0], b[1]), (b[2], b[3])


def host_semantics():
    """Name of the dihedral sign convention that yume-pdq's smart_kernel() uses on this host
    (src/kernel/mod.rs:79-176; ypdq_dropin_semantics): "avx2" on x86_64 with AVX2 and FMA,
    "scalar" on any other host, unless YUME_PDQ_DIHEDRAL_SEMANTICS overrides it."""
    import ctypes
    s = ctypes.c_int(-1)
    _lib.check(_lib.load().ypdq_dropin_semantics(ctypes.byref(s)))
    return ("exact", "avx2", "scalar")[s.value]


# Slot order of every batched output: the image, then visit_dihedrals' order.
SLOT_DIHEDRALS = [
    Dihedrals.NORMAL, Dihedrals.FLOPPED, Dihedrals.ROTATED_180, Dihedrals.FLIPPED,
    Dihedrals.ROTATED_90_FLOPPED, Dihedrals.ROTATED_270, Dihedrals.FLOPPED_ROTATED_270,
    Dihedrals.ROTATED_90,
]


class CudaKernel:
    """GPU implementation of the Kernel trait surface.

    semantics selects the dihedral sign convention ("exact" = Avx512F32Kernel, "avx2" =
    Avx2F32Kernel, "scalar" = the trait default); see include/ypdq.h.
    """

    InputDimension = 512
    OutputDimension = 16
    Buffer1WidthX = 128
    Buffer1LengthY = 128

    def __init__(self, ctx=None, semantics="exact", dct=_lib.DCT_FP32):
        self.ctx = ctx or core.Context(0)
        self.semantics = semantics
        self.dct = dct

    def ident(self):
        return "cuda_sm103a_f32_exact" if self.dct == _lib.DCT_FP32 else "cuda_sm103a_tensor"

    @staticmethod
    def required_hardware_features_met():
        try:
            _lib.load()
            return True
        except OSError:
            return False

    # -- batched fast path
    def hash_batch(self, images, want_pdqf=False, pdqf_slots=1):
        return core.hash_batch(self.ctx, images, semantics=self.semantics, dct=self.dct,
                               want_pdqf=want_pdqf, pdqf_slots=pdqf_slots)

    # -- trait methods (batch of one)
    def jarosz_compress(self, buffer, output):
        """Tent-filter compress 512x512 -> 127x127 into output[:127, :127]."""
        r = core.hash_batch(self.ctx, np.asarray(buffer, np.float32)[None], self.semantics,
                            self.dct, want_buf1=True)
        output[:127, :127] = r["buf1"][0]

    def quantize(self, input, output):
        """Median-threshold a 16x16 PDQF into output (32 bytes); returns the threshold."""
        r = self._quantize(input)
        output.reshape(-1)[:] = r[0]
        return r[1]

    def _quantize(self, pdqf):
        ctx = self.ctx
        p = np.ascontiguousarray(pdqf, np.float32).reshape(1, 256)
        d_p = ctx.to_device(p)
        d_h, d_q, d_t = ctx.alloc(256), ctx.alloc(32), ctx.alloc(32)
        _lib.check(ctx.lib.ypdq_dihedrals_batch(ctx.handle, d_p.ptr, None, 1,
                                                _lib.SEMANTICS[self.semantics], d_h.ptr, d_q.ptr,
                                                d_t.ptr, None, None))
        ctx.sync()
        h = d_h.download((8, 32), np.uint8)
        t = d_t.download((8,), np.float32)
        return h[0], float(t[0])

    @staticmethod
    def adjust_quality(gradient_sum):
        return min(float(np.float32(gradient_sum) / np.float32(QUALITY_ADJUST_DIVISOR)), 1.0)

    def dct2d(self, buffer, tmp_row_buffer, output):
        """Kernel::dct2d (src/kernel/mod.rs:484): the compressed buffer (127x127, or the
        reference's 128x128 padded Buffer1, first 127 rows and columns read) -> output
        16x16 PDQF. tmp_row_buffer is the reference's scratch row and is left untouched."""
        output[:] = core.dct2d_batch(self.ctx, np.asarray(buffer, np.float32)[None, :127])[0]

    def sum_of_gradients(self, input):
        """Kernel::sum_of_gradients (src/kernel/mod.rs:469)."""
        return float(core.sum_of_gradients_batch(self.ctx, np.asarray(input, np.float32)[None])[0])

    def _pdqf_op(self, pdqf, op, negate=False):
        pdqf[:] = core.pdqf_transform_batch(self.ctx, np.asarray(pdqf, np.float32)[None], op,
                                            negate, self.semantics)[0]

    def pdqf_t(self, input):
        """Kernel::pdqf_t (src/kernel/mod.rs:345): transpose in place."""
        self._pdqf_op(input, _lib.PDQF_T)

    def pdqf_negate_alt_cols(self, input, negate=False):
        """Kernel::pdqf_negate_alt_cols::<NEGATE> (src/kernel/mod.rs:368), in place, with
        this kernel's sign convention (the AVX2 kernel touches columns 0..7 only)."""
        self._pdqf_op(input, _lib.PDQF_NEGATE_ALT_COLS, negate)

    def pdqf_negate_alt_rows(self, input, negate=False):
        """Kernel::pdqf_negate_alt_rows::<NEGATE> (src/kernel/mod.rs:391), in place, with
        this kernel's sign convention (the AVX2/AVX-512 kernels negate the other rows)."""
        self._pdqf_op(input, _lib.PDQF_NEGATE_ALT_ROWS, negate)

    def pdqf_negate_off_diagonals(self, input):
        """Kernel::pdqf_negate_off_diagonals (src/kernel/mod.rs:413), in place."""
        self._pdqf_op(input, _lib.PDQF_NEGATE_OFF_DIAGONALS)

    def cvt_rgb8_to_luma8f(self, input, output, coeffs=core.BT601):
        """Kernel::cvt_rgb8_to_luma8f (src/kernel/mod.rs:303): a row of RGB8 pixels
        ([..., 3] u8) -> f32 luma in output."""
        output[...] = core.cvt_luma8f(self.ctx, np.asarray(input, np.uint8)[..., :3], coeffs)

    def cvt_rgba8_to_luma8f(self, input, output, coeffs=core.BT601):
        """Kernel::cvt_rgba8_to_luma8f (src/kernel/mod.rs:324): RGBA8 ([..., 4] u8, alpha
        ignored) -> f32 luma in output."""
        output[...] = core.cvt_luma8f(self.ctx, np.asarray(input, np.uint8), coeffs)


def hash_get_threshold(kernel, input, output, buf1, tmp, pdqf):
    """src/lib.rs:427-455. Fills output (32 B), buf1 (127x127 region), pdqf (16x16).

    Returns (quality, threshold)."""
    r = core.hash_batch(kernel.ctx, np.asarray(input, np.float32).reshape(1, 512, 512),
                        kernel.semantics, kernel.dct, want_pdqf=True, want_buf1=buf1 is not None)
    output.reshape(-1)[:] = r["hashes"][0, 0]
    if buf1 is not None:
        buf1[:127, :127] = r["buf1"][0]
    pdqf[:] = r["pdqf"][0, 0]
    return float(r["quality"][0, 0]), float(r["thresholds"][0, 0])


def hash(kernel, input, output, buf1, tmp, pdqf):
    """src/lib.rs:322-353: hash_get_threshold without the threshold. Returns quality."""
    return hash_get_threshold(kernel, input, output, buf1, tmp, pdqf)[0]


def hash_float(kernel, input, output, buf1, tmp):
    """src/lib.rs:464-479: the unquantized PDQF into output. Returns quality."""
    r = core.hash_batch(kernel.ctx, np.asarray(input, np.float32).reshape(1, 512, 512),
                        kernel.semantics, kernel.dct, want_pdqf=True, want_buf1=buf1 is not None)
    output[:] = r["pdqf"][0, 0]
    if buf1 is not None:
        buf1[:127, :127] = r["buf1"][0]
    return float(r["quality"][0, 0])


def visit_dihedrals(kernel, pdqf, output, threshold, f):
    """src/lib.rs:358-420. Calls f(dihedral, threshold, (quality, pdqf, output)) for the
    seven derived variants in the reference order; pdqf and output hold the variant while
    f runs. If f raises, the visit stops and the exception propagates (the Rust Err path)."""
    r = core.dihedrals_batch(kernel.ctx, np.asarray(pdqf, np.float32)[None],
                             np.array([threshold], np.float32), kernel.semantics)
    for s in range(1, 8):
        output.reshape(-1)[:] = r["hashes"][0, s]
        pdqf[:] = r["pdqf"][0, s]
        f(SLOT_DIHEDRALS[s], float(r["thresholds"][0, s]), (float(r["quality"][0, s]), pdqf, output))
