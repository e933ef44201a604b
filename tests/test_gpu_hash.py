"""GPU parity of the fused hash kernel against the oracle (yume-pdq's scalar f32 kernel).

The FP32 path is bit-exact: hashes, thresholds, qualities, PDQF and the compressed image
must equal the oracle's bit for bit. Every call goes through the C ABI.
"""
import ctypes
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def same_bits(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def same_values(a, b):
    """Equal as floats (-0.0 == +0.0), NaN positions equal."""
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


@pytest.mark.parametrize("semantics", ["exact", "avx2", "scalar"])
def test_hash_batch_bit_exact(ctx, yp, oracle, semantics):
    imgs, kind = yp.synth.mixed_images(24, seed=101)
    got = yp.hash_batch(ctx, imgs, semantics=semantics, want_pdqf=True, pdqf_slots=8)
    h, q, t, p = oracle.hash_batch(imgs, semantics=semantics, want_pdqf=True)
    assert np.array_equal(got["hashes"], h)
    assert same_bits(got["quality"], q)
    assert same_values(got["thresholds"], t)
    assert same_bits(got["pdqf"][:, 0], p)
    # every slot's matrix equals the oracle's visit_dihedrals buffer
    for n in range(len(imgs)):
        dh, dt, dq, dp = oracle.dihedrals(p[n], t[n, 0], semantics)
        assert same_bits(got["pdqf"][n, 1:], dp)
        assert np.array_equal(got["hashes"][n, 1:], dh)


def test_u8_input(ctx, yp, oracle):
    imgs = yp.synth.to_u8(yp.synth.mixed_images(16, seed=5)[0])
    got = yp.hash_batch(ctx, imgs)
    h, q, t, _ = oracle.hash_batch(imgs)
    assert np.array_equal(got["hashes"], h)
    assert same_bits(got["quality"], q)
    # u8 and the same values as f32 give the same result
    got32 = yp.hash_batch(ctx, imgs.astype(np.float32))
    assert np.array_equal(got32["hashes"], got["hashes"])


def test_compressed_image_bit_exact(ctx, yp, oracle):
    imgs = yp.synth.blob_images(3, seed=8)
    got = yp.hash_batch(ctx, imgs, want_buf1=True)
    for n in range(3):
        assert same_bits(got["buf1"][n], oracle.compress(imgs[n]))


@pytest.mark.parametrize("n", [1, 2, 7, 305, 1000])
def test_batch_sizes(ctx, yp, oracle, n):
    """More images than resident CTAs: each CTA loops, so the stage ring wraps many times."""
    rng = np.random.default_rng(n)
    imgs = rng.uniform(0, 255, (n, 512, 512)).astype(np.float32)
    imgs[::3] = yp.synth.blob_images(len(imgs[::3]), seed=n)
    got = yp.hash_batch(ctx, imgs)
    h, q, t, _ = oracle.hash_batch(imgs)
    assert np.array_equal(got["hashes"], h)
    assert same_bits(got["quality"], q)


def test_edge_images(ctx, yp, oracle):
    """Constant, black, white, single-pixel and negative/large-valued finite images."""
    imgs = np.zeros((7, 512, 512), np.float32)
    imgs[1] = 255.0
    imgs[2] = 77.0
    imgs[3, 200, 300] = 255.0
    imgs[4, 1, 6] = 200.0      # only a residue tap of the row-0 weights sees it
    imgs[4, 1, 9] = 13.0
    rng = np.random.default_rng(3)
    imgs[5] = rng.normal(0, 1e6, (512, 512))
    imgs[6] = rng.uniform(-1e-30, 1e-30, (512, 512))
    got = yp.hash_batch(ctx, imgs, want_pdqf=True, want_buf1=True)
    h, q, t, p = oracle.hash_batch(imgs, want_pdqf=True)
    assert np.array_equal(got["hashes"], h)
    assert same_bits(got["quality"], q)
    assert same_bits(got["pdqf"][:, 0], p)
    assert same_values(got["thresholds"], t)
    for n in range(len(imgs)):
        assert same_bits(got["buf1"][n], oracle.compress(imgs[n]))


def test_readme_kat_on_gpu(ctx, yp, oracle):
    kat = json.load(open(os.path.join(GOLDEN, "readme_fm_sine.json")))
    img = oracle.fm_sine_image()
    got = yp.hash_batch(ctx, img[None], want_pdqf=True)
    expected = np.frombuffer(bytes.fromhex(kat["expected_hash_hex"]), np.uint8)
    diff = int(np.unpackbits(got["hashes"][0, 0] ^ expected).sum())
    assert diff <= kat["max_bits_different"]
    assert np.all(np.abs(got["pdqf"][0, 0] - np.array(kat["pdqf_printed_1dp"])) <= 0.0500001)


def test_golden_vectors_on_gpu(ctx, yp):
    g = np.load(os.path.join(GOLDEN, "oracle_vectors.npz"))
    for sem in ("exact", "avx2", "scalar"):
        got = yp.hash_batch(ctx, g["images_u8"], semantics=sem)
        assert np.array_equal(got["hashes"], g["hashes_" + sem])
        assert same_bits(got["quality"], g["quality_" + sem])


@pytest.mark.parametrize("semantics", ["exact", "avx2", "scalar"])
def test_dihedrals_batch(ctx, yp, oracle, semantics):
    rng = np.random.default_rng(11)
    p = rng.normal(0, 50, (40, 16, 16)).astype(np.float32)
    thr = rng.normal(0, 5, 40).astype(np.float32)
    got = yp.core.dihedrals_batch(ctx, p, thr, semantics)
    for n in range(40):
        dh, dt, dq, dp = oracle.dihedrals(p[n], float(thr[n]), semantics)
        assert np.array_equal(got["hashes"][n, 1:], dh)
        assert same_values(got["thresholds"][n, 1:], dt)
        assert same_bits(got["quality"][n, 1:], dq)
        assert same_bits(got["pdqf"][n, 1:], dp)
        assert np.array_equal(got["hashes"][n, 0], oracle.threshold_2d(p[n], float(thr[n])))


def test_kernel_surface(ctx, yp, oracle):
    """The reference's pipeline functions (src/lib.rs) through the Kernel mirror."""
    k = yp.CudaKernel(ctx)
    img = yp.synth.blob_images(1, seed=77)[0]
    out = np.zeros(32, np.uint8)
    buf1 = np.zeros((128, 128), np.float32)
    pdqf = np.zeros((16, 16), np.float32)
    q, thr = yp.hash_get_threshold(k, img, out, buf1, None, pdqf)
    h0, t0, q0, b0, p0 = oracle.hash_get_threshold(img)
    assert np.array_equal(out, h0) and thr == t0 and q == q0
    assert same_bits(buf1[:127, :127], b0) and np.all(buf1[127] == 0) and np.all(buf1[:, 127] == 0)
    assert same_bits(pdqf, p0)
    hq, ht = k.quantize(p0, np.zeros(32, np.uint8)), None
    oh, ot = oracle.quantize(p0)
    o2 = np.zeros(32, np.uint8)
    assert k.quantize(p0, o2) == ot and np.array_equal(o2, oh)
    seen = []
    yp.visit_dihedrals(k, pdqf, out, thr, lambda d, t, x: seen.append((d, t, x[0], x[2].copy())))
    dh, dt, dq, dp = oracle.dihedrals(p0, t0, "exact")
    assert [s[0] for s in seen] == yp.SLOT_DIHEDRALS[1:]
    for v in range(7):
        assert np.array_equal(seen[v][3], dh[v]) and seen[v][1] == dt[v] and seen[v][2] == dq[v]


def test_dropin_hash_symbol(yp, oracle):
    """yume_pdq_hash_smart_kernel with the reference's calling convention (integration/hash.py)."""
    lib = yp._lib.load()
    img = yp.synth.blob_images(1, seed=55)[0]
    thr = ctypes.c_float(0.0)
    out = (ctypes.c_uint8 * 32)()
    buf1 = np.full((128, 128), 7.0, np.float32)  # padding must stay untouched
    tmp = np.zeros(128, np.float32)
    pdqf = np.zeros((16, 16), np.float32)
    q = lib.yume_pdq_hash_smart_kernel(img.ctypes.data_as(ctypes.c_void_p), ctypes.byref(thr), out,
                                       buf1.ctypes.data_as(ctypes.c_void_p),
                                       tmp.ctypes.data_as(ctypes.c_void_p),
                                       pdqf.ctypes.data_as(ctypes.c_void_p))
    h0, t0, q0, b0, p0 = oracle.hash_get_threshold(img)
    assert q == q0 and thr.value == t0
    assert bytes(out) == h0.tobytes()
    assert same_bits(buf1[:127, :127], b0) and np.all(buf1[127] == 7.0) and np.all(buf1[:, 127] == 7.0)
    assert same_bits(pdqf, p0)
    # NULL threshold is allowed
    q2 = lib.yume_pdq_hash_smart_kernel(img.ctypes.data_as(ctypes.c_void_p), None, out,
                                        buf1.ctypes.data_as(ctypes.c_void_p),
                                        tmp.ctypes.data_as(ctypes.c_void_p),
                                        pdqf.ctypes.data_as(ctypes.c_void_p))
    assert q2 == q0


def test_dropin_visit_symbol(yp, oracle):
    """yume_pdq_visit_dihedrals_smart_kernel derives the dihedrals with the sign convention
    of the kernel the reference's smart_kernel() picks on this host (the trait default on an
    aarch64 host, Avx2F32Kernel's on x86_64 with AVX2 and FMA)."""
    lib = yp._lib.load()
    sem = ctypes.c_int(-1)
    assert lib.ypdq_dropin_semantics(ctypes.byref(sem)) == 0
    img = yp.synth.blob_images(1, seed=56)[0]
    h0, t0, q0, b0, p0 = oracle.hash_get_threshold(img)
    dh, dt, dq, dp = oracle.dihedrals(p0, t0, ["exact", "avx2", "scalar"][sem.value])
    out = np.zeros(32, np.uint8)
    pdqf = p0.copy()
    calls = []

    @yp._lib.DihedralCallback
    def cb(ctxp, dihedral, threshold, quality):
        calls.append((dihedral, threshold, quality, out.copy(), pdqf.copy()))
        return True

    ok = lib.yume_pdq_visit_dihedrals_smart_kernel(None, t0, out.ctypes.data_as(ctypes.c_void_p),
                                                   pdqf.ctypes.data_as(ctypes.c_void_p), cb)
    assert ok and len(calls) == 7
    for v, (d, thr, q, o, p) in enumerate(calls):
        assert d == yp.SLOT_DIHEDRALS[v + 1]
        assert thr == np.float32(t0)  # the reference passes the outer threshold
        assert q == dq[v]
        assert np.array_equal(o, dh[v]) and same_bits(p, dp[v])
    # stop after the third callback
    pdqf[:] = p0
    calls.clear()

    @yp._lib.DihedralCallback
    def cb_stop(ctxp, dihedral, threshold, quality):
        calls.append(dihedral)
        return len(calls) < 3

    ok = lib.yume_pdq_visit_dihedrals_smart_kernel(None, t0, out.ctypes.data_as(ctypes.c_void_p),
                                                   pdqf.ctypes.data_as(ctypes.c_void_p), cb_stop)
    assert not ok and len(calls) == 3 and same_bits(pdqf, dp[2])


def test_invalid_arguments(ctx, yp):
    lib = ctx.lib
    d = ctx.alloc(1 << 20)
    bad = ctypes.c_void_p(d.address + 4)
    assert lib.ypdq_hash_batch(ctx.handle, bad, 1, 0, 0, 0, None, None, None, None, 1, None, None) == yp._lib.ERR_ALIGN
    assert lib.ypdq_hash_batch(ctx.handle, d.ptr, 1, 5, 0, 0, None, None, None, None, 1, None, None) == yp._lib.ERR_INVALID
    assert lib.ypdq_hash_batch(ctx.handle, d.ptr, 1, 0, 0, 9, None, None, None, None, 1, None, None) == yp._lib.ERR_INVALID
    assert lib.ypdq_hash_batch(ctx.handle, d.ptr, -1, 0, 0, 0, None, None, None, None, 1, None, None) == yp._lib.ERR_INVALID
    assert lib.ypdq_hash_batch(ctx.handle, d.ptr, 0, 0, 0, 0, None, None, None, None, 1, None, None) == 0
    ctx.check_device_errors()


@pytest.mark.parametrize("channels", [3, 4])
def test_rgb_input_bit_exact(ctx, yp, oracle, channels):
    """RGB8 / RGBA8 input: the kernel's fused BT.601 luma equals the reference's conversion
    followed by its f32 pipeline, bit for bit (hashes, thresholds, qualities, PDQF, buffer)."""
    imgs = yp.synth.color_images(10, seed=70 + channels, channels=channels)
    got = yp.hash_batch(ctx, imgs, want_pdqf=True, want_buf1=True)
    luma = oracle.luma(imgs)
    h, q, t, p = oracle.hash_batch(luma, want_pdqf=True)
    assert np.array_equal(got["hashes"], h)
    assert np.array_equal(got["quality"], q)
    assert np.array_equal(got["thresholds"], t)
    assert np.array_equal(got["pdqf"][:, 0].view(np.uint32), p.view(np.uint32))
    for n in (0, 9):
        assert np.array_equal(got["buf1"][n].view(np.uint32), oracle.compress(luma[n]).view(np.uint32))


@pytest.mark.parametrize("prec", [1, 2, 0x100, 0x102])
def test_rgb_input_variants_match_luma_input(ctx, yp, oracle, prec):
    """Every DCT / compress variant gives the same bits for RGB input as for the f32 luma
    image (the conversion is the only RGB-specific step); RGBA equals RGB."""
    rgba = yp.synth.color_images(6, seed=90, channels=4)
    rgb = np.ascontiguousarray(rgba[..., :3])
    luma = oracle.luma(rgb)
    a = yp.hash_batch(ctx, rgb, dct=prec, want_pdqf=True)
    b = yp.hash_batch(ctx, rgba, dct=prec, want_pdqf=True)
    c = yp.hash_batch(ctx, luma, dct=prec, want_pdqf=True)
    for k in ("hashes", "quality", "thresholds", "pdqf"):
        assert np.array_equal(a[k], c[k]), k
        assert np.array_equal(b[k], c[k]), k


JAROSZ = 0x200  # YPDQ_COMPRESS_JAROSZ


@pytest.mark.parametrize("u8,reps", [(False, 40), (True, 160)])
def test_reference_kernel_bit_exact(ctx, yp, oracle, u8, reps):
    """YPDQ_COMPRESS_JAROSZ = ReferenceKernel<f32>: full Jarosz filter, sequential DCT, the
    trait-default (scalar) dihedrals; bit-exact with the oracle. The u8 case (2,080 images)
    crosses the 2,048-image chunk boundary of the filter's scratch."""
    base, kind = yp.synth.mixed_images(13, seed=801)
    if u8:
        base = yp.synth.to_u8(base)
    imgs = np.concatenate([base] * reps)
    got = yp.hash_batch(ctx, imgs, dct=JAROSZ, semantics="scalar", want_pdqf=True, want_buf1=True)
    h, q, t, p, b = oracle.hash_batch_reference(base, semantics="scalar")
    for k in (0, reps // 2 + 1, reps - 1):  # repeats of the 13 distinct images
        sl = slice(13 * k, 13 * k + 13)
        assert np.array_equal(got["hashes"][sl], h)
        assert np.array_equal(got["quality"][sl], q)
        assert np.array_equal(got["thresholds"][sl], t)
        assert np.array_equal(got["pdqf"][sl, 0].view(np.uint32), p.view(np.uint32))
        assert np.array_equal(got["buf1"][sl].view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("channels", [3, 4])
def test_reference_kernel_color(ctx, yp, oracle, channels):
    """RGB8 / RGBA8 through the Jarosz path: BT.601 luma on load, then the f32 filter."""
    rgb = yp.synth.color_images(3, seed=802, channels=channels)
    got = yp.hash_batch(ctx, rgb, dct=JAROSZ, semantics="scalar", want_pdqf=True)
    h, q, t, p, b = oracle.hash_batch_reference(oracle.luma(rgb), semantics="scalar")
    assert np.array_equal(got["hashes"], h) and np.array_equal(got["quality"], q)
    assert np.array_equal(got["pdqf"][:, 0].view(np.uint32), p.view(np.uint32))


def test_disagreement_vs_avx2_kernel(ctx, yp, oracle):
    """Hash-bit disagreement of the bit-exact FP32 kernel (with the AVX2 sign patterns) with
    the restated Avx2F32Kernel, yume-pdq's smart_kernel on AVX2 hosts, over 512 mixed images
    (constant images excluded: their coefficients are rounding noise in every kernel).
    Measured: primary hashes 0 %, all 8 slots ~0.03 % (the transposed slots, through the
    quantizer's threshold value)."""
    imgs, kind = yp.synth.mixed_images(512, seed=2036)
    live = kind != 2
    got = yp.hash_batch(ctx, imgs, semantics="avx2")
    ha, qa, ta, pa = oracle.hash_batch_avx2(imgs)
    d0 = float(np.unpackbits(got["hashes"][live, 0] ^ ha[live, 0]).mean())
    dall = float(np.unpackbits(got["hashes"][live] ^ ha[live]).mean())
    print("disagreement vs Avx2F32Kernel: primary %.5f %%, all slots %.5f %%"
          % (100 * d0, 100 * dall))
    assert d0 <= 0.001 and dall <= 0.005
    # qualities are gradients of slightly different PDQFs (FMA rounding): equal to ~1e-7
    assert np.abs(got["quality"][live, 0] - qa[live, 0]).max() <= 1e-5

