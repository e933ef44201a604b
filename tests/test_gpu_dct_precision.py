"""Tensor-core DCT variants (TF32, BF16x3) against the FP64 oracle and the f32 reference.

Stage 1 of the DCT (16 x 127 x 127, 89 % of its MACs) runs on tcgen05 tensor cores with f32
accumulation; the compress and stage 2 stay f32. Per image the relative coefficient error
is max |P - P64| / max |P64|, where P64 is the FP64 DCT of the same (bit-exact) compressed
image. Tolerances written here:
  BF16x3 (split operands, hi*hi + hi*lo + lo*hi): relative error <= 1e-4
  TF32   (10-bit operands, round to nearest):     relative error <= 5e-3
Hash bits may flip only for coefficients near the median. Constant images are excluded
from the disagreement rate: their PDQF is rounding noise (about 1e-13 of the pixel value),
so their bits carry no information in any kernel.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {1: 5e-3, 2: 1e-4}
MAX_BIT_RATE = {0: 0.002, 1: 0.02, 2: 0.002}


def rel_errors(oracle, buf1, pdqf):
    errs = []
    for b, p in zip(buf1, pdqf):
        p64 = oracle.dct2d_f64(b)
        scale = np.max(np.abs(p64))
        errs.append(np.max(np.abs(p.astype(np.float64) - p64)) / scale if scale > 0 else 0.0)
    return np.array(errs)


@pytest.mark.parametrize("dct", [1, 2])
@pytest.mark.parametrize("u8", [False, True])
def test_tensor_core_dct_precision(ctx, yp, oracle, dct, u8):
    imgs, kind = yp.synth.mixed_images(96, seed=300 + dct)
    if u8:
        imgs = yp.synth.to_u8(imgs)
    ref = yp.hash_batch(ctx, imgs, dct=0, want_pdqf=True)
    got = yp.hash_batch(ctx, imgs, dct=dct, want_pdqf=True, want_buf1=True)
    # the compress stays f32 and bit-exact in every variant
    for n in range(0, len(imgs), 7):
        assert np.array_equal(got["buf1"][n].view(np.uint32),
                              oracle.compress(imgs[n].astype(np.float32)).view(np.uint32))
    live = kind != 2
    err = rel_errors(oracle, got["buf1"][live], got["pdqf"][live, 0])
    assert err.max() <= TOL[dct], err.max()
    # bit disagreement with the f32 reference kernel (slot 0 and all derived slots)
    diff = np.unpackbits(got["hashes"][live] ^ ref["hashes"][live]).sum()
    rate = diff / (live.sum() * 8 * 256)
    assert rate <= MAX_BIT_RATE[dct], rate
    # quality agrees
    assert np.max(np.abs(got["quality"][live] - ref["quality"][live])) <= 1e-3
    # the derived slots are consistent with the slot-0 PDQF of this variant
    h = np.unpackbits(got["hashes"][live][:, 0], axis=1).sum(1)
    assert np.all(np.abs(h - 128) <= 8)


@pytest.mark.parametrize("dct", [1, 2])
def test_tensor_core_dct_batch_sizes(ctx, yp, dct):
    """Several images per CTA: operand buffers and accumulators cycle through many phases."""
    imgs = yp.synth.blob_images(700, seed=77)
    ref = yp.hash_batch(ctx, imgs, dct=0)
    got = yp.hash_batch(ctx, imgs, dct=dct)
    rate = np.unpackbits(got["hashes"] ^ ref["hashes"]).mean()
    assert rate <= MAX_BIT_RATE[dct], rate
    got2 = yp.hash_batch(ctx, imgs, dct=dct)
    assert np.array_equal(got["hashes"], got2["hashes"])  # deterministic


def test_screen_host_with_tensor_core_dct(ctx, yp, oracle):
    imgs = yp.synth.blob_images(8, seed=61)
    got = yp.hash_batch(ctx, imgs, dct=2)
    queries = got["hashes"].reshape(-1, 32)
    rows = yp.synth.rows_128(20000, seed=62)
    yp.synth.plant(rows, queries, 100, 0, 31, seed=63)
    db = yp.Database(ctx, rows)
    hits = yp.screen_host(ctx, db, imgs, threshold=31, dct=2)
    want = oracle.find_all(rows, queries, 31)
    assert np.array_equal(hits[["index", "query", "distance"]], want[["index", "query", "distance"]])


SEPARABLE = 0x100  # YPDQ_COMPRESS_SEPARABLE
# FP32: the f32 DCT's own rounding (the bit-exact kernel measures ~2e-6 against FP64 too)
TOL_SEP = {0: 1e-5, 1: 5e-3, 2: 1e-4}


def separable_compress_f64(img):
    """(c^T X c) / 81 with c = (0,1,2,3,2,1,0), windows at 4i+1 .. 4i+7, in float64."""
    c = np.array([0, 1, 2, 3, 2, 1, 0], np.float64)
    idx = 4 * np.arange(127)[:, None] + 1 + np.arange(7)[None, :]
    x = img.astype(np.float64)
    rows = np.einsum("d,idc->ic", c, x[idx])  # 127 x 512
    return (rows[:, idx] @ c) / 81.0


@pytest.mark.parametrize("dct", [0, 1, 2])
@pytest.mark.parametrize("u8", [False, True])
def test_separable_compress_variants(ctx, yp, oracle, dct, u8):
    """YPDQ_COMPRESS_SEPARABLE: the compress is (c^T X c)/81, exact up to the final f32
    scale for u8; with the reference's compressed image as the FP64 baseline the PDQF stays
    within the variant's coefficient tolerance and the bits within its disagreement bound."""
    imgs, kind = yp.synth.mixed_images(64, seed=400 + dct)
    if u8:
        imgs = yp.synth.to_u8(imgs)
    got = yp.hash_batch(ctx, imgs, dct=dct | SEPARABLE, want_pdqf=True, want_buf1=True)
    ref = yp.hash_batch(ctx, imgs, dct=0)
    live = kind != 2
    for n in range(0, len(imgs), 5):
        want = separable_compress_f64(imgs[n])
        scale = max(np.abs(want).max(), 1.0)
        assert np.abs(got["buf1"][n].astype(np.float64) - want).max() / scale <= (2e-7 if u8 else 1e-6)
        exact = oracle.compress(imgs[n].astype(np.float32))
        assert np.abs(got["buf1"][n] - exact).max() / scale <= 2e-6
    errs = []
    for img, p in zip(imgs[live], got["pdqf"][live, 0]):
        p64 = oracle.dct2d_f64(oracle.compress(img.astype(np.float32)))
        errs.append(np.max(np.abs(p.astype(np.float64) - p64)) / np.max(np.abs(p64)))
    assert max(errs) <= TOL_SEP[dct], max(errs)
    rate = np.unpackbits(got["hashes"][live] ^ ref["hashes"][live]).mean()
    assert rate <= MAX_BIT_RATE.get(dct, 0.002), rate
