"""GPU parity of the per-stage Kernel entry points (ypdq_dct2d_batch,
ypdq_sum_of_gradients_batch, ypdq_pdqf_transform_batch, ypdq_cvt_luma8f) and of the
CudaKernel trait methods over them, against the oracle; and the drop-in interface used from
a C program built with gcc."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def same_bits(a, b):
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def compressed_buffers(yp, oracle, n, seed):
    """Compressed images of blob, noise and constant images, plus a raw noise buffer with
    values far outside 0..255 and an all-zero one."""
    imgs, _ = yp.synth.mixed_images(n, seed=seed)
    bufs = [oracle.compress(im) for im in imgs]
    rng = np.random.default_rng(seed)
    bufs.append(rng.normal(0, 1e4, (127, 127)).astype(np.float32))
    bufs.append(np.zeros((127, 127), np.float32))
    return np.stack(bufs)


@pytest.mark.parametrize("width", [127, 128])
def test_dct2d_batch_bit_exact(ctx, yp, oracle, width):
    """Kernel::dct2d of buffers with row stride 127 and with the reference's padded 128."""
    bufs = compressed_buffers(yp, oracle, 30, seed=width)
    padded = np.full((bufs.shape[0], 127, width), 9.0, np.float32)  # padding must be ignored
    padded[:, :, :127] = bufs
    got = yp.core.dct2d_batch(ctx, padded)
    for i in range(bufs.shape[0]):
        assert same_bits(got[i], oracle.dct2d(bufs[i])), i


def test_sum_of_gradients_batch_bit_exact(ctx, yp, oracle):
    rng = np.random.default_rng(3)
    p = np.concatenate([rng.normal(0, 50, (200, 16, 16)),
                        rng.normal(0, 1e-3, (20, 16, 16)),
                        np.zeros((1, 16, 16))]).astype(np.float32)
    got = yp.core.sum_of_gradients_batch(ctx, p)
    want = np.array([oracle.sum_of_gradients(x) for x in p], np.float32)
    assert same_bits(got, want)


@pytest.mark.parametrize("semantics", ["exact", "avx2", "scalar"])
def test_pdqf_transforms_each_kernel(ctx, yp, oracle, semantics):
    rng = np.random.default_rng(4)
    p = rng.normal(0, 30, (17, 16, 16)).astype(np.float32)
    for op in range(4):
        for negate in (False, True):
            got = yp.core.pdqf_transform_batch(ctx, p, op, negate, semantics)
            for i in range(p.shape[0]):
                assert same_bits(got[i], oracle.pdqf_transform(p[i], op, negate, semantics)), \
                    (op, negate, i)


def test_pdqf_transforms_compose_to_the_dihedrals(ctx, yp, oracle):
    """visit_dihedrals' FLOPPED variant (src/lib.rs:391-396) is negate_alt_cols::<false> of
    the PDQF; the fused kernel's dihedral slots agree with the per-stage call."""
    imgs = yp.synth.blob_images(3, seed=8)
    for sem in ("exact", "avx2", "scalar"):
        r = yp.hash_batch(ctx, imgs, semantics=sem, want_pdqf=True, pdqf_slots=8)
        flopped = yp.core.pdqf_transform_batch(ctx, r["pdqf"][:, 0], 1, False, sem)
        assert same_bits(flopped, r["pdqf"][:, 1]), sem


@pytest.mark.parametrize("channels", [3, 4])
def test_cvt_luma8f_bit_exact(ctx, yp, oracle, channels):
    rng = np.random.default_rng(channels)
    px = rng.integers(0, 256, (3, 512, channels), dtype=np.uint8)
    px[0, :8, :3] = [[0, 0, 0], [255, 255, 255], [255, 0, 0], [0, 255, 0], [0, 0, 255],
                     [1, 2, 3], [254, 253, 252], [128, 128, 128]]
    got = yp.core.cvt_luma8f(ctx, px)
    assert same_bits(got, oracle.luma(px))
    coeffs = (0.2126, 0.7152, 0.0722)  # another choice of the trait's generic coefficients
    assert same_bits(yp.core.cvt_luma8f(ctx, px, coeffs), oracle.luma_with(px, coeffs))


def test_kernel_methods_compose_the_pipeline(ctx, yp, oracle):
    """hash_get_threshold (src/lib.rs:427-455) rebuilt from the CudaKernel trait methods one
    stage at a time: compress, dct2d, sum_of_gradients, adjust_quality, quantize; each stage
    and the result equal the oracle's pipeline."""
    k = yp.CudaKernel(ctx, semantics="scalar")
    img = yp.synth.blob_images(1, seed=12)[0]
    h0, t0, q0, b0, p0 = oracle.hash_get_threshold(img)
    buf1 = np.zeros((128, 128), np.float32)
    k.jarosz_compress(img, buf1)
    assert same_bits(buf1[:127, :127], b0)
    pdqf = np.zeros((16, 16), np.float32)
    k.dct2d(buf1, np.zeros(128, np.float32), pdqf)
    assert same_bits(pdqf, p0)
    g = k.sum_of_gradients(pdqf)
    assert np.float32(g) == np.float32(oracle.sum_of_gradients(p0))
    assert k.adjust_quality(g) == q0
    out = np.zeros((16, 2), np.uint8)
    thr = k.quantize(pdqf, out)
    assert out.tobytes() == h0.tobytes() and np.float32(thr) == np.float32(t0)
    row = yp.synth.color_images(1, seed=5, channels=4)[0, 7]
    luma = np.zeros(512, np.float32)
    k.cvt_rgba8_to_luma8f(row, luma)
    assert same_bits(luma, oracle.luma(row))
    k.cvt_rgb8_to_luma8f(row[:, :3], luma)
    assert same_bits(luma, oracle.luma(row[:, :3]))
    t = pdqf.copy()
    k.pdqf_t(t)
    k.pdqf_negate_off_diagonals(t)
    assert same_bits(t, oracle.pdqf_transform(oracle.pdqf_transform(p0, 0), 3))
    r = pdqf.copy()
    k.pdqf_negate_alt_rows(r, negate=True)
    k.pdqf_negate_alt_cols(r)
    assert same_bits(r, oracle.pdqf_transform(oracle.pdqf_transform(p0, 2, True), 1))


def test_invalid_stage_arguments(ctx, yp):
    lib = ctx.lib
    d = ctx.alloc(1 << 16)
    bad = ctypes.c_void_p(d.address + 4)
    assert lib.ypdq_dct2d_batch(ctx.handle, d.ptr, 1, 126, d.ptr, None) == yp._lib.ERR_INVALID
    assert lib.ypdq_dct2d_batch(ctx.handle, bad, 1, 128, d.ptr, None) == yp._lib.ERR_ALIGN
    assert lib.ypdq_pdqf_transform_batch(ctx.handle, d.ptr, 1, 4, 0, 0, None) == yp._lib.ERR_INVALID
    assert lib.ypdq_pdqf_transform_batch(ctx.handle, d.ptr, 1, 0, 0, 3, None) == yp._lib.ERR_INVALID
    assert lib.ypdq_cvt_luma8f(ctx.handle, d.ptr, 4, 2, 1.0, 1.0, 1.0, d.ptr, None) == yp._lib.ERR_INVALID
    assert lib.ypdq_sum_of_gradients_batch(ctx.handle, d.ptr, -1, d.ptr, None) == yp._lib.ERR_INVALID
    for call in (lambda: lib.ypdq_dct2d_batch(ctx.handle, None, 0, 128, None, None),
                 lambda: lib.ypdq_sum_of_gradients_batch(ctx.handle, None, 0, None, None),
                 lambda: lib.ypdq_pdqf_transform_batch(ctx.handle, None, 0, 0, 0, 0, None),
                 lambda: lib.ypdq_cvt_luma8f(ctx.handle, None, 0, 3, 1.0, 1.0, 1.0, None, None)):
        assert call() == yp._lib.OK
    ctx.check_device_errors()


def build_consumer(tmp_path):
    lib_dir = os.path.join(ROOT, "yume-pdq_gb300", "_build")
    exe = str(tmp_path / "dropin_consumer")
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "dropin_consumer.c"), "-o", exe, "-L", lib_dir,
                    "-l:libyumepdq_gb300.so", "-Wl,-rpath," + lib_dir], check=True)
    return exe


def parse_fields(line):
    toks = line.split()
    return {toks[i]: toks[i + 1] for i in range(0, len(toks) - 1, 2)}


@pytest.mark.parametrize("stop_after", [0, 3, 7])
def test_c_consumer_against_oracle(yp, oracle, tmp_path, stop_after):
    """A gcc-built C program links the drop-in symbols (functions, the bool callback ABI,
    exported data symbols), hashes two ramp images and visits the dihedrals of the second;
    every printed value equals the oracle's, bit for bit."""
    exe = build_consumer(tmp_path)
    out = subprocess.run([exe, str(stop_after)], capture_output=True, text=True, timeout=300,
                         check=True).stdout.splitlines()
    sem = yp.kernel.host_semantics()
    for k in range(2):
        f = parse_fields(out[k])
        img = (np.arange(512 * 512, dtype=np.int64) + k).astype(np.float32).reshape(512, 512)
        h, t, q, b, p = oracle.hash_get_threshold(img)
        assert f["hash"] == h.tobytes().hex(), k
        assert np.float32(f["quality"]) == np.float32(q)
        assert np.float32(f["threshold"]) == np.float32(t)
        assert np.float32(f["buf1_0"]) == b[0, 0] and np.float32(f["pdqf0"]) == p[0, 0]
    dh, dt, dq, dp = oracle.dihedrals(p, t, sem)
    variants = [parse_fields(x) for x in out if x.startswith("variant")]
    assert len(variants) == (stop_after or 7)
    for v, f in enumerate(variants):
        assert int(f["dihedral"], 16) == yp.SLOT_DIHEDRALS[v + 1]
        assert np.float32(f["threshold"]) == np.float32(t)  # the outer threshold is passed
        assert np.float32(f["quality"]) == dq[v] and np.float32(f["pdqf0"]) == dp[v][0, 0]
        assert f["hash"] == dh[v].tobytes().hex()
    # a callback that returns false stops the visit, which then returns false (src/lib.rs:358-420)
    assert ("visited %d completed %d" % (stop_after or 7, 0 if stop_after else 1)) in out
    assert any(x.startswith("version 1.") for x in out)
    assert ("flipped %08x rotated_90 %08x" % (yp.Dihedrals.FLIPPED, yp.Dihedrals.ROTATED_90)) in out
