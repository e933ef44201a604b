"""CPU tests of the oracle: pinned against yume-pdq's golden vector and its own unit tests."""
import json
import os
import struct

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

F32_EPS = np.finfo(np.float32).eps


def bits_diff(a, b):
    return int(np.unpackbits(np.bitwise_xor(np.asarray(a, np.uint8), np.asarray(b, np.uint8))).sum())


def test_readme_fm_sine_kat(oracle):
    """README known-answer test (README.md:305-451): hash within 2 bits, PDQF to 1 decimal."""
    kat = json.load(open(os.path.join(GOLDEN, "readme_fm_sine.json")))
    img = oracle.fm_sine_image()
    h, thr, q, buf, p = oracle.hash_get_threshold(img)
    expected = np.frombuffer(bytes.fromhex(kat["expected_hash_hex"]), np.uint8)
    assert bits_diff(h, expected) <= kat["max_bits_different"]
    printed = np.array(kat["pdqf_printed_1dp"], np.float64)
    # "{:5.1}" rounding: each printed value is within 0.05 (+ float slack) of the real one
    assert np.all(np.abs(p.astype(np.float64) - printed) <= 0.0500001)
    assert q == 1.0


def test_avx2_kernel_readme_kat(oracle):
    """The Avx2F32Kernel restatement (FMA compress and DCT, residual-mean quantizer) against
    the README known-answer vector (README.md:305-451)."""
    kat = json.load(open(os.path.join(GOLDEN, "readme_fm_sine.json")))
    img = oracle.fm_sine_image()
    h, q, t, p = oracle.hash_batch_avx2(img[None])
    expected = np.frombuffer(bytes.fromhex(kat["expected_hash_hex"]), np.uint8)
    assert bits_diff(h[0, 0], expected) <= kat["max_bits_different"]
    printed = np.array(kat["pdqf_printed_1dp"], np.float64)
    assert np.all(np.abs(p[0].astype(np.float64) - printed) <= 0.0500001)
    assert q[0, 0] == 1.0


def test_avx2_dct_equivalence(oracle):
    """test_dct64_impl_avx2_equivalence (src/kernel/mod.rs:1249-1345) restated on the two
    DCT restatements: a matrix of ones and a ramp buffer (relative difference < 4e-7), then
    a constant buffer and a ramp matrix (< 8e-7)."""
    i, j = np.meshgrid(np.arange(127), np.arange(127), indexing="ij")
    cases = [
        (np.ones(16 * 127, np.float32),
         (i * 127 + j).astype(np.float32) * np.float32(0.00001), 4e-7),
        (np.arange(16 * 127).astype(np.float32),
         np.full((127, 127), np.float32(0.00001), np.float32), 8e-7),
    ]
    for D, b127, tol in cases:
        b128 = np.zeros((128, 128), np.float32)
        b128[:127, :127] = b127
        ref = oracle.dct2d_matrix(D, b127)
        got = oracle.dct2d_avx2_matrix(D, b128)
        assert np.all(np.abs(ref - got) / ref < tol)


def test_avx2_kernel_agrees_with_default(oracle, yp):
    """Seeded blob images: the Avx2F32Kernel and DefaultKernel restatements give the same
    primary hashes up to rare FMA-rounding flips; with the same sign patterns the derived
    slots differ only where the residual-mean quantizer's threshold value (which the
    transposed slots reuse) departs from the median."""
    imgs = yp.synth.blob_images(24, seed=77)
    ha, qa, ta, pa = oracle.hash_batch_avx2(imgs)
    hd = oracle.hash_batch(imgs, semantics="avx2")[0]
    assert np.unpackbits(ha[:, 0] ^ hd[:, 0]).mean() <= 0.002
    assert np.unpackbits(ha ^ hd).mean() <= 0.01


def test_constants_pinned(oracle, yp):
    """The oracle's tables equal the ones compiled into the library (both headers come from
    one generator: this checks that library and oracle were built from the same tables)."""
    import ctypes
    lib = yp._lib.load()
    dct = np.empty(16 * 127, np.float32)
    tent = np.empty(49, np.float32)
    yp._lib.check(lib.ypdq_constants(dct.ctypes.data_as(ctypes.c_void_p),
                                     tent.ctypes.data_as(ctypes.c_void_p)))
    assert np.array_equal(dct.view(np.uint32), oracle.dct_matrix_f32().ravel().view(np.uint32))
    assert np.array_equal(tent.view(np.uint32), oracle.tent_weights().ravel().view(np.uint32))


def test_constants_closed_form(oracle):
    """DCT rows: sqrt(2/127) cos(pi (i+1) (2j+1)/254); tent: (w w^T)/81, w = [0,1,2,3,2,1,0],
    except the 128-bit construction's residues (two subnormal taps in row 0; the mathematically
    zero cosines at column 63 of odd rows)."""
    d = oracle.dct_matrix_f32().astype(np.float64)
    i = np.arange(1, 17)[:, None]
    j = np.arange(127)[None, :]
    ref = np.sqrt(2.0 / 127) * np.cos(np.pi / 254 * i * (2 * j + 1))
    zero = (i * (2 * j + 1)) % 254 == 127
    assert np.all(np.abs(d - ref)[~zero] <= 1.5 * F32_EPS * np.abs(ref)[~zero] + 1e-12)
    assert np.all(np.abs(d[zero]) < 1e-37)
    w = np.array([0, 1, 2, 3, 2, 1, 0], np.float64)
    t = oracle.tent_weights().astype(np.float64)
    closed = np.outer(w, w) / 81
    assert np.array_equal(t[1:6, 1:6].astype(np.float32), closed[1:6, 1:6].astype(np.float32))
    resid = t.copy()
    resid[1:6, 1:6] = 0
    assert set(zip(*np.nonzero(resid))) == {(0, 4), (0, 5)}
    assert resid[0, 4] < 1e-38 and resid[0, 5] < 1e-38


def test_dct_against_f64(oracle):
    """src/kernel/mod.rs:1187-1246: DCT within 32 f32::EPSILON of the wide reference."""
    rng = np.random.default_rng(1)
    ii, jj = np.indices((127, 127))
    buf = np.where((ii + 2 * jj) % 20 < 10, rng.uniform(0, 1, (127, 127)),
                   rng.uniform(-1, 0, (127, 127))).astype(np.float32)
    p32 = oracle.dct2d(buf).astype(np.float64)
    p64 = oracle.dct2d_f64(buf)
    assert np.max(np.abs(p32 - p64)) <= 32 * F32_EPS


def test_torben_is_rank_127(oracle):
    rng = np.random.default_rng(2)
    for _ in range(200):
        v = rng.normal(size=256).astype(np.float32)
        if rng.random() < 0.3:
            v[rng.integers(0, 256, 40)] = v[0]  # ties
        assert oracle.torben_median(v) == np.sort(v)[127]


def test_rethreshold_identity(oracle, yp):
    """src/lib.rs:659-687: threshold_2d(pdqf, thr) equals quantize's output."""
    for img in yp.synth.blob_images(3, seed=4):
        h, thr, q, buf, p = oracle.hash_get_threshold(img)
        assert np.array_equal(oracle.threshold_2d(p, thr), h)


def test_bit_layout(oracle):
    """Element k = 16 i + j lands in byte 31 - k/8, bit k % 8 (src/kernel/mod.rs:605-606)."""
    for k in (0, 1, 7, 8, 100, 255):
        p = np.zeros(256, np.float32)
        p[k] = 1.0
        h = oracle.threshold_2d(p, 0.5)
        want = np.zeros(32, np.uint8)
        want[31 - k // 8] = 1 << (k % 8)
        assert np.array_equal(h, want)


def test_dihedral_semantics(oracle, yp):
    """The three sign conventions of yume-pdq, checked on their defining properties."""
    img = yp.synth.blob_images(1, seed=9)[0]
    h0, thr, q, buf, p = oracle.hash_get_threshold(img)
    he, te, qe, pe = oracle.dihedrals(p, thr, "exact")
    hs, ts, qs, ps = oracle.dihedrals(p, thr, "scalar")
    ha, ta, qa, pa = oracle.dihedrals(p, thr, "avx2")
    i, j = np.indices((16, 16))
    # exact: FLOPPED negates even columns, FLIPPED even rows, ROTATED_90_FLOPPED transposes
    assert np.array_equal(pe[0], np.where(j % 2 == 0, -p, p))
    assert np.array_equal(pe[2], np.where(i % 2 == 0, -p, p))
    assert np.array_equal(pe[3], p.T)
    # scalar negates odd rows: its FLIPPED is the negation of the exact FLIPPED, so the
    # bits are complemented except where values tie with the median
    assert np.array_equal(ps[2], -pe[2])
    assert bits_diff(hs[2], he[2]) >= 250
    # avx2 negates only columns 0, 2, 4, 6
    assert np.array_equal(pa[0], np.where((j % 2 == 0) & (j < 8), -p, p))
    # the transposed slot keeps the caller's threshold
    assert te[3] == thr and ts[3] == thr


def test_golden_oracle_vectors(oracle):
    """Regression pin: the oracle reproduces its committed vectors bit for bit."""
    g = np.load(os.path.join(GOLDEN, "oracle_vectors.npz"))
    imgs = g["images_u8"]
    for sem in ("exact", "avx2", "scalar"):
        h, q, t, p = oracle.hash_batch(imgs, semantics=sem, nthreads=2, want_pdqf=True)
        assert np.array_equal(h, g["hashes_" + sem])
        assert np.array_equal(q.view(np.uint32), g["quality_" + sem].view(np.uint32))
        assert np.array_equal(t.view(np.uint32), g["thresholds_" + sem].view(np.uint32))
        assert np.array_equal(p.view(np.uint32), g["pdqf"].view(np.uint32))
    assert np.array_equal(oracle.compress(imgs[0].astype(np.float32)), g["buf1_0"])
    for tt in (0, 16, 31, 48):
        hits = oracle.find_all(g["match_rows"], g["match_needles"], tt, nthreads=3)
        got = np.stack([hits["index"].astype(np.int64), hits["query"].astype(np.int64),
                        hits["distance"].astype(np.int64)], axis=1)
        assert np.array_equal(got.reshape(-1, 3), g["match_hits_t%d" % tt].reshape(-1, 3))


@pytest.mark.parametrize("n_needles", [8, 16, 24])
def test_matcher_planted_controls(oracle, yp, n_needles):
    """Structure of src/matching/mod.rs:460-553 with our own seeded RNG: random needles and
    2048 random rows give no hit at t = 31; a positive control with 31 flipped bits planted
    at every position is found exactly there."""
    rng = np.random.default_rng(0x79756D652D706471)
    needles = rng.integers(0, 256, (n_needles, 32), dtype=np.uint8)
    rows = rng.integers(0, 256, (2048, 32), dtype=np.uint8)
    assert oracle.count_all(rows, needles, 31) == 0
    for pos in range(0, 2048, 97):
        k = int(rng.integers(0, n_needles))
        planted = needles.copy()
        planted[k] = rows[pos]
        for _ in range(31):  # 31 random flips (repeats may cancel: distance <= 31)
            b = int(rng.integers(0, 256))
            planted[k, b // 8] ^= np.uint8(1 << (b % 8))
        hits = oracle.find_all(rows, planted, 31, nthreads=2)
        assert len(hits) == 1 and hits[0]["index"] == pos and hits[0]["query"] == k


def test_find_all_order_and_threads(oracle, yp):
    rows = yp.synth.rows_128(3000, seed=21)
    q = yp.synth.rows_128(9, seed=22)
    yp.synth.plant(rows, q, 200, 0, 50, seed=23)
    a = oracle.find_all(rows, q, 40, nthreads=1)
    b = oracle.find_all(rows, q, 40, nthreads=7)
    assert np.array_equal(a, b)
    key = a["index"].astype(np.int64) * 64 + a["query"]
    assert np.all(np.diff(key) > 0)
    # distances are the exact popcounts
    d = np.unpackbits(rows[a["index"]] ^ q[a["query"]], axis=1).sum(1)
    assert np.array_equal(d, a["distance"])


def test_clustered_rows_twin(oracle):
    """Clustered workload rows: member g of centre g // members sits at Hamming distance
    d ~ Binomial(trials, 1/2) from centre row g // members of the 128-bit generator."""
    members, trials, seed = 1000, 40, 77
    rows = oracle.synth_clustered(20_000, members, trials, seed, first=3_000_000)
    centres = oracle.synth_rows(20, seed, first=3_000)
    d = np.unpackbits(rows ^ np.repeat(centres, members, axis=0), axis=1).sum(1)
    assert d.max() <= trials and abs(d.mean() - trials / 2) < 0.2
    assert abs(d.std() - np.sqrt(trials) / 2) < 0.2
    # rows are a pure function of the global row number
    again = oracle.synth_clustered(100, members, trials, seed, first=3_000_000 + 500)
    assert np.array_equal(again, rows[500:600])


def test_luma_matches_reference_order(oracle):
    """Kernel::cvt_rgb8_to_luma8f (src/kernel/mod.rs:303-340): (0.299 r + 0.587 g) + 0.114 b
    in f32, left to right; the reference's own AVX2 test expects 0.299 * 255 for pure red
    (src/kernel/x86.rs:1510-1540)."""
    rng = np.random.default_rng(9)
    px = rng.integers(0, 256, (4096, 4), dtype=np.uint8)
    got3 = oracle.luma(px[:, :3])
    got4 = oracle.luma(px)
    r, g, b = (px[:, k].astype(np.float32) for k in range(3))
    want = (np.float32(0.299) * r + np.float32(0.587) * g) + np.float32(0.114) * b
    assert np.array_equal(got3.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(got4, got3)  # alpha ignored
    red = oracle.luma(np.array([[255, 0, 0]], np.uint8))[0]
    assert red == np.float32(0.299) * np.float32(255.0)


def test_jarosz_compress_semantics(oracle, yp):
    """ReferenceKernel<f32>::jarosz_compress (src/kernel/ref.rs): two passes of a box filter of
    window ceil(512/254) = 3 along rows then columns, windows shrinking to 2 at the edges,
    sampled at ((2 o + 1) 512) / 254. The oracle's f32 running sums agree with a direct FP64
    evaluation of that definition to f32 rounding."""
    img = yp.synth.blob_images(1, seed=12)[0]

    def box(a, axis):
        a = np.moveaxis(a, axis, -1)
        out = np.empty_like(a)
        for i in range(a.shape[-1]):
            out[..., i] = a[..., max(0, i - 1):i + 2].mean(-1)
        return np.moveaxis(out, -1, axis)

    y = img.astype(np.float64)
    for _ in range(2):
        y = box(box(y, 1), 0)
    idx = ((2 * np.arange(127) + 1) * 512) // 254
    want = y[np.ix_(idx, idx)]
    got = oracle.jarosz_compress(img)
    assert np.abs(got - want).max() / np.abs(want).max() < 1e-5
