"""GPU parity of the exact Hamming scan against the oracle's scalar matcher.

Hit sets must be identical (index, query, distance), in the scalar matcher's order once
sorted. Every call goes through the C ABI.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# YPDQ_SCAN_SIMT, YPDQ_SCAN_B1MMA, YPDQ_SCAN_TC, YPDQ_SCAN_TC_FP4, YPDQ_SCAN_TC_FP8
ALGOS = [1, 2, 3, 4, 5]


def as_tuples(h):
    return np.stack([h["index"].astype(np.int64), h["query"].astype(np.int64),
                     h["distance"].astype(np.int64)], axis=1) if len(h) else np.zeros((0, 3), np.int64)


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("n_rows,n_q", [(0, 8), (1, 1), (15, 3), (17, 8), (4099, 13), (20000, 64), (5000, 2049)])
def test_scan_matches_oracle(ctx, yp, oracle, algo, n_rows, n_q):
    rows = yp.synth.rows_128(n_rows, seed=n_rows + 1)
    q = yp.synth.rows_128(n_q, seed=n_q + 1000)
    if n_rows:
        yp.synth.plant(rows, q, min(n_rows, 60), 0, 96, seed=7)
    # both sides of the SIMT scan's prefix-bound switches (t = 34 / 35 and 62 / 63) and of
    # the tensor-core scan's 128-bit bound (t = 36 / 37)
    for t in (0, 16, 31, 34, 35, 36, 37, 48, 62, 63, 90):
        got = yp.scan(ctx, rows, q, t, algo=algo)
        want = oracle.find_all(rows, q, t)
        assert np.array_equal(as_tuples(got), as_tuples(want)), (t, len(got), len(want))


@pytest.mark.parametrize("algo", ALGOS)
def test_scan_thresholds_extremes(ctx, yp, oracle, algo):
    rows = np.random.default_rng(1).integers(0, 256, (300, 32), dtype=np.uint8)
    q = np.random.default_rng(2).integers(0, 256, (9, 32), dtype=np.uint8)
    rows[5] = q[3]
    for t in (0, 1, 100, 128, 255, 256):
        got = yp.scan(ctx, rows, q, t, algo=algo, capacity=4096)
        want = oracle.find_all(rows, q, t)
        assert np.array_equal(as_tuples(got), as_tuples(want))
    assert len(yp.scan(ctx, rows, q, 256, algo=algo)) == 300 * 9


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("n_q", [40, 100, 150, 300])
def test_dense_hits_per_row(ctx, yp, oracle, algo, n_q):
    """Rows that hit every query of a pass: queries are variants of one hash within 6 bits,
    planted rows within 10 bits of it, so each planted row hits all n_q queries at t >= 16
    (several hits per lane and column chunk in the tensor-core epilogue; 150 queries run
    one 192-query pass, 300 a 256-query pass plus a 44-query tail pass)."""
    rng = np.random.default_rng(n_q)
    base = yp.synth.rows_128(1, seed=77)[0]
    q = np.stack([yp.synth.flip_bits(base, int(rng.integers(0, 7)), rng) for _ in range(n_q)])
    rows = yp.synth.rows_128(3000, seed=78)
    pos = rng.choice(3000, size=45, replace=False)
    for p in pos:
        rows[p] = yp.synth.flip_bits(base, int(rng.integers(0, 11)), rng)
    for t in (16, 31, 48, 64, 90):
        got = yp.scan(ctx, rows, q, t, algo=algo, capacity=1 << 16)
        want = oracle.find_all(rows, q, t)
        assert len(want) >= 45 * n_q
        assert np.array_equal(as_tuples(got), as_tuples(want)), (t, len(got), len(want))
    # a hit buffer smaller than the hit count: the total is still exact, the stored hits a subset
    d_rows, d_q = ctx.to_device(rows), ctx.to_device(q)
    d_hits, d_cnt = ctx.alloc(1000 * 16), ctx.alloc(8)
    yp.core.scan_device(ctx, d_rows, 3000, d_q, n_q, 31, d_hits, 1000, d_cnt, algo)
    ctx.sync()
    want = {tuple(x) for x in as_tuples(oracle.find_all(rows, q, 31))}
    assert int(d_cnt.download((1,), np.uint64)[0]) == len(want)
    stored = {tuple(x) for x in as_tuples(d_hits.download((1000,), yp.HIT_DTYPE))}
    assert len(stored) == 1000 and stored <= want


@pytest.mark.parametrize("algo", ALGOS)
def test_planted_controls(ctx, yp, algo):
    """src/matching/mod.rs:460-553 structure on the GPU: no false hits, every control found."""
    rng = np.random.default_rng(0x79756D652D706471)
    needles = rng.integers(0, 256, (8, 32), dtype=np.uint8)
    rows = rng.integers(0, 256, (2048, 32), dtype=np.uint8)
    assert len(yp.scan(ctx, rows, needles, 31, algo=algo)) == 0
    for pos in range(0, 2048, 61):
        k = int(rng.integers(0, 8))
        planted = needles.copy()
        planted[k] = rows[pos]
        for _ in range(31):
            b = int(rng.integers(0, 256))
            planted[k, b // 8] ^= np.uint8(1 << (b % 8))
        hits = yp.scan(ctx, rows, planted, 31, algo=algo)
        assert len(hits) == 1 and hits[0]["index"] == pos and hits[0]["query"] == k


@pytest.mark.parametrize("algo", ALGOS)
def test_overflow_reports_total(ctx, yp, oracle, algo):
    rows = yp.synth.rows_128(5000, seed=3)
    q = yp.synth.rows_128(4, seed=4)
    yp.synth.plant(rows, q, 400, 0, 10, seed=5)
    d_rows, d_q = ctx.to_device(rows), ctx.to_device(q)
    d_hits, d_cnt = ctx.alloc(100 * 16), ctx.alloc(8)
    yp.core.scan_device(ctx, d_rows, 5000, d_q, 4, 31, d_hits, 100, d_cnt, algo)
    ctx.sync()
    total = int(d_cnt.download((1,), np.uint64)[0])
    assert total == len(oracle.find_all(rows, q, 31))
    stored = d_hits.download((100,), yp.HIT_DTYPE)
    full = {tuple(x) for x in as_tuples(oracle.find_all(rows, q, 31))}
    assert {tuple(x) for x in as_tuples(stored)} <= full


def test_sort_hits(ctx, yp):
    rng = np.random.default_rng(9)
    for n in (2, 3, 100, 1025, 70000):
        h = np.zeros(n, yp.HIT_DTYPE)
        h["index"] = rng.integers(0, 1 << 40, n)
        h["query"] = rng.integers(0, 5000, n)
        h["index"][: n // 3] = h["index"][0]  # ties on index
        d = ctx.to_device(h)
        yp.core.sort_hits_device(ctx, d, n)
        got = d.download((n,), yp.HIT_DTYPE)
        order = np.lexsort((h["query"], h["index"]))
        assert np.array_equal(got[["index", "query"]], h[order][["index", "query"]])


@pytest.mark.parametrize("algo", ALGOS)
def test_matcher_surface(ctx, yp, oracle, algo):
    rows = yp.synth.rows_128(3000, seed=31)
    q = yp.synth.rows_128(8, seed=32)
    yp.synth.plant(rows, q, 30, 0, 31, seed=33)
    db = yp.CudaVectorDatabase(ctx, rows)
    m = yp.CudaMatcher(ctx, db, 31, algo=algo)
    assert m.scan(q)
    assert not m.scan(yp.synth.rows_128(8, seed=99))
    want = oracle.find_all(rows, q, 31)
    first = m.find(q, lambda i, j: (i, j))
    assert first == (int(want[0]["index"]), int(want[0]["query"]))
    seen = []
    assert m.find(q, lambda i, j: seen.append((i, j))) is None
    assert seen == [(int(w["index"]), int(w["query"])) for w in want]


def test_full_size_10m_scan(ctx, yp, oracle):
    """10M-row database (320 MB) with 10,000 planted rows at distances 0..31: both kernels
    return the oracle's exact hit list for a batch of 8 and of 64 queries."""
    n = 10_000_000
    d_rows = ctx.alloc(n * 32)
    ctx.lib.ypdq_synth_rows(ctx.handle, d_rows.ptr, n, 0, 1234, None)
    ctx.sync()
    rows = d_rows.download((n, 32), np.uint8)
    assert np.all(yp.synth.popcount_rows(rows[:100000]) == 128)
    q = yp.synth.rows_128(64, seed=77)
    pos, qid, dist = yp.synth.plant(rows, q, 10_000, 0, 31, seed=78)
    d_rows.upload(rows)
    d_q = ctx.to_device(q)
    d_cnt = ctx.alloc(8)
    for nq in (8, 64):
        want = oracle.find_all(rows, q[:nq], 31)
        assert len(want) >= int(np.sum(qid < nq))
        for algo in ALGOS:
            d_hits = ctx.alloc(len(want) * 16 + 16)
            yp.core.scan_device(ctx, d_rows, n, d_q, nq, 31, d_hits, len(want) + 1, d_cnt, algo)
            ctx.sync()
            total = int(d_cnt.download((1,), np.uint64)[0])
            assert total == len(want)
            yp.core.sort_hits_device(ctx, d_hits, total)
            got = d_hits.download((total,), yp.HIT_DTYPE)
            assert np.array_equal(as_tuples(got), as_tuples(want))


def test_screen_host_end_to_end(ctx, yp, oracle):
    """ypdq_screen_host: host images in, sorted (index, query, distance) hits out."""
    imgs = yp.synth.blob_images(6, seed=41)
    h, q, t, _ = oracle.hash_batch(imgs)
    queries = h.reshape(-1, 32)
    rows = yp.synth.rows_128(50000, seed=42)
    yp.synth.plant(rows, queries, 500, 0, 40, seed=43)
    db = yp.Database(ctx, rows)
    hits, hashes = yp.screen_host(ctx, db, imgs, threshold=31, want_hashes=True)
    assert np.array_equal(hashes, h)
    want = oracle.find_all(rows, queries, 31)
    assert np.array_equal(as_tuples(hits), as_tuples(want))
    # capacity smaller than the hit count: the call grows and retries
    hits2 = yp.screen_host(ctx, db, imgs, threshold=31, capacity=3)
    assert np.array_equal(as_tuples(hits2), as_tuples(want))


def test_screen_64_images_against_100k_rows(ctx, yp, oracle):
    """The reference's small workload end to end: 64 seeded blob images hashed with their 8
    dihedrals and matched at t = 31 against 100,000 rows of exactly 128 set bits plus 1,000
    rows planted at distances U{0..40} from randomly chosen dihedral hashes of the images.
    Hashes equal the oracle's f32 pipeline; hits equal its scalar matcher's over them."""
    imgs = yp.synth.blob_images(64, seed=2025)
    h, q, t, _ = oracle.hash_batch(imgs)
    queries = h.reshape(-1, 32)
    rng = np.random.default_rng(2027)
    qid = rng.integers(0, queries.shape[0], 1000)
    dist = rng.integers(0, 41, 1000)
    planted = np.stack([yp.synth.flip_bits(queries[q_], int(d_), rng)
                        for q_, d_ in zip(qid, dist)])
    rows = np.concatenate([yp.synth.rows_128(100_000, seed=2026), planted])
    pos = np.arange(100_000, 101_000)
    db = yp.Database(ctx, rows)
    hits, hashes = yp.screen_host(ctx, db, imgs, threshold=31, want_hashes=True)
    db.close()
    assert np.array_equal(hashes, h)
    want = oracle.find_all(rows, queries, 31)
    assert np.array_equal(as_tuples(hits), as_tuples(want))
    # every planted row within the threshold is found at (at most) its planted distance
    found = {(int(i), int(qq)): int(d) for i, qq, d in as_tuples(hits)}
    for p_, q_, d_ in zip(pos, qid, dist):
        if d_ <= 31:
            assert found[(int(p_), int(q_))] <= d_


def test_screen_host_reference_kernel(ctx, yp, oracle):
    """ypdq_screen_host with YPDQ_COMPRESS_JAROSZ: the hashes are ypdq_hash_batch's
    ReferenceKernel hashes (pinned to the oracle in test_gpu_hash.py) and the hits are the
    scalar matcher's over them; 70 images span two screening chunks."""
    imgs = yp.synth.blob_images(70, seed=51)
    want_h = yp.hash_batch(ctx, imgs, dct=0x200)["hashes"]
    queries = want_h.reshape(-1, 32)
    rows = yp.synth.rows_128(40000, seed=52)
    yp.synth.plant(rows, queries, 400, 0, 40, seed=53)
    db = yp.Database(ctx, rows)
    hits, hashes = yp.screen_host(ctx, db, imgs, threshold=31, dct=0x200, want_hashes=True)
    assert np.array_equal(hashes, want_h)
    want = oracle.find_all(rows, queries, 31)
    assert len(want) > 0
    assert np.array_equal(as_tuples(hits), as_tuples(want))
    db.close()


@pytest.mark.parametrize("algo", [1, 3])
def test_row_sharded_scan(ctx, yp, oracle, algo):
    """A database row-sharded in 3 device slices (shard_rows), each scanned with the whole
    query batch, merged with its row offset (merge_shard_hits): the hits of one scan of the
    whole database. The shards run one after another on this GPU."""
    rows = yp.synth.rows_128(50021, seed=71)
    q = yp.synth.rows_128(96, seed=72)
    yp.synth.plant(rows, q, 600, 0, 40, seed=73)
    parts = []
    for rank in range(3):
        lo, hi = yp.shard_rows(rows.shape[0], 3, rank)
        parts.append((yp.scan(ctx, rows[lo:hi], q, 31, algo=algo), lo))
    merged = yp.merge_shard_hits(parts)
    want = oracle.find_all(rows, q, 31)
    assert len(want) > 0 and np.array_equal(as_tuples(merged), as_tuples(want))


def test_synth_rows_match_cpu_twin(ctx, yp, oracle):
    n = 20000
    d = ctx.alloc(n * 32)
    yp._lib.check(ctx.lib.ypdq_synth_rows(ctx.handle, d.ptr, n, 5, 42, None))
    ctx.sync()
    assert np.array_equal(d.download((n, 32), np.uint8), oracle.synth_rows(n, 42, first=5))


def test_screen_host_chunked(ctx, yp, oracle):
    """ypdq_screen_host with >= 256 images runs in chunks whose copies overlap compute; the
    hit list must still equal the oracle's, with query numbers image * 8 + slot."""
    imgs = yp.synth.blob_images(300, seed=44)
    h, q, t, _ = oracle.hash_batch(imgs)
    queries = h.reshape(-1, 32)
    rows = yp.synth.rows_128(60000, seed=45)
    yp.synth.plant(rows, queries, 2000, 0, 40, seed=46)
    db = yp.Database(ctx, rows)
    hits, hashes = yp.screen_host(ctx, db, imgs, threshold=31, want_hashes=True)
    assert np.array_equal(hashes, h)
    want = oracle.find_all(rows, queries, 31)
    assert np.array_equal(as_tuples(hits), as_tuples(want))
    u8 = yp.synth.to_u8(imgs)
    hu, _, _, _ = oracle.hash_batch(u8)
    hits_u8 = yp.screen_host(ctx, db, u8, threshold=31)
    assert np.array_equal(as_tuples(hits_u8), as_tuples(oracle.find_all(rows, hu.reshape(-1, 32), 31)))


def test_screen_host_growing_chunks(ctx, yp, oracle):
    """Against 4M rows a u8 image takes longer to hash and scan than to copy, so the chunks
    of ypdq_screen_host grow geometrically from 32 images (32, 64, 160, 344; the other
    screen tests run slowly growing chunks); the hit list must equal the oracle's."""
    imgs = yp.synth.to_u8(yp.synth.blob_images(600, seed=47))
    h, _, _, _ = oracle.hash_batch(imgs)
    queries = h.reshape(-1, 32)
    rows = oracle.synth_rows(4_000_000, 48)
    yp.synth.plant(rows, queries, 3000, 0, 40, seed=49)
    db = yp.Database(ctx, rows)
    hits = yp.screen_host(ctx, db, imgs, threshold=31)
    assert np.array_equal(as_tuples(hits), as_tuples(oracle.find_all(rows, queries, 31)))


def test_db_file_round_trip_and_scan(ctx, yp, oracle, tmp_path):
    """ypdq_db_load_file / ypdq_db_save_file: a flat row file, padded the reference's way to
    whole 2,048-row batches by repeating the last row, loads in chunks (a chunk size that
    does not divide the file) and scans exactly like the same rows from memory."""
    rows = yp.synth.rows_128(70_001, seed=31)
    q = yp.synth.rows_128(24, seed=32)
    yp.synth.plant(rows, q, 500, 0, 31, seed=33)
    pad = (-len(rows)) % 2048
    padded = np.concatenate([rows, np.repeat(rows[-1:], pad, axis=0)])
    path = tmp_path / "db.bin"
    padded.tofile(path)
    db = yp.Database.from_file(ctx, path, chunk_bytes=32 * 5000)
    assert db.n_rows == len(padded)
    d_rows, n = db.device_rows()
    d_q, d_hits, d_cnt = ctx.to_device(q), ctx.alloc(16 << 16), ctx.alloc(8)
    yp.core.scan_device(ctx, d_rows, n, d_q, len(q), 31, d_hits, 1 << 16, d_cnt)
    ctx.sync()
    total = int(d_cnt.download((1,), np.uint64)[0])
    yp.core.sort_hits_device(ctx, d_hits, total)
    ctx.sync()
    hits = d_hits.download((total,), yp.HIT_DTYPE)
    want = oracle.find_all(padded, q, 31)
    assert np.array_equal(hits[["index", "query", "distance"]], want[["index", "query", "distance"]])
    out = tmp_path / "db2.bin"
    db.save(out, chunk_bytes=32 * 7777)
    assert np.array_equal(np.fromfile(out, np.uint8).reshape(-1, 32), padded)
    db.close()
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"x" * 33)
    with pytest.raises(yp.YpdqError):
        yp.Database.from_file(ctx, bad)
    with pytest.raises(yp.YpdqError):
        yp.Database.from_file(ctx, tmp_path / "missing.bin")


@pytest.mark.parametrize("n_q", [257, 300, 511, 512, 513, 1025])
def test_pair_kernel_matches_oracle(ctx, yp, oracle, n_q):
    """YPDQ_SCAN_TC_FP8 past 256 queries at t <= 36 runs passes of 512 queries, two per f32
    accumulator column (the second scaled by 512); YPDQ_SCAN_TC and AUTO run the FP4 forms on
    the same cases. Odd counts leave a pair with one query; rows equal or
    complementary to a query on the 128-bit prefix put d = +-128 in either half of a column;
    thresholds cover 0..36 at one size and the range's edges at the others."""
    rows = yp.synth.rows_128(6000, seed=n_q)
    q = yp.synth.rows_128(n_q, seed=n_q + 1)
    yp.synth.plant(rows, q, 300, 0, 40, seed=3)
    rows[10], rows[11] = q[0], ~q[1]
    rows[12], rows[13] = q[n_q - 1], ~q[n_q - 1]
    rows[14, :16], rows[14, 16:] = q[2, :16], ~q[2, 16:]   # prefix equal, distance 128
    rows[15, :16], rows[15, 16:] = ~q[3, :16], q[3, 16:]   # prefix complement, distance 128
    rows[16] = q[n_q - 2]
    ts = range(37) if n_q == 513 else (0, 1, 16, 31, 35, 36)
    for t in ts:
        want = oracle.find_all(rows, q, t)
        for algo in (5, 3, 0):  # YPDQ_SCAN_TC_FP8, YPDQ_SCAN_TC, YPDQ_SCAN_AUTO
            got = yp.scan(ctx, rows, q, t, algo=algo)
            assert np.array_equal(as_tuples(got), as_tuples(want)), (t, algo, len(got), len(want))


@pytest.mark.parametrize("n_q", [513, 514, 515, 719, 720, 721, 722, 1441])
def test_fp4_triple_kernel_matches_oracle(ctx, yp, oracle, n_q):
    """YPDQ_SCAN_TC_FP4 past 512 queries: block-scaled e2m1 operands (K = 64 per MMA), three
    queries per f32 accumulator column (B scale factors 2^-1, 2^7, 2^15), passes of 720
    queries, the first 126 bits as the bound (up to 512 queries the row-triple scan runs,
    test_fp4_rows_kernel_matches_oracle). Pass boundaries, triples with one or two queries,
    rows equal or complementary to a query on the prefix (every field at its extreme), rows
    that differ from a query only in the two prefix bits the bound leaves out (distance 2:
    found, with the full distance), every threshold 0..36 at one size; above 36 the call runs
    the FP8 scan."""
    rows = yp.synth.rows_128(6000, seed=n_q + 900)
    q = yp.synth.rows_128(n_q, seed=n_q + 901)
    yp.synth.plant(rows, q, 300, 0, 40, seed=9)
    rows[10], rows[11] = q[0], ~q[n_q - 1]
    rows[14, :16], rows[14, 16:] = q[n_q // 2, :16], ~q[n_q // 2, 16:]
    rows[15, :16], rows[15, 16:] = ~q[n_q - 1, :16], q[n_q - 1, 16:]
    for i in range(3):                                 # one row per field of a triple
        rows[20 + i] = q[min(i, n_q - 1)]
        rows[20 + i, 15] ^= np.uint8(0xC0)             # bits 126 and 127 of the prefix
    rows[5999] = q[0]                                  # the last, partial tile
    rows[200:264] = q[np.arange(64) % n_q]             # many hits in one tile
    ts = range(37) if n_q == 721 else (0, 1, 2, 16, 31, 35, 36, 40)
    for t in ts:
        want = oracle.find_all(rows, q, t)
        got = yp.scan(ctx, rows, q, t, algo=yp._lib.SCAN_TC_FP4)
        assert np.array_equal(as_tuples(got), as_tuples(want)), (t, len(got), len(want))


@pytest.mark.parametrize("n_q,algo,t", [(64, 3, 40), (64, 3, 31), (256, 5, 31), (300, 5, 31),
                                         (300, 3, 31), (800, 4, 31)])
def test_device_wait_timeout_is_reported_and_recovered(ctx, yp, oracle, n_q, algo, t):
    """The timeout path of the tensor-core scans (64 queries: queries as A, FP8 at t = 40 and
    three rows per column, FP4, at t = 31; 256 with YPDQ_SCAN_TC_FP8: one pass of single
    queries; 300: FP8 pairs and three launches of row triples; 800: FP4 query triples).
    Under a 1 ms wait limit a launch whose producer issues nothing (ypdq_debug_stall_scans)
    stops with its waits run out: the stream sync reports YPDQ_ERR_TIMEOUT, and the next scan
    on the same context returns the oracle's hits. No trap, no fault, no unbounded wait."""
    lib = ctx.lib
    rows = yp.synth.rows_128(50_000, seed=n_q + 70)
    q = yp.synth.rows_128(n_q, seed=n_q + 71)
    yp.synth.plant(rows, q, 200, 0, t, seed=72)
    d_rows, d_q = ctx.to_device(rows), ctx.to_device(q)
    cap = 1 << 14
    d_hits, d_cnt = ctx.alloc(cap * 16), ctx.alloc(8)
    assert lib.ypdq_set_scan_wait_limit(1_000_000) == 0
    try:
        assert lib.ypdq_debug_stall_scans(1) == 0
        yp.core.scan_device(ctx, d_rows, rows.shape[0], d_q, n_q, t, d_hits, cap, d_cnt, algo)
        with pytest.raises(yp.YpdqError) as err:
            ctx.sync()
        assert err.value.status == yp._lib.ERR_TIMEOUT
    finally:
        lib.ypdq_debug_stall_scans(0)
        lib.ypdq_set_scan_wait_limit(0)
    got = yp.scan(ctx, rows, q, t, algo=algo)
    assert np.array_equal(as_tuples(got), as_tuples(oracle.find_all(rows, q, t)))
    assert lib.ypdq_set_scan_wait_limit(61 * 10 ** 9) == yp._lib.ERR_INVALID
    assert lib.ypdq_debug_stall_scans(-1) == yp._lib.ERR_INVALID


@pytest.mark.parametrize("n_q", [1, 2, 31, 33, 64, 100, 127, 128])
def test_rows_kernel_matches_oracle(ctx, yp, oracle, n_q):
    """Up to 128 queries the tensor-core scan takes the queries as the MMA's A operand: at
    t <= 36 with three database rows per column (FP4, 720 rows per MMA), above with 256 rows
    per MMA (FP8). Row counts that end mid-tile, rows equal or complementary to a query,
    several planted rows per 64-row chunk, and thresholds on both sides of each prefix-bound
    switch (36 / 37, 62 / 63) and at the range's ends."""
    rows = yp.synth.rows_128(6001, seed=n_q + 500)
    q = yp.synth.rows_128(n_q, seed=n_q + 501)
    yp.synth.plant(rows, q, min(600, 6001), 0, 70, seed=n_q)
    rows[5996], rows[5997] = q[0], ~q[n_q - 1]   # the last, partial tile
    rows[300:310] = q[np.arange(10) % n_q]       # ten hits in one 64-row chunk
    for t in (0, 1, 16, 31, 36, 37, 48, 62, 63, 90, 128, 255, 256):
        want = oracle.find_all(rows, q, t)
        got = yp.scan(ctx, rows, q, t, algo=3, capacity=1 << 20)
        assert np.array_equal(as_tuples(got), as_tuples(want)), (t, len(got), len(want))


@pytest.mark.parametrize("n_q", [1, 2, 3, 31, 32, 33, 64, 65, 100, 127, 128, 129, 200, 256,
                                 300, 385, 512])
def test_fp4_rows_kernel_matches_oracle(ctx, yp, oracle, n_q):
    """YPDQ_SCAN_TC_FP4 (and YPDQ_SCAN_TC) with at most 512 queries at t <= 36, one launch per
    128 queries: the queries are the MMA's A operand and three database rows share each f32
    accumulator column (rows 3j, 3j + 1, 3j + 2 of a 720-row tile with B scales 2^-1, 2^7,
    2^15), the first 126 bits as the bound. Row counts that end mid-tile and mid-column
    (6000 + 0, 1, 2 rows; 5761: one row in the last tile), the three rows of one column equal
    or complementary to queries (every field at its extreme), rows that differ from a query
    only in the two prefix bits the bound leaves out, a run of hits across the columns of one
    tile, lane quarters with and without queries, launches with a partial last 128, every
    threshold 0..36 at one size; above 36 the call runs the FP8 scan."""
    n_rows = 5761 if n_q == 64 else 6000 + n_q % 3  # 5761: one row in the last tile
    rows = yp.synth.rows_128(n_rows, seed=n_q + 1300)
    q = yp.synth.rows_128(n_q, seed=n_q + 1301)
    yp.synth.plant(rows, q, 400, 0, 40, seed=n_q + 1302)
    rows[30], rows[31], rows[32] = q[0], q[n_q - 1], ~q[n_q // 2]   # one column, three fields
    rows[33], rows[34], rows[35] = ~q[0], ~q[n_q - 1], q[n_q // 2]
    rows[40, :16], rows[40, 16:] = q[n_q // 2, :16], ~q[n_q // 2, 16:]
    rows[41, :16], rows[41, 16:] = ~q[n_q - 1, :16], q[n_q - 1, 16:]
    for i in range(3):                                 # one row per field of a column
        rows[60 + i] = q[min(i, n_q - 1)]
        rows[60 + i, 15] ^= np.uint8(0xC0)             # bits 126 and 127 of the prefix
    rows[1440:1536] = q[np.arange(96) % n_q]           # many hits in one tile
    rows[n_rows - 1] = q[0]                            # the last, partial tile
    rows[n_rows - 3] = q[n_q - 1]
    ts = range(37) if n_q == 33 else (0, 1, 2, 16, 31, 35, 36, 40)
    for t in ts:
        want = oracle.find_all(rows, q, t)
        for algo in (yp._lib.SCAN_TC_FP4, 3):
            got = yp.scan(ctx, rows, q, t, algo=algo, capacity=1 << 20)
            assert np.array_equal(as_tuples(got), as_tuples(want)), (t, algo, len(got), len(want))
