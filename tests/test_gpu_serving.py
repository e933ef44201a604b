"""The continuous-batching screening service (ypdq_server_*) through the C ABI.

Each request's result must not depend on what else was on the device: the hits of a request
screened alone, the hits of the same request inside a mix of concurrent requests, and the
hits of ypdq_screen_host on those images are the same (index, query, distance) lists, in
(index, query) order, bit for bit; so are its 8 dihedral hashes. That holds for every DCT
precision because each image is hashed independently of its batch neighbours (by one CTA,
or for the ReferenceKernel by per-line running sums within the image).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POOL = 200


def log_uniform_sizes(rng, n, hi=64):
    return np.clip(np.exp(rng.uniform(0.0, np.log(hi + 1), n)).astype(int), 1, hi)


@pytest.fixture(scope="module")
def workload(ctx, yp):
    imgs = yp.synth.blob_images(POOL, seed=1201)
    h = yp.hash_batch(ctx, imgs)["hashes"].reshape(-1, 32)
    rows = yp.synth.rows_128(300_000, seed=1202)
    yp.synth.plant(rows, h, 4000, 0, 40, seed=1203)
    db = yp.Database(ctx, rows)
    yield imgs, rows, db
    db.close()


def request_slices(rng, n_req):
    sizes = log_uniform_sizes(rng, n_req)
    return [(int(rng.integers(0, POOL - n + 1)), int(n)) for n in sizes]


@pytest.mark.parametrize("dct", [0, 2, 0x200])  # FP32, BF16x3, YPDQ_COMPRESS_JAROSZ
def test_same_alone_and_in_mix(ctx, yp, workload, dct):
    imgs, rows, db = workload
    reqs = request_slices(np.random.default_rng(40 + dct), 36)
    with yp.Server(ctx, db, threshold=31, dct=dct, max_step_images=256, slots=3) as srv:
        alone = {}
        for i, (s, n) in enumerate(reqs):
            srv.submit(imgs[s:s + n], want_hashes=True, tag=i)
            (r,) = srv.drain()
            alone[i] = r
        srv.stats(reset=True)
        for i, (s, n) in enumerate(reqs):
            srv.submit(imgs[s:s + n], want_hashes=True, tag=i)
        mix = {r.tag: r for r in srv.drain()}
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["rejected"] == 0
    assert st["steps"] < len(reqs)  # requests shared device steps
    assert 0 < st["p50_us"] <= st["p99_us"] <= st["max_us"]
    for i, (s, n) in enumerate(reqs):
        a, m = alone[i], mix[i]
        assert a.ok and m.ok and a.n_images == m.n_images == n
        assert a.n_hits == m.n_hits == len(m.hits)
        assert np.array_equal(a.hits, m.hits), i
        assert np.array_equal(a.hashes, m.hashes)
        assert np.array_equal(a.quality, m.quality)
        want, want_h = yp.screen_host(ctx, db, imgs[s:s + n], threshold=31, dct=dct,
                                      want_hashes=True)
        assert np.array_equal(m.hits, want), i
        assert np.array_equal(m.hashes, want_h)
    assert sum(r.n_hits for r in mix.values()) > 0


def test_hits_match_oracle(ctx, yp, oracle, workload):
    imgs, rows, db = workload
    reqs = request_slices(np.random.default_rng(5), 10)
    with yp.Server(ctx, db, threshold=31, max_step_images=128, slots=2) as srv:
        for i, (s, n) in enumerate(reqs):
            srv.submit(imgs[s:s + n], want_hashes=True, tag=i)
        res = {r.tag: r for r in srv.drain()}
    for i, (s, n) in enumerate(reqs):
        r = res[i]
        want = oracle.find_all(rows, r.hashes.reshape(-1, 32), 31)
        assert np.array_equal(r.hits[["index", "query", "distance"]],
                              want[["index", "query", "distance"]])
        ref_hashes = oracle.hash_batch(imgs[s:s + n], semantics="exact")[0]
        assert np.array_equal(r.hashes, ref_hashes)


def test_admission_bounds_queue(ctx, yp, workload):
    imgs, rows, db = workload
    with yp.Server(ctx, db, max_step_images=64, slots=1, max_queued_images=100) as srv:
        with pytest.raises(yp.YpdqError) as e:
            srv.submit(imgs[:65])
        assert e.value.status == yp._lib.ERR_INVALID
        accepted, busy = [], 0
        for k in range(200):
            rid = srv.try_submit(imgs[k % 100:k % 100 + 30])
            if rid is None:
                busy += 1
                if busy >= 5:
                    break
            else:
                accepted.append(rid)
        done = srv.drain()
        st = srv.stats()
    assert busy >= 1
    assert st["rejected"] == busy and st["completed"] == len(accepted) == len(done)
    assert all(r.ok for r in done)
    assert st["mean_step_images"] <= 64


def test_overflow_and_exact_rescan(ctx, yp, workload):
    """A request capacity below its hits reports OVERFLOW with the true count and the first
    hits in order; a step whose hits exceed the device buffer is re-scanned exactly."""
    imgs, rows, db = workload
    want = [yp.screen_host(ctx, db, imgs[i:i + 8], threshold=31) for i in (0, 8, 16)]
    assert all(len(w) > 8 for w in want)
    with yp.Server(ctx, db, max_step_images=32, slots=1, step_hit_capacity=16) as srv:
        srv.submit(imgs[0:8], hit_capacity=1 << 16, tag=0)
        srv.submit(imgs[8:16], hit_capacity=1 << 16, tag=1)
        srv.submit(imgs[16:24], hit_capacity=5, tag=2)
        res = {r.tag: r for r in srv.drain()}
        st = srv.stats()
    assert st["rescans"] >= 1
    for t in (0, 1):
        assert res[t].ok and np.array_equal(res[t].hits, want[t])
    r = res[2]
    assert r.status == yp._lib.ERR_OVERFLOW and r.n_hits == len(want[2])
    assert np.array_equal(r.hits, want[2][:5])


def test_hits_past_the_copied_prefix(ctx, yp, workload):
    """At threshold 110 an image matches ~1-2 % of random rows (tens of thousands of hits),
    more than every step copies back by default; the rest is fetched after the step."""
    imgs, rows, db = workload
    want = [yp.screen_host(ctx, db, imgs[i:i + 1], threshold=110, capacity=1 << 20)
            for i in (3, 4)]
    assert min(len(w) for w in want) > 8192
    with yp.Server(ctx, db, threshold=110, max_step_images=8, slots=2) as srv:
        srv.submit(imgs[3:4], hit_capacity=1 << 20, tag=0)
        srv.submit(imgs[4:5], hit_capacity=1 << 20, tag=1)
        res = {r.tag: r for r in srv.drain()}
    for t in (0, 1):
        assert res[t].ok and np.array_equal(res[t].hits, want[t])


def test_u8_input(ctx, yp, workload):
    imgs, rows, db = workload
    u8 = yp.synth.to_u8(imgs[:40])
    with yp.Server(ctx, db, input_kind="u8", max_step_images=64) as srv:
        for i, (s, n) in enumerate([(0, 7), (7, 20), (27, 13)]):
            srv.submit(u8[s:s + n], tag=i)
        res = {r.tag: r for r in srv.drain()}
    for i, (s, n) in enumerate([(0, 7), (7, 20), (27, 13)]):
        assert np.array_equal(res[i].hits, yp.screen_host(ctx, db, u8[s:s + n], threshold=31))


def test_autotune_table_and_target(ctx, yp, workload):
    imgs, rows, db = workload
    with yp.Server(ctx, db, max_step_images=64, autotune=True) as srv:
        st = srv.stats()
        assert [b["images"] for b in st["buckets"]] == [1, 2, 4, 8, 16, 32, 64]
        assert all(b["ms"] > 0 and b["algo"] in ("simt", "tc", "tc pairs", "tc rows",
                                                 "tc fp4 triples", "tc fp4 rows")
                   for b in st["buckets"])
        # FP8 pair passes are timed from 17 images; FP4 triple passes run past 64 images only
        assert all(b["algo"] != "tc pairs" or b["images"] > 16 for b in st["buckets"])
        assert all(b["algo"] != "tc fp4 triples" for b in st["buckets"])
        # queries as the MMA's A operand: FP8 up to 16 images (128 queries, t > 36 only),
        # FP4 with three rows per column up to 64 images (512 queries, 128 per launch)
        assert all(b["algo"] != "tc rows" for b in st["buckets"])
        assert all(b["algo"] != "tc fp4 rows" or b["n_tile"] == 128 for b in st["buckets"])
        srv.submit(imgs[:50], tag=0)
        (r,) = srv.drain()
        assert np.array_equal(r.hits, yp.screen_host(ctx, db, imgs[:50], threshold=31))
    # a step-time target below every bucket keeps only the smallest one
    with yp.Server(ctx, db, max_step_images=8, autotune=True, target_step_ms=1e-6) as srv:
        assert srv.stats()["max_step_images"] == 1
        with pytest.raises(yp.YpdqError):
            srv.submit(imgs[:2])
        srv.submit(imgs[:1])
        (r,) = srv.drain()
        assert r.ok


def test_pinned_images(ctx, yp, workload):
    imgs, rows, db = workload
    pin = yp.PinnedArray(ctx, (48, 512, 512), np.float32)
    pin.array[:] = imgs[:48]
    with yp.Server(ctx, db, max_step_images=64) as srv:
        srv.submit(pin.array[:16], tag=0)
        srv.submit(pin.array[16:48], tag=1)
        res = {r.tag: r for r in srv.drain()}
    assert np.array_equal(res[0].hits, yp.screen_host(ctx, db, imgs[:16], threshold=31))
    assert np.array_equal(res[1].hits, yp.screen_host(ctx, db, imgs[16:48], threshold=31))
    pin.free()


def test_rgba_requests(ctx, yp, workload):
    imgs, rows, db = workload
    rgba = yp.synth.color_images(9, seed=77, channels=4)
    with yp.Server(ctx, db, input_kind="rgba8", max_step_images=16) as srv:
        srv.submit(rgba[:4], tag=0)
        srv.submit(rgba[4:], tag=1)
        res = {r.tag: r for r in srv.drain()}
    assert np.array_equal(res[0].hits, yp.screen_host(ctx, db, rgba[:4], threshold=31))
    assert np.array_equal(res[1].hits, yp.screen_host(ctx, db, rgba[4:], threshold=31))


def test_native_replay(ctx, yp, workload):
    """ypdq_server_replay, the native load generator: an open-loop trace (arrivals spread over
    20 ms) and a closed loop over the same requests. Every request completes, its hits (in
    (index, query) order, query numbers local to the request) equal ypdq_screen_host's on its
    images, its true hit count is reported, and the server's window counts the requests."""
    imgs, rows, db = workload
    rng = np.random.default_rng(1290)
    reqs = request_slices(rng, 24)
    first = np.array([s for s, _ in reqs])
    n = np.array([k for _, k in reqs])
    want = [yp.screen_host(ctx, db, imgs[s:s + k], threshold=31) for s, k in reqs]
    cap = max(len(w) for w in want) + 8
    with yp.Server(ctx, db, max_step_images=64, slots=2, max_queued_images=4096) as srv:
        for arrival in (np.sort(rng.integers(0, 20_000_000, len(reqs))), None):
            srv.stats(reset=True)
            sub, rej, n_hits, hits = srv.replay(imgs, first, n, arrival, duration_s=10.0,
                                                hit_capacity=cap)
            assert (sub, rej) == (len(reqs), 0)
            st = srv.stats()
            assert st["completed"] == len(reqs) and st["images_completed"] == n.sum()
            for i, w in enumerate(want):
                assert n_hits[i] == len(w), i
                assert np.array_equal(hits[i, :len(w)], w), i
        # a pool range outside the pool is refused before anything is submitted
        with pytest.raises(yp.YpdqError):
            srv.replay(imgs, np.array([POOL - 1]), np.array([2]))
