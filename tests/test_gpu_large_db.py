"""Large database with heavy hits: 100,000,000 rows (3.2 GB resident) in 10^5 clusters.

Every row is a member of a cluster: the cluster centre has 128 set bits, and the member
sits at Hamming distance d ~ Binomial(40, 1/2) from it (about 20). Queries are 1,024
cluster centres; at thresholds 16, 31, 48 and 64 a batch returns ~1.3e5 to ~1.0e6 hits.

Checks, each independent of the others:
  * the tensor-core scan and the SIMT scan (different kernels, different arithmetic)
    return the same sorted (index, query, distance) list over all 100M rows;
  * the hits contain every member of a query's cluster within the threshold, with its
    distance computed on the CPU from the oracle's twin of the generator, and every other
    hit (there are none with random centres, but none are assumed) has the distance of
    its row;
  * on a 2,000,000-row slice the hits equal the oracle's scalar matcher.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_CENTRES, MEMBERS, TRIALS, SEED = 100_000, 1000, 40, 4242
N_ROWS = N_CENTRES * MEMBERS
N_QUERIES = 1024
SLICE = 2_000_000


@pytest.fixture(scope="module")
def large_db(ctx, yp):
    d_rows = ctx.alloc(N_ROWS * 32)
    yp._lib.check(ctx.lib.ypdq_synth_clustered_rows(ctx.handle, d_rows.ptr, N_ROWS, 0, MEMBERS,
                                                    TRIALS, SEED, None))
    d_c = ctx.alloc(N_CENTRES * 32)
    yp._lib.check(ctx.lib.ypdq_synth_rows(ctx.handle, d_c.ptr, N_CENTRES, 0, SEED, None))
    ctx.sync()
    centres = d_c.download((N_CENTRES, 32), np.uint8)
    d_c.free()
    rng = np.random.default_rng(11)
    qc = np.sort(rng.choice(N_CENTRES, N_QUERIES, replace=False))
    queries = np.ascontiguousarray(centres[qc])
    d_q = ctx.to_device(queries)
    yield d_rows, centres, qc, queries, d_q
    d_q.free()
    d_rows.free()


def scan_sorted(ctx, yp, d_rows, d_q, t, algo, cap=1 << 21):
    d_hits = ctx.alloc(cap * 16)
    d_cnt = ctx.alloc(8)
    yp.core.scan_device(ctx, d_rows, N_ROWS, d_q, N_QUERIES, t, d_hits, cap, d_cnt, algo)
    ctx.sync()
    n = int(d_cnt.download((1,), np.uint64)[0])
    assert n <= cap
    yp.core.sort_hits_device(ctx, d_hits, n)
    ctx.sync()
    hits = d_hits.download((n,), yp.HIT_DTYPE)
    d_hits.free()
    d_cnt.free()
    return hits


def keys(h):
    return h["index"].astype(np.int64) * N_QUERIES + h["query"].astype(np.int64)


def test_generator_matches_oracle(ctx, yp, oracle, large_db):
    d_rows, centres, qc, queries, d_q = large_db
    assert np.array_equal(centres[:1000], oracle.synth_rows(1000, SEED))
    for first in (0, 57_123_000, N_ROWS - 50_000):
        got = d_rows.download((50_000, 32), np.uint8, offset=first * 32)
        assert np.array_equal(got, oracle.synth_clustered(50_000, MEMBERS, TRIALS, SEED, first=first))


@pytest.mark.parametrize("t", [16, 31, 48, 64])
def test_heavy_hits_100m_rows(ctx, yp, oracle, large_db, t):
    d_rows, centres, qc, queries, d_q = large_db
    tc = scan_sorted(ctx, yp, d_rows, d_q, t, yp._lib.SCAN_TC)
    simt = scan_sorted(ctx, yp, d_rows, d_q, t, yp._lib.SCAN_SIMT)
    assert np.array_equal(tc, simt)

    # every member of each query's cluster within t, distances from the generator's twin
    exp_idx, exp_q, exp_d = [], [], []
    for q, c in enumerate(qc):
        members = oracle.synth_clustered(MEMBERS, MEMBERS, TRIALS, SEED, first=int(c) * MEMBERS,
                                         nthreads=1)
        d = np.unpackbits(members ^ queries[q], axis=1).sum(1)
        m = np.nonzero(d <= t)[0]
        exp_idx.append(int(c) * MEMBERS + m)
        exp_q.append(np.full(len(m), q))
        exp_d.append(d[m])
    exp = np.zeros(sum(len(x) for x in exp_idx), yp.HIT_DTYPE)
    exp["index"] = np.concatenate(exp_idx)
    exp["query"] = np.concatenate(exp_q)
    exp["distance"] = np.concatenate(exp_d)
    k_tc, k_exp = keys(tc), keys(exp)
    inside = np.isin(k_tc, k_exp)
    assert inside.sum() == len(exp)
    order = np.argsort(k_exp)
    assert np.array_equal(tc[inside]["distance"], exp[order]["distance"])
    for h in tc[~inside][:1000]:  # hits outside the query clusters: check from the rows
        row = d_rows.download((1, 32), np.uint8, offset=int(h["index"]) * 32)[0]
        assert np.unpackbits(row ^ queries[h["query"]]).sum() == h["distance"] <= t
    if t >= 31:
        assert len(tc) > 990_000  # ~1,000 members per query cluster

    # scalar matcher on a slice of the database
    rows = d_rows.download((SLICE, 32), np.uint8)
    want = oracle.find_all(rows, queries, t)
    got = tc[tc["index"] < SLICE]
    assert np.array_equal(got[["index", "query", "distance"]], want[["index", "query", "distance"]])
