#!/usr/bin/env python3
"""Benchmark: images screened per second against a 10M-hash database.

One step screens a batch of B synthetic 512x512 f32 images: hash each (FP32, bit-exact with
yume-pdq's scalar kernel), derive its 8 dihedral hashes, and scan all 8B hashes exactly
against a device-resident 10,000,000-row database at Hamming threshold 31. `value` is
images/s with inputs already in HBM. `e2e` is the same metric for a stream of such batches
from pinned host memory through the C ABI's serving loop (ypdq_server_*), sorted hits back
in host memory, every copy inside the timed region; `e2e_blocking` through one blocking
ypdq_screen_host call per batch.

--impl reference times yume-pdq's CPU path (the CPU oracle, a restatement of its scalar
kernel and scalar matcher) on this host's cores on a bounded sample of the same workload.

Multi-GPU: one process per GPU (torchrun), each a replica with the full database screening
its own batch (weak scaling; the path needs no collective).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "images screened/s vs 10M-hash DB (hash+8-dihedral scan); p50/p99 latency"
UNIT = "images/s"
L2_BYTES = 129 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=1024, help="images per step")
    ap.add_argument("--db-rows", type=int, default=10_000_000)
    ap.add_argument("--planted", type=int, default=10_000)
    ap.add_argument("--threshold", type=int, default=31)
    ap.add_argument("--algo", type=int, default=0, help="scan algorithm (0 auto, 1 SIMT, 2 B1MMA)")
    ap.add_argument("--seed", type=int, default=2025)
    ap.add_argument("--dct", type=int, default=0, choices=[0, 1, 2],
                    help="DCT stage 1: 0 FP32 SIMT (bit-exact), 1 TF32, 2 BF16x3 tensor cores")
    ap.add_argument("--cpu-sample", type=int, default=256,
                    help="images per CPU-baseline sample (about 10 s of work on 16 cores)")
    ap.add_argument("--serve-rates", default="2000,4000,8000",
                    help="Poisson request rates (req/s) for the serving loop; '' skips it")
    ap.add_argument("--serve-seconds", type=float, default=2.0,
                    help="arrival window per serving rate (and for the saturation run)")
    ap.add_argument("--large-rows", type=int, default=100_000_000,
                    help="rows of the clustered heavy-hit database (0 skips it)")
    ap.add_argument("--scan-sweep", type=int, default=1,
                    help="1: report the 1/8/64/256/1024-query scan sweep (0 skips the section)")
    ap.add_argument("--dct-variants", type=int, default=1,
                    help="1: time and check the FP32 / TF32 / BF16x3 hash variants")
    ap.add_argument("--peaks", action="store_true",
                    help="only measure the dense FP8 burst of GPU 0 and print it as JSON")
    ap.add_argument("--kernel", choices=["hash", "scan"],
                    help="only time one kernel configuration with CUDA events and print one "
                         "line per repetition (for profiling): `hash` runs ypdq_hash_batch on "
                         "--images device-resident images of --input kind with --dct (plus "
                         "--separable / --jarosz); `scan` runs ypdq_scan of --queries random "
                         "hashes against --db-rows generated rows with --algo at --threshold")
    ap.add_argument("--input", choices=["f32", "u8", "rgb8", "rgba8"], default="f32")
    ap.add_argument("--images", type=int, default=4096)
    ap.add_argument("--separable", action="store_true",
                    help="with --kernel hash: YPDQ_COMPRESS_SEPARABLE (not bit-exact)")
    ap.add_argument("--jarosz", action="store_true",
                    help="with --kernel hash: YPDQ_COMPRESS_JAROSZ (ReferenceKernel<f32>)")
    ap.add_argument("--queries", type=int, default=64)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--ranks-only", action="store_true",
                    help="only join the replicas' process group and print this rank's view "
                         "(tests the multi-process launch without a GPU)")
    return ap.parse_args()


def launch_replicas(argv, n):
    """`bench.py --gpus N` started outside torchrun: run N replica processes of this script,
    one per GPU (RANK = LOCAL_RANK = i, WORLD_SIZE = N, rendezvous on 127.0.0.1 at a free
    port), as torchrun would. Returns the first non-zero exit status, else 0. Rank 0 prints
    the JSON line."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n),
                   LOCAL_WORLD_SIZE=str(n), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, os.path.abspath(__file__)] + list(argv),
                                      env=env))
    rcs = [p.wait() for p in procs]
    return next((rc for rc in rcs if rc), 0)


def aggregate_over_ranks(pg, local_ms, world, images_per_rank):
    """Replicas: every rank screened `images_per_rank` images in its own `local_ms`. The job
    time is the slowest rank's (all-reduce MAX over the process group, if any) and the
    job's value is all ranks' images over that time, in images/s."""
    t = float(local_ms)
    if pg is not None:
        import torch
        x = torch.tensor([t], dtype=torch.float64)
        pg.all_reduce(x, op=pg.ReduceOp.MAX)
        t = float(x.item())
    return t, world * images_per_rank / (t / 1000.0)


def dist_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class ClockSampler:
    """nvidia-smi clock/throttle samples taken while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    """(HBM GB/s, dense bf16 TFLOP/s burst, source) from MEASURED_PEAKS.json, else fallback."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d["hbm_gbs"], d["bf16_tflops"], "measured"
    return 6800.0, 1900.0, "fallback"


# DRAM bytes (read + write) per 512-query pass of the pair scan over 10M rows: an ncu
# capture of one launch of 4 passes (2,048 queries, t = 31) read 1.2797 GB and wrote 3.4 MB.
NCU_DRAM_BYTES_PER_PASS_10M = (1.2797e9 + 3.4e6) / 4


def fp8_dense_burst(device=0, n=8192, reps=10):
    """Dense FP8 (e4m3) tensor-core rate of this GPU in TFLOP/s: torch._scaled_mm of two
    n x n e4m3 matrices (per-tensor unit scales, bf16 out), best of `reps` launches timed
    with CUDA events on torch's stream, 2 n^3 FLOP each. The method of the bf16 burst in
    MEASURED_PEAKS.json with the FP8 operand type. None if torch or FP8 GEMMs are absent."""
    try:
        import torch
        dev = torch.device("cuda", device)
        a = torch.randn(n, n, device=dev).to(torch.float8_e4m3fn)
        b = torch.randn(n, n, device=dev).to(torch.float8_e4m3fn).t()  # column-major
        one = torch.ones((), device=dev)

        def mm():
            return torch._scaled_mm(a, b, one, one, out_dtype=torch.bfloat16)

        for _ in range(3):
            mm()
        best = float("inf")
        for _ in range(reps):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            mm()
            e.record()
            e.synchronize()
            best = min(best, s.elapsed_time(e))
        del a, b
        torch.cuda.empty_cache()
        return 2.0 * n ** 3 / (best / 1e3) / 1e12
    except Exception as exc:  # reported, never silently replaced by a guess
        sys.stderr.write("fp8 burst not measured: %s\n" % exc)
        return None


def fp4_dense_burst(device=0, n=8192, reps=10):
    """Dense block-scaled FP4 tensor-core rate of this GPU in TFLOP/s: torch._scaled_mm of two
    n x n e2m1 matrices with unit e4m3 scales per 16 elements along K (the block-scaled FP4
    GEMM this torch build offers; bf16 out), best of `reps` launches timed with CUDA events,
    2 n^3 FLOP each. None if this torch build has no FP4 GEMM."""
    try:
        import torch
        dev = torch.device("cuda", device)
        x4 = torch.float4_e2m1fn_x2
        a = torch.randint(0, 256, (n, n // 2), dtype=torch.uint8, device=dev).view(x4)
        b = torch.randint(0, 256, (n, n // 2), dtype=torch.uint8, device=dev).view(x4).t()
        scale = torch.ones(n * (n // 16), device=dev).to(torch.float8_e4m3fn)

        def mm():
            return torch._scaled_mm(a, b, scale, scale, out_dtype=torch.bfloat16)

        for _ in range(3):
            mm()
        best = float("inf")
        for _ in range(reps):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            mm()
            e.record()
            e.synchronize()
            best = min(best, s.elapsed_time(e))
        del a, b, scale
        torch.cuda.empty_cache()
        return 2.0 * n ** 3 / (best / 1e3) / 1e12
    except Exception as exc:  # reported, never silently replaced by a guess
        sys.stderr.write("fp4 burst not measured: %s\n" % exc)
        return None


def scan_algo_used(algo, nq, threshold):
    """The algorithm ypdq_scan runs for YPDQ_SCAN_AUTO (mirrors auto_scan_algo in scan.cu)."""
    if algo == 0:
        simt_max = (9 if threshold <= 34 else 6 if threshold <= 36 else
                    24 if threshold <= 62 else 12)
        return 1 if nq <= simt_max else 3
    return algo


def setup_workload(yp, ctx, args, rank):
    """Images on the device and the database with its planted near-duplicates, on the device
    and (for the CPU baseline and the parity check) on the host. The rows are
    ypdq_synth_rows(seed); args.planted of them become copies of the step's dihedral hashes
    at distances 0..31 (synth.plant_near_duplicates, the same edit the CPU arm makes)."""
    batch = yp.synth.blob_images(args.batch, seed=args.seed + 1000 * rank)
    d_img = ctx.to_device(batch)
    n = args.db_rows
    d_rows = ctx.alloc(n * 32)
    yp._lib.check(ctx.lib.ypdq_synth_rows(ctx.handle, d_rows.ptr, n, 0, args.seed, None))
    d_hash = ctx.alloc(args.batch * 256)
    d_q = ctx.alloc(args.batch * 32)
    yp.core.hash_batch_device(ctx, d_img, args.batch, yp._lib.INPUT_F32, d_hash, d_q)
    ctx.sync()
    queries = d_hash.download((args.batch * 8, 32), np.uint8)
    rows = d_rows.download((n, 32), np.uint8)
    yp.synth.plant_near_duplicates(rows, queries, args.planted, args.seed + 99)
    d_rows.upload(rows)
    return batch, d_img, rows, d_rows, d_hash, d_q


def serve_run(yp, srv, pool, rate, seconds, rng, hit_cap=1024):
    """Open-loop Poisson arrivals at `rate` req/s (rate None: submit whenever the queue has
    room, i.e. saturation) of log-uniform 1..64-image requests sliced from `pool`, for
    `seconds`. The arrival times are drawn here and the requests submitted by the library's
    native load generator (ypdq_server_replay), so no pause of this interpreter shifts an
    arrival. Returns the server's window statistics once every accepted request has
    completed."""
    n_pool = pool.shape[0]
    m = int((rate if rate is not None else 20000.0) * seconds * 1.25) + 16
    n = np.minimum(64, np.maximum(1, np.exp(rng.uniform(0.0, np.log(65.0), m)).astype(np.int64)))
    first = rng.integers(0, n_pool - n + 1)
    arrival = (None if rate is None else
               (np.cumsum(rng.exponential(1.0 / rate, m)) * 1e9).astype(np.uint64))
    srv.stats(reset=True)
    srv.replay(pool, first, n, arrival, duration_s=seconds, hit_capacity=hit_cap)
    st = srv.stats()
    return {"offered_req_s": rate, "seconds": round(st["elapsed_s"], 3),
            "completed_req_s": st["completed"] / st["elapsed_s"],
            "images_s": st["images_completed"] / st["elapsed_s"],
            "p50_ms": st["p50_us"] / 1e3, "p99_ms": st["p99_us"] / 1e3,
            "mean_ms": st["mean_us"] / 1e3, "max_ms": st["max_us"] / 1e3,
            "requests": st["completed"], "rejected": st["rejected"],
            "steps": st["steps"], "mean_step_images": st["mean_step_images"],
            "hits": st["hits_completed"]}


def serving(yp, ctx, db, batch, args):
    """The continuous-batching service on the same database: Poisson sweep + saturation."""
    rates = [float(r) for r in args.serve_rates.split(",") if r.strip()]
    if not rates:
        return None
    pin = yp.PinnedArray(ctx, batch.shape, np.float32)
    pin.array[:] = batch
    rng = np.random.default_rng(args.seed + 7)
    t_tune = time.perf_counter()
    srv = yp.Server(ctx, db, threshold=args.threshold, dct=args.dct, max_step_images=1024,
                    slots=3, autotune=True)
    t_tune = time.perf_counter() - t_tune
    serve_run(yp, srv, pin.array, rates[0], min(0.5, args.serve_seconds), rng)  # warm-up
    points = [serve_run(yp, srv, pin.array, r, args.serve_seconds, rng) for r in rates]
    sat = serve_run(yp, srv, pin.array, None, args.serve_seconds, rng)
    table = srv.stats()["buckets"]
    srv.close()
    pin.free()
    return {"workload": "Poisson arrivals, 1-64 images per request (log-uniform), hash + 8 "
                        "dihedrals + exact scan vs %d rows at t=%d" % (db.n_rows, args.threshold),
            "images_pool": int(batch.shape[0]), "slots": 3, "max_step_images": 1024,
            "points": points, "saturation": sat, "autotune_s": round(t_tune, 3),
            "buckets": table}


def large_db(yp, ctx, args, members=1000, trials=40, n_queries=1024):
    """Heavy hits: 1,024 cluster-centre queries vs a clustered database (members at distance
    ~Binomial(40, 1/2) from 128-bit centres) at t = 16, 31, 48, 64; scan + sort of the hits."""
    n = args.large_rows
    if n <= 0:
        return None
    n_centres = n // members
    d_rows = ctx.alloc(n * 32)
    yp._lib.check(ctx.lib.ypdq_synth_clustered_rows(ctx.handle, d_rows.ptr, n, 0, members,
                                                    trials, args.seed, None))
    rng = np.random.default_rng(args.seed + 3)
    qc = np.sort(rng.choice(n_centres, n_queries, replace=False))
    d_c = ctx.alloc(n_centres * 32)
    yp._lib.check(ctx.lib.ypdq_synth_rows(ctx.handle, d_c.ptr, n_centres, 0, args.seed, None))
    ctx.sync()
    d_q = ctx.to_device(d_c.download((n_centres, 32), np.uint8)[qc])
    d_c.free()
    cap = 1 << 22
    d_hits = ctx.alloc(cap * 16)
    d_cnt = ctx.alloc(8)
    stream = ctx.stream()
    e = [ctx.event() for _ in range(3)]
    points = []
    for t in (16, 31, 48, 64):
        scan_ms, sort_ms = [], []
        for rep in range(4):
            ctx.record(e[0], stream)
            yp.core.scan_device(ctx, d_rows, n, d_q, n_queries, t, d_hits, cap, d_cnt,
                                yp._lib.SCAN_TC, stream)
            ctx.record(e[1], stream)
            ctx.sync(stream)
            hits = int(d_cnt.download((1,), np.uint64)[0])
            yp.core.sort_hits_device(ctx, d_hits, min(hits, cap), stream)
            ctx.record(e[2], stream)
            ctx.sync(stream)
            if rep:  # first repetition is warm-up
                scan_ms.append(ctx.elapsed_ms(e[0], e[1]))
                sort_ms.append(ctx.elapsed_ms(e[1], e[2]))
        ms = statistics.median(scan_ms)
        points.append({"t": t, "hits": hits, "scan_ms": ms, "sort_ms": statistics.median(sort_ms),
                       "G_pairs_s": n * n_queries / (ms / 1e3) / 1e9,
                       "hit_bytes_written": hits * 16})
    d_rows.free()
    d_hits.free()
    return {"workload": "%d clustered rows (%d centres x %d members, distance ~Binomial(%d, 1/2)) "
                        "vs %d centre queries, tensor-core scan + bitonic sort of the hits"
                        % (n, n_centres, members, trials, n_queries),
            "db_bytes": n * 32, "points": points}


def scan_sweep(yp, ctx, d_rows, n, d_hash, args, qs=(1, 8, 64, 256, 1024), reps=6):
    """Scan only against the bench database: query batches of 1, 8, 64, 256 and 1,024 hashes
    (the step's own dihedral hashes, whose near-duplicates are planted in the database) at
    the bench threshold, through the SIMT scan, the tensor-core scans (FP8 and FP4) and
    YPDQ_SCAN_AUTO:
    launch time (median of reps - 1 after one warm launch), database stream rate and its
    fraction of the measured HBM copy rate. Every launch reads the whole database (larger
    than L2)."""
    hbm_peak, _, peak_kind = measured_peaks()
    stream = ctx.stream()
    e0, e1 = ctx.event(), ctx.event()
    cap = 1 << 20
    d_hits, d_cnt = ctx.alloc(cap * 16), ctx.alloc(8)
    out = {"db_rows": n, "threshold": args.threshold, "hbm_peak_gbs": hbm_peak,
           "peak_source": peak_kind, "points": []}
    for q in qs:
        pt = {"queries": q, "auto_algo": {1: "simt", 3: "tc"}[scan_algo_used(0, q, args.threshold)]}
        for name, algo in (("simt", 1), ("tc", 3), ("tc_fp4", 4), ("auto", 0)):
            ms = []
            for rep in range(reps):
                ctx.record(e0, stream)
                yp.core.scan_device(ctx, d_rows, n, d_hash, q, args.threshold, d_hits, cap, d_cnt,
                                    algo, stream)
                ctx.record(e1, stream)
                ctx.sync(stream)
                if rep:
                    ms.append(ctx.elapsed_ms(e0, e1))
            t = statistics.median(ms)
            gbs = n * 32 / (t / 1e3) / 1e9
            pt[name] = {"ms": t, "db_GB_s": gbs, "frac_hbm": gbs / hbm_peak,
                        "Gpairs_s": n * q / (t / 1e3) / 1e9}
        pt["hits"] = int(d_cnt.download((1,), np.uint64)[0])
        out["points"].append(pt)
    d_hits.free()
    d_cnt.free()
    return out


def dct_variants(yp, ctx, args, n_distinct=512, n_launch=4096):
    """4,096 images per launch (blob images with 25 % noise and 5 % constant ones), f32 and
    u8 input, DCT stage 1 in FP32 SIMT / TF32 / BF16x3, each with the reference-order and the
    separable compress, and the ReferenceKernel (full Jarosz filter, sequential DCT): launch
    throughput, coefficient error against an FP64 DCT of the variant's own compressed
    images, hash-bit disagreement with the exact FP32 kernel."""
    import ctypes
    imgs, kind = yp.synth.mixed_images(n_distinct, seed=args.seed + 11)
    live = kind != 2  # constant images: PDQF is rounding noise, bits carry no information
    d = np.arange(127)
    d64 = np.sqrt(2.0 / 127.0) * np.cos(np.pi * np.outer(np.arange(1, 17), 2 * d + 1) / 254.0)
    stream = ctx.stream()
    e0, e1 = ctx.event(), ctx.event()
    out = {"images_per_launch": n_launch, "distinct_images": n_distinct,
           "mix": "%d blob, %d noise, %d constant" % ((kind == 0).sum(), (kind == 1).sum(),
                                                      (kind == 2).sum()), "variants": []}
    for name, data in (("f32", imgs), ("u8", yp.synth.to_u8(imgs))):
        ik = yp._lib.INPUT_U8 if name == "u8" else yp._lib.INPUT_F32
        d_img = ctx.to_device(np.concatenate([data] * (n_launch // n_distinct)))
        d_h, d_q = ctx.alloc(n_launch * 256), ctx.alloc(n_launch * 32)
        ref = yp.hash_batch(ctx, data, dct=0)
        # 0x100: YPDQ_COMPRESS_SEPARABLE; 0x200: YPDQ_COMPRESS_JAROSZ (ReferenceKernel<f32>)
        for dct in (0, 1, 2, 0x100, 0x101, 0x102, 0x200):
            ms = []
            for rep in range(6):
                ctx.record(e0, stream)
                yp.core.hash_batch_device(ctx, d_img, n_launch, ik, d_h, d_q, dct=dct,
                                          stream=stream)
                ctx.record(e1, stream)
                ctx.sync(stream)
                if rep:
                    ms.append(ctx.elapsed_ms(e0, e1))
            t = statistics.median(ms)
            ctas = None
            if dct != 0x200:
                c = ctypes.c_int()
                yp._lib.check(ctx.lib.ypdq_hash_occupancy(ctx.handle, ik, dct, ctypes.byref(c)))
                ctas = c.value
            v = {"input": name,
                 "dct": "fp32 sequential" if dct == 0x200 else ("fp32", "tf32", "bf16x3")[dct & 0xFF],
                 "compress": ("jarosz filter (ReferenceKernel)" if dct == 0x200 else
                              "separable" if dct & 0x100 else "reference order"), "ms": t,
                 "images_s": n_launch / (t / 1e3), "ctas_per_sm": ctas,
                 "input_GB_s": n_launch * data[0].nbytes / (t / 1e3) / 1e9}
            got = yp.hash_batch(ctx, data, dct=dct, want_pdqf=True, want_buf1=True)
            b = got["buf1"][live].astype(np.float64)
            p64 = np.einsum("ki,nij,lj->nkl", d64, b, d64)
            err = np.abs(got["pdqf"][live, 0].astype(np.float64) - p64).max(axis=(1, 2))
            scale = np.abs(p64).max(axis=(1, 2))
            v["max_abs_coef_err"] = float(err.max())
            v["max_rel_coef_err"] = float((err / np.maximum(scale, 1e-30)).max())
            v["bit_disagreement_vs_fp32"] = float(
                np.unpackbits(got["hashes"][live] ^ ref["hashes"][live]).mean())
            v["quality_max_abs_diff_vs_fp32"] = float(
                np.abs(got["quality"][live] - ref["quality"][live]).max())
            out["variants"].append(v)
        d_img.free()
    return out


def join_ranks(args):
    """(rank, world, local rank, process group or None); the world must be --gpus."""
    rank, world, local = dist_info()
    if world != args.gpus:
        raise SystemExit("bench.py: %d ranks running for --gpus %d" % (world, args.gpus))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return rank, world, local, pg


def run_ours(args):
    import __graft_entry__ as g
    yp = g.load_package()
    rank, world, local, pg = join_ranks(args)
    ctx = yp.Context(local)
    batch, d_img, rows, d_rows, d_hash, d_q = setup_workload(yp, ctx, args, rank)
    n, B = args.db_rows, args.batch
    nq = 8 * B
    cap = 1 << 22
    d_hits = ctx.alloc(cap * 16)
    d_cnt = ctx.alloc(8)
    stream = ctx.stream()
    ev = [ctx.event() for _ in range(3)]

    def step(record=False):
        if record:
            ctx.record(ev[0], stream)
        yp.core.hash_batch_device(ctx, d_img, B, yp._lib.INPUT_F32, d_hash, d_q, dct=args.dct,
                                  stream=stream)
        if record:
            ctx.record(ev[1], stream)
        yp.core.scan_device(ctx, d_rows, n, d_hash, nq, args.threshold, d_hits, cap, d_cnt,
                            args.algo, stream)
        if record:
            ctx.record(ev[2], stream)

    for _ in range(args.warmup):
        step()
    ctx.sync(stream)
    hits_per_step = int(d_cnt.download((1,), np.uint64)[0])

    # device-resident timed region
    t_start, t_end = ctx.event(), ctx.event()
    hash_ms, scan_ms = [], []
    if pg:
        pg.barrier()
    ctx.sync(stream)
    clocks = ClockSampler(local)
    clocks.start()
    ctx.record(t_start, stream)
    for _ in range(args.steps):
        step(record=True)
        ctx.sync(stream)
        hash_ms.append(ctx.elapsed_ms(ev[0], ev[1]))
        scan_ms.append(ctx.elapsed_ms(ev[1], ev[2]))
    ctx.record(t_end, stream)
    ctx.sync(stream)
    total_ms = ctx.elapsed_ms(t_start, t_end)
    clk = clocks.stop()
    total_ms, value = aggregate_over_ranks(pg, total_ms, world, B * args.steps)
    ms_per_step = total_ms / args.steps
    # the last timed step's hits in the scalar matcher's order, for the parity check
    step_hits = int(d_cnt.download((1,), np.uint64)[0])
    yp.core.sort_hits_device(ctx, d_hits, min(step_hits, cap), stream)
    ctx.sync(stream)
    gpu_step_hits = d_hits.download((min(step_hits, cap),), yp.HIT_DTYPE)

    # end to end through the public C ABI from pinned host memory
    db = yp.Database(ctx, device_buffer=d_rows, n_rows=n)
    import ctypes
    h_img = ctypes.c_void_p()
    yp._lib.check(ctx.lib.ypdq_malloc_host(ctx.handle, batch.nbytes, ctypes.byref(h_img)))
    ctypes.memmove(h_img, batch.ctypes.data, batch.nbytes)
    h_hits = np.zeros(max(hits_per_step, 1) * 2, yp.HIT_DTYPE)
    nh = ctypes.c_uint64()

    def e2e_step():
        yp._lib.check(ctx.lib.ypdq_screen_host(
            ctx.handle, db.handle, h_img, B, yp._lib.INPUT_F32, args.dct, 0, args.threshold,
            h_hits.ctypes.data_as(ctypes.c_void_p), len(h_hits), ctypes.byref(nh), None, None))

    for _ in range(max(1, args.warmup)):
        e2e_step()
    lat = []
    if pg:
        pg.barrier()
    import gc
    gc.collect()
    gc.disable()  # the calling loop runs with Python's collector paused
    t0 = time.perf_counter()
    try:
        for _ in range(args.steps):
            s = time.perf_counter()
            e2e_step()
            lat.append(time.perf_counter() - s)
    finally:
        gc.enable()
    # like the device-resident value: all ranks' images over the slowest rank's time
    _, e2e_value = aggregate_over_ranks(pg, (time.perf_counter() - t0) * 1e3, world,
                                        B * args.steps)
    e2e_hits = h_hits[:min(nh.value, len(h_hits))].copy()
    ctx.lib.ypdq_free_host(ctx.handle, h_img)
    stream_e2e = e2e_stream(yp, ctx, db, batch, args, pg, world, hits_per_step)
    link = host_link(batch.nbytes, B) if rank == 0 else None
    # the serving sweep, the heavy-hit database and the precision variants describe one GPU:
    # rank 0 runs them (the other replicas wait at the final barrier)
    serve = serving(yp, ctx, db, batch, args) if rank == 0 else None
    large = large_db(yp, ctx, args) if rank == 0 else None
    sweep = scan_sweep(yp, ctx, d_rows, n, d_hash, args) if args.scan_sweep and rank == 0 else None
    dctv = dct_variants(yp, ctx, args) if args.dct_variants and rank == 0 else None

    hbm_peak, bf16_peak, peak_kind = measured_peaks()
    hash_avg = statistics.mean(hash_ms)
    scan_avg = statistics.mean(scan_ms)
    algo = scan_algo_used(args.algo, nq, args.threshold)
    # the tensor-core form launch_scan_tc takes (mirrors it): at t <= 36 FP4 row triples up
    # to 512 queries (launches of 128), FP4 query triples past that (passes of 720), or with
    # YPDQ_SCAN_TC_FP8 FP8 query pairs past 256 (passes of 512) and single queries below;
    # above t = 36 single queries (passes of 256)
    low_t = args.threshold <= 36
    if low_t and args.algo != 5:
        form = "rows3" if nq <= 512 else "triples"
    elif low_t:
        form = "pairs" if nq > 256 else "single"
    else:
        form = "single"
    rows3_launches = (nq + 127) // 128
    scan_launches = ((rows3_launches if form == "rows3" else 1) if algo in (3, 4, 5)
                     else (nq + 2047) // 2048)
    if scan_avg >= hash_avg and algo in (3, 4, 5):
        # tensor-core scan, one launch per step: FP8 flops the MMAs execute per (row, query)
        # pair, 2 * K: K = 128 at t <= 36 and 192 for passes of 256 queries at t <= 62 (the
        # prefix bound; mirrors launch_scan_tc), else 256. Peak: the dense FP8 burst measured
        # on this GPU in this run (else twice the measured bf16 burst, the nominal ratio).
        k_bits = (128 if args.threshold <= 36 else
                  192 if (nq > 128 and args.threshold <= 62) else 256)
        flops = 2.0 * k_bits * nq * n
        achieved = flops / (scan_avg / 1000.0) / 1e12
        triples = form in ("triples", "rows3")  # the FP4 forms
        pairs = form != "single"  # several queries (or rows) per accumulator column
        per_pass = {"triples": 720, "rows3": 128, "pairs": 512}.get(form, 256)
        passes = (nq + per_pass - 1) // per_pass
        if triples:
            fp4 = fp4_dense_burst(local) if rank == 0 else None
            peak = fp4 if fp4 else 2 * fp8_dense_burst(local)
            peak_source = ("measured fp4 burst (torch._scaled_mm, e2m1 with e4m3 scales per 16, "
                           "8192^3, best of 10, this GPU, this run)" if fp4 else
                           "measured fp8 burst x 2 (fp4 dense)")
            kernel = ("scan_pair_kernel<2> (tcgen05 kind::mxf4 block-scaled e2m1, three queries "
                      "per f32 accumulator column)" if form == "triples" else
                      "scan_rows3_kernel (tcgen05 kind::mxf4 block-scaled e2m1, queries as A, "
                      "three database rows per f32 accumulator column)")
        else:
            fp8 = fp8_dense_burst(local) if rank == 0 else None
            peak = fp8 if fp8 else 2 * bf16_peak
            peak_source = ("measured fp8 burst (torch._scaled_mm e4m3 8192^3, best of 10, this "
                           "GPU, this run)" if fp8 else "%s bf16 burst x 2 (fp8 dense)" % peak_kind)
            kernel = ("scan_pair_kernel<0> (tcgen05 kind::f8f6f4, e5m2, two queries per f32 "
                      "accumulator column)" if pairs else "scan_tc_kernel (tcgen05 kind::f8f6f4)")
        if form == "rows3":
            # launches of <= 128 queries stream the database once each: HBM-bound
            launch_ms = scan_avg / scan_launches
            achieved_gbs = (n * 32 + hits_per_step * 16.0 / scan_launches) / (launch_ms / 1e3) / 1e9
            roofline_hbm = {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak,
                            "unit": "GB/s", "frac": achieved_gbs / hbm_peak,
                            "peak_source": peak_kind}
        roofline = {"bound": "tensor",
                    "kernel": kernel,
                    "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak,
                    "peak_source": peak_source,
                    "traffic": (passes * NCU_DRAM_BYTES_PER_PASS_10M * (n / 1e7)
                                + hits_per_step * 16.0 if pairs else None),
                    "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of a "
                                       "4-pass launch over 10M rows (1.283 GB) per pass, scaled "
                                       "by this launch's passes and rows" if pairs else None),
                    "traffic_computed": passes * 32.0 * n + hits_per_step * 16.0,
                    "traffic_note": "traffic_computed = 32 B x rows x %d query passes of %d + 16 B "
                                    "per hit (the database streams once per pass), computed, not "
                                    "a counter" % (passes, per_pass),
                    "mma_flop_note": "2 x %d FLOP per (row, query) pair: the K the MMAs execute "
                                     "per query" % k_bits,
                    "launch_ms": scan_avg / scan_launches, "launches_per_step": scan_launches,
                    "mma_k_bits": k_bits,
                    "pairs_per_s": nq * n / (scan_avg / 1e3),
                    "db_stream_gbs": (n * 32 * passes) / (scan_avg / 1e3) / 1e9,
                    "query_passes": passes}
        if form == "rows3":
            roofline.update(roofline_hbm)
            roofline["mma_flop_note"] += " (the launch is bound by its database stream)"
    elif scan_avg >= hash_avg:
        # SIMT scan: one launch reads the whole database once for up to 2048 queries
        dom_ms = scan_avg / scan_launches
        alg_bytes = n * 32 + (hits_per_step / scan_launches) * 16
        achieved = alg_bytes / (dom_ms / 1000.0) / 1e9
        roofline = {"bound": "hbm", "kernel": "scan_simt_kernel", "achieved": achieved,
                    "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                    "traffic": None, "peak_source": peak_kind, "launch_ms": dom_ms,
                    "launches_per_step": scan_launches}
    else:
        # hash kernel: reads every image once, writes 8 hashes + 8 qualities per image
        alg_bytes = B * (512 * 512 * 4) + B * (8 * 32 + 8 * 4)
        achieved = alg_bytes / (hash_avg / 1000.0) / 1e9
        roofline = {"bound": "hbm", "kernel": "hash_kernel<float>", "achieved": achieved,
                    "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                    "traffic": None, "peak_source": peak_kind, "launch_ms": hash_avg,
                    "launches_per_step": 1}
    hash_gbs = (B * (512 * 512 * 4 + 288)) / (hash_avg / 1000.0) / 1e9
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {0: "f32", 1: "f32 (DCT stage 1 tf32)", 2: "f32 (DCT stage 1 bf16x3)"}[args.dct],
        "data": "synthetic (seeded blob images; 10M rows of exactly 128 set bits + planted near-duplicates)",
        "config": {"workload": "screen %d f32 images x 8 dihedrals vs %d-row DB at t=%d" % (B, n, args.threshold),
                   "images_per_step": B, "queries_per_step": nq, "db_rows": n,
                   "threshold": args.threshold, "hits_per_step": hits_per_step,
                   "l2": "inputs larger than L2 (images %d MiB, DB %d MiB > 129 MB L2)"
                         % (B * 4 * 512 * 512 >> 20, n * 32 >> 20),
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "scan_algo": ({1: "simt", 2: "b1mma"}.get(algo) or
                                 {"triples": "tcgen05 fp4 triples",
                                  "rows3": "tcgen05 fp4 row triples"}.get(form, "tcgen05 fp8"))},
        "kernels_ms": {"hash": hash_avg, "scan": scan_avg},
        "latency_ms": ({"p50": serve["points"][0]["p50_ms"], "p99": serve["points"][0]["p99_ms"],
                        "at": "serving loop, %g req/s Poisson" % serve["points"][0]["offered_req_s"]}
                       if serve else None),
        "batch_latency_ms": {"p50": 1000 * statistics.median(lat),
                             "p99": 1000 * float(np.percentile(lat, 99)),
                             "all": [round(1000 * x, 3) for x in lat],
                             "at": "ypdq_screen_host of %d images" % B},
        "serving": serve,
        "scan_sweep": sweep,
        "large_db": large,
        "dct_variants": dctv,
        "e2e": {"value": stream_e2e["value"], "unit": UNIT,
                "h2d_bytes_per_step": B * 512 * 512 * 4,
                "d2h_bytes_per_step": hits_per_step * 16 + 8,
                "path": "ypdq_server_* (the C ABI's serving loop, 3 slots): %d requests of %d "
                        "pinned host f32 images each, hits back to host memory; the copies of "
                        "one step overlap the hash and scan of another" % (args.steps, B),
                "ms_per_step": stream_e2e["ms_per_step"],
                "request_latency_ms": stream_e2e["latency_ms"],
                "frac_of_host_link": (stream_e2e["value"] / link["images_per_s_ceiling"]
                                      if link else None)},
        "host_link": link,
        "e2e_blocking": {"value": e2e_value, "unit": UNIT,
                         "path": "one blocking ypdq_screen_host call per batch of %d pinned "
                                 "host images (copies and compute overlap inside the call "
                                 "only)" % B},
        "roofline": roofline,
        "hash_kernel": {"ms": hash_avg, "GB/s": hash_gbs, "frac_hbm": hash_gbs / hbm_peak},
        "gpu_launches": args.steps * (1 + scan_launches),
        "clocks": clk,
    }
    if rank == 0:
        out["cpu_baseline"] = cpu_baseline(args, args.cpu_sample,
                                           workload=(batch[:args.cpu_sample], rows))
        out["parity"] = parity_check(args, batch, rows, gpu_step_hits, step_hits, e2e_hits,
                                     stream_e2e["hits"])
        print(json.dumps(out))
    if pg:
        pg.barrier()
    ctx.close()


def cpu_workload(args, sample):
    """Images and database of the CPU arm: the GPU arm's generators and its planted rows.
    The rows come from the CPU twin of ypdq_synth_rows; the step's args.batch images are
    hashed by the oracle (bit-identical to the GPU's hashes) and args.planted rows become
    copies of those hashes (synth.plant_near_duplicates, the GPU arm's edit). Returns the
    first `sample` images and the rows."""
    import oracle  # noqa: the oracle, timed here as yume-pdq's CPU path
    import __graft_entry__ as g
    yp = g.load_package()
    imgs = yp.synth.blob_images(args.batch, seed=args.seed)
    rows = oracle.synth_rows(args.db_rows, args.seed, nthreads=os.cpu_count() or 1)
    hashes, _, _, _ = oracle.hash_batch(imgs)
    yp.synth.plant_near_duplicates(rows, hashes, args.planted, args.seed + 99)
    return imgs[:sample], rows


def host_link(nbytes, images, reps=5):
    """The host link's H2D rate: copies of nbytes from pinned host memory to the device by the
    copy engine (torch, CUDA events on the copy's stream, median of reps after one warm copy),
    and the images/s a stream of nbytes-sized batches could not exceed."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    ms = []
    with torch.cuda.stream(s):
        for rep in range(reps + 1):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            d.copy_(h, non_blocking=True)
            e1.record(s)
            e1.synchronize()
            if rep:
                ms.append(e0.elapsed_time(e1))
    t = statistics.median(ms)
    del h, d
    return {"bytes": nbytes, "ms": t, "h2d_GB_s": nbytes / (t / 1e3) / 1e9,
            "images_per_s_ceiling": images / (t / 1e3),
            "how": "torch copy of pinned host memory to the device, CUDA events, median of %d"
                   % reps}


def e2e_stream(yp, ctx, db, batch, args, pg, world, hits_per_step):
    """The same metric for a stream of batches through the serving loop (ypdq_server_*):
    --steps requests of the step's B pinned host images each, hashed and matched exactly at
    the bench threshold. Every request's 1 GiB image copy and its hit list's copy back are
    inside the timed region; the server overlaps one step's copies with another step's
    hash and scan (3 slots), which one blocking ypdq_screen_host call per batch cannot do.
    Returns images/s (all ranks' images over the slowest rank's time), the request
    latencies and the last request's hits (sorted, query numbers local to the request)."""
    B = batch.shape[0]
    pin = yp.PinnedArray(ctx, batch.shape, np.float32)
    pin.array[:] = batch
    cap = max(hits_per_step, 1) * 2
    srv = yp.Server(ctx, db, threshold=args.threshold, dct=args.dct, max_step_images=B,
                    slots=3, max_queued_images=3 * B)

    def run(k):
        done, sent = [], 0
        while sent < k:
            if srv.try_submit(pin.array, hit_capacity=cap) is not None:
                sent += 1
            else:
                done.extend(srv.poll(timeout_us=-1))
        done.extend(srv.drain())
        return done

    run(max(1, args.warmup))
    if pg:
        pg.barrier()
    # the submitting loop runs with Python's collector paused, as the serving sweep's does
    import gc
    gc.collect()
    gc.disable()
    t0 = time.perf_counter()
    try:
        res = run(args.steps)
    finally:
        gc.enable()
    wall_ms = (time.perf_counter() - t0) * 1e3
    _, value = aggregate_over_ranks(pg, wall_ms, world, B * args.steps)
    assert all(r.ok for r in res) and len(res) == args.steps
    last = max(res, key=lambda r: r.request_id)
    lat = sorted(r.latency_us / 1e3 for r in res)
    srv.close()
    pin.free()
    return {"value": value, "ms_per_step": wall_ms / args.steps,
            "latency_ms": {"p50": statistics.median(lat), "max": lat[-1]},
            "hits": last.hits.copy()}


def parity_check(args, imgs, rows, gpu_hits, gpu_count, e2e_hits, stream_hits=None):
    """The timed step against the oracle, once, after the timed regions: the oracle hashes
    the step's images (its f32 pipeline) and its scalar matcher lists every hit of the 8B
    hashes in the same planted rows. Equal when the GPU step's sorted hit list and the last
    ypdq_screen_host call's are both that list."""
    import oracle
    import __graft_entry__ as g
    yp = g.load_package()
    t0 = time.perf_counter()
    hashes, _, _, _ = oracle.hash_batch(imgs)
    want = oracle.find_all(rows, hashes.reshape(-1, 32), args.threshold)

    def same(h):
        return (len(h) == len(want) and all(np.array_equal(h[f], want[f])
                                            for f in ("index", "query", "distance")))
    out = {"gpu_hits": int(gpu_count), "oracle_hits": int(len(want)),
           "equal": bool(gpu_count == len(want) and same(gpu_hits)),
           "e2e_equal": bool(same(e2e_hits)),
           "oracle_s": round(time.perf_counter() - t0, 2),
           "what": "sorted (index, query, distance) lists of the timed step, of the last "
                   "ypdq_screen_host call and of the last streamed request vs the oracle's "
                   "scalar matcher over all %d x %d pairs of the same planted rows"
                   % (8 * len(imgs), rows.shape[0])}
    if stream_hits is not None:
        out["e2e_stream_equal"] = bool(same(stream_hits))
    return out


def cpu_time(args, imgs, rows):
    """yume-pdq's CPU path (scalar kernel + scalar matcher, restated in C) on all host
    cores: hash the images with their dihedrals, scan all 8n hashes against the rows."""
    import oracle
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    h, q, t, _ = oracle.hash_batch(imgs, nthreads=cores)
    t1 = time.perf_counter()
    oracle.count_all(rows, h.reshape(-1, 32), args.threshold, nthreads=cores)
    t2 = time.perf_counter()
    return t2 - t0, t1 - t0, t2 - t1


# The reference's own single-core figures (README.md:184-216, Zen 4 at 5.1 GHz): the scalar
# matcher scans 478M database rows/s against 8 needles at once, and the scalar
# auto-vectorized pipeline hashes 1,600 frames/s.
REF_ROWS_PER_S_8_NEEDLES = 478e6
REF_HASH_FPS = 1600.0


def published_rate_estimate(n_images, db_rows, cores):
    """images/s of yume-pdq's CPU path if every host core ran at the reference's published
    single-core rates: an optimistic upper bound, reported beside the measured port."""
    scan_s = n_images * db_rows / (REF_ROWS_PER_S_8_NEEDLES * cores)
    hash_s = n_images / (REF_HASH_FPS * cores)
    return n_images / (scan_s + hash_s)


def host_cpu():
    """'<vendor> <model name>' of this host's CPU from lscpu (None if unavailable)."""
    try:
        info = dict(line.split(":", 1) for line in subprocess.run(
            ["lscpu"], capture_output=True, text=True, timeout=10).stdout.splitlines()
            if ":" in line)
        return " ".join(info[k].strip() for k in ("Vendor ID", "Model name") if k in info) or None
    except (OSError, subprocess.SubprocessError, ValueError):
        return None


def cpu_baseline(args, sample, workload=None, reps=1):
    imgs, rows = workload or cpu_workload(args, sample)
    cores = os.cpu_count() or 1
    times = [cpu_time(args, imgs, rows) for _ in range(reps)]
    tot, th, ts = min(times)
    return {"value": len(imgs) / tot, "unit": UNIT, "cores": cores, "kind": "port",
            "cpu": host_cpu(),
            "sample": "%d images hashed (+7 dihedrals each) and %d hashes scanned vs %d rows "
                      "(the planted database of the GPU step) at t=%d; hash %.3f s, scan %.3f s"
                      % (len(imgs), 8 * len(imgs), args.db_rows, args.threshold, th, ts),
            "published_rate_upper_bound": {
                "value": published_rate_estimate(len(imgs), args.db_rows, cores), "unit": UNIT,
                "basis": "reference README single-core rates (478M rows/s x 8 needles scalar "
                         "matcher, 1,600 frames/s hashing, Zen 4 5.1 GHz) times %d cores" % cores}}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    work = cpu_workload(args, args.cpu_sample)
    for _ in range(args.warmup):
        cpu_time(args, *work)
    vals = []
    base = None
    for _ in range(max(1, args.steps)):
        base = cpu_baseline(args, args.cpu_sample, workload=work)
        vals.append(base["value"])
    v = statistics.median(vals)
    base["value"] = v
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "config": {"workload": "screen %d f32 images x 8 dihedrals vs %d-row DB at t=%d per step"
                               % (args.cpu_sample, args.db_rows, args.threshold)},
        "cpu_baseline": base,
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def kernel_mode(args):
    """One kernel configuration timed with CUDA events, one line per repetition (the first
    includes first-launch costs). Hash: 64 distinct seeded images repeated to --images;
    scan: --queries random 128-bit hashes against ypdq_synth_rows(seed 1)."""
    import ctypes
    import __graft_entry__ as g
    yp = g.load_package()
    ctx = yp.Context(0)
    stream = ctx.stream()
    e0, e1 = ctx.event(), ctx.event()
    if args.kernel == "hash":
        kind = {"f32": yp._lib.INPUT_F32, "u8": yp._lib.INPUT_U8, "rgb8": yp._lib.INPUT_RGB8,
                "rgba8": yp._lib.INPUT_RGBA8}[args.input]
        if kind in (yp._lib.INPUT_RGB8, yp._lib.INPUT_RGBA8):
            ch = 3 if kind == yp._lib.INPUT_RGB8 else 4
            base = np.concatenate([yp.synth.color_images(16, seed=3, channels=ch)] * 4)
        else:
            base = yp.synth.blob_images(64, seed=3)
            if kind == yp._lib.INPUT_U8:
                base = yp.synth.to_u8(base)
        d_img = ctx.to_device(np.concatenate([base] * ((args.images + 63) // 64))[: args.images])
        d_h, d_q = ctx.alloc(args.images * 256), ctx.alloc(args.images * 32)
        prec = 0x200 if args.jarosz else args.dct | (0x100 if args.separable else 0)
        if not args.jarosz:
            c = ctypes.c_int()
            yp._lib.check(ctx.lib.ypdq_hash_occupancy(ctx.handle, kind, prec, ctypes.byref(c)))
            print("hash_kernel input %s dct %d separable %d: %d CTAs per SM"
                  % (args.input, args.dct, args.separable, c.value))
        for _ in range(args.reps):
            ctx.record(e0, stream)
            yp.core.hash_batch_device(ctx, d_img, args.images, kind, d_h, d_q, dct=prec,
                                      stream=stream)
            ctx.record(e1, stream)
            ctx.sync(stream)
            ms = ctx.elapsed_ms(e0, e1)
            print("images %d ms %.4f Mimg/s %.3f" % (args.images, ms, args.images / ms / 1e3),
                  flush=True)
    else:
        n = args.db_rows
        d_rows = ctx.alloc(n * 32)
        yp._lib.check(ctx.lib.ypdq_synth_rows(ctx.handle, d_rows.ptr, n, 0, 1, None))
        d_q = ctx.to_device(yp.synth.rows_128(args.queries, seed=5))
        cap = 1 << 20
        d_hits, d_cnt = ctx.alloc(cap * 16), ctx.alloc(8)
        for _ in range(args.reps):
            ctx.record(e0, stream)
            yp.core.scan_device(ctx, d_rows, n, d_q, args.queries, args.threshold, d_hits, cap,
                                d_cnt, args.algo, stream)
            ctx.record(e1, stream)
            ctx.sync(stream)
            ms = ctx.elapsed_ms(e0, e1)
            print("rows %d queries %d ms %.4f Gpairs/s %.1f DB GB/s %.1f"
                  % (n, args.queries, ms, n * args.queries / ms / 1e6, n * 32 / ms / 1e6),
                  flush=True)
    ctx.close()


def main():
    args = parse()
    if args.kernel:
        kernel_mode(args)
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    if args.peaks:
        print(json.dumps({"fp8_e4m3_dense_tflops": fp8_dense_burst(),
                          "fp4_dense_tflops": fp4_dense_burst(),
                          "how": "torch._scaled_mm 8192^3 (e4m3 with unit per-tensor scales; "
                                 "e2m1 with unit e4m3 scales per 16 elements), bf16 out, best "
                                 "of 10, CUDA events"}))
        return
    if args.impl == "ours" and args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_replicas(sys.argv[1:], args.gpus))
    if args.ranks_only:
        rank, world, local, pg = join_ranks(args)
        t, v = aggregate_over_ranks(pg, float(rank + 1), world, 1)
        print(json.dumps({"rank": rank, "world": world, "local_rank": local, "max_ms": t}))
        if pg:
            pg.destroy_process_group()
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
