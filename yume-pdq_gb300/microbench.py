"""Time one kernel configuration of the library with CUDA events (a tuning aid).

    python yume-pdq_gb300/microbench.py hash --input u8 --dct 2 --images 4096
    python yume-pdq_gb300/microbench.py hash --input u8 --jarosz --images 2048
    python yume-pdq_gb300/microbench.py scan --rows 10000000 --queries 2048 --algo 3

`hash` times ypdq_hash_batch on device-resident seeded blob images (64 distinct images
repeated); `scan` times ypdq_scan of random 128-bit queries against generated rows. Each
prints one line per repetition; the first repetition includes first-launch costs.
"""
import argparse
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main(argv=None):
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="what", required=True)
    h = sub.add_parser("hash")
    h.add_argument("--input", choices=["f32", "u8", "rgb8", "rgba8"], default="f32")
    h.add_argument("--dct", type=int, choices=[0, 1, 2], default=0)
    h.add_argument("--images", type=int, default=4096)
    h.add_argument("--separable", action="store_true",
                   help="YPDQ_COMPRESS_SEPARABLE (not bit-exact with the reference)")
    h.add_argument("--jarosz", action="store_true",
                   help="YPDQ_COMPRESS_JAROSZ (ReferenceKernel<f32>; --dct is ignored)")
    s = sub.add_parser("scan")
    s.add_argument("--rows", type=int, default=10_000_000)
    s.add_argument("--queries", type=int, default=64)
    s.add_argument("--algo", type=int, default=3)
    s.add_argument("--threshold", type=int, default=31)
    for p in (h, s):
        p.add_argument("--reps", type=int, default=5)
    a = ap.parse_args(argv)

    import __graft_entry__ as g
    yp = g.load_package()
    ctx = yp.Context(0)
    stream = ctx.stream()
    e0, e1 = ctx.event(), ctx.event()
    if a.what == "hash":
        kind = {"f32": yp._lib.INPUT_F32, "u8": yp._lib.INPUT_U8, "rgb8": yp._lib.INPUT_RGB8,
                "rgba8": yp._lib.INPUT_RGBA8}[a.input]
        if kind in (yp._lib.INPUT_RGB8, yp._lib.INPUT_RGBA8):
            base = yp.synth.color_images(16, seed=3, channels=3 if kind == yp._lib.INPUT_RGB8 else 4)
            base = np.concatenate([base] * 4)
        else:
            base = yp.synth.blob_images(64, seed=3)
            if kind == yp._lib.INPUT_U8:
                base = yp.synth.to_u8(base)
        reps = (a.images + 63) // 64
        d_img = ctx.to_device(np.concatenate([base] * reps)[: a.images])
        d_h, d_q = ctx.alloc(a.images * 256), ctx.alloc(a.images * 32)
        prec = a.dct | (0x100 if a.separable else 0)
        if a.jarosz:
            prec = 0x200
            print("jarosz input %s" % a.input)
        else:
            c = ctypes.c_int()
            yp._lib.check(ctx.lib.ypdq_hash_occupancy(ctx.handle, kind, prec, ctypes.byref(c)))
            print("hash_kernel input %s dct %d separable %d: %d CTAs per SM"
                  % (a.input, a.dct, a.separable, c.value))
        for _ in range(a.reps):
            ctx.record(e0, stream)
            yp.core.hash_batch_device(ctx, d_img, a.images, kind, d_h, d_q, dct=prec,
                                      stream=stream)
            ctx.record(e1, stream)
            ctx.sync(stream)
            ms = ctx.elapsed_ms(e0, e1)
            print("images %d ms %.4f Mimg/s %.3f" % (a.images, ms, a.images / ms / 1e3),
                  flush=True)
    else:
        d_rows = ctx.alloc(a.rows * 32)
        yp._lib.check(ctx.lib.ypdq_synth_rows(ctx.handle, d_rows.ptr, a.rows, 0, 1, None))
        d_q = ctx.to_device(yp.synth.rows_128(a.queries, seed=5))
        cap = 1 << 20
        d_hits, d_cnt = ctx.alloc(cap * 16), ctx.alloc(8)
        for _ in range(a.reps):
            ctx.record(e0, stream)
            yp.core.scan_device(ctx, d_rows, a.rows, d_q, a.queries, a.threshold, d_hits, cap,
                                d_cnt, a.algo, stream)
            ctx.record(e1, stream)
            ctx.sync(stream)
            ms = ctx.elapsed_ms(e0, e1)
            print("rows %d queries %d ms %.4f Gpairs/s %.1f DB GB/s %.1f"
                  % (a.rows, a.queries, ms, a.rows * a.queries / ms / 1e6,
                     a.rows * 32 / ms / 1e6), flush=True)
    ctx.close()


if __name__ == "__main__":
    main()
