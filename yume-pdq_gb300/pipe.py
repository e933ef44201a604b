"""Raw-frame stream front-end: yume-pdq's `pipe` command (src/main.rs:391-836, 1091-1304)
over the GPU library.

    python yume-pdq_gb300/pipe.py -i frames.raw --input-format rgb8 -f q+hex+lf --dihedrals
    python yume-pdq_gb300/pipe.py -i - -f hex+lf --db hashes.bin --threshold 31

Input: consecutive 512x512 frames of luma8 (1 byte per pixel), rgb8 (3) or rgba8 (4), read
whole (a partial frame at the end of the stream is an error, as in the reference). Output,
per frame, the hash and with --dihedrals the 7 derived hashes in visit order, each in the
reference's formats (src/main.rs:683-773):
  raw / Raw / RAW      the 32 hash bytes
  q+raw                f32 quality (little-endian) then the 32 bytes
  hex / HEX            64 hex digits, lower / upper case
  bin / BIN            256 '0'/'1' characters, byte by byte, most significant bit first
  q+hex, q+HEX, q+bin  prefixed with the quality x 100 as "{:02.3}" and ':'
  diagnostic           per hash: its dihedral, its index in the frame, quality, threshold,
                       the 256 bits and the 16 x 16 PDQF with '*' on coefficients above the
                       threshold (src/main.rs:738-773)
  ...+lf / +crlf / +cr / +nul / +nl   a separator after every hash
With --db the frames go through the continuous-batching server (ypdq_server_*), which also
matches all 8 hashes of each frame against the database; after a frame's hashes one line
per hit follows in text formats: "match <slot> <row index> <distance>" (not in the reference).
--reference-kernel hashes with ReferenceKernel<f32> (not in the reference's CLI, which always
uses its default kernel).
"""
import argparse
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

FRAME_PIXELS = 512 * 512
BYTES_PER_PIXEL = {"luma8": 1, "rgb8": 3, "rgba8": 4}
SEPARATORS = {"nl": b"\n", "lf": b"\n", "crlf": b"\r\n", "cr": b"\r", "nul": b"\0", "null": b"\0"}
FORMATS = {  # name -> (kind, upper, quality prefix)
    "raw": ("raw", False, False), "Raw": ("raw", False, False), "RAW": ("raw", False, False),
    "q+raw": ("raw", False, True), "q+Raw": ("raw", False, True), "q+RAW": ("raw", False, True),
    "hex": ("hex", False, False), "HEX": ("hex", True, False),
    "bin": ("bin", False, False), "BIN": ("bin", False, False),
    "q+hex": ("hex", False, True), "q+HEX": ("hex", True, True),
    "q+bin": ("bin", False, True), "q+BIN": ("bin", False, True),
    "diagnostic": ("diagnostic", False, False),
}
# The diagnostic header of each slot: the reference prints `{:?}` of its name, "original"
# for the hash itself and the Dihedrals value (a u32 of four big-endian i8 matrix entries,
# src/lib.rs:85-134) for each derived hash, in visit order (src/lib.rs:358-420).
DIHEDRAL_PACKED = (None, 0xFF000001, 0xFF0000FF, 0x010000FF, 0x00FFFF00, 0x00010100, 0x00FF0100,
                   0x0001FF00)


def slot_name(slot):
    return '"original"' if slot == 0 else "Dihedrals { packed: %d }" % DIHEDRAL_PACKED[slot]


def parse_format(spec):
    """(kind, upper, quality prefix, separator bytes) of a --format value such as q+hex+lf."""
    parts = spec.split("+")
    sep = b""
    if len(parts) > 1 and parts[-1].lower() in SEPARATORS:
        sep = SEPARATORS[parts[-1].lower()]
        spec = "+".join(parts[:-1])
    if spec not in FORMATS:
        raise ValueError("invalid output format %r" % spec)
    kind, upper, quality = FORMATS[spec]
    return kind, upper, quality, sep


def quality_prefix(quality):
    """The reference's "{0:02.3}:" of quality * 100 (the product taken in f32; qualities are
    in [0, 1], so the width of 2 never pads)."""
    q100 = float(np.float32(quality) * np.float32(100.0))
    return ("%.3f" % q100).encode() + b":"


def format_hash(hash32, quality, kind, upper, with_quality, sep):
    """One hash (32 bytes) in the reference's output format."""
    h = bytes(hash32)
    if kind == "raw":
        out = (struct.pack("<f", float(quality)) if with_quality else b"") + h
    else:
        pre = quality_prefix(quality) if with_quality else b""
        if kind == "hex":
            body = h.hex().upper() if upper else h.hex()
            out = pre + body.encode()
        else:
            out = pre + "".join(format(b, "08b") for b in h).encode()
    return out + sep


def format_diagnostic(slot, index, hash32, quality, threshold, pdqf, sep):
    """One hash in the reference's diagnostic format: `[name]`, `Index: i` (the hash's position
    among the frame's outputs), `Quality: {0:02.3}` of quality x 100, `Threshold: {0:.7}`,
    `Hash:` and its 256 bits on one line, `PDQF:` and 16 rows of 16 tab-separated `{:.5}`
    values, each prefixed by '*' when it exceeds the threshold (all f32)."""
    t = np.float32(threshold)
    q100 = float(np.float32(quality) * np.float32(100.0))
    bits = "".join(format(b, "08b") for b in bytes(hash32))
    rows = []
    for row in np.asarray(pdqf, np.float32).reshape(16, 16):
        rows.append("\t".join(("*" if v > t else "") + "%.5f" % float(v) for v in row))
    text = ("[%s]\nIndex: %d\nQuality: %.3f\nThreshold: %.7f\nHash:\n%s\nPDQF:\n%s\n"
            % (slot_name(slot), index, q100, float(t), bits, "\n".join(rows)))
    return text.encode() + sep


def read_frames(stream, bpp, max_frames):
    """Up to max_frames whole frames from a binary stream as a uint8 array, or None at EOF."""
    frame = FRAME_PIXELS * bpp
    want = frame * max_frames
    buf = bytearray()
    while len(buf) < want:
        chunk = stream.read(want - len(buf))
        if not chunk:
            break
        buf += chunk
    if not buf:
        return None
    if len(buf) % frame:
        raise EOFError("unexpected end of stream in the middle of a frame")
    a = np.frombuffer(bytes(buf), np.uint8)
    n = len(buf) // frame
    return a.reshape(n, 512, 512) if bpp == 1 else a.reshape(n, 512, 512, bpp)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("-i", "--input", default="-", help="input file, - for stdin")
    ap.add_argument("-o", "--output", default="-", help="output file, - for stdout")
    ap.add_argument("--input-format", default="luma8", type=str.lower,
                    choices=sorted(BYTES_PER_PIXEL))
    ap.add_argument("-f", "--format", default="bin")
    ap.add_argument("--dihedrals", action="store_true", help="output all 8 hashes per frame")
    ap.add_argument("--semantics", default="host", choices=["host", "exact", "avx2", "scalar"],
                    help="dihedral sign convention (the reference's kernels differ); host: "
                         "the one the reference's smart_kernel uses on this host")
    ap.add_argument("--reference-kernel", action="store_true",
                    help="hash with ReferenceKernel<f32> (full Jarosz filter, "
                         "YPDQ_COMPRESS_JAROSZ) instead of the default kernel (an extension)")
    ap.add_argument("--batch", type=int, default=256, help="frames per GPU launch")
    ap.add_argument("--db", help="database file of 32-byte rows: screen every frame")
    ap.add_argument("--threshold", type=int, default=31)
    a = ap.parse_args(argv)
    kind, upper, with_quality, sep = parse_format(a.format)
    bpp = BYTES_PER_PIXEL[a.input_format]

    sys.path.insert(0, os.path.dirname(HERE))
    import __graft_entry__ as g
    yp = g.load_package()
    ctx = yp.Context(0)
    if a.semantics == "host":
        a.semantics = yp.kernel.host_semantics()
    fin = sys.stdin.buffer if a.input == "-" else open(a.input, "rb")
    fout = sys.stdout.buffer if a.output == "-" else open(a.output, "wb")
    slots = 8 if a.dihedrals else 1
    text = kind != "raw"
    diag = kind == "diagnostic"
    dct = 0x200 if a.reference_kernel else 0  # YPDQ_COMPRESS_JAROSZ or the FP32 default

    def hash_frames(frames):
        return yp.hash_batch(ctx, frames, semantics=a.semantics, dct=dct, want_pdqf=diag,
                             pdqf_slots=8 if diag else 1)

    def emit(hashes, quality, hits_per_frame, extra=None):
        for f in range(hashes.shape[0]):
            for s in range(slots):
                if diag:
                    fout.write(format_diagnostic(s, s, hashes[f, s], quality[f, s],
                                                 extra["thresholds"][f, s], extra["pdqf"][f, s],
                                                 sep))
                    continue
                fout.write(format_hash(hashes[f, s], quality[f, s], kind, upper, with_quality, sep))
            if hits_per_frame is not None and text:
                for h in hits_per_frame[f]:
                    fout.write(b"match %d %d %d\n" % (h["query"] % 8, h["index"], h["distance"]))

    if a.db is None:
        while True:
            frames = read_frames(fin, bpp, a.batch)
            if frames is None:
                break
            out = hash_frames(frames)
            emit(out["hashes"], out["quality"], None, out)
            fout.flush()
    else:
        db = yp.Database.from_file(ctx, a.db)
        in_kind = {1: "u8", 3: "rgb8", 4: "rgba8"}[bpp]
        batch = 1 << max(0, (a.batch - 1).bit_length())
        with yp.Server(ctx, db, threshold=a.threshold, input_kind=in_kind, dct=dct,
                       semantics=a.semantics, max_step_images=batch) as srv:
            pending, done, frames_of = [], {}, {}

            def flush_ready():
                # results in stream order: emit the oldest requests that have completed
                while pending and pending[0] in done:
                    r = done.pop(pending.pop(0))
                    if not r.ok:
                        raise RuntimeError("request %d failed with status %d"
                                           % (r.request_id, r.status))
                    per_frame = [r.hits[(r.hits["query"] >> 3) == f] for f in range(r.n_images)]
                    # the server returns hashes and qualities; the diagnostic format also
                    # needs each slot's threshold and PDQF, from the hash path
                    fr = frames_of.pop(r.request_id)
                    emit(r.hashes, r.quality, per_frame, hash_frames(fr) if diag else None)

            while True:
                frames = read_frames(fin, bpp, batch)
                if frames is None:
                    break
                while True:
                    rid = srv.try_submit(frames, hit_capacity=1 << 20, want_hashes=True)
                    if rid is not None:
                        break
                    done.update((r.request_id, r) for r in srv.poll(timeout_us=1000))
                    flush_ready()
                pending.append(rid)
                frames_of[rid] = frames if diag else None
                done.update((r.request_id, r) for r in srv.poll(timeout_us=0))
                flush_ready()
            done.update((r.request_id, r) for r in srv.drain())
            flush_ready()
        fout.flush()
        db.close()
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
