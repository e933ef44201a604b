#!/usr/bin/env python3
"""Generate ``ypdq_tables.h``: the f32 constant tables compiled into the CUDA library.

This is a build step of the library. Its output is committed because the build
machines have no arbitrary-precision package. The oracle's header (oracle/ypdq_constants.h,
with the f64 matrix too) is generated from the same functions by oracle/gen_constants.py;
the construction itself is checked against the closed form and the README known-answer
vector.

This restates the constant generation in yume-pdq's build script, which runs in
MPFR at 128 bits and rounds once to f32/f64:

* DCT matrix ``D[i-1][j] = sqrt(2/127) * cos(pi / (2*127) * i * (2j + 1))`` for i in 1..=16,
  j in 0..127. The order of operations follows ``d_value`` in build.rs:316-325. The rows are
  written out for ``i = 1..=16`` in build.rs:591-602 (f32) and build.rs:625-637 (f64).
* Tent filter: the 7x7 impulse response of two passes of the 3-wide pdqhash box filter.
  The filter truncates its window at the edges, as ``mean_box::box_one_d_float`` does in
  build.rs:203-261. It is measured at the centre pixel, following
  ``tent_filter_weights`` (build.rs:334-381, asserted 7x7 with offset 3 at build.rs:652).
* Sample offsets ``round(4 * (i + 1))`` from ``lerp(0, 512, i, 127)``
  (build.rs:383-387, build.rs:771-773).

mpmath stands in for MPFR: both round each operation to nearest at a 128-bit mantissa.
Each value is then rounded once, directly from 128 bits to 24 or 53 bits, so no value
is rounded twice.
"""
import os
import sys

import mpmath
from mpmath import mp, mpf

PREC = 128


def round_to_bits(x, bits):
    """Round an mpf once to a ``bits``-bit mantissa (round to nearest even) and return a float."""
    with mpmath.workprec(bits):
        y = +x
    return float(y)


def f32_bits(x):
    import struct
    v = round_to_bits(x, 24)
    return struct.unpack("<I", struct.pack("<f", v))[0], v


def f64_bits(x):
    import struct
    v = round_to_bits(x, 53)
    return struct.unpack("<Q", struct.pack("<d", v))[0], v


def d_value(i, j, n):
    # build.rs:316-325: (two / n).sqrt() * (pi / (two * n) * i * (two * j + one)).cos()
    n1, i1, j1 = mpf(n), mpf(i), mpf(j)
    one = mpf(1)
    two = one + one
    pi = mp.pi
    return mpmath.sqrt(two / n1) * mpmath.cos(pi / (two * n1) * i1 * (two * j1 + one))


def box_one_d(invec, start, outvec, length, stride, full_window):
    """Restates the edge-truncated running box mean of build.rs:203-261."""
    half = (full_window + 2) // 2
    p1 = half - 1
    p2 = full_window - half + 1
    oi_off = p1 * stride
    li_off = p2 * stride
    s = mpf(0)
    cur = mpf(0)
    p1_end = oi_off + start
    for ri in range(start, p1_end, stride):
        s += invec[ri]
        cur += 1
    p2_end = full_window * stride + start
    for ri in range(p1_end, p2_end, stride):
        oi = ri - oi_off
        s += invec[ri]
        cur += 1
        outvec[oi] = s / cur
    p3_end = length * stride + start
    for ri in range(p2_end, p3_end, stride):
        oi = ri - oi_off
        li = oi - li_off
        s += invec[ri]
        s -= invec[li]
        outvec[oi] = s / cur
    p4_start = (length - half + 1) * stride + start
    for oi in range(p4_start, p3_end, stride):
        li = oi - li_off
        s -= invec[li]
        cur -= 1
        outvec[oi] = s / cur


def jarosz(buf, rows, cols, wr, wc, nreps):
    """build.rs:283-303: nreps x (box along rows, then box along columns)."""
    tmp = [mpf(0)] * len(buf)
    for _ in range(nreps):
        for i in range(rows):
            box_one_d(buf, i * cols, tmp, cols, 1, wr)
        for j in range(cols):
            box_one_d(tmp, j, buf, rows, cols, wc)


def tent_weights(old_dim=512, new_dim=127):
    window = -(-old_dim // (2 * new_dim))  # div_ceil, build.rs:310-312
    er = ec = 2 * window + 1
    out = [mpf(0)] * (er * ec)
    for di in range(er):
        for dj in range(ec):
            tmp = [mpf(0)] * (er * ec)
            tmp[di * ec + dj] = mpf(1)
            total = sum(tmp, mpf(0))
            tmp = [x / total for x in tmp]
            jarosz(tmp, er, ec, window, window, 2)
            mid = tmp[window * ec + window]
            if float(mid) > 0.0:
                out[di * ec + dj] = mid
    return (ec - 1) // 2, er, ec, out


def main(path):
    mp.prec = PREC
    lines = []
    w = lines.append
    w("/* Generated by gen_tables.py (mpmath at 128 bits). Do not edit. */")
    w("#pragma once")
    w("#include <stdint.h>")
    dct32 = []
    dct64 = []
    for i in range(1, 17):
        for j in range(127):
            v = d_value(i, j, 127)
            dct32.append(f32_bits(v)[0])
            dct64.append(f64_bits(v)[0])
    w("static const uint32_t YPDQ_DCT_F32_BITS[16 * 127] = {")
    for r in range(16):
        w("  " + ", ".join("0x%08xu" % b for b in dct32[r * 127:(r + 1) * 127]) + ",")
    w("};")
    offset, er, ec, tent = tent_weights()
    assert (offset, er, ec) == (3, 7, 7)
    w("#define YPDQ_TENT_OFFSET %d" % offset)
    w("#define YPDQ_TENT_ROWS %d" % er)
    w("#define YPDQ_TENT_COLS %d" % ec)
    w("static const uint32_t YPDQ_TENT_F32_BITS[49] = {")
    w("  " + ", ".join("0x%08xu" % f32_bits(x)[0] for x in tent) + ",")
    w("};")
    # one macro per tap, for compile-time immediates in device code
    for di in range(er):
        for dj in range(ec):
            w("#define YPDQ_TENT_BITS_%d_%d 0x%08xu" % (di, dj, f32_bits(tent[di * ec + dj])[0]))
    offs = []
    for i in range(127):
        step = (512.0 - 0.0) / 128
        offs.append(int(round(0.0 + step * (i + 1))))
    w("static const int YPDQ_CONV_OFFSET[127] = {")
    w("  " + ", ".join(str(o) for o in offs) + ",")
    w("};")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    # report the tent weights as k/81 to document the closed form
    ks = [round(float(x) * 81) for x in tent]
    print("tent weights x81:")
    for r in range(7):
        print("  ", ks[r * 7:(r + 1) * 7])


if __name__ == "__main__":
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(__file__), "ypdq_tables.h")
    main(out)
