#!/usr/bin/env python3
"""Generate ``oracle/ypdq_constants.h``: the PDQ constant tables at 128-bit precision.

TEST INFRASTRUCTURE. Only the oracle and the tests use the header this script writes.

The tables come from the library's one generator, ``yume-pdq_gb300/csrc/gen_tables.py``
(imported here), which restates the 128-bit MPFR construction of yume-pdq's build script
(build.rs:203-387, 557-643): the DCT matrix rounded once to f32 and f64, the 7x7 tent
weights and the 127 sample offsets. This script adds the f64 DCT matrix the FP64 oracle
needs and writes the oracle's header format. Generating both headers from one
implementation means the equality of the two f32 tables (test_constants_pinned) is a
check of the build, not of the construction; what checks the construction independently
is the closed-form comparison (test_constants_closed_form) and the README known-answer
vector, which the oracle reproduces to 0 bits.
"""
import importlib.util
import os
import sys

from mpmath import mp

_GEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), os.pardir, "yume-pdq_gb300",
                    "csrc", "gen_tables.py")
_spec = importlib.util.spec_from_file_location("ypdq_gen_tables", _GEN)
gen = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(gen)
PREC, d_value, f32_bits, f64_bits, tent_weights = (gen.PREC, gen.d_value, gen.f32_bits,
                                                   gen.f64_bits, gen.tent_weights)


def main(path):
    mp.prec = PREC
    lines = []
    w = lines.append
    w("/* Generated by oracle/gen_constants.py (mpmath at 128 bits). Do not edit. */")
    w("/* TEST INFRASTRUCTURE: constant tables for the CPU oracle. */")
    w("#pragma once")
    w("#include <stdint.h>")
    dct32 = []
    dct64 = []
    for i in range(1, 17):
        for j in range(127):
            v = d_value(i, j, 127)
            dct32.append(f32_bits(v)[0])
            dct64.append(f64_bits(v)[0])
    w("static const uint32_t YPDQO_DCT_F32_BITS[16 * 127] = {")
    for r in range(16):
        w("  " + ", ".join("0x%08xu" % b for b in dct32[r * 127:(r + 1) * 127]) + ",")
    w("};")
    w("static const uint64_t YPDQO_DCT_F64_BITS[16 * 127] = {")
    for r in range(16):
        w("  " + ", ".join("0x%016xull" % b for b in dct64[r * 127:(r + 1) * 127]) + ",")
    w("};")
    offset, er, ec, tent = tent_weights()
    assert (offset, er, ec) == (3, 7, 7)
    w("#define YPDQO_TENT_OFFSET %d" % offset)
    w("#define YPDQO_TENT_ROWS %d" % er)
    w("#define YPDQO_TENT_COLS %d" % ec)
    w("static const uint32_t YPDQO_TENT_F32_BITS[49] = {")
    w("  " + ", ".join("0x%08xu" % f32_bits(x)[0] for x in tent) + ",")
    w("};")
    offs = []
    for i in range(127):
        step = (512.0 - 0.0) / 128
        offs.append(int(round(0.0 + step * (i + 1))))
    w("static const int YPDQO_CONV_OFFSET[127] = {")
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
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(__file__), "ypdq_constants.h")
    main(out)
