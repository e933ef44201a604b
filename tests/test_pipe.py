"""The raw-frame front-end's output formats (yume-pdq `pipe`, src/main.rs:683-773,
1106-1133), checked on the CPU against the formats' definitions."""
import importlib.util
import os
import struct

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def pipe():
    spec = importlib.util.spec_from_file_location(
        "ypdq_pipe", os.path.join(ROOT, "yume-pdq_gb300", "pipe.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_format_specs(pipe):
    assert pipe.parse_format("q+hex+lf") == ("hex", False, True, b"\n")
    assert pipe.parse_format("HEX+crlf") == ("hex", True, False, b"\r\n")
    assert pipe.parse_format("bin") == ("bin", False, False, b"")
    assert pipe.parse_format("q+raw+nul") == ("raw", False, True, b"\0")
    with pytest.raises(ValueError):
        pipe.parse_format("json")


def test_hash_outputs(pipe):
    h = bytes(range(0, 256, 8))  # 32 bytes
    assert pipe.format_hash(h, 1.0, "hex", False, False, b"\n") == h.hex().encode() + b"\n"
    assert pipe.format_hash(h, 1.0, "hex", True, False, b"") == h.hex().upper().encode()
    bits = pipe.format_hash(h, 1.0, "bin", False, False, b"")
    assert len(bits) == 256 and bits[:16] == b"0000000000001000"  # bytes 0x00, 0x08, MSB first
    raw = pipe.format_hash(h, 0.5, "raw", False, True, b"")
    assert raw[:4] == struct.pack("<f", 0.5) and raw[4:] == h
    # quality x 100 in f32 with 3 decimals, as "{0:02.3}"
    assert pipe.format_hash(h, 1.0, "hex", False, True, b"")[:8] == b"100.000:"
    assert pipe.quality_prefix(np.float32(0.123456)) == b"12.346:"
    assert pipe.quality_prefix(0.0) == b"0.000:"


def test_read_frames(pipe):
    import io
    data = np.arange(2 * 512 * 512 * 3, dtype=np.uint64).astype(np.uint8).tobytes()
    f = pipe.read_frames(io.BytesIO(data), 3, 8)
    assert f.shape == (2, 512, 512, 3)
    with pytest.raises(EOFError):
        pipe.read_frames(io.BytesIO(data[:-1]), 3, 8)
    assert pipe.read_frames(io.BytesIO(b""), 1, 8) is None


def test_diagnostic_format(pipe):
    """The reference's diagnostic output (src/main.rs:738-773): header, index, quality x 100
    with 3 decimals, threshold with 7, the 256 bits on one line, the PDQF rows with '*' on
    values above the threshold, each value with 5 decimals."""
    h = bytes(range(0, 256, 8))
    pdqf = np.arange(256, dtype=np.float32).reshape(16, 16) / np.float32(7.0) - np.float32(10.0)
    out = pipe.format_diagnostic(0, 0, h, np.float32(0.5), np.float32(1.25), pdqf, b"\n").decode()
    lines = out.split("\n")
    assert lines[:5] == ['["original"]', "Index: 0", "Quality: 50.000", "Threshold: 1.2500000",
                         "Hash:"]
    assert lines[5] == "".join(format(b, "08b") for b in h)
    assert lines[6] == "PDQF:"
    rows = lines[7:23]
    assert len(rows) == 16 and lines[23] == "" and out.endswith("\n\n")
    first = rows[0].split("\t")
    assert first[0] == "%.5f" % float(pdqf[0, 0]) and not first[0].startswith("*")
    assert rows[15].split("\t")[15] == "*%.5f" % float(pdqf[15, 15])
    assert sum(v.startswith("*") for r in rows for v in r.split("\t")) == int(np.sum(pdqf > 1.25))
    # derived hashes are named by their Dihedrals value (four big-endian i8 matrix entries)
    assert pipe.format_diagnostic(1, 1, h, 0.5, 1.25, pdqf, b"").startswith(
        b"[Dihedrals { packed: 4278190081 }]\nIndex: 1\n")
    assert pipe.slot_name(7) == "Dihedrals { packed: %d }" % 0x0001FF00
    assert pipe.parse_format("diagnostic+lf") == ("diagnostic", False, False, b"\n")
