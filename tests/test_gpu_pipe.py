"""The raw-frame front-end end to end: frames in, the reference CLI's output formats out,
hashes equal to the oracle's (which restates the reference's f32 pipeline)."""
import importlib.util
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

PIPE = os.path.join(ROOT, "yume-pdq_gb300", "pipe.py")


def load_pipe():
    spec = importlib.util.spec_from_file_location("ypdq_pipe", PIPE)
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def run(args, data):
    r = subprocess.run([sys.executable, PIPE] + args, input=data, capture_output=True, cwd=ROOT,
                       timeout=600)
    assert r.returncode == 0, r.stderr.decode()[-2000:]
    return r.stdout


def expected(pipe, hashes, quality, fmt, slots):
    kind, upper, q, sep = pipe.parse_format(fmt)
    return b"".join(pipe.format_hash(hashes[f, s], quality[f, s], kind, upper, q, sep)
                    for f in range(hashes.shape[0]) for s in range(slots))


def test_luma8_stream_all_dihedrals(yp, oracle):
    pipe = load_pipe()
    frames = yp.synth.to_u8(yp.synth.blob_images(3, seed=501))
    out = run(["-f", "q+hex+lf", "--dihedrals", "--batch", "2"], frames.tobytes())
    # the CLI's default: the sign convention of the reference's smart_kernel on this host
    h, q, t, _ = oracle.hash_batch(frames, semantics=yp.kernel.host_semantics())
    assert out == expected(pipe, h, q, "q+hex+lf", 8)
    assert out.count(b"\n") == 24


def test_rgb8_stream_bin(yp, oracle):
    pipe = load_pipe()
    frames = yp.synth.color_images(2, seed=502, channels=3)
    out = run(["--input-format", "rgb8", "-f", "bin"], frames.tobytes())
    h, q, t, _ = oracle.hash_batch(oracle.luma(frames))
    assert out == expected(pipe, h, q, "bin", 1)


def test_reference_kernel_stream(yp, oracle):
    """--reference-kernel: ReferenceKernel<f32> hashes (oracle restatement of ref.rs), scalar
    dihedral semantics as that kernel's trait defaults."""
    pipe = load_pipe()
    frames = yp.synth.to_u8(yp.synth.blob_images(3, seed=503))
    out = run(["-f", "hex+lf", "--dihedrals", "--semantics", "scalar", "--reference-kernel"],
              frames.tobytes())
    h, q, t, p, b = oracle.hash_batch_reference(frames, semantics="scalar")
    assert out == expected(pipe, h, q, "hex+lf", 8)


def test_partial_frame_is_an_error(yp):
    r = subprocess.run([sys.executable, PIPE, "-f", "hex"], input=b"\0" * 1000,
                       capture_output=True, cwd=ROOT, timeout=600)
    assert r.returncode != 0 and b"middle of a frame" in r.stderr


def test_screening_stream_with_database(yp, oracle, tmp_path):
    pipe = load_pipe()
    frames = yp.synth.to_u8(yp.synth.blob_images(5, seed=503))
    h, q, t, _ = oracle.hash_batch(frames, semantics=yp.kernel.host_semantics())
    rows = yp.synth.rows_128(50_000, seed=504)
    yp.synth.plant(rows, h.reshape(-1, 32), 300, 0, 31, seed=505)
    db = tmp_path / "db.bin"
    rows.tofile(db)
    out = run(["-f", "hex+lf", "--batch", "2", "--db", str(db), "--threshold", "31"],
              frames.tobytes())
    want = oracle.find_all(rows, h.reshape(-1, 32), 31)
    lines = out.split(b"\n")[:-1]
    got_hashes, got_hits = [], []
    frame = -1
    for line in lines:
        if line.startswith(b"match "):
            slot, idx, dist = map(int, line.split()[1:])
            got_hits.append((idx, 8 * frame + slot, dist))
        else:
            frame += 1
            got_hashes.append(line)
    assert got_hashes == [bytes(x).hex().encode() for x in h[:, 0]]
    assert sorted(got_hits) == sorted(zip(want["index"].tolist(), want["query"].tolist(),
                                          want["distance"].tolist()))


def test_diagnostic_stream(yp, oracle):
    """The diagnostic format end to end: each slot's quality, threshold, hash and PDQF (as the
    reference's buffer holds it at that visit) equal the oracle's, printed as the reference
    prints them."""
    pipe = load_pipe()
    frames = yp.synth.to_u8(yp.synth.blob_images(2, seed=507))
    sem = yp.kernel.host_semantics()
    out = run(["-f", "diagnostic", "--dihedrals"], frames.tobytes())
    h, q, t, p = oracle.hash_batch(frames, semantics=sem, want_pdqf=True)
    want = []
    for f in range(len(frames)):
        dh, dt, dq, dp = oracle.dihedrals(p[f], t[f, 0], sem)
        pdqfs = [p[f]] + list(dp)
        for s in range(8):
            want.append(pipe.format_diagnostic(s, s, h[f, s], q[f, s], t[f, s], pdqfs[s], b""))
    assert out == b"".join(want)
    assert out.count(b"Index: 0\n") == 2 and out.count(b"[Dihedrals") == 14
