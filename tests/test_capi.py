"""CPU tests of the C-ABI library: it loads, exports every symbol include/*.h declares, and
its host-only logic (constants, argument checks without a device) behaves."""
import ctypes
import os
import re

import numpy as np

from conftest import ROOT


def declared_symbols():
    funcs, data = set(), set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if not name.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", name)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b((?:ypdq|yume_pdq)_\w+)\s*\(", text):
            funcs.add(m.group(1))
        for m in re.finditer(r"extern\s+const\s+[\w\s]+?\b(YUME_PDQ_\w+)", text):
            data.add(m.group(1))
    return funcs, data


def test_library_exports_declared_symbols(yp):
    lib = yp._lib.load()
    funcs, data = declared_symbols()
    assert len(funcs) >= 30 and len(data) == 12
    for f in sorted(funcs | data):
        assert hasattr(lib, f), "missing export " + f
    assert funcs <= set(yp._lib.SIGNATURES), "binding does not cover " + str(funcs - set(yp._lib.SIGNATURES))
    assert data == set(yp._lib.DATA_SYMBOLS)


def test_dihedral_constants_match_reference(yp):
    """Dihedrals::from_tuples (src/lib.rs:97-134): big-endian packed i8 matrices."""
    lib = yp._lib.load()
    want = {
        "NORMAL": ((1, 0), (0, 1)), "FLIPPED": ((1, 0), (0, -1)), "FLOPPED": ((-1, 0), (0, 1)),
        "ROTATED_180": ((-1, 0), (0, -1)), "ROTATED_90": ((0, 1), (-1, 0)),
        "ROTATED_270": ((0, 1), (1, 0)), "ROTATED_90_FLOPPED": ((0, -1), (-1, 0)),
        "FLOPPED_ROTATED_270": ((0, -1), (1, 0)),
    }
    for name, tup in want.items():
        v = ctypes.c_uint32.in_dll(lib, "YUME_PDQ_DIHEDRAL_" + name).value
        assert yp.Dihedrals.into_tuples(v) == tup
        assert getattr(yp.Dihedrals, name) == v
    assert ctypes.c_uint32.in_dll(lib, "YUME_PDQ_VERSION_MAJOR").value == 1
    assert ctypes.c_char_p.in_dll is not None


def test_slot_order(yp):
    assert yp.SLOT_DIHEDRALS[1:] == [
        yp.Dihedrals.FLOPPED, yp.Dihedrals.ROTATED_180, yp.Dihedrals.FLIPPED,
        yp.Dihedrals.ROTATED_90_FLOPPED, yp.Dihedrals.ROTATED_270,
        yp.Dihedrals.FLOPPED_ROTATED_270, yp.Dihedrals.ROTATED_90]


def test_ctx_create_without_device_reports_error(yp):
    """On a machine without a GPU the context call fails with a status, not a crash."""
    lib = yp._lib.load()
    h = ctypes.c_void_p()
    st = lib.ypdq_ctx_create(0, ctypes.byref(h))
    if st == 0:  # a GPU is present: nothing to check here
        lib.ypdq_ctx_destroy(h)
        return
    assert st in (yp._lib.ERR_CUDA, yp._lib.ERR_INVALID)
    assert lib.ypdq_last_error()


def test_null_ctx_rejected(yp):
    lib = yp._lib.load()
    assert lib.ypdq_hash_batch(None, None, 0, 0, 0, 0, None, None, None, None, 1, None, None) == yp._lib.ERR_INVALID
    assert lib.ypdq_scan(None, None, 0, None, 0, 31, None, 0, None, 0, None) == yp._lib.ERR_INVALID


def test_synth_rows_have_128_bits(yp):
    rows = yp.synth.rows_128(1000, seed=5)
    assert np.all(yp.synth.popcount_rows(rows) == 128)
    assert len({r.tobytes() for r in rows}) == 1000


def test_plant_distances_exact(yp):
    rng = np.random.default_rng(3)
    rows = yp.synth.rows_128(500, seed=1)
    q = yp.synth.rows_128(10, seed=2)
    pos, qid, dist = yp.synth.plant(rows, q, 50, 0, 40, seed=4)
    d = np.unpackbits(rows[pos] ^ q[qid], axis=1).sum(1)
    assert np.array_equal(d, dist)


def test_server_config_default_and_argument_checks(yp):
    """ypdq_server_config_default is host-only; create/submit/poll reject NULL handles."""
    lib = yp._lib.load()
    cfg = yp._lib.ServerConfig()
    assert lib.ypdq_server_config_default(ctypes.byref(cfg)) == yp._lib.OK
    assert (cfg.threshold, cfg.max_step_images, cfg.slots) == (31, 1024, 3)
    assert (cfg.input_kind, cfg.dct_precision, cfg.semantics) == (0, 0, 0)
    assert cfg.step_hit_capacity == 1 << 20 and cfg.autotune == 0
    assert lib.ypdq_server_config_default(None) == yp._lib.ERR_INVALID
    out = ctypes.c_void_p()
    assert lib.ypdq_server_create(None, None, ctypes.byref(cfg), ctypes.byref(out)) == yp._lib.ERR_INVALID
    n = ctypes.c_uint32()
    assert lib.ypdq_server_poll(None, None, 0, ctypes.byref(n), 0) == yp._lib.ERR_INVALID
    assert lib.ypdq_server_submit(None, None, 1, None, 0, None, None, 0, None) == yp._lib.ERR_INVALID
    assert lib.ypdq_server_destroy(None) == yp._lib.ERR_INVALID


def test_screen_chunk_plan(yp):
    """ypdq_screen_plan (host-only): the chunks of ypdq_screen_host cover [0, n) in order,
    are whole multiples of 32 images (90 at t <= 36: one pass of 720 queries in triples)
    except the last and number at most 32. They grow geometrically when hashing and scanning
    an image takes longer than copying it, and slowly (by the hash kernel's fixed cost per
    chunk) when it does not; then a remainder smaller than a pass is the last chunk."""
    lib = yp._lib.load()
    bounds = (ctypes.c_int64 * 33)()
    k = ctypes.c_int()

    def plan(n, kind, rows, t, dct=0):
        assert lib.ypdq_screen_plan(n, kind, dct, rows, t, bounds, ctypes.byref(k)) == yp._lib.OK
        return [bounds[i] for i in range(k.value + 1)]

    cases = [(0, 10_000_000, 31), (1, 4_000_000, 31), (0, 60_000, 31), (0, 10_000_000, 64),
             (3, 100_000_000, 48), (0, 0, 0)]
    for n in (0, 1, 31, 32, 33, 63, 64, 65, 300, 1024, 4096, 100_000, 10_000_000):
        for kind, rows, t in cases:
            b = plan(n, kind, rows, t)
            sizes = np.diff(b)
            assert b[0] == 0 and b[-1] == n and (sizes > 0).all() and len(sizes) <= 32
            assert (sizes[:-1] % (90 if t <= 36 else 32) == 0).all()
    # 1,024 f32 images against 10M rows at t = 31: ~5 us of hash and scan per image against
    # ~5 us of copy, so whole 90-image passes, growing slowly, and the remainder last
    sizes = np.diff(plan(1024, 0, 10_000_000, 31))
    assert sizes[0] == 90 and (sizes[:-1] % 90 == 0).all() and sizes[-1] <= 180
    assert 6 <= len(sizes) <= 16
    # at 100M rows the scan is ten times longer than the copy: chunks grow geometrically
    big = np.diff(plan(1024, 0, 100_000_000, 31))
    assert big[0] == 90 and (big[:-1] % 90 == 0).all() and big.max() >= 180 and len(big) < 10
    # above t = 36 passes hold 256 queries: chunks of whole 32-image passes
    sizes48 = np.diff(plan(1024, 0, 10_000_000, 48))
    assert sizes48[0] == 32 and (sizes48 % 32 == 0).all()
    # a small database: copying dominates and a chunk's compute is mostly the hash kernel's
    # one round over its images, so chunks grow only by that fixed cost
    small = np.diff(plan(1024, 0, 60_000, 31))
    assert (np.diff(small[:-1]) >= 0).all() and len(small) >= len(sizes) and small.max() <= 304
    # the Jarosz filter (dct_precision 0x200) adds ~1 us of compute per image: where the scan
    # dominates (30M rows: ~11 us of scan per image against ~5 us of copy), its chunks grow
    # at least as fast
    assert len(plan(1024, 0, 30_000_000, 31, dct=0x200)) <= len(plan(1024, 0, 30_000_000, 31))
    assert lib.ypdq_screen_plan(10, 9, 0, 1, 31, bounds, ctypes.byref(k)) == yp._lib.ERR_INVALID
    assert lib.ypdq_screen_plan(-1, 0, 0, 1, 31, bounds, ctypes.byref(k)) == yp._lib.ERR_INVALID
    assert lib.ypdq_screen_plan(10, 0, 0, 1, 31, None, ctypes.byref(k)) == yp._lib.ERR_INVALID


LAYOUT_PROBE = r"""
#include <stddef.h>
#include <stdio.h>
#include "ypdq.h"
#define F(T, m) printf(#T " " #m " %zu\n", offsetof(T, m))
int main(void) {
  printf("ypdq_server_config size %zu\n", sizeof(ypdq_server_config));
  printf("ypdq_completion size %zu\n", sizeof(ypdq_completion));
  printf("ypdq_server_stats size %zu\n", sizeof(ypdq_server_stats));
  printf("ypdq_hit size %zu\n", sizeof(ypdq_hit));
  F(ypdq_server_config, target_step_ms); F(ypdq_server_config, autotune);
  F(ypdq_completion, latency_us); F(ypdq_completion, n_hits);
  F(ypdq_server_stats, p50_us); F(ypdq_server_stats, n_buckets);
  F(ypdq_server_stats, bucket_ms); F(ypdq_server_stats, bucket_steps);
  return 0;
}
"""


def test_struct_layouts_match_header(yp, tmp_path):
    """The ctypes mirrors of the server structs have the C compiler's layout of include/ypdq.h."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    src = tmp_path / "probe.c"
    src.write_text(LAYOUT_PROBE)
    exe = tmp_path / "probe"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        t, m, v = line.split()
        got[(t, m)] = int(v)
    L = yp._lib
    mirrors = {"ypdq_server_config": L.ServerConfig, "ypdq_completion": L.Completion,
               "ypdq_server_stats": L.ServerStats}
    for (t, m), v in got.items():
        if t == "ypdq_hit":
            assert v == L.HIT_DTYPE.itemsize
        elif m == "size":
            assert ctypes.sizeof(mirrors[t]) == v, t
        else:
            assert getattr(mirrors[t], m).offset == v, (t, m)


def _host_dropin_semantics():
    """What yume-pdq's smart_kernel() computes on this host in its default build
    (src/kernel/mod.rs:79-176): Avx2F32Kernel's signs on x86_64 with AVX2 and FMA, the
    trait default elsewhere."""
    import platform
    flags = set()
    try:
        for line in open("/proc/cpuinfo"):
            if line.startswith("flags"):
                flags |= set(line.split(":", 1)[1].split())
    except OSError:
        pass
    if platform.machine() in ("x86_64", "AMD64") and {"avx2", "fma"} <= flags:
        return 1  # YPDQ_DIHEDRAL_AVX2
    return 2      # YPDQ_DIHEDRAL_SCALAR


def _dropin_semantics_in_child(env_value):
    import subprocess
    import sys
    code = ("import sys, ctypes; sys.path.insert(0, %r); import __graft_entry__ as g; "
            "yp = g.load_package(); s = ctypes.c_int(-1); "
            "assert yp._lib.load().ypdq_dropin_semantics(ctypes.byref(s)) == 0; print(s.value)"
            % ROOT)
    env = dict(os.environ)
    env.pop("YUME_PDQ_DIHEDRAL_SEMANTICS", None)
    if env_value is not None:
        env["YUME_PDQ_DIHEDRAL_SEMANTICS"] = env_value
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    return int(r.stdout.strip())


def test_dropin_semantics_default_follows_host():
    """The drop-in symbols derive dihedrals with the sign convention the replaced library
    uses on the same host, and the environment variable overrides it."""
    assert _dropin_semantics_in_child(None) == _host_dropin_semantics()
    for name, want in (("exact", 0), ("avx2", 1), ("scalar", 2)):
        assert _dropin_semantics_in_child(name) == want
    assert _dropin_semantics_in_child("bogus") == _host_dropin_semantics()


REFERENCE_CONSUMER = "/root/reference/integration/dummy.c"  # yume-pdq's own C example


def test_reference_c_consumer_links_unchanged(tmp_path):
    """yume-pdq's C example (integration/dummy.c), compiled unchanged with gcc, links
    against libyumepdq_gb300.so in place of libyume_pdq.so. Only where the reference tree is
    present (running it needs a GPU; tests/dropin_consumer.c covers the run on one)."""
    import pytest
    import subprocess
    if not os.path.exists(REFERENCE_CONSUMER):
        pytest.skip("reference tree not present")
    lib_dir = os.path.join(ROOT, "yume-pdq_gb300", "_build")
    exe = str(tmp_path / "dummy")
    r = subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), "-o", exe, REFERENCE_CONSUMER,
                        "-L", lib_dir, "-l:libyumepdq_gb300.so"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nm = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True, text=True)
    assert "yume_pdq_hash_smart_kernel" in nm.stdout
