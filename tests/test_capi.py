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
