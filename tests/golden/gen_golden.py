#!/usr/bin/env python3
"""Regenerate the golden fixtures in tests/golden/.

1. readme_fm_sine.json: yume-pdq's own known-answer vector. The expected 32-byte hash and
   the printed 16x16 PDQF come from the "API Usage" example of the reference README
   (README.md:305-451), read from a reference checkout given as argv[1]. That checkout is
   needed only to regenerate this file; the tests read the committed JSON.
2. oracle_vectors.npz: regression vectors from the CPU oracle. Three seeded u8 images
   (blob, noise, constant), their hashes, qualities, thresholds and PDQF under all three
   dihedral sign conventions, and a small matcher case with planted hits.

Usage: python tests/golden/gen_golden.py /path/to/yume-pdq
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def readme_vector(ref_root):
    text = open(os.path.join(ref_root, "README.md"), encoding="utf-8").read()
    m = re.search(r"let expected = \[(.*?)\];", text, re.S)
    expected = [int(x, 16) for x in re.findall(r"0x([0-9a-fA-F]{2})", m.group(1))]
    assert len(expected) == 32
    m = re.search(r"You should see:\n(.*?)\*/", text, re.S)
    rows = []
    for line in m.group(1).strip().splitlines():
        vals = [float(v) for v in line.split()]
        if len(vals) == 16:
            rows.append(vals)
    assert len(rows) == 16
    return {
        "source": "yume-pdq README.md, section 'API Usage (and dihedral transformations)'",
        "expected_hash_hex": bytes(expected).hex(),
        "max_bits_different": 2,
        "pdqf_printed_1dp": rows,
    }


def oracle_vectors(path):
    import oracle
    sys.path.insert(0, ROOT)
    import __graft_entry__ as g
    synth = g.load_package().synth
    rng = np.random.default_rng(20250)
    imgs = np.stack([synth.blob_image(rng), synth.noise_image(rng), synth.constant_image(rng)])
    imgs_u8 = synth.to_u8(imgs)
    out = {"images_u8": imgs_u8}
    for sem in ("exact", "avx2", "scalar"):
        h, q, t, p = oracle.hash_batch(imgs_u8, semantics=sem, nthreads=1, want_pdqf=True)
        out["hashes_" + sem] = h
        out["quality_" + sem] = q
        out["thresholds_" + sem] = t
        out["pdqf"] = p
    out["buf1_0"] = oracle.compress(imgs_u8[0].astype(np.float32))
    # matcher: 512 random rows, 16 needles, 40 planted rows at distance 0..40
    rows = synth.rows_128(512, seed=11)
    needles = synth.rows_128(16, seed=12)
    synth.plant(rows, needles, 40, 0, 40, seed=13)
    out["match_rows"] = rows
    out["match_needles"] = needles
    for t in (0, 16, 31, 48):
        hits = oracle.find_all(rows, needles, t, nthreads=1)
        out["match_hits_t%d" % t] = np.stack([hits["index"].astype(np.int64),
                                             hits["query"].astype(np.int64),
                                             hits["distance"].astype(np.int64)], axis=1)
    np.savez_compressed(path, **out)


def main():
    if len(sys.argv) > 1:
        with open(os.path.join(HERE, "readme_fm_sine.json"), "w") as f:
            json.dump(readme_vector(sys.argv[1]), f, indent=1)
    oracle_vectors(os.path.join(HERE, "oracle_vectors.npz"))


if __name__ == "__main__":
    main()
