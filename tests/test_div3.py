"""The Jarosz kernels' division-free x / 3 (div3_rn, yume-pdq_gb300/csrc/jarosz.cu) equals
IEEE division for every float: the same IEEE operations compiled for the host and run over
all 2^31 non-negative bit patterns (tests/div3_exhaustive.c)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_div3_exhaustive(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "div3_exhaustive")
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-o", exe,
                    os.path.join(HERE, "div3_exhaustive.c"), "-lm", "-lpthread"], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
