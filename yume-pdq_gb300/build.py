"""Build libyumepdq_gb300.so in-tree with nvcc for sm_103a (no CMake, no torch)."""
import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_NAME = "libyumepdq_gb300.so"
LIB_PATH = os.path.join(BUILD_DIR, LIB_NAME)

SOURCES = ["hash.cu", "scan.cu", "scan_tc.cu", "synth.cu", "capi.cu", "noalloc.cu", "serve.cu",
           "dbfile.cu", "jarosz.cu", "stages.cu"]
HEADERS = ["ypdq_internal.cuh", "ypdq_tables.h", "capi_internal.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills",
]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    deps = [os.path.join(CSRC, h) for h in HEADERS]
    deps += [os.path.join(INCLUDE, h) for h in os.listdir(INCLUDE) if h.endswith(".h")]
    deps.append(os.path.abspath(__file__))
    return deps


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose=False, force=False, extra_flags=()):
    """Compile every .cu for sm_103a and link the shared library. Returns its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    cc = nvcc()
    deps = _deps()
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + deps):
            cmd = [cc, "-c", s, "-o", o, "-I", INCLUDE, "-I", CSRC] + NVCC_FLAGS + list(extra_flags)
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed for %s" % cmd[2])
    if force or _stale(LIB_PATH, objs):
        cmd = [cc, "-shared", "-o", LIB_PATH] + objs + ARCH + ["-cudart", "shared"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("link failed")
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
