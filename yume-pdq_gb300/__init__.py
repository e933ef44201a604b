"""GB300-native yume-pdq hot path: batched PDQ hashing with dihedrals and exact Hamming scan.

Everything computes in libyumepdq_gb300.so (CUDA, sm_103a) behind the C ABI in include/.
This package is a thin host layer: ctypes bindings (`_lib`), device buffers and batched
calls (`core`), the reference's pipeline/Kernel surface (`kernel`), its PDQMatcher surface
(`matching`), the continuous-batching screening service (`serving`) and seeded synthetic
workloads (`synth`).

The directory name contains a hyphen, so import it through `load_package()` in
`__graft_entry__` or register it under the name `yume_pdq_gb300` with importlib.
"""
from . import _lib, build, core, kernel, matching, serving, synth  # noqa: F401
from ._lib import HIT_DTYPE, YpdqError  # noqa: F401
from .core import (Context, Database, DeviceBuffer, hash_batch, merge_shard_hits,  # noqa: F401
                   scan, screen_host, shard_rows)
from .kernel import (CudaKernel, Dihedrals, SLOT_DIHEDRALS, hash, hash_float,  # noqa: F401
                     hash_get_threshold, visit_dihedrals)
from .matching import CudaMatcher, CudaVectorDatabase  # noqa: F401
from .serving import PinnedArray, Result, Server  # noqa: F401
