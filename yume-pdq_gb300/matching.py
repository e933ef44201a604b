"""The reference's matcher surface (PDQMatcher) backed by the CUDA scan.

Mirrors src/matching/mod.rs:50-105 (the PDQMatcher trait) in the accelerator style of
src/matching/vulkan.rs: the matcher owns the haystack (a device-resident database) and is
queried with needles. Unlike VulkanMatcher (FindsAllMatches = B0), this matcher returns
every hit with its distance, as CpuMatcher does.
"""
import numpy as np

from . import _lib, core


class CudaVectorDatabase(core.Database):
    """Device-resident haystack; mirror of VulkanVectorDatabase::new (vulkan.rs:46-64)."""

    def __init__(self, ctx, data):
        super().__init__(ctx, rows=data)
        self.num_vectors = self.n_rows


class CudaMatcher:
    """PDQMatcher over a CudaVectorDatabase with a fixed threshold."""

    InputDimension = 32
    NoFalseNegative = True
    NoFalsePositive = True
    FindsAllMatches = True

    def __init__(self, ctx, haystack, threshold, algo=_lib.SCAN_AUTO):
        if not 0 <= int(threshold) <= 256:
            raise ValueError("threshold must be in [0, 256]")
        self.ctx = ctx
        self.haystack = haystack
        self.threshold = int(threshold)
        self.algo = algo
        self._cnt = ctx.alloc(8)

    @staticmethod
    def ident():
        return "CUDA sm_103a exact matcher"

    def _queries(self, needles):
        q = np.ascontiguousarray(needles, np.uint8).reshape(-1, 32)
        return q, (self.ctx.to_device(q) if q.shape[0] else self.ctx.alloc(32))

    def scan(self, needles):
        """True if any haystack row is within the threshold of any needle."""
        q, d_q = self._queries(needles)
        d_rows, n = self.haystack.device_rows()
        core.scan_device(self.ctx, d_rows, n, d_q, q.shape[0], self.threshold, None, 0,
                         self._cnt, self.algo)
        self.ctx.sync()
        return int(self._cnt.download((1,), np.uint64)[0]) > 0

    def find_all(self, needles, capacity=1 << 16):
        """Every hit (index, query, distance), sorted by (index, query)."""
        q, d_q = self._queries(needles)
        d_rows, n = self.haystack.device_rows()
        while True:
            d_hits = self.ctx.alloc(max(capacity, 1) * 16)
            core.scan_device(self.ctx, d_rows, n, d_q, q.shape[0], self.threshold, d_hits,
                             capacity, self._cnt, self.algo)
            self.ctx.sync()
            total = int(self._cnt.download((1,), np.uint64)[0])
            if total <= capacity:
                break
            capacity = total
        if total > 1:
            core.sort_hits_device(self.ctx, d_hits, total)
        return d_hits.download((total,), _lib.HIT_DTYPE) if total else np.zeros(0, _lib.HIT_DTYPE)

    def find(self, needles, f):
        """Call f(haystack_index, needle_index) for hits in (index, needle) order until it
        returns something other than None, and return that (PDQMatcher::find)."""
        for h in self.find_all(needles):
            r = f(int(h["index"]), int(h["query"]))
            if r is not None:
                return r
        return None
