// Exact linear Hamming scan of 256-bit rows against a batch of 256-bit queries, with
// warp-aggregated hit compaction.
//
// Reference: CpuMatcher::find (scalar, src/matching/mod.rs:336-362) reports every
// (row, needle) with popcount(row ^ needle) <= threshold; the WGSL matcher
// (src/matching/vulkan.rs:98-147) evaluates the same predicate, one row per thread.
// Both kernels here return the full hit set with distances. They differ only in how
// they compute distances:
//   SIMT   one row per thread, eight 32-bit XOR + POPC per (row, query);
//   B1MMA  16 rows x 8 queries per warp instruction with the binary tensor-core MMA
//          (mma.sync m16n8k256 .b1 .xor.popc), whose accumulator is the distance.
#include "ypdq_internal.cuh"

namespace ypdq {

constexpr int kScanThreads = 256;
constexpr uint32_t kMaxSmemQueries = 2048;  // queries per launch (64 KiB of shared memory)

// Hit emission from lanes that found a hit in the same converged step: one atomic per warp.
__device__ __forceinline__ void emit_hits_ballot(bool pred, uint64_t row, uint32_t query,
                                                 uint32_t dist, ypdq_hit* hits, uint64_t cap,
                                                 unsigned long long* count) {
  const uint32_t ballot = __ballot_sync(0xffffffffu, pred);
  if (ballot == 0) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(ballot) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(count, static_cast<unsigned long long>(__popc(ballot)));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (pred) {
    const uint64_t pos = base + __popc(ballot & lanemask_lt());
    if (pos < cap) {
      ypdq_hit h;
      h.index = row;
      h.query = query;
      h.distance = dist;
      hits[pos] = h;
    }
  }
}

__device__ __forceinline__ uint4 ld_stream(const uint4* p) {
  uint4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}

// ------------------------------------------------------------------- SIMT

// Popcounts of several words through carry-save adders: a full adder turns three words into
// a sum word and a carry word with x0 + x1 + x2 = s + 2 c bit by bit, so fewer popcounts
// (the scarce pipe) are needed; the adders are single three-input logic ops.
__device__ __forceinline__ void csa(uint32_t a, uint32_t b, uint32_t c, uint32_t& s, uint32_t& cy) {
  s = a ^ b ^ c;
  cy = (a & b) | (c & (a ^ b));
}
__device__ __forceinline__ uint32_t popc3(uint32_t x0, uint32_t x1, uint32_t x2) {
  uint32_t s, c;
  csa(x0, x1, x2, s, c);
  return __popc(s) + 2 * __popc(c);
}
__device__ __forceinline__ uint32_t popc5(uint32_t x0, uint32_t x1, uint32_t x2, uint32_t x3,
                                          uint32_t x4) {
  uint32_t s1, c1, s2, c2;
  csa(x0, x1, x2, s1, c1);
  csa(s1, x3, x4, s2, c2);
  return __popc(s2) + 2 * (__popc(c1) + __popc(c2));
}
__device__ __forceinline__ uint32_t popc8(uint4 x, uint4 y) {
  uint32_t s1, c1, s2, c2, s3, c3, t1, f1;
  csa(x.x, x.y, x.z, s1, c1);
  csa(x.w, y.x, y.y, s2, c2);
  csa(s1, s2, y.z, s3, c3);
  const uint32_t ones = s3 ^ y.w, c4 = s3 & y.w;
  csa(c1, c2, c3, t1, f1);
  const uint32_t twos = t1 ^ c4, f2 = t1 & c4;
  const uint32_t fours = f1 ^ f2, eights = f1 & f2;
  return __popc(ones) + 2 * __popc(twos) + 4 * __popc(fours) + 8 * __popc(eights);
}

// kPrefix words (3, 5 or 8 of 8) are counted first. Their popcount is a lower bound of the
// distance, so once it exceeds t in every lane of the warp no pair of this query can be a
// hit; rows that pass are finished exactly, so hits and distances do not change. The host
// picks kPrefix by threshold: a random row is 48 +- 5 bits from a query in 96 bits and
// 80 +- 6 in 160, so for t <= 34 (or <= 62) nearly every warp stops after 2 (or 3) of the
// 8 popcounts that a plain count needs; above that the whole row is counted with 4.
// Rows per thread and resident blocks per SM of each variant (register-bound). With a
// prefix bound a thread takes two rows, so each query's shared load, vote and loop step
// serve both; the full count (4 popcounts per pair) runs out of registers first and keeps
// one row at higher occupancy. The grid-stride grid is exactly this many blocks per SM so
// that no block starts late.
__host__ __device__ constexpr int simt_rows(int prefix) { return prefix == 8 ? 1 : 2; }
__host__ __device__ constexpr int simt_blocks_per_sm(int prefix) { return prefix == 8 ? 6 : 4; }

template <int kPrefix>
__global__ void __launch_bounds__(kScanThreads, simt_blocks_per_sm(kPrefix))
    scan_simt_kernel(const uint4* __restrict__ rows, uint64_t n_rows,
                     const uint4* __restrict__ queries, uint32_t nq, uint32_t q_base,
                     uint32_t t, ypdq_hit* hits, uint64_t cap, unsigned long long* count,
                     const uint32_t* nq_dev) {
  constexpr int R = simt_rows(kPrefix);
  extern __shared__ uint4 sq[];
  if (nq_dev) nq = min(*nq_dev, nq);
  for (uint32_t i = threadIdx.x; i < 2 * nq; i += blockDim.x) sq[i] = queries[i];
  __syncthreads();
  // A warp owns 32 R consecutive rows per step, lane l rows l + 32 i. Every lane of a warp
  // runs the same number of steps so the ballots stay converged.
  const int lane = threadIdx.x & 31;
  const uint64_t stride = static_cast<uint64_t>(R) * gridDim.x * blockDim.x;
  const uint64_t warp_first =
      ((static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5) * (32 * R);
  // the next step's rows are in flight while the queries run over the current ones
  uint4 na[R], nb[R];
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const uint64_t r = warp_first + lane + 32 * i;
    na[i] = nb[i] = make_uint4(0, 0, 0, 0);
    if (r < n_rows) {
      na[i] = ld_stream(rows + 2 * r);
      nb[i] = ld_stream(rows + 2 * r + 1);
    }
  }
  for (uint64_t base = warp_first; base < n_rows; base += stride) {
    uint64_t r[R];
    bool v[R];
    uint4 a[R], b[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
      r[i] = base + lane + 32 * i;
      v[i] = r[i] < n_rows;
      a[i] = na[i];
      b[i] = nb[i];
      if (r[i] + stride < n_rows) {
        na[i] = ld_stream(rows + 2 * (r[i] + stride));
        nb[i] = ld_stream(rows + 2 * (r[i] + stride) + 1);
      }
    }
#pragma unroll(R == 1 ? 4 : 2)
    for (uint32_t q = 0; q < nq; ++q) {
      const uint4 qa = sq[2 * q];
      uint32_t d[R];
      if constexpr (kPrefix == 3) {
        bool near = false;
#pragma unroll
        for (int i = 0; i < R; ++i) {
          d[i] = popc3(a[i].x ^ qa.x, a[i].y ^ qa.y, a[i].z ^ qa.z);
          near |= d[i] <= t;
        }
        if (!__any_sync(0xffffffffu, near)) continue;
        const uint4 qb = sq[2 * q + 1];
#pragma unroll
        for (int i = 0; i < R; ++i)
          d[i] += popc5(a[i].w ^ qa.w, b[i].x ^ qb.x, b[i].y ^ qb.y, b[i].z ^ qb.z, b[i].w ^ qb.w);
      } else if constexpr (kPrefix == 5) {
        const uint4 qb = sq[2 * q + 1];
        bool near = false;
#pragma unroll
        for (int i = 0; i < R; ++i) {
          d[i] = popc5(a[i].x ^ qa.x, a[i].y ^ qa.y, a[i].z ^ qa.z, a[i].w ^ qa.w, b[i].x ^ qb.x);
          near |= d[i] <= t;
        }
        if (!__any_sync(0xffffffffu, near)) continue;
#pragma unroll
        for (int i = 0; i < R; ++i) d[i] += popc3(b[i].y ^ qb.y, b[i].z ^ qb.z, b[i].w ^ qb.w);
      } else {
        const uint4 qb = sq[2 * q + 1];
#pragma unroll
        for (int i = 0; i < R; ++i)
          d[i] = popc8(make_uint4(a[i].x ^ qa.x, a[i].y ^ qa.y, a[i].z ^ qa.z, a[i].w ^ qa.w),
                       make_uint4(b[i].x ^ qb.x, b[i].y ^ qb.y, b[i].z ^ qb.z, b[i].w ^ qb.w));
      }
      bool h[R], any_hit = false;
#pragma unroll
      for (int i = 0; i < R; ++i) {
        h[i] = v[i] && d[i] <= t;
        any_hit |= h[i];
      }
      if (__any_sync(0xffffffffu, any_hit)) {
#pragma unroll
        for (int i = 0; i < R; ++i) emit_hits_ballot(h[i], r[i], q_base + q, d[i], hits, cap, count);
      }
    }
  }
}

// ------------------------------------------------------------------ B1 MMA

__device__ __forceinline__ void mma_b1_xor_popc(uint32_t a0, uint32_t a1, uint32_t a2,
                                                uint32_t a3, uint32_t b0, uint32_t b1,
                                                uint32_t& d0, uint32_t& d1, uint32_t& d2,
                                                uint32_t& d3) {
  asm volatile(
      "mma.sync.aligned.m16n8k256.row.col.s32.b1.b1.s32.xor.popc "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%10,%10,%10,%10};"
      : "=r"(d0), "=r"(d1), "=r"(d2), "=r"(d3)
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1), "r"(0));
}

// Fragment layout of m16n8k256 (.b1): lane = 4*g + tq holds
//   a0: row g,   k = 32 tq .. 32 tq + 31      a2: row g,   k = 128 + 32 tq ..
//   a1: row g+8, k = 32 tq ..                 a3: row g+8, k = 128 + 32 tq ..
//   b0: col (query) g, k = 32 tq ..           b1: col g,   k = 128 + 32 tq ..
//   d0,d1: row g, queries 2tq, 2tq+1          d2,d3: row g+8, queries 2tq, 2tq+1
// The distance is a popcount over all k, so any fixed word <-> k-slot assignment works as
// long as rows and queries use the same one: k-slot tq <-> word 2tq, slot 128+32tq <->
// word 2tq+1. Each lane then loads one 8-byte pair of words per row.
__global__ void __launch_bounds__(kScanThreads)
    scan_b1_kernel(const uint2* __restrict__ rows, uint64_t n_rows,
                   const uint2* __restrict__ queries, uint32_t nq, uint32_t q_base, uint32_t t,
                   ypdq_hit* hits, uint64_t cap, unsigned long long* count) {
  extern __shared__ uint2 sfrag[];  // [chunks][32 lanes]
  const uint32_t chunks = (nq + 7) / 8;
  for (uint32_t idx = threadIdx.x; idx < chunks * 32; idx += blockDim.x) {
    const uint32_t c = idx >> 5, l = idx & 31, g = l >> 2, tq = l & 3;
    const uint32_t qi = 8 * c + g;
    sfrag[idx] = qi < nq ? queries[qi * 4 + tq] : make_uint2(0, 0);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const uint32_t g = lane >> 2, tq = lane & 3;
  const uint64_t warp = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const uint64_t n_warps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  const uint64_t n_tiles = (n_rows + 15) / 16;
  for (uint64_t tile = warp; tile < n_tiles; tile += n_warps) {
    const uint64_t r0 = tile * 16 + g, r1 = r0 + 8;
    uint2 A0 = make_uint2(0, 0), A1 = make_uint2(0, 0);
    if (r0 < n_rows) A0 = rows[r0 * 4 + tq];
    if (r1 < n_rows) A1 = rows[r1 * 4 + tq];
    for (uint32_t c = 0; c < chunks; ++c) {
      const uint2 B = sfrag[c * 32 + lane];
      uint32_t d0, d1, d2, d3;
      mma_b1_xor_popc(A0.x, A1.x, A0.y, A1.y, B.x, B.y, d0, d1, d2, d3);
      const uint32_t q0 = 8 * c + 2 * tq, q1 = q0 + 1;
      const bool h0 = r0 < n_rows && q0 < nq && d0 <= t;
      const bool h1 = r0 < n_rows && q1 < nq && d1 <= t;
      const bool h2 = r1 < n_rows && q0 < nq && d2 <= t;
      const bool h3 = r1 < n_rows && q1 < nq && d3 <= t;
      if (__any_sync(0xffffffffu, h0 | h1 | h2 | h3)) {
        emit_hits_ballot(h0, r0, q_base + q0, d0, hits, cap, count);
        emit_hits_ballot(h1, r0, q_base + q1, d1, hits, cap, count);
        emit_hits_ballot(h2, r1, q_base + q0, d2, hits, cap, count);
        emit_hits_ballot(h3, r1, q_base + q1, d3, hits, cap, count);
      }
    }
  }
}

cudaError_t scan_init() {
  const int smem = static_cast<int>(kMaxSmemQueries * 32);
  cudaError_t e = cudaSuccess;
  for (const void* f : {reinterpret_cast<const void*>(scan_simt_kernel<3>),
                        reinterpret_cast<const void*>(scan_simt_kernel<5>),
                        reinterpret_cast<const void*>(scan_simt_kernel<8>)}) {
    e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
  }
  e = cudaFuncSetAttribute(scan_b1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  return scan_tc_init();
}

// SIMT is HBM-bound up to a few queries; past that it is bound by its popcount and logic
// pipes, at 2, 3 or 4 popcounts per pair depending on the threshold (the prefix bound in
// scan_simt_kernel). A narrow tensor-core pass (at most 128 queries) costs about the time of
// 9 SIMT queries at t <= 34 (10M rows: 0.072-0.078 ms against 0.066 ms for 8 SIMT queries
// and 0.080 ms for 10), 6 at t = 35..36 (the SIMT side at three popcounts: 0.071 ms for 6,
// 0.088 ms for 8), 24 at t <= 62 and 12 above (the FP8 passes, neither side pruned as far).
int auto_scan_algo(uint32_t n_queries, uint32_t threshold) {
  const uint32_t simt_max = threshold <= 34 ? 9 : threshold <= 36 ? 6 : threshold <= 62 ? 24 : 12;
  return n_queries <= simt_max ? YPDQ_SCAN_SIMT : YPDQ_SCAN_TC;
}

cudaError_t launch_scan(const ScanLaunch& p, int algo, int num_sms, cudaStream_t s) {
  cudaError_t e = p.append ? cudaSuccess : cudaMemsetAsync(p.count, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess || p.n_rows == 0 || p.n_queries == 0) return e;
  if (algo == YPDQ_SCAN_AUTO) algo = auto_scan_algo(p.n_queries, p.threshold);
  if (algo == YPDQ_SCAN_TC) return launch_scan_tc(p, num_sms, s);
  if (algo == YPDQ_SCAN_TC_FP4) {
    ScanLaunch q = p;
    if (p.threshold <= 36) q.pair_n = kPairFp4N;  // FP4, three queries per column
    return launch_scan_tc(q, num_sms, s);
  }
  if (algo == YPDQ_SCAN_TC_FP8) {
    // FP8 at t <= 36 too: query pairs past 256 queries, else one pass of up to 256
    ScanLaunch q = p;
    if (p.threshold <= 36) {
      if (p.n_queries > 256)
        q.pair_n = 256;
      else
        q.n_tile = (p.n_queries + 63u) & ~63u;
    }
    return launch_scan_tc(q, num_sms, s);
  }
  // a device-side query count needs the whole query set in one launch
  if (p.nq_dev && (algo != YPDQ_SCAN_SIMT || p.n_queries > kMaxSmemQueries))
    return cudaErrorInvalidValue;
  for (uint32_t q0 = 0; q0 < p.n_queries; q0 += kMaxSmemQueries) {
    const uint32_t nq = (p.n_queries - q0) < kMaxSmemQueries ? (p.n_queries - q0) : kMaxSmemQueries;
    const uint8_t* qptr = p.queries + static_cast<size_t>(q0) * 32;
    if (algo == YPDQ_SCAN_B1MMA) {
      const uint64_t tiles = (p.n_rows + 15) / 16;
      uint64_t blocks = (tiles + (kScanThreads / 32) - 1) / (kScanThreads / 32);
      const uint64_t cap_blocks = static_cast<uint64_t>(num_sms) * 8;
      if (blocks > cap_blocks) blocks = cap_blocks;
      const size_t smem = static_cast<size_t>((nq + 7) / 8) * 32 * sizeof(uint2);
      scan_b1_kernel<<<static_cast<unsigned>(blocks), kScanThreads, smem, s>>>(
          reinterpret_cast<const uint2*>(p.rows), p.n_rows, reinterpret_cast<const uint2*>(qptr),
          nq, p.query_base + q0, p.threshold, p.hits, p.capacity, p.count);
    } else {
      const size_t smem = static_cast<size_t>(nq) * 32;
      const int prefix = p.threshold <= 34 ? 3 : p.threshold <= 62 ? 5 : 8;
      auto kern = prefix == 3 ? scan_simt_kernel<3> : prefix == 5 ? scan_simt_kernel<5>
                                                                  : scan_simt_kernel<8>;
      // blocks per SM: registers allow simt_blocks_per_sm; the queries' shared memory (plus
      // the 1 KiB the runtime reserves per block, of 228 KiB per SM) may allow fewer
      const uint64_t fit = (228u << 10) / (smem + 1024);
      const uint64_t bps = static_cast<uint64_t>(simt_blocks_per_sm(prefix));
      const uint64_t rows_per_block = static_cast<uint64_t>(kScanThreads) * simt_rows(prefix);
      uint64_t blocks = (p.n_rows + rows_per_block - 1) / rows_per_block;
      const uint64_t cap_blocks = static_cast<uint64_t>(num_sms) * (fit < bps ? fit : bps);
      if (blocks > cap_blocks) blocks = cap_blocks;
      kern<<<static_cast<unsigned>(blocks), kScanThreads, smem, s>>>(
          reinterpret_cast<const uint4*>(p.rows), p.n_rows, reinterpret_cast<const uint4*>(qptr),
          nq, p.query_base + q0, p.threshold, p.hits, p.capacity, p.count, p.nq_dev);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// ---------------------------------------------------------------- hit sorting

// Order by (index, query): the scalar matcher's visit order.
__device__ __forceinline__ bool hit_less(const ypdq_hit& a, const ypdq_hit& b) {
  return a.index < b.index || (a.index == b.index && a.query < b.query);
}

// One compare-exchange step of a bitonic sort in the "flip" form: every comparison puts
// the smaller hit at the lower index, so the virtual +infinity padding past n (up to the
// next power of two) never has to move and is never stored.
__global__ void bitonic_step_kernel(ypdq_hit* h, uint64_t n, uint64_t k, uint64_t j, int flip) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t l;
  if (flip) {
    if (i & (k >> 1)) return;
    l = i ^ (k - 1);
  } else {
    if (i & j) return;
    l = i ^ j;
  }
  if (l >= n) return;  // partner is padding: the real element is already the smaller
  const ypdq_hit a = h[i], b = h[l];
  if (hit_less(b, a)) {
    h[i] = b;
    h[l] = a;
  }
}

// The steps of the same sort whose partners lie inside one 2,048-hit block, done in shared
// memory in one launch. full != 0: every stage k = 2 .. k_last (<= 2,048), each its flip
// step and then j = k/4 .. 1. full == 0: the steps j = 1,024 .. 1 of stage k_last (> 2,048),
// whose wider steps ran as global launches. Positions past n hold a +infinity hit, which
// compares above every real one exactly as the global kernel's skipped padding does.
constexpr int kSortBlock = 2048;
__global__ void __launch_bounds__(kSortBlock / 2)
    bitonic_block_kernel(ypdq_hit* h, uint64_t n, uint64_t k_last, int full) {
  __shared__ ypdq_hit sh[kSortBlock];
  const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kSortBlock;
  const int t = threadIdx.x;
  ypdq_hit inf;
  inf.index = ~0ull;
  inf.query = ~0u;
  inf.distance = ~0u;
  for (int x = t; x < kSortBlock; x += kSortBlock / 2)
    sh[x] = base + x < n ? h[base + x] : inf;
  __syncthreads();
  auto step = [&](uint32_t j, bool flip, uint32_t k) {
    // thread t owns the pair whose lower position has bit j clear
    const uint32_t i = ((t & ~(j - 1)) << 1) | (t & (j - 1));
    const uint32_t l = flip ? (i ^ (k - 1)) : (i | j);
    const ypdq_hit a = sh[i], b = sh[l];
    if (hit_less(b, a)) {
      sh[i] = b;
      sh[l] = a;
    }
    __syncthreads();
  };
  if (full) {
    for (uint32_t k = 2; k <= k_last; k <<= 1) {
      step(k >> 1, true, k);
      for (uint32_t j = k >> 2; j > 0; j >>= 1) step(j, false, k);
    }
  } else {
    for (uint32_t j = kSortBlock / 2; j > 0; j >>= 1) step(j, false, 0);
  }
  for (int x = t; x < kSortBlock; x += kSortBlock / 2)
    if (base + x < n) h[base + x] = sh[x];
}

cudaError_t launch_sort_hits(ypdq_hit* hits, uint64_t n, cudaStream_t s) {
  if (n < 2) return cudaSuccess;
  uint64_t padded = 1;
  while (padded < n) padded <<= 1;
  const unsigned threads = 256;
  const unsigned blocks = static_cast<unsigned>((n + threads - 1) / threads);
  const unsigned sblocks = static_cast<unsigned>((n + kSortBlock - 1) / kSortBlock);
  const uint64_t first = padded < static_cast<uint64_t>(kSortBlock) ? padded : kSortBlock;
  bitonic_block_kernel<<<sblocks, kSortBlock / 2, 0, s>>>(hits, n, first, 1);
  for (uint64_t k = 2 * kSortBlock; k <= padded; k <<= 1) {
    bitonic_step_kernel<<<blocks, threads, 0, s>>>(hits, n, k, k >> 1, 1);
    for (uint64_t j = k >> 2; j >= static_cast<uint64_t>(kSortBlock); j >>= 1)
      bitonic_step_kernel<<<blocks, threads, 0, s>>>(hits, n, k, j, 0);
    bitonic_block_kernel<<<sblocks, kSortBlock / 2, 0, s>>>(hits, n, k, 0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

}  // namespace ypdq
