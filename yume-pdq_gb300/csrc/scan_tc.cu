// Exact Hamming scan on the 5th-generation tensor cores (tcgen05, kind::f8f6f4).
//
// Each bit b of a 256-bit hash becomes the FP8 (e4m3) value s = 1 - 2b, i.e. +1.0 or -1.0.
// For a database row r and a query q the dot product of the two sign vectors is
//     sum_k s_r[k] s_q[k] = 256 - 2 * popcount(r ^ q),
// an integer in [-256, 256]. Every product is exactly +-1 and every partial sum an integer
// of magnitude <= 256, so even an f16 accumulator (11-bit significand) holds it exactly and
//     distance = (256 - dot) / 2,    hit  <=>  dot >= 256 - 2 * threshold.
// The hit set equals the scalar matcher's (CpuMatcher::find, src/matching/mod.rs:336-362).
//
// CTA (one per SM, persistent over 128-row database tiles; 14 warps, 15 with kDual):
//   warps 0-7   epilogue: tcgen05.ld the 128 x N f16 accumulator, two warps per TMEM lane
//               quarter (warp w reads lanes 32(w%4).. = tile rows; the two groups take
//               alternate 64-column chunks, or with kDual and N = 64 alternate tiles),
//               hand the stage back, then a half2 max per 64 columns against the
//               threshold; the rare chunk with a hit becomes a per-lane column mask whose
//               hits are written with one atomic per warp. One f16 is read per (row, query)
//               pair, so the readout gets twice the warps of the other roles (four per
//               quarter were slower: the extra warps take issue slots from the expanders).
//   warp 8      producer: one lane bulk-copies packed tiles (128 rows x 32 B) into a ring.
//   warps 9, 14 MMA: one lane issues kKSteps tcgen05.mma (M=128, N, K=32) per tile into a
//               double-buffered accumulator and commits to mbarriers (tcgen05.commit tracks
//               the issuing thread's own MMAs). Issuing and its barrier handoffs keep one
//               thread busy ~1,100 clk per tile, longer than the MMAs of a pass of <= 128
//               queries take on the tensor core; there (kDual) the two warps take alternate
//               tiles, one accumulator stage each. Wider passes launch without warp 14.
//               Warp 9 also allocates and frees TMEM.
//   warps 10-13 expanders: packed bits -> FP8 +-1. The queries (B, once per pass) go to
//               shared memory in the 128B-swizzled K-major layout that the MMA descriptors
//               describe. The database tiles (A) go there too for passes of 192-256
//               queries; with kDual they go straight into tensor memory with tcgen05.st (row
//               r = TMEM lane r, K in column order) and the MMA reads A from there: a narrow
//               pass is otherwise bound by shared-memory traffic (expansion stores plus the
//               MMA's operand reads), and the columns the accumulators leave free hold 4-8
//               tiles in flight.
// Queries are processed in passes of N <= 256; the database streams once per pass. The
// shared memory left after the operands holds as many packed tiles in flight as fit.
//
// kKSteps < 8 (a prefix bound): only the first 32 * kKSteps bits of rows and queries are
// expanded and multiplied (kKSteps MMAs per tile instead of 8): 128 bits at t <= 36 (any
// pass width), 192 bits at t <= 62 (passes of 256 queries). Their distance is a lower bound
// of the full one, so a pair can only be a hit if that partial distance is <= t; the
// epilogue re-checks every such candidate exactly with popcounts of the packed row and
// query and reports the exact distance. For random rows a 128-bit partial distance is
// 64 +- 6 and a 192-bit one 96 +- 7, so candidates are rare and the hit set is the full
// scan's.
#include <cuda_fp16.h>

#include <atomic>
#include <type_traits>

#include "capi_internal.h"
#include "ypdq_internal.cuh"

namespace ypdq {

namespace tc {

constexpr int kEpilogueWarps = 8;  // warps 0..7
constexpr int kProducerWarp = 8;
constexpr int kMmaWarp = 9;
constexpr int kExpandWarp0 = 10;   // warps 10..13
constexpr int kMmaWarp2 = 14;      // the second MMA issuer (kDual only)
__host__ __device__ constexpr int threads_of(bool dual) { return (dual ? 15 : 14) * 32; }
constexpr int kTileRows = 128;
constexpr int kMaxN = 256;
constexpr int kMaxPackStages = 16;
constexpr int kAStages = 4;       // A tiles in shared memory (32 KiB each)
constexpr int kMaxAStages = 8;    // A tiles in tensor memory (kDual; 64 or 32 columns each)
constexpr int kAccStages = 2;
constexpr int kTmemCols = 512;
constexpr int kChunkBytes = kTileRows * 128;  // one 128-byte K-chunk of a 128-row tile
constexpr int kPackBytes = kTileRows * 32;
constexpr size_t kSmemLimit = 227 * 1024;

// Fixed part of shared memory; the expanded tiles (shared-memory A only: kAStages x 2
// K-chunks of 128 rows x 128 B), the expanded queries (2 K-chunks of N x 128 B) and the
// packed ring follow it at 1024-byte aligned offsets computed per launch.
struct Smem {
  uint64_t pk_full[kMaxPackStages], pk_empty[kMaxPackStages];
  uint64_t a_full[kMaxAStages], a_empty[kMaxAStages];
  uint64_t acc_full[kAccStages], acc_empty[kAccStages];
  uint64_t b_full, b_empty, epi_exit, exp_exit, mma_done;
  uint32_t tmem_base;
  int abort_flag;
};
constexpr size_t kFixedBytes = (sizeof(Smem) + 1023) & ~static_cast<size_t>(1023);

__device__ __forceinline__ void mma_f8(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                       uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// The same with A read from tensor memory (128 lanes = rows, K along the columns).
__device__ __forceinline__ void mma_f8_ta(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], [%1], %2, %3, p;\n\t}" ::"r"(tmem_d),
      "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// Store 32 consecutive 32-bit columns of this warp's 32 TMEM lanes (one row per lane).
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
}
__device__ __forceinline__ void tmem_st_wait() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// Issue a load of 32 consecutive columns of this warp's 32 TMEM lanes. The registers are
// written asynchronously: read them only through tmem_take() after tmem_ld_wait().
__device__ __forceinline__ void tmem_ld32_nowait(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
}
// After tmem_ld_wait(): pass the registers through an empty volatile asm so that no use of
// them can be scheduled above the wait.
__device__ __forceinline__ void tmem_take(uint32_t (&r)[32], float (&v)[32]) {
  asm volatile("" : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]), "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]), "+r"(r[29]), "+r"(r[30]), "+r"(r[31]));
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Issue a load of 64 consecutive columns of this warp's 32 TMEM lanes holding 16-bit
// values; column pairs (2i, 2i+1) arrive packed in r[i]. Valid only after tmem_ld_wait().
__device__ __forceinline__ void tmem_ld64_pack16_nowait(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.pack::16b.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
}

// Instruction descriptor: D f16, A and B e4m3, both K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t idesc_f8(uint32_t n) {
  return (0u << 4) | (0u << 7) | (0u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

// 4 bits -> 4 e4m3 bytes: bit 0 -> 0x38 (+1.0), bit 1 -> 0xB8 (-1.0).
// Expand one packed 32-byte row (database row or query) into the 128B-swizzled K-major e4m3
// operand, +1 (0x38) for a clear bit and -1 (0xB8) for a set bit. The dot product of two
// expanded rows is 256 - 2 * Hamming distance for ANY bijection between the 256 bit
// positions and the 256 K positions, as long as rows and queries use the same one. This one
// makes each 4-byte output word a shift, a mask and an OR: byte i of output word m (m = 0..7)
// of packed word p holds bit 8i + 7 - m of that word, which `<< m` moves to the byte's sign
// bit. Output word (p, m) goes to K chunk p / 4, 16-byte unit 2 (p % 4) + m / 4.
// kWords < 8: only packed words 0 .. kWords - 1 (the first 32 * kWords bits).
// kOne: the magnitude's byte, repeated (e4m3 1.0 = 0x38; the pair kernel below uses e5m2
// 1.0 = 0x3C and 512.0 = 0x60); the data bit becomes the sign bit.
template <int kWords = 8, uint32_t kOne = 0x38383838u>
__device__ __forceinline__ void expand_row(const uint4 w0, const uint4 w1, uint8_t* chunk0,
                                           uint8_t* chunk1, int row) {
  const uint32_t words[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
  const int sw = row & 7;
#pragma unroll
  for (int p = 0; p < kWords; ++p) {
    uint8_t* base = (p < 4 ? chunk0 : chunk1) + row * 128;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint32_t w = words[p];
      uint4 out;
      out.x = ((w << (4 * h + 0)) & 0x80808080u) | kOne;
      out.y = ((w << (4 * h + 1)) & 0x80808080u) | kOne;
      out.z = ((w << (4 * h + 2)) & 0x80808080u) | kOne;
      out.w = ((w << (4 * h + 3)) & 0x80808080u) | kOne;
      const int unit = 2 * (p & 3) + h;
      *reinterpret_cast<uint4*>(base + ((unit ^ sw) << 4)) = out;
    }
  }
}

// The expansion of expand_row as 64 column words of one TMEM lane: K element 4 c + i is
// byte i of column c. Output word (p, m) of expand_row holds K elements 32 p + 4 m .. + 3,
// so it is column 8 p + m, and rows and queries keep the same bijection. kHalf: the first
// 32 columns only (packed words 0..3, the first 128 bits).
template <bool kHalf = false>
__device__ __forceinline__ void expand_row_tmem(const uint4 w0, const uint4 w1,
                                                uint32_t taddr) {
  const uint32_t words[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
  for (int half = 0; half < (kHalf ? 1 : 2); ++half) {
    uint32_t r[32];
#pragma unroll
    for (int pp = 0; pp < 4; ++pp) {
      const uint32_t w = words[4 * half + pp];
#pragma unroll
      for (int m = 0; m < 8; ++m) r[8 * pp + m] = ((w << m) & 0x80808080u) | 0x38383838u;
    }
    tmem_st32(taddr + 32 * half, r);
  }
}

struct Params {
  const uint8_t* rows;
  uint64_t n_rows;
  const uint8_t* queries;
  uint32_t n_queries;
  uint32_t n_tile;       // N: queries per pass (multiple of 32, <= 256)
  uint32_t threshold;
  ypdq_hit* hits;
  uint64_t capacity;
  unsigned long long* count;
  int* dev_err;
  uint32_t query_base;    // added to reported query numbers
  const uint32_t* nq_dev; // device-side query count (graph replay), bounded by n_queries
  uint32_t nq_off;        // scan_rows3_kernel: this launch's first query of the *nq_dev ones
  uint32_t pack_stages;   // packed tiles in flight (<= kMaxPackStages)
  uint32_t pack_offset;   // byte offset of the packed ring in shared memory
  uint32_t a_stages;      // expanded tiles in flight
  uint32_t b_offset;      // byte offset of the expanded queries
  uint64_t wait_ns;       // longest barrier wait before the kernel gives up (timeout flag)
  int stall;              // testing: the producer issues no copies, so the waits run out
};

__device__ __forceinline__ uint32_t popc256(uint4 a0, uint4 a1, uint4 b0, uint4 b1) {
  return __popc(a0.x ^ b0.x) + __popc(a0.y ^ b0.y) + __popc(a0.z ^ b0.z) + __popc(a0.w ^ b0.w) +
         __popc(a1.x ^ b1.x) + __popc(a1.y ^ b1.y) + __popc(a1.z ^ b1.z) + __popc(a1.w ^ b1.w);
}

// Bit j set when column j of the 64 in raw (f16 pairs, one row) holds a dot product of at
// least dot_min: a hit, or with a prefix bound a candidate.
__device__ __forceinline__ uint64_t candidate_mask(const uint32_t (&raw)[32], float dot_min) {
  uint32_t lo = 0, hi = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const __half2 a = *reinterpret_cast<const __half2*>(&raw[i]);
    const __half2 b = *reinterpret_cast<const __half2*>(&raw[16 + i]);
    lo |= (__low2float(a) >= dot_min ? 1u : 0u) << (2 * i);
    lo |= (__high2float(a) >= dot_min ? 1u : 0u) << (2 * i + 1);
    hi |= (__low2float(b) >= dot_min ? 1u : 0u) << (2 * i);
    hi |= (__high2float(b) >= dot_min ? 1u : 0u) << (2 * i + 1);
  }
  return (static_cast<uint64_t>(hi) << 32) | lo;
}

// Report this lane's candidates (bit j of cand: query q_first + j against `row`): the exact
// distance of each from popcounts of the packed row and query, the ones within the threshold
// written as hits at positions taken with one atomic per warp. Called by all 32 lanes; a
// lane without candidates passes cand = 0. The loops run once per candidate of the lane,
// which keeps this rare path short: it runs while the tile's epilogue warp holds up the next
// tile, and a planted near-duplicate row makes it run for several queries of a pass.
// (stride: bit j of cand stands for query q_first + stride * j; 1 unless given.)
__device__ __forceinline__ void emit_candidates(uint64_t cand, uint64_t row, uint64_t q_first,
                                                uint32_t n_queries, const Params& prm,
                                                int lane, uint32_t stride = 1) {
  {
    // bits whose query is past the end
    const uint64_t lim = q_first >= n_queries ? 0 : (n_queries - q_first + stride - 1) / stride;
    if (lim < 64) cand &= (1ull << lim) - 1;
  }
  uint4 r0 = make_uint4(0, 0, 0, 0), r1 = r0;
  if (cand) {
    const uint4* rp = reinterpret_cast<const uint4*>(prm.rows + row * 32);
    r0 = __ldg(rp);
    r1 = __ldg(rp + 1);
  }
  const uint8_t* const qbase = prm.queries + q_first * 32;
  uint64_t hits = 0;
  for (uint64_t m = cand; m; m &= m - 1) {
    const int j = __ffsll(static_cast<long long>(m)) - 1;
    const uint4* qp = reinterpret_cast<const uint4*>(qbase + static_cast<uint64_t>(stride) * j * 32);
    if (popc256(r0, r1, __ldg(qp), __ldg(qp + 1)) <= prm.threshold) hits |= 1ull << j;
  }
  const uint32_t mine = static_cast<uint32_t>(__popcll(hits));
  uint32_t incl = mine;  // inclusive prefix sum over the lanes
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  if (total == 0) return;
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(prm.count, static_cast<unsigned long long>(total));
  base = __shfl_sync(0xffffffffu, base, 0);
  uint64_t pos = base + incl - mine;
  for (uint64_t m = hits; m; m &= m - 1, ++pos) {
    if (pos >= prm.capacity) break;
    const int j = __ffsll(static_cast<long long>(m)) - 1;
    const uint4* qp = reinterpret_cast<const uint4*>(qbase + static_cast<uint64_t>(stride) * j * 32);
    ypdq_hit h;
    h.index = row;
    h.query = static_cast<uint32_t>(q_first + static_cast<uint64_t>(stride) * j) + prm.query_base;
    h.distance = popc256(r0, r1, __ldg(qp), __ldg(qp + 1));
    prm.hits[pos] = h;
  }
}

// emit_candidates as a call: the pair kernel's epilogue reaches it only on the rare tiles with a
// candidate, and inlined at each of its chunks it would crowd the registers of the common path.
__device__ __noinline__ void emit_candidates_call(uint64_t cand, uint64_t row, uint64_t q_first,
                                                  uint32_t n_queries, const Params* prm,
                                                  int lane, uint32_t stride) {
  emit_candidates(cand, row, q_first, n_queries, *prm, lane, stride);
}

__device__ __forceinline__ void raise_abort(Smem& sm, int* dev_err) {
  *reinterpret_cast<volatile int*>(&sm.abort_flag) = 1;
  atomicOr(dev_err, kDevErrTimeout);
}

template <bool kDual, int kKSteps>
__global__ void __launch_bounds__(threads_of(kDual), 1) scan_tc_kernel(const Params prm) {
  static_assert(kKSteps == 4 || kKSteps == 8 || (!kDual && kKSteps == 6), "K steps");
  constexpr uint32_t kACols = kKSteps == 4 ? 32 : 64;  // TMEM columns of one A tile (kDual)
  extern __shared__ uint8_t smem_raw[];
  // Align by offsetting the shared array itself so the compiler keeps the shared address
  // space (an integer round trip would turn every access into a generic one).
  uint8_t* const smem_base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  Smem& sm = *reinterpret_cast<Smem*>(smem_base);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t N = prm.n_tile;
  const uint32_t n_pack = prm.pack_stages;
  const uint32_t n_queries = prm.nq_dev ? min(*prm.nq_dev, prm.n_queries) : prm.n_queries;
  const uint32_t n_a = kDual ? prm.a_stages : static_cast<uint32_t>(kAStages);
  uint8_t* const a_smem = smem_base + kFixedBytes;    // [kAStages][2][kChunkBytes] (!kDual)
  uint8_t* const bchunk0 = smem_base + prm.b_offset;  // N rows x 128 B (K 0..127)
  uint8_t* const bchunk1 = bchunk0 + N * 128;         // N rows x 128 B (K 128..255)
  uint8_t* const packed = smem_base + prm.pack_offset;
  const uint64_t n_tiles = (prm.n_rows + kTileRows - 1) / kTileRows;
  const uint32_t n_passes = (n_queries + N - 1) / N;
  // tiles of this CTA: blockIdx.x, blockIdx.x + gridDim.x, ...
  const uint64_t my_tiles =
      blockIdx.x < n_tiles ? (n_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  volatile int* abort_flag = &sm.abort_flag;

  if (tid == 0) {
    for (uint32_t s = 0; s < n_pack; ++s) {
      mbar_init(&sm.pk_full[s], 1);
      mbar_init(&sm.pk_empty[s], 4);
    }
    for (uint32_t s = 0; s < n_a; ++s) {
      mbar_init(&sm.a_full[s], 4);
      mbar_init(&sm.a_empty[s], 1);
    }
    for (int s = 0; s < kAccStages; ++s) {
      mbar_init(&sm.acc_full[s], 1);
      // kDual with N = 64: each epilogue group drains one accumulator stage (alternate tiles)
      mbar_init(&sm.acc_empty[s], kDual && N <= 64 ? kEpilogueWarps / 2 : kEpilogueWarps);
    }
    mbar_init(&sm.b_full, 4);
    mbar_init(&sm.b_empty, kDual ? 2 : 1);   // one commit per MMA issuer
    mbar_init(&sm.epi_exit, kEpilogueWarps);
    mbar_init(&sm.exp_exit, 4);
    mbar_init(&sm.mma_done, kDual ? 2 : 1);
    sm.abort_flag = 0;
    fence_mbar_init();
  }
  // columns: kAccStages accumulators of N, then (kDual) n_a A tiles of 64 columns
  const uint32_t tmem_cols =
      kDual ? static_cast<uint32_t>(kTmemCols)
            : (2 * N <= 32 ? 32 : (2 * N <= 64 ? 64 : (2 * N <= 128 ? 128 : (2 * N <= 256 ? 256 : 512))));
  const uint32_t a_col0 = kAccStages * N;
  if (warp == kMmaWarp) {
    tmem_alloc(&sm.tmem_base, tmem_cols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = sm.tmem_base;
  if (my_tiles == 0) {
    if (warp == kMmaWarp) tmem_dealloc(tmem_base, tmem_cols);
    return;
  }

  if (warp == kProducerWarp) {
    if (lane == 0 && !prm.stall) {
      uint32_t slot = 0, phase = 0, issued = 0;
      bool ok = true;
      for (uint32_t p = 0; p < n_passes && ok; ++p) {
        for (uint64_t k = 0; k < my_tiles; ++k) {
          const uint64_t tile = blockIdx.x + k * gridDim.x;
          if (!mbar_wait(&sm.pk_empty[slot], phase ^ 1u, abort_flag, prm.wait_ns)) {
            ok = false;
            break;
          }
          const uint64_t r0 = tile * kTileRows;
          const uint64_t nr = (prm.n_rows - r0) < kTileRows ? (prm.n_rows - r0) : kTileRows;
          const uint32_t bytes = static_cast<uint32_t>(nr * 32);
          mbar_arrive_expect_tx(&sm.pk_full[slot], bytes);
          bulk_g2s(packed + slot * kPackBytes, prm.rows + r0 * 32, bytes, &sm.pk_full[slot],
                   policy_evict_first());
          ++issued;
          if (++slot == n_pack) {
            slot = 0;
            phase ^= 1u;
          }
        }
      }
      if (!ok) {
        raise_abort(sm, prm.dev_err);
        // let the copies already issued land (bounded): they sit in the n_pack slots before
        // `slot`; those at or past `slot` were issued in the previous phase
        for (uint32_t k = 1; k <= n_pack && k <= issued; ++k) {
          const uint32_t sl = (slot + n_pack - k) % n_pack;
          const uint32_t ph = (k <= slot) ? phase : (phase ^ 1u);
          const uint64_t t0 = globaltimer_ns();
          while (!mbar_try_wait(&sm.pk_full[sl], ph))
            if (globaltimer_ns() - t0 > prm.wait_ns / 4) break;
        }
      }
    }
    return;
  }

  if (warp >= kExpandWarp0 && warp < kExpandWarp0 + 4) {
    const int e = tid - kExpandWarp0 * 32;  // 0..127: query row
    // tile row: a warp may only access its own quarter of the TMEM lanes (warp % 4)
    const int arow = kDual ? 32 * (warp & 3) + lane : e;
    const uint32_t a_lane = static_cast<uint32_t>(32 * (warp & 3)) << 16;
    uint32_t slot = 0, phase = 0, ga = 0, as_t = 0, aph_t = 0;  // as_t, aph_t: kDual stages
    for (uint32_t p = 0; p < n_passes; ++p) {
      // queries of this pass into B (N rows; padding rows are zero = contributes nothing)
      if (!mbar_wait(&sm.b_empty, (p & 1u) ^ 1u, abort_flag, prm.wait_ns)) goto fail;
      for (uint32_t qr = e; qr < N; qr += 128) {
        const uint64_t qi = static_cast<uint64_t>(p) * N + qr;
        if (qi < n_queries) {
          const uint4* src = reinterpret_cast<const uint4*>(prm.queries + qi * 32);
          expand_row<kKSteps>(src[0], src[1], bchunk0, bchunk1, static_cast<int>(qr));
        } else {
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            *reinterpret_cast<uint4*>(bchunk0 + qr * 128 + u * 16) = make_uint4(0, 0, 0, 0);
            *reinterpret_cast<uint4*>(bchunk1 + qr * 128 + u * 16) = make_uint4(0, 0, 0, 0);
          }
        }
      }
      fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.b_full);

      for (uint64_t k = 0; k < my_tiles; ++k, ++ga) {
        const uint32_t as = kDual ? as_t : ga % kAStages;
        const uint32_t aph = kDual ? aph_t : (ga / kAStages) & 1u;
        if (!mbar_wait(&sm.pk_full[slot], phase, abort_flag, prm.wait_ns)) goto fail;
        const uint4* src = reinterpret_cast<const uint4*>(packed + slot * kPackBytes + arow * 32);
        const uint4 w0 = src[0], w1 = src[1];
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.pk_empty[slot]);
        if (++slot == n_pack) {
          slot = 0;
          phase ^= 1u;
        }
        if (!mbar_wait(&sm.a_empty[as], aph ^ 1u, abort_flag, prm.wait_ns)) goto fail;
        if constexpr (kDual) {
          __syncwarp();  // tcgen05.st is .sync.aligned: the lanes leave the wait one by one
          expand_row_tmem<kKSteps == 4>(w0, w1, tmem_base + a_lane + a_col0 + kACols * as);
          tmem_st_wait();
          tc_fence_before();
          if (++as_t == n_a) {
            as_t = 0;
            aph_t ^= 1u;
          }
        } else {
          uint8_t* a = a_smem + static_cast<size_t>(as) * 2 * kChunkBytes;
          expand_row<kKSteps>(w0, w1, a, a + kChunkBytes, arow);
          fence_proxy_async_smem();
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.a_full[as]);
      }
    }
    // no TMEM access by this warp after this point
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.exp_exit);
    return;
  fail:
    if (lane == 0) {
      raise_abort(sm, prm.dev_err);
      mbar_arrive(&sm.exp_exit);
    }
    return;
  }

  if (warp == kMmaWarp || (kDual && warp == kMmaWarp2)) {
    const uint32_t idesc = idesc_f8(N);
    const uint32_t issuer = warp == kMmaWarp ? 0u : 1u;  // kDual: takes the tiles ga % 2 == issuer
    uint32_t ga = 0, as_t = 0, aph_t = 0;  // as_t, aph_t: kDual stages, advanced every tile
    bool ok = true;
    if (lane == 0) {
      for (uint32_t p = 0; p < n_passes && ok; ++p) {
        if (!mbar_wait(&sm.b_full, p & 1u, abort_flag, prm.wait_ns)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t b0 = smem_u32(bchunk0), b1 = smem_u32(bchunk1);
        for (uint64_t k = 0; k < my_tiles; ++k, ++ga) {
          const uint32_t as = kDual ? as_t : ga % kAStages;
          const uint32_t aph = kDual ? aph_t : (ga / kAStages) & 1u;
          if (kDual && ++as_t == n_a) {
            as_t = 0;
            aph_t ^= 1u;
          }
          if (kDual && (ga & 1u) != issuer) continue;
          const uint32_t ac = ga % kAccStages;
          if (!mbar_wait(&sm.a_full[as], aph, abort_flag, prm.wait_ns) ||
              !mbar_wait(&sm.acc_empty[ac], ((ga / kAccStages) & 1u) ^ 1u, abort_flag, prm.wait_ns)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t d = tmem_base + ac * N;
          if constexpr (kDual) {
            const uint32_t ta = tmem_base + a_col0 + kACols * as;  // lane 0; K = 32 per 8 columns
#pragma unroll
            for (int ks = 0; ks < kKSteps; ++ks) {
              const uint64_t bd = sw128_desc((ks < 4 ? b0 : b1) + (ks & 3) * 32);
              mma_f8_ta(d, ta + 8 * ks, bd, idesc, ks > 0 ? 1u : 0u);
            }
          } else {
            const uint32_t a0 = smem_u32(a_smem + static_cast<size_t>(as) * 2 * kChunkBytes);
            const uint32_t a1 = a0 + kChunkBytes;
#pragma unroll
            for (int ks = 0; ks < kKSteps; ++ks) {
              const uint32_t off = (ks & 3) * 32;
              const uint64_t ad = sw128_desc((ks < 4 ? a0 : a1) + off);
              const uint64_t bd = sw128_desc((ks < 4 ? b0 : b1) + off);
              mma_f8(d, ad, bd, idesc, ks > 0 ? 1u : 0u);
            }
          }
          mma_commit(&sm.a_empty[as]);
          mma_commit(&sm.acc_full[ac]);
        }
        if (ok) mma_commit(&sm.b_empty);
      }
      if (!ok) raise_abort(sm, prm.dev_err);
      // every MMA of both issuers has completed once both commits arrive
      mma_commit(&sm.mma_done);
      const uint64_t t0 = globaltimer_ns();
      while (!mbar_try_wait(&sm.mma_done, 0))
        if (globaltimer_ns() - t0 > prm.wait_ns) {
          raise_abort(sm, prm.dev_err);
          break;
        }
    }
    __syncwarp();
    if (kDual && warp == kMmaWarp2) return;
    // the epilogue warps arrive on epi_exit when they stop reading TMEM, the expanders on
    // exp_exit when they stop writing it
    {
      const uint64_t t0 = globaltimer_ns();
      while (!mbar_try_wait(&sm.epi_exit, 0))
        if (globaltimer_ns() - t0 > prm.wait_ns) {
          raise_abort(sm, prm.dev_err);
          break;
        }
      const uint64_t t1 = globaltimer_ns();
      while (!mbar_try_wait(&sm.exp_exit, 0))
        if (globaltimer_ns() - t1 > prm.wait_ns) {
          raise_abort(sm, prm.dev_err);
          break;
        }
    }
    tc_fence_after();
    tmem_dealloc(tmem_base, tmem_cols);
    return;
  }

  // ---- epilogue warps 0..7: rows (warp % 4) * 32 + lane of the tile; warp / 4 picks
  // alternate 64-column chunks of the accumulator, or with kDual and N = 64 alternate tiles
  // (one accumulator stage each), so that both groups work on a narrow pass
  {
    // the accumulator holds 32 * kKSteps - 2 * (distance over the first 32 * kKSteps bits)
    const float dot_min = 32.0f * kKSteps - 2.0f * static_cast<float>(prm.threshold);
    const uint32_t quarter = static_cast<uint32_t>(warp & 3);
    const uint32_t group = static_cast<uint32_t>(warp >> 2);
    const uint32_t lane_addr = (quarter * 32) << 16;
    const bool by_tile = kDual && N <= 64;
    uint32_t ga = 0;
    bool ok = true;
    for (uint32_t p = 0; p < n_passes && ok; ++p) {
      const uint64_t q0 = static_cast<uint64_t>(p) * N;
      for (uint64_t k = 0; k < my_tiles; ++k, ++ga) {
        if (by_tile && (ga & 1u) != group) continue;
        const uint64_t tile = blockIdx.x + k * gridDim.x;
        const uint32_t ac = ga % kAccStages;
        if (!mbar_wait(&sm.acc_full[ac], (ga / kAccStages) & 1u, abort_flag, prm.wait_ns)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint64_t row = tile * kTileRows + quarter * 32 + lane;
        const bool row_ok = row < prm.n_rows;
        // the 64 accumulator columns c0 .. c0 + 63 in raw: any hit (or candidate) in them?
        auto scan_chunk = [&](const uint32_t (&raw)[32], uint32_t c0) {
          __half2 mh = *reinterpret_cast<const __half2*>(&raw[0]);
#pragma unroll
          for (int i = 1; i < 32; ++i) mh = __hmax2(mh, *reinterpret_cast<const __half2*>(&raw[i]));
          const float m = fmaxf(__low2float(mh), __high2float(mh));
          if (__any_sync(0xffffffffu, row_ok && m >= dot_min)) {
            const uint64_t cand = row_ok && m >= dot_min ? candidate_mask(raw, dot_min) : 0;
            emit_candidates(cand, row, q0 + c0, n_queries, prm, lane);
          }
        };
        // hand the accumulator stage back once its last columns are in registers, before
        // the (rarely slow) hit reporting
        auto release_acc = [&]() {
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&sm.acc_empty[ac]);
        };
        float unused[32];
        if constexpr (!kDual && kKSteps == 4) {
          // N = 192 or 256 with the 128-bit bound: group g reads chunks g and g + 2 with
          // both loads in flight before one wait (the readout is on the pass's critical path
          // once the MMAs are cut to a quarter of the tile's time; with 6 or 8 MMAs the extra
          // registers cost more than the overlap gains)
          const uint32_t c0 = 64 * group, c1 = c0 + 128;
          const bool two = c1 < N;
          uint32_t raw0[32], raw1[32];
          tmem_ld64_pack16_nowait(tmem_base + lane_addr + ac * N + c0, raw0);
          if (two) tmem_ld64_pack16_nowait(tmem_base + lane_addr + ac * N + c1, raw1);
          tmem_ld_wait();
          tmem_take(raw0, unused);
          if (two) tmem_take(raw1, unused);
          release_acc();
          scan_chunk(raw0, c0);
          if (two) scan_chunk(raw1, c1);
        } else {
          const uint32_t step = 64 * (kEpilogueWarps / 4);
          bool released = false;
          for (uint32_t c0 = by_tile ? 0u : 64 * group; c0 < N; c0 += step) {
            uint32_t raw[32];
            tmem_ld64_pack16_nowait(tmem_base + lane_addr + ac * N + c0, raw);
            tmem_ld_wait();
            tmem_take(raw, unused);
            if (c0 + step >= N) {
              release_acc();
              released = true;
            }
            scan_chunk(raw, c0);
          }
          if (!released) release_acc();
        }
      }
    }
    if (!ok && lane == 0) raise_abort(sm, prm.dev_err);
    tc_fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.epi_exit);
  }
}

// ---------------------------------------------------------------------------------------
// scan_pair_kernel: two queries per f32 accumulator column (passes of 512 queries, t <= 36).
//
// The 128-bit prefix bound of scan_tc_kernel<false, 4>, with a pass's queries taken in pairs
// (2j, 2j+1). The operands are e5m2: a database row's prefix bits become +-1 (A), query 2j's
// +-1 (B chunk 0, row j) and query 2j+1's +-512 (B chunk 1, row j). For each 128-row tile one
// thread issues 8 MMAs of M = 128, N = 256 (pairs), K = 32 into one f32 accumulator stage:
//   MMA k     (k < 4): A K-chunk k x B0 K-chunk k  ->  d1 = 128 - 2 * (prefix distance of 2j)
//   MMA 4 + k        : A K-chunk k x B1 K-chunk k  ->  512 * d2 (the same for query 2j + 1)
// Column j then holds v = d1 + 512 d2, an integer of magnitude <= 65,664: every product is
// +-1 or +-512 and every partial sum an integer below 2^24, so f32 accumulation is exact
// (checked on the GPU for all three orders of the 8 MMAs, including d = +-128).
//
// Decoding both halves at once. With f = d + 128 in [0, 256] (even, as d is),
// v + 65,664 = f1 + 512 f2. A pair member is a candidate when d >= dot_min = 128 - 2t.
// Adding c = 384 - dot_min to each 9-bit field makes it carry out exactly then, so with
// MAGIC = 2^23 + 65,664 + 513 c (an integer below 2^24, exact in f32) the sum v + MAGIC lies
// in [2^23, 2^24), where the f32 mantissa is the integer itself, and
//   bit 9 of its bits   <=>  query 2j   is a candidate
//   bit 18 of its bits  <=>  query 2j+1 is a candidate
// (field 2 + c is even, so field 1's carry lands in a clear bit 9 and cannot change whether
// field 2 carries). A 32-column chunk costs 32 FADD and 16 three-input ORs; a chunk with a
// candidate becomes a 64-query mask that emit_candidates re-checks over all 256 bits.
//
// Why pairs: reading the accumulator costs about the same per byte whatever its type, so f32
// pairs read no more than f16 singles per query, but a pass of 512 queries puts twice the
// MMA work behind each accumulator stage. The two stages of 256 columns then give the
// readout and the barrier handoffs a whole tile of MMAs (~1,060 clk) to hide behind, where
// passes of 256 f16 queries gave them ~540 clk and left the tensor pipe ~40 % idle. Eight
// MMAs per commit also keep the issuing thread (~60 clk per MMA) off the critical path.
// Roles and barriers are those of scan_tc_kernel<false, 4>.
constexpr int kPairN = 256;                 // pairs per pass (MMA N), 512 queries
constexpr int kPairAStages = 4;             // A tiles in shared memory (16 KiB each)

// The FP4 forms use block-scaled e2m1 operands, K = 64 per MMA, whose scale factors live in
// tensor memory beside the accumulators: a stage holds 240 columns (stage s at columns
// 256 s .. 256 s + 239).
constexpr int kPair4N = static_cast<int>(kPairFp4N);
constexpr uint32_t kPairStageCols = 256;

// The triple form (kForm 2): three queries per f32 column, FP4 operands. The bound is the
// first 126 bits (the queries' bits 126 and 127 expand to 0.0): per query the dot product d
// is even and in [-126, 126], so e = d / 2 fits 7 bits. With B scale factors 2^-1, 2^7 and
// 2^15 for queries 3j, 3j + 1 and 3j + 2 (A's scale 1), column j holds
// v = e_a + 256 e_b + 65536 e_c: every 32-element block adds an integer (its 32 products of
// +-1 sum to an even number), so every partial sum is an integer below 2^23 in magnitude and
// f32 accumulation is exact. The tile's first MMA overwrites the stage; the epilogue adds the
// decoding constant in registers (v + MAGIC, an integer in [2^23, 2^24), exact), so a stage
// goes back to the MMA issuer as soon as its loads have landed, with no reset stores to wait
// for (presetting the stages to MAGIC and writing it back after each read cost ~5 % more at
// 8,192 queries). Scale regions of 8
// columns in the two gaps the stages leave (columns 240-255 and 496-511): 2^0 at 240 (A),
// 2^-1 at 248, 2^7 at 496, 2^15 at 504. A block-scaled MMA with N = 240 reads more than 4
// columns of B scale factors (4-column regions made the last read run past column 511, an
// illegal access) and at most 8 (8-column regions at 496 and 504 of an earlier pair form
// gave exact results). Passes of 720 queries.
__host__ __device__ constexpr uint32_t sf_tri_col(int i) {
  return i == 0 ? 240u : i == 1 ? 248u : i == 2 ? 496u : 504u;
}
__host__ __device__ constexpr uint32_t sf_tri_val(int i) {
  return i == 0 ? 0x7F7F7F7Fu : i == 1 ? 0x7E7E7E7Eu : i == 2 ? 0x86868686u : 0x8E8E8E8Eu;
}
// forms of scan_pair_kernel
constexpr int kFormFp8Pairs = 0, kFormFp4Triples = 2;
__host__ __device__ constexpr int form_columns(int form) { return form == 0 ? kPairN : kPair4N; }
__host__ __device__ constexpr int form_queries(int form) {
  return (form == 2 ? 3 : 2) * form_columns(form);
}

// Both forms read their accumulator stage with 8 epilogue warps, two per TMEM lane quarter,
// each warp half the stage's columns (128 for FP8 pairs, 120 for FP4 triples) in two rounds.
__host__ __device__ constexpr int pair_epilogue_warps(bool) { return 8; }
__host__ __device__ constexpr int pair_threads(bool fp4) {
  return (pair_epilogue_warps(fp4) + 6) * 32;
}

// Instruction descriptor: D f32, A and B e5m2, both K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t idesc_e5m2_f32(uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

// Instruction descriptor of the block-scaled kind::mxf4 (D is f32): A and B e2m1 (format 1,
// bits 7-9 and 10-12), both K-major, scale factors UE8M0 (bit 23), N >> 3 at bits 17-22,
// M >> 4 at bits 24-28, scale-factor IDs 0 (bits 4-5 for B, 29-30 for A), dense K = 64
// (bit 31 clear).
__host__ __device__ constexpr uint32_t idesc_mxf4(uint32_t n) {
  return (1u << 7) | (1u << 10) | ((n >> 3) << 17) | (1u << 23) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void mma_mxf4(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t tmem_sfa, uint32_t tmem_sfb,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %6, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::mxf4.block_scale.scale_vec::2X [%0], %1, %2, %3, [%4], "
      "[%5], p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(tmem_sfa), "r"(tmem_sfb), "r"(accumulate)
      : "memory");
}

// Store 16 consecutive 32-bit columns of this warp's 32 TMEM lanes, all with the value v.
__device__ __forceinline__ void tmem_st16_fill(uint32_t taddr, uint32_t v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(taddr),
      "r"(v)
      : "memory");
}
// Store 8 consecutive 32-bit columns of this warp's 32 TMEM lanes, all with the value v.
__device__ __forceinline__ void tmem_st8_fill(uint32_t taddr, uint32_t v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(taddr),
      "r"(v)
      : "memory");
}

// Issue a load of 16 consecutive columns of this warp's 32 TMEM lanes into r[0..15].
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}

// Two f32 additions in one instruction (add.rn.f32x2): (a + m.lo, b + m.hi) as bit patterns,
// a in the low half of the result.
__device__ __forceinline__ uint64_t fadd2_rn(uint32_t a, uint32_t b, uint64_t m2) {
  uint64_t r;
  asm("{\n\t.reg .b64 t;\n\tmov.b64 t, {%1, %2};\n\tadd.rn.f32x2 %0, t, %3;\n\t}"
      : "=l"(r)
      : "r"(a), "r"(b), "l"(m2));
  return r;
}

// Issue a load of 8 consecutive columns of this warp's 32 TMEM lanes into r[0..7].
__device__ __forceinline__ void tmem_ld8_nowait(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
}

// tmem_take for the 8 registers of tmem_ld8_nowait.
__device__ __forceinline__ void tmem_take8(uint32_t (&r)[8]) {
  asm volatile("" : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]));
}

// tmem_take for the 16 registers of tmem_ld16_nowait.
__device__ __forceinline__ void tmem_take16(uint32_t (&r)[16]) {
  asm volatile("" : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]));
}

// The 128-bit prefix of a packed row as e2m1 (two per byte), +1.0 (0x2) for a clear bit and
// -1.0 (0xA) for a set bit, into the 128B-swizzled K-major operand (bytes 0-63 of the row;
// one MMA of K = 64 reads 32 of them). Packed word p becomes 16-byte unit p; its output word
// m (m = 0..3) holds bits m, m + 4, ..., m + 28 of the word in nibbles 0..7, which `<< (3 - m)`
// moves to each nibble's sign bit. Rows and queries share the bijection, so the dot product
// of two expanded rows is 128 - 2 * (prefix distance).
// kUnit0: the first of the four 16-byte units written (0, or 4 for bytes 64-127 of the row).
// kDrop2: the prefix's last two bits (126, 127: nibble 7 of output words 2 and 3 of packed
// word 3) become 0.0, so the dot product covers the first 126 bits only.
template <int kUnit0 = 0, bool kDrop2 = false>
__device__ __forceinline__ void expand_row_fp4(const uint4 w0, uint8_t* chunk, int row) {
  const uint32_t words[4] = {w0.x, w0.y, w0.z, w0.w};
  uint8_t* const base = chunk + row * 128;
  const int sw = row & 7;
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const uint32_t w = words[p];
    uint4 out;
    out.x = ((w << 3) & 0x88888888u) | 0x22222222u;
    out.y = ((w << 2) & 0x88888888u) | 0x22222222u;
    out.z = ((w << 1) & 0x88888888u) | 0x22222222u;
    out.w = (w & 0x88888888u) | 0x22222222u;
    if (kDrop2 && p == 3) {
      out.z &= 0x0FFFFFFFu;
      out.w &= 0x0FFFFFFFu;
    }
    *reinterpret_cast<uint4*>(base + (((kUnit0 + p) ^ sw) << 4)) = out;
  }
}

// All MMAs accumulate: the stage holds the decoding constant when the tile's MMAs start.
__device__ __forceinline__ void mma_pair_issue(uint32_t d, uint32_t a0, uint32_t b0,
                                               uint32_t b1, uint32_t idesc) {
#pragma unroll
  for (int ks = 0; ks < 4; ++ks)
    mma_f8(d, sw128_desc(a0 + 32 * ks), sw128_desc(b0 + 32 * ks), idesc, 1u);
#pragma unroll
  for (int ks = 0; ks < 4; ++ks)
    mma_f8(d, sw128_desc(a0 + 32 * ks), sw128_desc(b1 + 32 * ks), idesc, 1u);
}

// FP4 triples: two MMAs of K = 64 per query; queries 3j and 3j + 1 share B chunk 0 (bytes
// 0-63 and 64-127 of a row), query 3j + 2 is B chunk 1. acc_first: the first MMA adds to the
// stage (1: it holds the decoding constant) or overwrites it (0).
__device__ __forceinline__ void mma_triple4_issue(uint32_t d, uint32_t a0, uint32_t b0,
                                                  uint32_t b1, uint32_t idesc, uint32_t sf,
                                                  uint32_t acc_first = 1u) {
#pragma unroll
  for (int ks = 0; ks < 2; ++ks)
    mma_mxf4(d, sw128_desc(a0 + 32 * ks), sw128_desc(b0 + 32 * ks), idesc, sf + sf_tri_col(0),
             sf + sf_tri_col(1), ks == 0 ? acc_first : 1u);
#pragma unroll
  for (int ks = 0; ks < 2; ++ks)
    mma_mxf4(d, sw128_desc(a0 + 32 * ks), sw128_desc(b0 + 64 + 32 * ks), idesc,
             sf + sf_tri_col(0), sf + sf_tri_col(2), 1u);
#pragma unroll
  for (int ks = 0; ks < 2; ++ks)
    mma_mxf4(d, sw128_desc(a0 + 32 * ks), sw128_desc(b1 + 32 * ks), idesc, sf + sf_tri_col(0),
             sf + sf_tri_col(3), 1u);
}

// OR of N consecutive registers as a balanced tree (depth log2 N), not one dependent chain:
// the triple decode runs it on the stage hand-off path.
template <int N>
__device__ __forceinline__ uint32_t or_tree(const uint32_t* r) {
  if constexpr (N == 1)
    return r[0];
  else
    return or_tree<N / 2>(r) | or_tree<N - N / 2>(r + N / 2);
}

template <int kForm>
__global__ void __launch_bounds__(pair_threads(kForm != 0), 1)
    scan_pair_kernel(const __grid_constant__ Params prm) {
  constexpr bool kFp4 = kForm != kFormFp8Pairs;
  constexpr bool kTriples = kForm == kFormFp4Triples;
  constexpr int kN = form_columns(kForm);     // accumulator columns (pairs or triples) a pass
  constexpr int kQueries = form_queries(kForm);
  // roles: epilogue warps 0 .. kEpi - 1, then the producer, the MMA issuer, four expanders
  constexpr int kEpi = pair_epilogue_warps(kFp4);
  constexpr int kProducerWarp = kEpi, kMmaWarp = kEpi + 1, kExpandWarp0 = kEpi + 2;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* const smem_base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  Smem& sm = *reinterpret_cast<Smem*>(smem_base);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t n_pack = prm.pack_stages;
  const uint32_t n_queries = prm.nq_dev ? min(*prm.nq_dev, prm.n_queries) : prm.n_queries;
  uint8_t* const a_smem = smem_base + kFixedBytes;    // [kPairAStages][kChunkBytes]
  uint8_t* const bchunk0 = smem_base + prm.b_offset;  // 256 pair rows x 128 B: queries 2j
  uint8_t* const bchunk1 = bchunk0 + kPairN * 128;    // 256 pair rows x 128 B: 2j + 1 (x512)
  uint8_t* const packed = smem_base + prm.pack_offset;
  const uint64_t n_tiles = (prm.n_rows + kTileRows - 1) / kTileRows;
  const uint32_t n_passes = (n_queries + kQueries - 1) / kQueries;
  const uint64_t my_tiles =
      blockIdx.x < n_tiles ? (n_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  volatile int* abort_flag = &sm.abort_flag;

  if (tid == 0) {
    for (uint32_t s = 0; s < n_pack; ++s) {
      mbar_init(&sm.pk_full[s], 1);
      mbar_init(&sm.pk_empty[s], 4);
    }
    for (int s = 0; s < kPairAStages; ++s) {
      mbar_init(&sm.a_full[s], 4);
      mbar_init(&sm.a_empty[s], 1);
    }
    for (int s = 0; s < kAccStages; ++s) {
      mbar_init(&sm.acc_full[s], 1);
      mbar_init(&sm.acc_empty[s], kEpi);
    }
    mbar_init(&sm.b_full, 4);
    mbar_init(&sm.b_empty, 1);
    mbar_init(&sm.epi_exit, kEpi);
    mbar_init(&sm.exp_exit, 4);
    mbar_init(&sm.mma_done, 1);
    sm.abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == kMmaWarp) {
    tmem_alloc(&sm.tmem_base, kTmemCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = sm.tmem_base;
  if (my_tiles == 0 || n_passes == 0) {
    if (warp == kMmaWarp) tmem_dealloc(tmem_base, kTmemCols);
    return;
  }
  // FP8 pairs: the decoding constant (see the epilogue) goes into every accumulator column,
  // of both stages, before any MMA is issued; each epilogue warp writes its own columns.
  // Triples: the scale-factor regions (group 0 those at 240 and 248, group 1 those at 496
  // and 504); their stages are not preset.
  const float dot_min = 128.0f - 2.0f * static_cast<float>(prm.threshold);
  // triples: 2^23 + 63 (1 + 256 + 65536) + 257 (t + 2), an integer below 2^24
  const uint32_t magic_bits =
      kTriples ? __float_as_uint(8388608.0f + 4144959.0f +
                                 257.0f * (static_cast<float>(prm.threshold) + 2.0f))
               : __float_as_uint(8388608.0f + 65664.0f + 513.0f * (384.0f - dot_min));
  constexpr uint32_t kGroupCols = kFp4 ? 120 : 128;
  // (16 columns per store: a store's source is a block of consecutive registers)
  auto fill_cols = [&](uint32_t taddr, auto cols) {
    constexpr int kCols = decltype(cols)::value;
#pragma unroll
    for (int c = 0; c + 16 <= kCols; c += 16) tmem_st16_fill(taddr + c, magic_bits);
    if constexpr (kCols % 16 == 8) tmem_st8_fill(taddr + kCols - 8, magic_bits);
  };
  auto fill_group = [&](uint32_t taddr) {
    fill_cols(taddr, std::integral_constant<int, static_cast<int>(kGroupCols)>{});
  };
  if (warp < kEpi) {
    const uint32_t lanes = (static_cast<uint32_t>(warp & 3) * 32) << 16;
    const uint32_t g = static_cast<uint32_t>(warp >> 2);
    if constexpr (!kTriples)
      for (uint32_t st = 0; st < kAccStages; ++st)
        fill_group(tmem_base + lanes + st * kPairStageCols + kGroupCols * g);
    if constexpr (kTriples) {
      tmem_st8_fill(tmem_base + lanes + sf_tri_col(2 * g), sf_tri_val(2 * g));
      tmem_st8_fill(tmem_base + lanes + sf_tri_col(2 * g + 1), sf_tri_val(2 * g + 1));
    }
    tmem_st_wait();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();

  if (warp == kProducerWarp) {
    if (lane == 0 && !prm.stall) {
      uint32_t slot = 0, phase = 0, issued = 0;
      bool ok = true;
      for (uint32_t p = 0; p < n_passes && ok; ++p) {
        for (uint64_t k = 0; k < my_tiles; ++k) {
          const uint64_t tile = blockIdx.x + k * gridDim.x;
          if (!mbar_wait(&sm.pk_empty[slot], phase ^ 1u, abort_flag, prm.wait_ns)) {
            ok = false;
            break;
          }
          const uint64_t r0 = tile * kTileRows;
          const uint64_t nr = (prm.n_rows - r0) < kTileRows ? (prm.n_rows - r0) : kTileRows;
          const uint32_t bytes = static_cast<uint32_t>(nr * 32);
          mbar_arrive_expect_tx(&sm.pk_full[slot], bytes);
          bulk_g2s(packed + slot * kPackBytes, prm.rows + r0 * 32, bytes, &sm.pk_full[slot],
                   policy_evict_first());
          ++issued;
          if (++slot == n_pack) {
            slot = 0;
            phase ^= 1u;
          }
        }
      }
      if (!ok) {
        raise_abort(sm, prm.dev_err);
        // let the copies already issued land (bounded), as in scan_tc_kernel
        for (uint32_t k = 1; k <= n_pack && k <= issued; ++k) {
          const uint32_t sl = (slot + n_pack - k) % n_pack;
          const uint32_t ph = (k <= slot) ? phase : (phase ^ 1u);
          const uint64_t t0 = globaltimer_ns();
          while (!mbar_try_wait(&sm.pk_full[sl], ph))
            if (globaltimer_ns() - t0 > prm.wait_ns / 4) break;
        }
      }
    }
    return;
  }

  if (warp >= kExpandWarp0 && warp < kExpandWarp0 + 4) {
    const int e = tid - kExpandWarp0 * 32;  // 0..127: tile row; pairs e and e + 128
    uint32_t slot = 0, phase = 0, ga = 0;
    for (uint32_t p = 0; p < n_passes; ++p) {
      if (!mbar_wait(&sm.b_empty, (p & 1u) ^ 1u, abort_flag, prm.wait_ns)) goto fail;
      if constexpr (kTriples) {
        // triple j: queries 3j and 3j + 1 in bytes 0-63 and 64-127 of chunk 0's row j, query
        // 3j + 2 in bytes 0-63 of chunk 1's row j (126-bit prefixes); a query past the end
        // is zero
        for (uint32_t j = e; j < static_cast<uint32_t>(kN); j += 128) {
          const uint64_t q0 = static_cast<uint64_t>(p) * kQueries + 3 * j;
          const uint4 zero = make_uint4(0, 0, 0, 0);
          auto src = [&](uint64_t q) {
            return q < n_queries ? *reinterpret_cast<const uint4*>(prm.queries + q * 32) : zero;
          };
          expand_row_fp4<0, true>(src(q0), bchunk0, static_cast<int>(j));
          expand_row_fp4<4, true>(src(q0 + 1), bchunk0, static_cast<int>(j));
          expand_row_fp4<0, true>(src(q0 + 2), bchunk1, static_cast<int>(j));
          // zero words of a query past the end expand to +-1 values: clear those units
          const int sw = static_cast<int>(j) & 7;
#pragma unroll
          for (int f = 0; f < 3; ++f) {
            if (q0 + f < n_queries) continue;
            uint8_t* const rowp = (f == 2 ? bchunk1 : bchunk0) + j * 128;
            const int u0 = f == 1 ? 4 : 0;
#pragma unroll
            for (int u = 0; u < 4; ++u)
              *reinterpret_cast<uint4*>(rowp + (((u0 + u) ^ sw) << 4)) = zero;
          }
        }
      } else
      for (uint32_t j = e; j < static_cast<uint32_t>(kN); j += 128) {
        const uint64_t q0 = static_cast<uint64_t>(p) * kQueries + 2 * j;
        const uint4 zero = make_uint4(0, 0, 0, 0);
        // a query past the end gives a zero B row: its products are all 0
        if (q0 < n_queries) {
          const uint4* src = reinterpret_cast<const uint4*>(prm.queries + q0 * 32);
          expand_row<4, 0x3C3C3C3Cu>(src[0], src[1], bchunk0, nullptr, static_cast<int>(j));
        } else {
#pragma unroll
          for (int u = 0; u < 8; ++u)
            *reinterpret_cast<uint4*>(bchunk0 + j * 128 + u * 16) = zero;
        }
        if (q0 + 1 < n_queries) {
          const uint4* src = reinterpret_cast<const uint4*>(prm.queries + (q0 + 1) * 32);
          expand_row<4, 0x60606060u>(src[0], src[1], bchunk1, nullptr, static_cast<int>(j));
        } else {
#pragma unroll
          for (int u = 0; u < 8; ++u)
            *reinterpret_cast<uint4*>(bchunk1 + j * 128 + u * 16) = zero;
        }
      }
      fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.b_full);

      for (uint64_t k = 0; k < my_tiles; ++k, ++ga) {
        const uint32_t as = ga % kPairAStages;
        const uint32_t aph = (ga / kPairAStages) & 1u;
        if (!mbar_wait(&sm.pk_full[slot], phase, abort_flag, prm.wait_ns)) goto fail;
        const uint4* src = reinterpret_cast<const uint4*>(packed + slot * kPackBytes + e * 32);
        const uint4 w0 = src[0], w1 = src[1];
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.pk_empty[slot]);
        if (++slot == n_pack) {
          slot = 0;
          phase ^= 1u;
        }
        if (!mbar_wait(&sm.a_empty[as], aph ^ 1u, abort_flag, prm.wait_ns)) goto fail;
        if constexpr (kFp4)
          expand_row_fp4(w0, a_smem + static_cast<size_t>(as) * kChunkBytes, e);
        else
          expand_row<4, 0x3C3C3C3Cu>(w0, w1, a_smem + static_cast<size_t>(as) * kChunkBytes,
                                     nullptr, e);
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.a_full[as]);
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.exp_exit);
    return;
  fail:
    if (lane == 0) {
      raise_abort(sm, prm.dev_err);
      mbar_arrive(&sm.exp_exit);
    }
    return;
  }

  if (warp == kMmaWarp) {
    if (lane == 0) {
      const uint32_t idesc = kFp4 ? idesc_mxf4(kN) : idesc_e5m2_f32(kN);
      const uint32_t b0 = smem_u32(bchunk0), b1 = smem_u32(bchunk1);
      uint32_t ga = 0;
      bool ok = true;
      for (uint32_t p = 0; p < n_passes && ok; ++p) {
        if (!mbar_wait(&sm.b_full, p & 1u, abort_flag, prm.wait_ns)) {
          ok = false;
          break;
        }
        tc_fence_after();
        for (uint64_t k = 0; k < my_tiles; ++k, ++ga) {
          const uint32_t as = ga % kPairAStages;
          const uint32_t ac = ga % kAccStages;
          if (!mbar_wait(&sm.a_full[as], (ga / kPairAStages) & 1u, abort_flag, prm.wait_ns) ||
              !mbar_wait(&sm.acc_empty[ac], ((ga / kAccStages) & 1u) ^ 1u, abort_flag, prm.wait_ns)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a0 = smem_u32(a_smem + static_cast<size_t>(as) * kChunkBytes);
          if constexpr (kTriples)
            mma_triple4_issue(tmem_base + ac * kPairStageCols, a0, b0, b1, idesc, tmem_base, 0u);
          else
            mma_pair_issue(tmem_base + ac * kPairStageCols, a0, b0, b1, idesc);
          mma_commit(&sm.a_empty[as]);
          mma_commit(&sm.acc_full[ac]);
        }
        if (ok) mma_commit(&sm.b_empty);
      }
      if (!ok) raise_abort(sm, prm.dev_err);
      mma_commit(&sm.mma_done);
      const uint64_t t0 = globaltimer_ns();
      while (!mbar_try_wait(&sm.mma_done, 0))
        if (globaltimer_ns() - t0 > prm.wait_ns) {
          raise_abort(sm, prm.dev_err);
          break;
        }
    }
    __syncwarp();
    // the epilogue warps arrive on epi_exit when they stop reading TMEM, the expanders on
    // exp_exit when they stop writing shared memory the MMAs read
    {
      const uint64_t t0 = globaltimer_ns();
      while (!mbar_try_wait(&sm.epi_exit, 0))
        if (globaltimer_ns() - t0 > prm.wait_ns) {
          raise_abort(sm, prm.dev_err);
          break;
        }
      const uint64_t t1 = globaltimer_ns();
      while (!mbar_try_wait(&sm.exp_exit, 0))
        if (globaltimer_ns() - t1 > prm.wait_ns) {
          raise_abort(sm, prm.dev_err);
          break;
        }
    }
    tc_fence_after();
    tmem_dealloc(tmem_base, kTmemCols);
    return;
  }

  // ---- epilogue warps 0..7: rows (warp % 4) * 32 + lane; group g = warp / 4 reads pairs
  // kGroupCols g .. + kGroupCols - 1 of the stage in two rounds: 64 columns (two loads of 32),
  // then the rest (FP8: two loads of 32; FP4: loads of 32, 16 and 8). FP8 pairs: each column
  // holds v + MAGIC (the stage was filled with MAGIC before its MMAs), so the common case (no
  // candidate in the round's columns) costs one three-input OR per two columns and one vote;
  // the warp writes MAGIC back into its columns before it hands the stage to the MMA issuer.
  // Triples: the warp adds MAGIC to each column in registers and hands the stage back once
  // its second round of loads has landed.
  {
    const uint32_t quarter = static_cast<uint32_t>(warp & 3);
    const uint32_t group = static_cast<uint32_t>(warp >> 2);
    const uint32_t lane_addr = (quarter * 32) << 16;
    auto chunk_any = [&](const uint32_t* raw, auto cols) -> uint32_t {
      constexpr int kCols = decltype(cols)::value;
      uint32_t any = 0;
#pragma unroll
      for (int i = 0; i < kCols; i += 2) any |= raw[i] | raw[i + 1];
      return any;
    };
    // the rare path: the 2 kCols-query candidate mask of one chunk (bits 2i and 2i + 1 are pair
    // i's two queries)
    auto chunk_mask = [&](const uint32_t* raw, auto cols) -> uint64_t {
      constexpr int kCols = decltype(cols)::value;
      uint64_t mask = 0;
#pragma unroll
      for (int i = 0; i < kCols; ++i) {
        mask |= static_cast<uint64_t>((raw[i] >> 9) & 1u) << (2 * i);
        mask |= static_cast<uint64_t>((raw[i] >> 18) & 1u) << (2 * i + 1);
      }
      return mask;
    };
    using C8 = std::integral_constant<int, 8>;
    using C16 = std::integral_constant<int, 16>;
    using C32 = std::integral_constant<int, 32>;
    // Triples: bit 7 / bit 15 of a column's bits mark a candidate for its first / second
    // query; its third query is a candidate when the bits (a float in [2^23, 2^24), so
    // ordered as integers) reach 2^23 + 65536 (126 - t).
    const uint32_t tc_bits =
        __float_as_uint(8388608.0f + 65536.0f * (126.0f - static_cast<float>(prm.threshold)));
    // The common-case test, one FADD and half a three-input OR per column: with MAGIC2 =
    // MAGIC + 65536 (t + 2), v + MAGIC2 has bits 7 and 15 of v + MAGIC (fields a and b) and
    // reaches 2^24 exactly when field c is a candidate, which sets bit 23 of its bits (the
    // exponent's low bit). A sum at or past 2^24 may round its low bits, but its column is
    // flagged either way and the masks come from v + MAGIC (exact).
    const float magic_f = __uint_as_float(magic_bits);
    const float magic2_f = magic_f + 65536.0f * (static_cast<float>(prm.threshold) + 2.0f);
    auto tri_any = [&](const uint32_t* raw, auto cols) -> bool {
      constexpr int kCols = decltype(cols)::value;
      uint32_t x[kCols];
#pragma unroll
      for (int i = 0; i < kCols; ++i)
        x[i] = __float_as_uint(__fadd_rn(__uint_as_float(raw[i]), magic2_f));
      return (or_tree<kCols>(x) & 0x808080u) != 0;
    };
    // the rare path: one lane's candidate masks of one chunk, bit i for triple i of the chunk
    // (from v + MAGIC: bits 7 and 15, and field c's test on the whole value)
    auto tri_masks = [&](const uint32_t* raw, auto cols, uint32_t (&m)[3]) {
      constexpr int kCols = decltype(cols)::value;
#pragma unroll
      for (int i = 0; i < kCols; ++i) {
        const uint32_t r = __float_as_uint(__fadd_rn(__uint_as_float(raw[i]), magic_f));
        m[0] |= ((r >> 7) & 1u) << i;
        m[1] |= ((r >> 15) & 1u) << i;
        m[2] |= (r >= tc_bits ? 1u : 0u) << i;
      }
    };
    auto triple_tile = [&](uint32_t cols, uint64_t row, bool row_ok, uint64_t q_first,
                           uint32_t n_q, uint32_t (&raw0)[32], uint32_t (&raw1)[32],
                           float (&unused)[32], uint32_t ac) {
      // chunk c (triples kChunkTriple[c] ..) of the group: its candidates re-checked exactly
      // (all lanes take part)
      auto report = [&](const uint32_t (&m)[3], uint32_t first_triple) {
#pragma unroll
        for (int f = 0; f < 3; ++f)
          if (__any_sync(0xffffffffu, m[f] != 0))
            emit_candidates_call(m[f], row, q_first + 3 * first_triple + f, n_q, &prm, lane, 3);
      };
      tmem_ld32_nowait(cols, raw0);
      tmem_ld32_nowait(cols + 32, raw1);
      tmem_ld_wait();
      tmem_take(raw0, unused);
      tmem_take(raw1, unused);
      const bool mine1 = row_ok & (tri_any(raw0, C32{}) | tri_any(raw1, C32{}));
      if (__any_sync(0xffffffffu, mine1)) {
        // rare: report round 1's candidates now, while its columns are in registers (the
        // stage is handed back a little later)
        uint32_t m0[3] = {}, m1[3] = {};
        if (mine1) {
          tri_masks(raw0, C32{}, m0);
          tri_masks(raw1, C32{}, m1);
        }
        report(m0, 0);
        report(m1, 32);
      }
      uint32_t raw2[16], raw3[8];
      tmem_ld32_nowait(cols + 64, raw0);
      tmem_ld16_nowait(cols + 96, raw2);
      tmem_ld8_nowait(cols + 112, raw3);
      tmem_ld_wait();
      tmem_take(raw0, unused);
      tmem_take16(raw2);
      tmem_take8(raw3);
      // all of the warp's columns are in registers: hand the stage back
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.acc_empty[ac]);
      const bool mine2 =
          row_ok & (tri_any(raw0, C32{}) | tri_any(raw2, C16{}) | tri_any(raw3, C8{}));
      uint32_t m2[3] = {}, m3[3] = {}, m4[3] = {};
      if (mine2) {
        tri_masks(raw0, C32{}, m2);
        tri_masks(raw2, C16{}, m3);
        tri_masks(raw3, C8{}, m4);
      }
      if (__any_sync(0xffffffffu, mine2)) {
        report(m2, 64);
        report(m3, 96);
        report(m4, 112);
      }
    };
    uint32_t ga = 0;
    bool ok = true;
    for (uint32_t p = 0; p < n_passes && ok; ++p) {
      const uint64_t pass_q = static_cast<uint64_t>(p) * kQueries;
      for (uint64_t k = 0; k < my_tiles; ++k, ++ga) {
        const uint64_t tile = blockIdx.x + k * gridDim.x;
        const uint32_t ac = ga % kAccStages;
        if (!mbar_wait(&sm.acc_full[ac], (ga / kAccStages) & 1u, abort_flag, prm.wait_ns)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint64_t row = tile * kTileRows + quarter * 32 + lane;
        const bool row_ok = row < prm.n_rows;
        const uint32_t cols = tmem_base + lane_addr + ac * kPairStageCols + kGroupCols * group;
        const uint64_t q_first =
            pass_q + (kTriples ? 3 : 2) * static_cast<uint64_t>(kGroupCols * group);
        uint32_t raw0[32], raw1[32];
        float unused[32];
        if constexpr (kTriples) {
          triple_tile(cols, row, row_ok, q_first, n_queries, raw0, raw1, unused, ac);
          continue;
        }
        // round 1: pairs 0..63 of the group
        tmem_ld32_nowait(cols, raw0);
        tmem_ld32_nowait(cols + 32, raw1);
        tmem_ld_wait();
        tmem_take(raw0, unused);
        tmem_take(raw1, unused);
        const bool mine1 = row_ok && ((chunk_any(raw0, C32{}) | chunk_any(raw1, C32{})) & 0x40200u);
        const bool need1 = __any_sync(0xffffffffu, mine1);
        uint64_t m0 = 0, m1 = 0, m2 = 0, m3 = 0;
        if (need1 && mine1) {
          m0 = chunk_mask(raw0, C32{});
          m1 = chunk_mask(raw1, C32{});
        }
        // round 2: pairs 64.. of the group
        bool mine2;
        tmem_ld32_nowait(cols + 64, raw0);
        tmem_ld32_nowait(cols + 96, raw1);
        tmem_ld_wait();
        tmem_take(raw0, unused);
        tmem_take(raw1, unused);
        mine2 = row_ok && ((chunk_any(raw0, C32{}) | chunk_any(raw1, C32{})) & 0x40200u);
        if (mine2) {
          m2 = chunk_mask(raw0, C32{});
          m3 = chunk_mask(raw1, C32{});
        }
        // decoded: reset the warp's columns (one wait for all stores: a store's source
        // registers stay reserved until then) and hand the stage back before any hit reporting
        fill_group(cols);
        tmem_st_wait();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.acc_empty[ac]);
        // each chunk's candidates re-checked exactly (all lanes take part); the chunk starts
        // at pair `pair` of the group
        auto report = [&](uint64_t m, uint32_t pair) {
          if (__any_sync(0xffffffffu, m != 0))
            emit_candidates_call(m, row, q_first + 2 * pair, n_queries, &prm, lane, 1);
        };
        if (need1) {
          report(m0, 0);
          report(m1, 32);
        }
        if (__any_sync(0xffffffffu, mine2)) {
          report(m2, 64);
          report(m3, 96);

        }
      }
    }
    if (!ok && lane == 0) raise_abort(sm, prm.dev_err);
    tc_fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.epi_exit);
  }
}

// ---------------------------------------------------------------------------------------
// scan_rows_kernel: narrow passes (<= 128 queries) with the operands swapped, at t > 36
// (at t <= 36 scan_rows3_kernel runs them).
//
// The queries are the MMA's A operand (M = 128 rows; a query past the end is a zero row,
// whose dot products are 0 and never reach dot_min) and the database tiles its B operand,
// N = 256 rows per MMA. An M = 128, K = 32 MMA costs ~120 clk whatever its N up to 128 and
// ~128 clk at N = 256, so scan_tc_kernel's narrow passes (N = 64 queries, 128 rows per MMA)
// pay four times the MMA instructions per database row that these do. The accumulator of a
// tile is 128 lanes (queries) x 256 columns (rows), f16 as in scan_tc_kernel (two stages);
// epilogue warp w reads queries 32 (w % 4) .. + 31 (its lanes) and rows 128 (w / 4) .. + 127
// as two 64-column loads. A candidate column becomes a 64-row mask per lane, re-checked with
// popcounts of the packed row and the lane's query (emit_rows). The queries are expanded
// once per launch; each 256-row tile is expanded once (two rows per expander thread).
// Roles: warps 0-7 epilogue, 8 producer (bulk copies of 8 KiB packed tiles), 9 MMA and
// TMEM allocation, 10-13 expanders.
constexpr int kRowsN = 256;                  // database rows per tile (MMA N)
// expanded tiles in shared memory: 3 of 32 KiB (128-bit prefix) or 2 of 64 KiB
__host__ __device__ constexpr int rows_b_stages(int k_steps) { return k_steps > 4 ? 2 : 3; }
constexpr int kRowsPackBytes = kRowsN * 32;  // one packed tile
constexpr int kRowsChunkBytes = kRowsN * 128;  // one 128-byte K-chunk of an expanded tile
constexpr int kRowsMaxQueries = kTileRows;   // queries per launch (MMA M)

// Report the candidate rows of one lane (bit j of cand: row row0 + j against the lane's
// query q): the exact distance of each from popcounts, hits within the threshold written at
// positions taken with one atomic per warp. Called by all 32 lanes; a lane without
// candidates passes cand = 0.
// (stride: bit j of cand stands for row row0 + stride * j; 1 unless given.)
__device__ __forceinline__ void emit_rows(uint64_t cand, uint64_t row0, uint32_t q,
                                          const Params& prm, int lane, uint32_t stride = 1) {
  {
    // bits whose row is past the end
    const uint64_t lim = row0 >= prm.n_rows ? 0 : (prm.n_rows - row0 + stride - 1) / stride;
    if (lim < 64) cand &= (1ull << lim) - 1;
  }
  uint4 q0 = make_uint4(0, 0, 0, 0), q1 = q0;
  if (cand) {
    const uint4* qp = reinterpret_cast<const uint4*>(prm.queries + static_cast<uint64_t>(q) * 32);
    q0 = __ldg(qp);
    q1 = __ldg(qp + 1);
  }
  uint64_t hits = 0;
  for (uint64_t m = cand; m; m &= m - 1) {
    const int j = __ffsll(static_cast<long long>(m)) - 1;
    const uint4* rp = reinterpret_cast<const uint4*>(prm.rows + (row0 + stride * j) * 32);
    if (popc256(__ldg(rp), __ldg(rp + 1), q0, q1) <= prm.threshold) hits |= 1ull << j;
  }
  const uint32_t mine = static_cast<uint32_t>(__popcll(hits));
  uint32_t incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  if (total == 0) return;
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(prm.count, static_cast<unsigned long long>(total));
  base = __shfl_sync(0xffffffffu, base, 0);
  uint64_t pos = base + incl - mine;
  for (uint64_t m = hits; m; m &= m - 1, ++pos) {
    if (pos >= prm.capacity) break;
    const int j = __ffsll(static_cast<long long>(m)) - 1;
    const uint4* rp = reinterpret_cast<const uint4*>(prm.rows + (row0 + stride * j) * 32);
    ypdq_hit h;
    h.index = row0 + stride * j;
    h.query = q + prm.query_base;
    h.distance = popc256(__ldg(rp), __ldg(rp + 1), q0, q1);
    prm.hits[pos] = h;
  }
}

template <int kKSteps>
__global__ void __launch_bounds__(threads_of(false), 1) scan_rows_kernel(const Params prm) {
  static_assert(kKSteps == 4 || kKSteps == 6 || kKSteps == 8, "K steps");
  constexpr int kChunks = kKSteps > 4 ? 2 : 1;  // 128-byte K-chunks per expanded row
  constexpr int kRowsBStages = rows_b_stages(kKSteps);
  extern __shared__ uint8_t smem_raw[];
  uint8_t* const smem_base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  Smem& sm = *reinterpret_cast<Smem*>(smem_base);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t n_pack = prm.pack_stages;
  const uint32_t n_queries = prm.nq_dev ? min(*prm.nq_dev, prm.n_queries) : prm.n_queries;
  uint8_t* const q_smem = smem_base + kFixedBytes;                  // [kChunks][128 x 128 B]
  uint8_t* const b_smem = q_smem + kChunks * kChunkBytes;           // [stages][kChunks][32 KB]
  uint8_t* const packed = smem_base + prm.pack_offset;
  const uint64_t n_tiles = (prm.n_rows + kRowsN - 1) / kRowsN;
  const uint64_t my_tiles =
      blockIdx.x < n_tiles ? (n_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  volatile int* abort_flag = &sm.abort_flag;

  if (tid == 0) {
    for (uint32_t s = 0; s < n_pack; ++s) {
      mbar_init(&sm.pk_full[s], 1);
      mbar_init(&sm.pk_empty[s], 4);
    }
    for (int s = 0; s < kRowsBStages; ++s) {
      mbar_init(&sm.a_full[s], 4);   // expanded tile stage s is ready
      mbar_init(&sm.a_empty[s], 1);  // the MMAs reading it have completed
    }
    for (int s = 0; s < kAccStages; ++s) {
      mbar_init(&sm.acc_full[s], 1);
      mbar_init(&sm.acc_empty[s], kEpilogueWarps);
    }
    mbar_init(&sm.b_full, 4);  // the queries are expanded
    mbar_init(&sm.epi_exit, kEpilogueWarps);
    mbar_init(&sm.exp_exit, 4);
    mbar_init(&sm.mma_done, 1);
    sm.abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == kMmaWarp) {
    tmem_alloc(&sm.tmem_base, kTmemCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = sm.tmem_base;
  if (my_tiles == 0 || n_queries == 0) {
    if (warp == kMmaWarp) tmem_dealloc(tmem_base, kTmemCols);
    return;
  }

  if (warp == kProducerWarp) {
    if (lane == 0 && !prm.stall) {
      uint32_t slot = 0, phase = 0, issued = 0;
      bool ok = true;
      for (uint64_t k = 0; k < my_tiles; ++k) {
        const uint64_t tile = blockIdx.x + k * gridDim.x;
        if (!mbar_wait(&sm.pk_empty[slot], phase ^ 1u, abort_flag, prm.wait_ns)) {
          ok = false;
          break;
        }
        const uint64_t r0 = tile * kRowsN;
        const uint64_t nr = (prm.n_rows - r0) < kRowsN ? (prm.n_rows - r0) : kRowsN;
        const uint32_t bytes = static_cast<uint32_t>(nr * 32);
        mbar_arrive_expect_tx(&sm.pk_full[slot], bytes);
        bulk_g2s(packed + slot * kRowsPackBytes, prm.rows + r0 * 32, bytes, &sm.pk_full[slot],
                 policy_evict_first());
        ++issued;
        if (++slot == n_pack) {
          slot = 0;
          phase ^= 1u;
        }
      }
      if (!ok) {
        raise_abort(sm, prm.dev_err);
        // let the copies already issued land (bounded), as in scan_tc_kernel
        for (uint32_t k = 1; k <= n_pack && k <= issued; ++k) {
          const uint32_t sl = (slot + n_pack - k) % n_pack;
          const uint32_t ph = (k <= slot) ? phase : (phase ^ 1u);
          const uint64_t t0 = globaltimer_ns();
          while (!mbar_try_wait(&sm.pk_full[sl], ph))
            if (globaltimer_ns() - t0 > prm.wait_ns / 4) break;
        }
      }
    }
    return;
  }

  if (warp >= kExpandWarp0 && warp < kExpandWarp0 + 4) {
    const int e = tid - kExpandWarp0 * 32;  // 0..127: query e; tile rows e and e + 128
    uint8_t* const q1 = q_smem + (kChunks > 1 ? kChunkBytes : 0);
    if (static_cast<uint32_t>(e) < n_queries) {
      const uint4* src = reinterpret_cast<const uint4*>(prm.queries + static_cast<uint64_t>(e) * 32);
      expand_row<kKSteps>(src[0], src[1], q_smem, q1, e);
    } else {
      for (int c = 0; c < kChunks; ++c)
#pragma unroll
        for (int u = 0; u < 8; ++u)
          *reinterpret_cast<uint4*>(q_smem + c * kChunkBytes + e * 128 + u * 16) =
              make_uint4(0, 0, 0, 0);
    }
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.b_full);
    uint32_t slot = 0, phase = 0;
    for (uint64_t k = 0; k < my_tiles; ++k) {
      const uint32_t bs = static_cast<uint32_t>(k % kRowsBStages);
      const uint32_t bph = static_cast<uint32_t>(k / kRowsBStages) & 1u;
      if (!mbar_wait(&sm.pk_full[slot], phase, abort_flag, prm.wait_ns)) goto fail;
      const uint4* src0 = reinterpret_cast<const uint4*>(packed + slot * kRowsPackBytes + e * 32);
      const uint4* src1 = src0 + 2 * 128;  // row e + 128
      const uint4 a0 = src0[0], a1 = src0[1], c0 = src1[0], c1 = src1[1];
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.pk_empty[slot]);
      if (++slot == n_pack) {
        slot = 0;
        phase ^= 1u;
      }
      if (!mbar_wait(&sm.a_empty[bs], bph ^ 1u, abort_flag, prm.wait_ns)) goto fail;
      uint8_t* const b0 = b_smem + static_cast<size_t>(bs) * kChunks * kRowsChunkBytes;
      uint8_t* const b1 = b0 + (kChunks > 1 ? kRowsChunkBytes : 0);
      expand_row<kKSteps>(a0, a1, b0, b1, e);
      expand_row<kKSteps>(c0, c1, b0, b1, e + 128);
      fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.a_full[bs]);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.exp_exit);
    return;
  fail:
    if (lane == 0) {
      raise_abort(sm, prm.dev_err);
      mbar_arrive(&sm.exp_exit);
    }
    return;
  }

  if (warp == kMmaWarp) {
    if (lane == 0) {
      const uint32_t idesc = idesc_f8(kRowsN);
      bool ok = mbar_wait(&sm.b_full, 0, abort_flag, prm.wait_ns);
      tc_fence_after();
      const uint32_t qa0 = smem_u32(q_smem), qa1 = qa0 + kChunkBytes;
      for (uint64_t k = 0; k < my_tiles && ok; ++k) {
        const uint32_t bs = static_cast<uint32_t>(k % kRowsBStages);
        const uint32_t ac = static_cast<uint32_t>(k % kAccStages);
        if (!mbar_wait(&sm.a_full[bs], static_cast<uint32_t>(k / kRowsBStages) & 1u, abort_flag,
                       prm.wait_ns) ||
            !mbar_wait(&sm.acc_empty[ac], (static_cast<uint32_t>(k / kAccStages) & 1u) ^ 1u,
                       abort_flag, prm.wait_ns)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t b0 = smem_u32(b_smem + static_cast<size_t>(bs) * kChunks * kRowsChunkBytes);
        const uint32_t b1 = b0 + kRowsChunkBytes;
        const uint32_t d = tmem_base + ac * kRowsN;
#pragma unroll
        for (int ks = 0; ks < kKSteps; ++ks) {
          const uint32_t off = (ks & 3) * 32;
          mma_f8(d, sw128_desc((ks < 4 ? qa0 : qa1) + off), sw128_desc((ks < 4 ? b0 : b1) + off),
                 idesc, ks > 0 ? 1u : 0u);
        }
        mma_commit(&sm.a_empty[bs]);
        mma_commit(&sm.acc_full[ac]);
      }
      if (!ok) raise_abort(sm, prm.dev_err);
      mma_commit(&sm.mma_done);
      const uint64_t t0 = globaltimer_ns();
      while (!mbar_try_wait(&sm.mma_done, 0))
        if (globaltimer_ns() - t0 > prm.wait_ns) {
          raise_abort(sm, prm.dev_err);
          break;
        }
    }
    __syncwarp();
    {
      const uint64_t t0 = globaltimer_ns();
      while (!mbar_try_wait(&sm.epi_exit, 0))
        if (globaltimer_ns() - t0 > prm.wait_ns) {
          raise_abort(sm, prm.dev_err);
          break;
        }
      const uint64_t t1 = globaltimer_ns();
      while (!mbar_try_wait(&sm.exp_exit, 0))
        if (globaltimer_ns() - t1 > prm.wait_ns) {
          raise_abort(sm, prm.dev_err);
          break;
        }
    }
    tc_fence_after();
    tmem_dealloc(tmem_base, kTmemCols);
    return;
  }

  // ---- epilogue warps 0..7: queries (warp % 4) * 32 + lane; group warp / 4 reads the tile's
  // rows 128 g .. 128 g + 127 as two 64-column loads
  {
    const float dot_min = 32.0f * kKSteps - 2.0f * static_cast<float>(prm.threshold);
    const uint32_t quarter = static_cast<uint32_t>(warp & 3);
    const uint32_t group = static_cast<uint32_t>(warp >> 2);
    const uint32_t lane_addr = (quarter * 32) << 16;
    const uint32_t q = quarter * 32 + lane;
    const bool q_ok = q < n_queries;
    // a lane quarter that holds no query (fewer than 97, 65 or 33 queries) has nothing to
    // read: its warps only hand each stage back
    const bool active = quarter * 32 < n_queries;
    bool ok = true;
    for (uint64_t k = 0; k < my_tiles && ok; ++k) {
      const uint64_t tile = blockIdx.x + k * gridDim.x;
      const uint32_t ac = static_cast<uint32_t>(k % kAccStages);
      if (!mbar_wait(&sm.acc_full[ac], static_cast<uint32_t>(k / kAccStages) & 1u, abort_flag,
                     prm.wait_ns)) {
        ok = false;
        break;
      }
      tc_fence_after();
      if (!active) {
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.acc_empty[ac]);
        continue;
      }
      const uint32_t c0 = 128 * group;
      uint32_t raw0[32], raw1[32];
      float unused[32];
      tmem_ld64_pack16_nowait(tmem_base + lane_addr + ac * kRowsN + c0, raw0);
      tmem_ld64_pack16_nowait(tmem_base + lane_addr + ac * kRowsN + c0 + 64, raw1);
      tmem_ld_wait();
      tmem_take(raw0, unused);
      tmem_take(raw1, unused);
      // both chunks are in registers: hand the stage back before the hit reporting
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.acc_empty[ac]);
      const uint64_t row0 = tile * kRowsN + c0;
      auto scan_chunk = [&](const uint32_t (&raw)[32], uint64_t r0) {
        __half2 mh = *reinterpret_cast<const __half2*>(&raw[0]);
#pragma unroll
        for (int i = 1; i < 32; ++i) mh = __hmax2(mh, *reinterpret_cast<const __half2*>(&raw[i]));
        const float m = fmaxf(__low2float(mh), __high2float(mh));
        if (__any_sync(0xffffffffu, q_ok && m >= dot_min))
          emit_rows(q_ok && m >= dot_min ? candidate_mask(raw, dot_min) : 0, r0, q, prm, lane);
      };
      scan_chunk(raw0, row0);
      scan_chunk(raw1, row0 + 64);
    }
    if (!ok && lane == 0) raise_abort(sm, prm.dev_err);
    tc_fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.epi_exit);
  }
}

// ---------------------------------------------------------------------------------------
// scan_rows3_kernel: narrow passes (<= 128 queries a launch; the launcher runs up to 512 as
// launches of 128) at t <= 36 with three database rows per f32 accumulator column and
// block-scaled FP4 operands.
//
// The triple form of scan_pair_kernel with the operands swapped: the queries (126-bit
// prefixes) are A, M = 128 lanes, expanded once per launch; a tile of 720 database rows is B,
// rows 3j, 3j + 1 and 3j + 2 in column j (fields a, b and c: see the chunk layout below, with
// B scales 2^-1, 2^7 and 2^15). Column j of lane q then holds
// e_a + 256 e_b + 65536 e_c over the decoding constant, e = 63 - (distance over the prefix),
// decoded by the same bit tests. Per database row the tensor core runs 6 MMAs of N = 240 for
// 720 rows (~1.4 clk) where scan_rows_kernel runs 4 FP8 MMAs of N = 256 for 256 rows (~2 clk),
// and the epilogue reads 240 columns per 720 rows instead of 256 per 256. TMEM, scale regions
// and the decoding (MAGIC added in registers) are those of the triple form. Epilogue warp w
// reads queries 32 (w % 4) + lane and the 120 columns 120 (w / 4) ..; a lane quarter without
// queries (A rows zero) only hands each stage back. Rows past the end of the last tile are
// zero B units (their fields stay 0, below every candidate test).
// Roles: warps 0-7 epilogue, 8 producer (bulk copies of 22.5 KiB packed tiles), 9 MMA and
// TMEM allocation, 10-13 expanders (thread e: the rows of columns e and e + 128).
constexpr int kRows3Cols = kPair4N;                 // accumulator columns per tile (MMA N)
constexpr int kRows3Rows = 3 * kRows3Cols;          // database rows per tile
constexpr int kRows3PackBytes = kRows3Rows * 32;    // one packed tile
constexpr int kRows3ChunkBytes = kRows3Cols * 128;  // one B chunk (240 rows x 128 B)
// Three expanded tiles in five chunks of 240 rows x 128 B, every byte used: stage s's fields
// a and b are chunk s (bytes 0-63 and 64-127 of row j); the fields c of stages 0 and 1 are
// chunk 3 (bytes 0-63 and 64-127), that of stage 2 bytes 0-63 of chunk 4, whose bytes
// 64-127 of rows 0-127 hold the queries (A). Three stages let the expanders run up to two
// tiles ahead of the MMAs (an expander warp that shares its scheduler with busy epilogue
// warps runs slower than the others); the five chunks leave room for three packed tiles in
// flight.
constexpr int kRows3BStages = 3;
constexpr int kRows3BChunks = 5;
static_assert(kRows3ChunkBytes % 1024 == 0, "B chunks stay 1024-byte aligned");

// expand_row_fp4 with the first unit chosen at run time; keep = 0 writes zero units
__device__ __forceinline__ void expand_prefix_fp4(const uint4 w0, uint8_t* chunk, int row,
                                                  int unit0, uint32_t keep) {
  const uint32_t words[4] = {w0.x, w0.y, w0.z, w0.w};
  uint8_t* const base = chunk + row * 128;
  const int sw = row & 7;
  const uint32_t sign = 0x88888888u & keep, one = 0x22222222u & keep;
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const uint32_t w = words[p];
    uint4 out;
    out.x = ((w << 3) & sign) | one;
    out.y = ((w << 2) & sign) | one;
    out.z = ((w << 1) & sign) | one;
    out.w = (w & sign) | one;
    *reinterpret_cast<uint4*>(base + (((unit0 + p) ^ sw) << 4)) = out;
  }
}

// emit_rows out of line (the rare path; keeps the epilogue's registers for its loads)
__device__ __noinline__ void emit_rows_call(uint64_t cand, uint64_t row0, uint32_t q,
                                            const Params* prm, int lane, uint32_t stride) {
  emit_rows(cand, row0, q, *prm, lane, stride);
}

__global__ void __launch_bounds__(threads_of(false), 1)
    scan_rows3_kernel(const __grid_constant__ Params prm) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* const smem_base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  Smem& sm = *reinterpret_cast<Smem*>(smem_base);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t n_pack = prm.pack_stages;
  // a launch covers queries nq_off .. nq_off + n_queries - 1 of a device-side count
  uint32_t n_queries = prm.n_queries;
  if (prm.nq_dev) {
    const uint32_t nq = *prm.nq_dev;
    n_queries = nq > prm.nq_off ? min(nq - prm.nq_off, prm.n_queries) : 0u;
  }
  uint8_t* const b_smem = smem_base + kFixedBytes;  // [kRows3BChunks][240 x 128 B]
  uint8_t* const q_smem = b_smem + 4 * kRows3ChunkBytes;  // queries: bytes 64-127 of rows
  uint8_t* const packed = smem_base + prm.pack_offset;
  const uint64_t n_tiles = (prm.n_rows + kRows3Rows - 1) / kRows3Rows;
  const uint64_t my_tiles =
      blockIdx.x < n_tiles ? (n_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  volatile int* abort_flag = &sm.abort_flag;

  if (tid == 0) {
    for (uint32_t s = 0; s < n_pack; ++s) {
      mbar_init(&sm.pk_full[s], 1);
      mbar_init(&sm.pk_empty[s], 4);
    }
    for (int s = 0; s < kRows3BStages; ++s) {
      mbar_init(&sm.a_full[s], 4);   // expanded tile stage s is ready
      mbar_init(&sm.a_empty[s], 1);  // the MMAs reading it have completed
    }
    for (int s = 0; s < kAccStages; ++s) {
      mbar_init(&sm.acc_full[s], 1);
      mbar_init(&sm.acc_empty[s], kEpilogueWarps);
    }
    mbar_init(&sm.b_full, 4);  // the queries are expanded
    mbar_init(&sm.epi_exit, kEpilogueWarps);
    mbar_init(&sm.exp_exit, 4);
    mbar_init(&sm.mma_done, 1);
    sm.abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == kMmaWarp) {
    tmem_alloc(&sm.tmem_base, kTmemCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = sm.tmem_base;
  if (my_tiles == 0 || n_queries == 0) {
    if (warp == kMmaWarp) tmem_dealloc(tmem_base, kTmemCols);
    return;
  }
  // The scale regions, as in the triple form. The stages are not preset: a tile's first MMA
  // overwrites its stage, and the epilogue adds the decoding constant in registers (exact:
  // v and the sum are integers below 2^24), so it hands a stage back as soon as its loads
  // have landed, with no tensor-memory stores to wait for.
  const float magic = 8388608.0f + 4144959.0f + 257.0f * (static_cast<float>(prm.threshold) + 2.0f);
  constexpr int kGroupCols = kRows3Cols / 2;  // 120 columns per epilogue warp
  if (warp < kEpilogueWarps) {
    const uint32_t lanes = (static_cast<uint32_t>(warp & 3) * 32) << 16;
    const uint32_t g = static_cast<uint32_t>(warp >> 2);
    tmem_st8_fill(tmem_base + lanes + sf_tri_col(2 * g), sf_tri_val(2 * g));
    tmem_st8_fill(tmem_base + lanes + sf_tri_col(2 * g + 1), sf_tri_val(2 * g + 1));
    tmem_st_wait();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();

  if (warp == kProducerWarp) {
    if (lane == 0 && !prm.stall) {
      uint32_t slot = 0, phase = 0, issued = 0;
      bool ok = true;
      for (uint64_t k = 0; k < my_tiles; ++k) {
        const uint64_t tile = blockIdx.x + k * gridDim.x;
        if (!mbar_wait(&sm.pk_empty[slot], phase ^ 1u, abort_flag, prm.wait_ns)) {
          ok = false;
          break;
        }
        const uint64_t r0 = tile * kRows3Rows;
        const uint64_t nr = (prm.n_rows - r0) < kRows3Rows ? (prm.n_rows - r0) : kRows3Rows;
        const uint32_t bytes = static_cast<uint32_t>(nr * 32);
        mbar_arrive_expect_tx(&sm.pk_full[slot], bytes);
        bulk_g2s(packed + slot * kRows3PackBytes, prm.rows + r0 * 32, bytes, &sm.pk_full[slot],
                 policy_evict_first());
        ++issued;
        if (++slot == n_pack) {
          slot = 0;
          phase ^= 1u;
        }
      }
      if (!ok) {
        raise_abort(sm, prm.dev_err);
        // let the copies already issued land (bounded), as in scan_tc_kernel
        for (uint32_t k = 1; k <= n_pack && k <= issued; ++k) {
          const uint32_t sl = (slot + n_pack - k) % n_pack;
          const uint32_t ph = (k <= slot) ? phase : (phase ^ 1u);
          const uint64_t t0 = globaltimer_ns();
          while (!mbar_try_wait(&sm.pk_full[sl], ph))
            if (globaltimer_ns() - t0 > prm.wait_ns / 4) break;
        }
      }
    }
    return;
  }

  if (warp >= kExpandWarp0 && warp < kExpandWarp0 + 4) {
    const int e = tid - kExpandWarp0 * 32;  // 0..127: query e; the rows of columns e, e + 128
    // Thread e expands columns j = e and e + 128 (< 240), the three rows of each: in one
    // store instruction the lanes write one field of consecutive columns, so eight lanes
    // (one wavefront of 16-byte stores) cover eight distinct swizzled units. (Consecutive
    // rows per lane put fields a and c of a column, same unit of chunks 0 and 1, in one
    // wavefront: twice the store wavefronts.)
    constexpr int kHalves = (kRows3Cols + 127) / 128;
    {
      const uint4 w = static_cast<uint32_t>(e) < n_queries
                          ? __ldg(reinterpret_cast<const uint4*>(prm.queries +
                                                                  static_cast<uint64_t>(e) * 32))
                          : make_uint4(0, 0, 0, 0);
      if (static_cast<uint32_t>(e) < n_queries)
        expand_row_fp4<4, true>(w, q_smem, e);
      else
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if ((u ^ (e & 7)) >= 4)  // units 4-7 (swizzled); 0-3 are stage 2's fields c
            *reinterpret_cast<uint4*>(q_smem + e * 128 + u * 16) = make_uint4(0, 0, 0, 0);
    }
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.b_full);
    uint32_t slot = 0, phase = 0;
    for (uint64_t k = 0; k < my_tiles; ++k) {
      const uint64_t tile = blockIdx.x + k * gridDim.x;
      const uint32_t bs = static_cast<uint32_t>(k % kRows3BStages);
      const uint32_t bph = static_cast<uint32_t>(k / kRows3BStages) & 1u;
      const uint64_t r0 = tile * kRows3Rows;
      const uint32_t nr = static_cast<uint32_t>(
          (prm.n_rows - r0) < kRows3Rows ? (prm.n_rows - r0) : kRows3Rows);
      if (!mbar_wait(&sm.pk_full[slot], phase, abort_flag, prm.wait_ns)) goto fail;
      uint4 w[kHalves][3];
#pragma unroll
      for (int h = 0; h < kHalves; ++h) {
        const int j = e + 128 * h;
#pragma unroll
        for (int f = 0; f < 3; ++f)
          w[h][f] = j < kRows3Cols ? *reinterpret_cast<const uint4*>(
                                         packed + slot * kRows3PackBytes + (3 * j + f) * 32)
                                   : make_uint4(0, 0, 0, 0);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.pk_empty[slot]);
      if (++slot == n_pack) {
        slot = 0;
        phase ^= 1u;
      }
      if (!mbar_wait(&sm.a_empty[bs], bph ^ 1u, abort_flag, prm.wait_ns)) goto fail;
      {
        uint8_t* const b0 = b_smem + static_cast<size_t>(bs) * kRows3ChunkBytes;
        uint8_t* const b1 = b_smem + (bs < 2 ? 3 : 4) * kRows3ChunkBytes;
#pragma unroll
        for (int h = 0; h < kHalves; ++h) {
          const int j = e + 128 * h;
          if (j >= kRows3Cols) continue;
#pragma unroll
          for (int f = 0; f < 3; ++f)
            expand_prefix_fp4(w[h][f], f == 2 ? b1 : b0, j,
                              f == 1 || (f == 2 && bs == 1) ? 4 : 0,
                              static_cast<uint32_t>(3 * j + f) < nr ? 0xFFFFFFFFu : 0u);
        }
      }
      fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.a_full[bs]);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.exp_exit);
    return;
  fail:
    if (lane == 0) {
      raise_abort(sm, prm.dev_err);
      mbar_arrive(&sm.exp_exit);
    }
    return;
  }

  if (warp == kMmaWarp) {
    if (lane == 0) {
      const uint32_t idesc = idesc_mxf4(kRows3Cols);
      bool ok = mbar_wait(&sm.b_full, 0, abort_flag, prm.wait_ns);
      tc_fence_after();
      const uint32_t qa = smem_u32(q_smem) + 64;  // bytes 64-127 of the rows
      for (uint64_t k = 0; k < my_tiles && ok; ++k) {
        const uint32_t bs = static_cast<uint32_t>(k % kRows3BStages);
        const uint32_t ac = static_cast<uint32_t>(k % kAccStages);
        if (!mbar_wait(&sm.a_full[bs], static_cast<uint32_t>(k / kRows3BStages) & 1u, abort_flag,
                       prm.wait_ns) ||
            !mbar_wait(&sm.acc_empty[ac], (static_cast<uint32_t>(k / kAccStages) & 1u) ^ 1u,
                       abort_flag, prm.wait_ns)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t b0 = smem_u32(b_smem + static_cast<size_t>(bs) * kRows3ChunkBytes);
        const uint32_t b1 = smem_u32(b_smem + (bs < 2 ? 3 : 4) * kRows3ChunkBytes) + (bs == 1 ? 64 : 0);
        mma_triple4_issue(tmem_base + ac * kPairStageCols, qa, b0, b1, idesc, tmem_base, 0u);
        mma_commit(&sm.a_empty[bs]);
        mma_commit(&sm.acc_full[ac]);
      }
      if (!ok) raise_abort(sm, prm.dev_err);
      mma_commit(&sm.mma_done);
      const uint64_t t0 = globaltimer_ns();
      while (!mbar_try_wait(&sm.mma_done, 0))
        if (globaltimer_ns() - t0 > prm.wait_ns) {
          raise_abort(sm, prm.dev_err);
          break;
        }
    }
    __syncwarp();
    {
      const uint64_t t0 = globaltimer_ns();
      while (!mbar_try_wait(&sm.epi_exit, 0))
        if (globaltimer_ns() - t0 > prm.wait_ns) {
          raise_abort(sm, prm.dev_err);
          break;
        }
      const uint64_t t1 = globaltimer_ns();
      while (!mbar_try_wait(&sm.exp_exit, 0))
        if (globaltimer_ns() - t1 > prm.wait_ns) {
          raise_abort(sm, prm.dev_err);
          break;
        }
    }
    tc_fence_after();
    tmem_dealloc(tmem_base, kTmemCols);
    return;
  }

  // ---- epilogue warps 0..7: query q = 32 (warp % 4) + lane; group warp / 4 reads the
  // stage's columns 120 g .. 120 g + 119 (database rows 360 g .. + 359 of the tile) in two
  // rounds, 32 + 32 then 32 + 16 + 8, adds the decoding constant to each column and tests
  // the bits as scan_pair_kernel's triple form does; the stage goes back to the MMA issuer
  // once the second round's loads have landed
  {
    const uint32_t quarter = static_cast<uint32_t>(warp & 3);
    const uint32_t group = static_cast<uint32_t>(warp >> 2);
    const uint32_t lane_addr = (quarter * 32) << 16;
    const uint32_t q = quarter * 32 + lane;
    const bool q_ok = q < n_queries;
    const bool active = quarter * 32 < n_queries;
    // field c's test: the column's bits (a float in [2^23, 2^24)) reach 2^23 + 65536 (126 - t)
    const uint32_t tc_bits =
        __float_as_uint(8388608.0f + 65536.0f * (126.0f - static_cast<float>(prm.threshold)));
    // the common-case test and the rare path's masks of scan_pair_kernel's triple form
    const float magic2 = magic + 65536.0f * (static_cast<float>(prm.threshold) + 2.0f);
    auto tri_any = [&](const uint32_t* raw, auto cols) -> bool {
      constexpr int kCols = decltype(cols)::value;
      uint32_t x[kCols];
#pragma unroll
      for (int i = 0; i < kCols; ++i)
        x[i] = __float_as_uint(__fadd_rn(__uint_as_float(raw[i]), magic2));
      return (or_tree<kCols>(x) & 0x808080u) != 0;
    };
    auto tri_masks = [&](const uint32_t* raw, auto cols, uint32_t (&m)[3]) {
      constexpr int kCols = decltype(cols)::value;
#pragma unroll
      for (int i = 0; i < kCols; ++i) {
        const uint32_t r = __float_as_uint(__fadd_rn(__uint_as_float(raw[i]), magic));
        m[0] |= ((r >> 7) & 1u) << i;
        m[1] |= ((r >> 15) & 1u) << i;
        m[2] |= (r >= tc_bits ? 1u : 0u) << i;
      }
    };
    using C8 = std::integral_constant<int, 8>;
    using C16 = std::integral_constant<int, 16>;
    using C32 = std::integral_constant<int, 32>;
    bool ok = true;
    for (uint64_t k = 0; k < my_tiles && ok; ++k) {
      const uint64_t tile = blockIdx.x + k * gridDim.x;
      const uint32_t ac = static_cast<uint32_t>(k % kAccStages);
      if (!mbar_wait(&sm.acc_full[ac], static_cast<uint32_t>(k / kAccStages) & 1u, abort_flag,
                     prm.wait_ns)) {
        ok = false;
        break;
      }
      tc_fence_after();
      if (!active) {
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.acc_empty[ac]);
        continue;
      }
      const uint32_t cols = tmem_base + lane_addr + ac * kPairStageCols + kGroupCols * group;
      // database row of field f of the group's column i: row_g + 3 i + f
      const uint64_t row_g = tile * kRows3Rows + 3ull * kGroupCols * group;
      auto report = [&](const uint32_t (&m)[3], uint32_t first) {
#pragma unroll
        for (int f = 0; f < 3; ++f)
          if (__any_sync(0xffffffffu, m[f] != 0))
            emit_rows_call(m[f], row_g + 3 * first + f, q, &prm, lane, 3);
      };
      uint32_t raw0[32], raw1[32];
      float unused[32];
      tmem_ld32_nowait(cols, raw0);
      tmem_ld32_nowait(cols + 32, raw1);
      tmem_ld_wait();
      tmem_take(raw0, unused);
      tmem_take(raw1, unused);
      const bool mine1 = q_ok & (tri_any(raw0, C32{}) | tri_any(raw1, C32{}));
      if (__any_sync(0xffffffffu, mine1)) {
        uint32_t m0[3] = {}, m1[3] = {};
        if (mine1) {
          tri_masks(raw0, C32{}, m0);
          tri_masks(raw1, C32{}, m1);
        }
        report(m0, 0);
        report(m1, 32);
      }
      uint32_t raw2[16], raw3[8];
      tmem_ld32_nowait(cols + 64, raw0);
      tmem_ld16_nowait(cols + 96, raw2);
      tmem_ld8_nowait(cols + 112, raw3);
      tmem_ld_wait();
      tmem_take(raw0, unused);
      tmem_take16(raw2);
      tmem_take8(raw3);
      // all of the warp's columns are in registers: hand the stage back
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.acc_empty[ac]);
      const bool mine2 =
          q_ok & (tri_any(raw0, C32{}) | tri_any(raw2, C16{}) | tri_any(raw3, C8{}));
      uint32_t m2[3] = {}, m3[3] = {}, m4[3] = {};
      if (mine2) {
        tri_masks(raw0, C32{}, m2);
        tri_masks(raw2, C16{}, m3);
        tri_masks(raw3, C8{}, m4);
      }
      if (__any_sync(0xffffffffu, mine2)) {
        report(m2, 64);
        report(m3, 96);
        report(m4, 112);
      }
    }
    if (!ok && lane == 0) raise_abort(sm, prm.dev_err);
    tc_fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.epi_exit);
  }
}

}  // namespace tc

cudaError_t scan_tc_init() {
  for (const void* f : {reinterpret_cast<const void*>(tc::scan_tc_kernel<true, 4>),
                        reinterpret_cast<const void*>(tc::scan_tc_kernel<true, 8>),
                        reinterpret_cast<const void*>(tc::scan_tc_kernel<false, 4>),
                        reinterpret_cast<const void*>(tc::scan_tc_kernel<false, 6>),
                        reinterpret_cast<const void*>(tc::scan_tc_kernel<false, 8>),
                        reinterpret_cast<const void*>(tc::scan_pair_kernel<tc::kFormFp8Pairs>),
                        reinterpret_cast<const void*>(tc::scan_pair_kernel<tc::kFormFp4Triples>),
                        reinterpret_cast<const void*>(tc::scan_rows_kernel<6>),
                        reinterpret_cast<const void*>(tc::scan_rows_kernel<8>),
                        reinterpret_cast<const void*>(tc::scan_rows3_kernel)}) {
    const cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               static_cast<int>(tc::kSmemLimit));
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_scan_tc(const ScanLaunch& p, int num_sms, cudaStream_t s) {
  tc::Params prm{};
  prm.rows = p.rows;
  prm.n_rows = p.n_rows;
  prm.queries = p.queries;
  prm.n_queries = p.n_queries;
  // N is a multiple of 64 so every 64-column TMEM load stays inside one accumulator.
  uint32_t n = (p.n_queries + 63u) & ~63u;
  prm.n_tile = n > static_cast<uint32_t>(tc::kMaxN) ? static_cast<uint32_t>(tc::kMaxN) : n;
  if (p.n_tile) {
    if (p.n_tile % 64u != 0 || p.n_tile > static_cast<uint32_t>(tc::kMaxN) || p.pair_n)
      return cudaErrorInvalidValue;
    prm.n_tile = p.n_tile;
  }
  prm.threshold = p.threshold;
  prm.hits = p.hits;
  prm.capacity = p.capacity;
  prm.count = p.count;
  prm.dev_err = p.dev_err;
  prm.query_base = p.query_base;
  prm.nq_dev = p.nq_dev;
  prm.wait_ns = scan_wait_limit_ns();
  prm.stall = take_scan_stall() ? 1 : 0;
  // at a small threshold the first 128 bits bound the distance (kKSteps = 4)
  const bool half_k = p.threshold <= 36;
  const uint64_t tiles = (p.n_rows + tc::kTileRows - 1) / tc::kTileRows;
  const uint64_t grid = tiles < static_cast<uint64_t>(num_sms) ? tiles : num_sms;
  // At t <= 36 with no pass width or FP8 pairs asked for, up to 512 queries: queries as A,
  // three database rows per accumulator column (scan_rows3_kernel), one launch per 128
  // queries. On 10M rows a launch takes 0.072-0.079 ms for 1 to 128 queries, so 2 to 4 of
  // them beat one 256-query pass of scan_tc_kernel (0.23 ms) and one 720-query triple pass
  // (0.327 ms); past 512 queries the triple passes cost less.
  if (half_k && !p.n_tile && p.pair_n != static_cast<uint32_t>(tc::kPairN) &&
      p.n_queries <= 4u * static_cast<uint32_t>(tc::kRowsMaxQueries)) {
    const size_t b_end = tc::kFixedBytes +
                         static_cast<size_t>(tc::kRows3BChunks) * tc::kRows3ChunkBytes;
    size_t stages = (tc::kSmemLimit - 1024 - b_end) / tc::kRows3PackBytes;
    if (stages > static_cast<size_t>(tc::kMaxPackStages)) stages = tc::kMaxPackStages;
    if (stages < 2) return cudaErrorInvalidConfiguration;
    prm.n_tile = tc::kRowsMaxQueries;
    prm.pack_stages = static_cast<uint32_t>(stages);
    prm.pack_offset = static_cast<uint32_t>(b_end);
    const size_t smem = b_end + stages * tc::kRows3PackBytes + 1024;
    const uint64_t rtiles = (p.n_rows + tc::kRows3Rows - 1) / tc::kRows3Rows;
    const unsigned g = static_cast<unsigned>(rtiles < static_cast<uint64_t>(num_sms) ? rtiles : num_sms);
    for (uint32_t q0 = 0; q0 < p.n_queries; q0 += tc::kRowsMaxQueries) {
      tc::Params c = prm;
      c.queries = p.queries + static_cast<size_t>(q0) * 32;
      c.n_queries = p.n_queries - q0 < static_cast<uint32_t>(tc::kRowsMaxQueries)
                        ? p.n_queries - q0
                        : static_cast<uint32_t>(tc::kRowsMaxQueries);
      c.query_base = p.query_base + q0;
      c.nq_off = q0;
      c.stall = q0 == 0 ? prm.stall : 0;
      tc::scan_rows3_kernel<<<g, tc::threads_of(false), smem, s>>>(c);
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  // at most 128 queries at t > 36 and no pass width asked for: queries as A, 256 database
  // rows per MMA (scan_rows_kernel)
  if (!half_k && !p.n_tile && !p.pair_n &&
      p.n_queries <= static_cast<uint32_t>(tc::kRowsMaxQueries)) {
    const int ks = p.threshold <= 62 ? 6 : 8;
    const int chunks = ks > 4 ? 2 : 1;
    const size_t b_end = tc::kFixedBytes + static_cast<size_t>(chunks) * tc::kChunkBytes +
                         static_cast<size_t>(tc::rows_b_stages(ks)) * chunks * tc::kRowsChunkBytes;
    size_t stages = (tc::kSmemLimit - 1024 - b_end) / tc::kRowsPackBytes;
    if (stages > static_cast<size_t>(tc::kMaxPackStages)) stages = tc::kMaxPackStages;
    if (stages < 2) return cudaErrorInvalidConfiguration;
    prm.n_tile = tc::kRowsMaxQueries;
    prm.pack_stages = static_cast<uint32_t>(stages);
    prm.pack_offset = static_cast<uint32_t>(b_end);
    const size_t smem = b_end + stages * tc::kRowsPackBytes + 1024;
    const uint64_t rtiles = (p.n_rows + tc::kRowsN - 1) / tc::kRowsN;
    const unsigned g = static_cast<unsigned>(rtiles < static_cast<uint64_t>(num_sms) ? rtiles : num_sms);
    if (ks == 6)
      tc::scan_rows_kernel<6><<<g, tc::threads_of(false), smem, s>>>(prm);
    else
      tc::scan_rows_kernel<8><<<g, tc::threads_of(false), smem, s>>>(prm);
    return cudaGetLastError();
  }
  if (p.pair_n && (!half_k || (p.pair_n != static_cast<uint32_t>(tc::kPairN) &&
                                p.pair_n != kPairFp4N)))
    return cudaErrorInvalidValue;  // pairs need the 128-bit bound (t <= 36)
  // at t <= 36 past 512 queries (or when asked for): several queries per accumulator column
  // (scan_pair_kernel), FP4 triples in passes of 720 or, with pair_n = 256, FP8 pairs in
  // passes of 512. A triple pass costs less than a pair pass (0.327 against 0.36 ms on 10M
  // rows) and covers more queries, so without a form asked for the triples run.
  if (half_k && !p.n_tile && (p.pair_n || p.n_queries > static_cast<uint32_t>(tc::kMaxN))) {
    const int form = p.pair_n == static_cast<uint32_t>(tc::kPairN) ? tc::kFormFp8Pairs
                                                                   : tc::kFormFp4Triples;
    prm.n_tile = static_cast<uint32_t>(tc::form_queries(form));
    prm.a_stages = tc::kPairAStages;
    // layout: [fixed Smem][A: 4 x 16 KB][B: 2 x 256 pairs x 128 B][packed ring], 1024-aligned
    prm.b_offset = static_cast<uint32_t>(tc::kFixedBytes +
                                         static_cast<size_t>(tc::kPairAStages) * tc::kChunkBytes);
    const size_t b_end = prm.b_offset + 2 * static_cast<size_t>(tc::kPairN) * 128;
    size_t stages = (tc::kSmemLimit - 1024 - b_end) / tc::kPackBytes;
    if (stages > static_cast<size_t>(tc::kMaxPackStages)) stages = tc::kMaxPackStages;
    prm.pack_stages = static_cast<uint32_t>(stages);
    prm.pack_offset = static_cast<uint32_t>(b_end);
    const size_t smem = b_end + stages * tc::kPackBytes + 1024;
    const unsigned g = static_cast<unsigned>(grid);
    if (form == tc::kFormFp4Triples)
      tc::scan_pair_kernel<tc::kFormFp4Triples><<<g, tc::pair_threads(true), smem, s>>>(prm);
    else
      tc::scan_pair_kernel<tc::kFormFp8Pairs><<<g, tc::pair_threads(false), smem, s>>>(prm);
    return cudaGetLastError();
  }
  // passes of <= 128 queries: two MMA issuers and A in tensor memory (the pass is bound by
  // issuing and shared-memory traffic, not by the tensor core)
  const bool dual = prm.n_tile <= 128;
  uint32_t a_stages = tc::kAStages;
  if (dual) {
    a_stages = (tc::kTmemCols - tc::kAccStages * prm.n_tile) / (half_k ? 32 : 64);
    if (a_stages > static_cast<uint32_t>(tc::kMaxAStages)) a_stages = tc::kMaxAStages;
  }
  prm.a_stages = a_stages;
  // layout: [fixed Smem][A (shared-memory A only): 4 x 2 x 16 KB][B: 2 x N x 128]
  //         [packed ring: stages x 4 KB], base aligned to 1024
  prm.b_offset = static_cast<uint32_t>(
      tc::kFixedBytes + (dual ? 0 : static_cast<size_t>(tc::kAStages) * 2 * tc::kChunkBytes));
  const size_t b_end = prm.b_offset + 2 * static_cast<size_t>(prm.n_tile) * 128;
  const size_t avail = tc::kSmemLimit - 1024 - b_end;
  size_t stages = avail / tc::kPackBytes;
  if (stages > static_cast<size_t>(tc::kMaxPackStages)) stages = tc::kMaxPackStages;
  if (stages < 2) return cudaErrorInvalidConfiguration;
  prm.pack_stages = static_cast<uint32_t>(stages);
  prm.pack_offset = static_cast<uint32_t>(b_end);
  const size_t smem = b_end + stages * tc::kPackBytes + 1024;
  // passes of 256 queries at t <= 62: the first 192 bits bound the distance
  const bool prefix192 = !dual && !half_k && p.threshold <= 62;
  const unsigned g = static_cast<unsigned>(grid);
  if (dual && half_k)
    tc::scan_tc_kernel<true, 4><<<g, tc::threads_of(true), smem, s>>>(prm);
  else if (dual)
    tc::scan_tc_kernel<true, 8><<<g, tc::threads_of(true), smem, s>>>(prm);
  else if (half_k)
    tc::scan_tc_kernel<false, 4><<<g, tc::threads_of(false), smem, s>>>(prm);
  else if (prefix192)
    tc::scan_tc_kernel<false, 6><<<g, tc::threads_of(false), smem, s>>>(prm);
  else
    tc::scan_tc_kernel<false, 8><<<g, tc::threads_of(false), smem, s>>>(prm);
  return cudaGetLastError();
}

namespace {
std::atomic<uint64_t> g_scan_wait_ns{kWaitLimitNs};
std::atomic<int> g_scan_stalls{0};
}  // namespace

uint64_t scan_wait_limit_ns() { return g_scan_wait_ns.load(std::memory_order_relaxed); }

bool take_scan_stall() {
  int n = g_scan_stalls.load();
  while (n > 0)
    if (g_scan_stalls.compare_exchange_weak(n, n - 1)) return true;
  return false;
}

}  // namespace ypdq

extern "C" ypdq_status ypdq_set_scan_wait_limit(uint64_t ns) {
  if (ns > 60ull * 1000 * 1000 * 1000)
    return ypdq::fail(YPDQ_ERR_INVALID, "wait limit %llu ns > 60 s", (unsigned long long)ns);
  ypdq::g_scan_wait_ns.store(ns ? ns : ypdq::kWaitLimitNs);
  return YPDQ_OK;
}

extern "C" ypdq_status ypdq_debug_stall_scans(int n) {
  if (n < 0) return ypdq::fail(YPDQ_ERR_INVALID, "n < 0");
  ypdq::g_scan_stalls.store(n);
  return YPDQ_OK;
}
