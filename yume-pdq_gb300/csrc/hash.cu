// Fused PDQ hash kernel: 512x512 image -> tent compress -> DCT -> quality -> exact median
// quantize -> the 8 dihedral hashes, for a batch of images, one image per CTA at a time.
//
// Reference semantics (yume-pdq):
//   compress  DefaultKernel::jarosz_compress   src/kernel/mod.rs:644-666
//   DCT       DefaultKernel::dct2d_impl        src/kernel/mod.rs:543-574
//   quality   sum_of_gradients / adjust_quality src/kernel/mod.rs:611-642
//   median    torben_median                    src/kernel/mod.rs:212-253 (the 128th smallest)
//   packing   quantize / threshold_2d_f32      src/kernel/mod.rs:595-608, threshold.rs:37-119
//   dihedrals visit_dihedrals                  src/lib.rs:358-420
//
// The FP32 path reproduces the reference's f32 results bit for bit for finite inputs.
// Every product and sum is a separately rounded __fmul_rn / __fadd_rn (the reference is
// Rust, which never contracts a*b+c). Sums run in the reference's order: taps row by row;
// the DCT in four interleaved partial sums combined as ((s0+s1)+s2)+s3. The tent table is
// 7x7, but only 27 taps are nonzero: the 5x5 centre (k/81) and two subnormal residues in
// row 0 that the reference's 128-bit constant generation leaves behind. A zero tap adds +0
// to a finite partial sum, which changes nothing, so the kernel skips those taps.
//
// CTA layout (192 threads):
//   warps 0-3  compute: thread j owns output column j (j < 127) of the compressed image,
//              accumulates DCT stage 1 (16 x 127 x 127) as each compressed row appears,
//              then computes the 16 x 16 stage 2 together.
//   warp 4     producer: one lane streams the image into a shared-memory ring with 1-D
//              bulk async copies (4 input rows = one stage), NSTAGE stages deep.
//   warp 5     epilogue: quality, exact medians, bits and dihedrals of image k while the
//              compute warps already work on image k+1 (double-buffered PDQF).
#include <cuda_bf16.h>

#include <cstring>

#include <type_traits>

#include "ypdq_internal.cuh"
#include "ypdq_tables.h"

namespace ypdq {

__device__ float g_dct[16 * 127];  // D[k][i] = sqrt(2/127) cos(pi (k+1) (2i+1) / 254), f32

constexpr int kStagesPerImage = 128;  // stage s holds rows 4s+1 .. 4s+4 (stage 127: 509, 510)
constexpr int kComputeThreads = 128;
constexpr int kProducerWarp = 4;
constexpr int kEpilogueWarp = 5;
constexpr int kMmaWarpHash = 6;   // tensor-core DCT only: allocates TMEM, issues the MMAs
template <int kDct>
constexpr int hash_threads() { return kDct == 0 ? 192 : 224; }
// RGB8 / RGBA8 pixels, converted to f32 luma once per stage (see convert_stage).
struct rgb8_t {
  uint8_t c[3];
};
struct rgba8_t {
  uint8_t c[4];
};
template <typename Tin>
constexpr bool is_rgb() {
  return std::is_same<Tin, rgb8_t>::value || std::is_same<Tin, rgba8_t>::value;
}

// Depth of the input ring (4-row stages). The tensor-core variants with f32 input use 6
// stages so that two CTAs fit on an SM next to their operand buffers.
#ifndef YPDQ_RING_U8
#define YPDQ_RING_U8 8
#endif
#ifndef YPDQ_RING_U8_TC
#define YPDQ_RING_U8_TC 16
#endif
#ifndef YPDQ_U8_TC_CTAS
#define YPDQ_U8_TC_CTAS 2
#endif
template <typename Tin, int kDct>
constexpr int ring_stages() {
  return is_rgb<Tin>() ? (kDct != 0 ? 3 : 6)
                       : (sizeof(Tin) == 4 ? (kDct != 0 ? 6 : 8)
                                           : (kDct != 0 ? YPDQ_RING_U8_TC : YPDQ_RING_U8));
}
template <typename Tin>
constexpr int conv_slots() { return is_rgb<Tin>() ? 3 : 0; }
// The tensor-core variants need no DCT accumulators in registers: with u8 input (issue-
// bound, not HBM-bound) they run 3 CTAs per SM.
template <typename Tin, int kDct>
constexpr int hash_min_blocks() { return (kDct != 0 && sizeof(Tin) == 1) ? YPDQ_U8_TC_CTAS : 2; }
constexpr int kComputeBarrier = 1;  // named barrier id used by the 128 compute threads
constexpr int kConvRow = 136;       // floats per row of an RGB luma staging (128 + 4, padded)

// Stage 1 of the DCT on tensor cores (kDct = 1: TF32, 2: BF16x3). The compressed values
// are written, chunk by chunk of compressed rows, into a 128-byte-swizzled K-major operand
// A[j][i] (M = 128 columns j, K = rows i); B is the DCT matrix D[k][i] (N = 16).
template <int kDct>
struct DctTraits {
  static constexpr int kRowsPerChunk = 128;  // unused for kDct = 0
  static constexpr int kBufBytes = 16;
  static constexpr int kDBytes = 16;
};
template <>
struct DctTraits<1> {  // TF32: 32 rows x 4 B = 128 B per column per chunk
  static constexpr int kRowsPerChunk = 32;
  static constexpr int kBufBytes = 128 * 128;
  static constexpr int kDBytes = 4 * 2048;  // 4 K-chunks x 16 rows x 128 B
  static constexpr int kDChunkBytes = 2048;
  static constexpr int kKSteps = 4;         // MMAs of K = 8 (32 B) per chunk
};
template <>
struct DctTraits<2> {  // BF16x3: 32 rows x 2 B (64-byte swizzle), hi at +0 and lo at +8192
  static constexpr int kRowsPerChunk = 32;
  static constexpr int kBufBytes = 2 * 128 * 64;
  static constexpr int kDBytes = 2 * 4 * 1024;  // hi, lo x 4 K-chunks x 16 rows x 64 B
  static constexpr int kDChunkBytes = 1024;
  static constexpr int kKSteps = 2;             // MMAs of K = 16 (32 B) per chunk
  static constexpr int kALo = 8192, kDLo = 4096;  // byte offsets of the lo operands
};

template <int kStageBytes, int kNumStages, int kDct, int kConvSlots>
struct HashSmem {
  // RGB input only: per compute warp, f32 luma of its columns of the last 3 stages
  alignas(16) float conv[kConvSlots > 0 ? 4 : 1][kConvSlots > 0 ? kConvSlots : 1]
                        [kConvSlots > 0 ? 4 * kConvRow : 4];
  alignas(1024) uint8_t ops[2][DctTraits<kDct>::kBufBytes];  // A operand, double-buffered
  alignas(1024) uint8_t dops[DctTraits<kDct>::kDBytes];      // B operand (DCT matrix)
  alignas(128) unsigned char ring[kNumStages][kStageBytes];
  alignas(16) float dt[kDct == 0 ? 128 : 1][16];  // dt[i][k] = D[k][i]; row 127 is zero
  float dr[16][129];              // D[k][m], padded against bank conflicts
  float t[16][129];               // DCT stage 1 result T = D * B
  alignas(16) float p[2][256];    // PDQF, double-buffered between compute and epilogue
  uint64_t full[kNumStages];
  uint64_t empty[kNumStages];
  uint64_t pfull[2];
  uint64_t pempty[2];
  uint64_t a_full[2], a_empty[2], acc_full[2], acc_empty[2], tc_exit, mma_done;
  uint32_t tmem_base;
  int abort_flag;
};

template <typename Tin>
struct InputTraits;
template <>
struct InputTraits<float> {
  static constexpr int kRowBytes = 512 * 4;
};
template <>
struct InputTraits<uint8_t> {
  static constexpr int kRowBytes = 512;
};
template <>
struct InputTraits<rgb8_t> {
  static constexpr int kRowBytes = 512 * 3;
};
template <>
struct InputTraits<rgba8_t> {
  static constexpr int kRowBytes = 512 * 4;
};
// The element type the compress reads: the input itself, or f32 luma for RGB input.
template <typename Tin, bool kRgb = is_rgb<Tin>()>
struct CompressIn {
  using T = Tin;
};
template <typename Tin>
struct CompressIn<Tin, true> {
  using T = float;
};

// ITU-R BT.601 luma in the reference's scalar order (Kernel::cvt_rgb8_to_luma8f,
// src/kernel/mod.rs:303-340, coefficients src/kernel/constants.rs:23):
// (0.299 r + 0.587 g) + 0.114 b, each product and sum rounded to f32, no fused multiply-add.
__device__ __forceinline__ float luma_bt601(float r, float g, float b) {
  return __fadd_rn(__fadd_rn(__fmul_rn(0.299f, r), __fmul_rn(0.587f, g)), __fmul_rn(0.114f, b));
}
// Byte k (0..3) of w as an exact float: the byte placed in the mantissa of 2^23 by a byte
// permute, then 2^23 subtracted (keeps the conversion off the quarter-rate I2F path).
template <int k>
__device__ __forceinline__ float byte_f(uint32_t w) {
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7650 | k)) - 8388608.0f;
}
// Luma staging of one 4-row stage for one compute warp: warp w reads input columns
// 128w .. 128w+131 (its 32 compressed columns need 4j .. 4j+7), stored as 4 rows of
// kConvRow floats from column 128w on. Lane l converts columns 128w+4l .. +3 of each row;
// lanes 0..15 also convert the 4 columns past the warp's 128 (row l/4), 0 past the image.
__device__ __forceinline__ uint32_t rgb_word(const unsigned char* p) {  // 4-byte aligned
  return *reinterpret_cast<const uint32_t*>(p);
}
template <typename Tin>
__device__ __forceinline__ void convert_stage_warp(const unsigned char* raw, float* out, int w,
                                                   int lane) {
  constexpr int kRowBytes = InputTraits<Tin>::kRowBytes;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int c0 = 128 * w + 4 * lane;
    const unsigned char* row = raw + r * kRowBytes;
    float l[4];
    if constexpr (sizeof(Tin) == 4) {
      const uint4 v = *reinterpret_cast<const uint4*>(row + 4 * c0);
      const uint32_t px[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int k = 0; k < 4; ++k) l[k] = luma_bt601(byte_f<0>(px[k]), byte_f<1>(px[k]), byte_f<2>(px[k]));
    } else {
      const unsigned char* p = row + 3 * c0;  // 12 bytes: r g b r | g b r g | b r g b
      const uint32_t a = rgb_word(p), b = rgb_word(p + 4), c = rgb_word(p + 8);
      l[0] = luma_bt601(byte_f<0>(a), byte_f<1>(a), byte_f<2>(a));
      l[1] = luma_bt601(byte_f<3>(a), byte_f<0>(b), byte_f<1>(b));
      l[2] = luma_bt601(byte_f<2>(b), byte_f<3>(b), byte_f<0>(c));
      l[3] = luma_bt601(byte_f<1>(c), byte_f<2>(c), byte_f<3>(c));
    }
    *reinterpret_cast<float4*>(out + r * kConvRow + 4 * lane) = make_float4(l[0], l[1], l[2], l[3]);
  }
  if (lane < 16) {
    const int r = lane >> 2, c = 128 * w + 128 + (lane & 3);
    float v = 0.0f;
    if (c < 512) {
      const unsigned char* p = raw + r * kRowBytes + c * static_cast<int>(sizeof(Tin));
      v = luma_bt601(static_cast<float>(p[0]), static_cast<float>(p[1]), static_cast<float>(p[2]));
    }
    out[r * kConvRow + 128 + (lane & 3)] = v;
  }
}

// Columns 4j .. 4j+7 of one input row held in shared memory.
__device__ __forceinline__ void load_row8(const float* row, int j, float x[8]) {
  const float4* r = reinterpret_cast<const float4*>(row);
  float4 a = r[j], b = r[j + 1];
  x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
  x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
}
// u8 columns as exact floats through a byte permute and one add (byte_f), which keeps the
// 27 conversions per compressed value off the quarter-rate conversion pipe.
__device__ __forceinline__ void load_row8(const uint8_t* row, int j, float x[8]) {
  const uint32_t* r = reinterpret_cast<const uint32_t*>(row);
  uint32_t a = r[j], b = r[j + 1];
  x[0] = byte_f<0>(a); x[1] = byte_f<1>(a); x[2] = byte_f<2>(a); x[3] = byte_f<3>(a);
  x[4] = byte_f<0>(b); x[5] = byte_f<1>(b); x[6] = byte_f<2>(b); x[7] = byte_f<3>(b);
}

#define YPDQ_W(di, dj) __uint_as_float(YPDQ_TENT_BITS_##di##_##dj)
#define YPDQ_TAP(acc, di, dj, x) acc = __fadd_rn(acc, __fmul_rn(YPDQ_W(di, dj), (x)))
#define YPDQ_ROW_TAPS(acc, di, x)     \
  YPDQ_TAP(acc, di, 1, x[2]);         \
  YPDQ_TAP(acc, di, 2, x[3]);         \
  YPDQ_TAP(acc, di, 3, x[4]);         \
  YPDQ_TAP(acc, di, 4, x[5]);         \
  YPDQ_TAP(acc, di, 5, x[6])

// Compressed value (i, j) in the reference's tap order: rows 4i+1 .. 4i+6 come from stage i
// (rows 0..3) and stage i+1 (rows 0..1); tap (di, dj) reads input column 4j+1+dj, which is
// x[1+dj]; row 4i+1 holds only the two residue taps. Called for consecutive output rows of
// one column: the first two input rows of output row i + 1 (4i + 5, 4i + 6) are the last
// two of row i, so their converted values (x[5], x[6] of the first; x[2..6] of the second)
// stay in registers instead of being read and converted twice.
struct CompressCarry {
  float a5, a6;   // row 4i + 1: the residue taps' inputs
  float b[5];     // row 4i + 2: x[2..6]
};
template <typename Tin, int kRow = 512>
__device__ __forceinline__ float compress_next(const Tin* st0, const Tin* st1, int j, bool first,
                                               CompressCarry& c) {
  float x[8];
  float s = 0.0f;
  if (first) {
    load_row8(st0 + 0 * kRow, j, x);
    c.a5 = x[5];
    c.a6 = x[6];
    load_row8(st0 + 1 * kRow, j, x);
#pragma unroll
    for (int e = 0; e < 5; ++e) c.b[e] = x[2 + e];
  }
  YPDQ_TAP(s, 0, 4, c.a5);
  YPDQ_TAP(s, 0, 5, c.a6);
  YPDQ_TAP(s, 1, 1, c.b[0]);
  YPDQ_TAP(s, 1, 2, c.b[1]);
  YPDQ_TAP(s, 1, 3, c.b[2]);
  YPDQ_TAP(s, 1, 4, c.b[3]);
  YPDQ_TAP(s, 1, 5, c.b[4]);
  load_row8(st0 + 2 * kRow, j, x);
  YPDQ_ROW_TAPS(s, 2, x);
  load_row8(st0 + 3 * kRow, j, x);
  YPDQ_ROW_TAPS(s, 3, x);
  load_row8(st1 + 0 * kRow, j, x);
  YPDQ_ROW_TAPS(s, 4, x);
  c.a5 = x[5];
  c.a6 = x[6];
  load_row8(st1 + 1 * kRow, j, x);
  YPDQ_ROW_TAPS(s, 5, x);
#pragma unroll
  for (int e = 0; e < 5; ++e) c.b[e] = x[2 + e];
  return s;
}

// Separable compress (YPDQ_COMPRESS_SEPARABLE; not the reference's operation order). The
// tent weights are W[di][dj] = c[di] c[dj] / 81 with c = (0, 1, 2, 3, 2, 1, 0) (the 128-bit
// table also holds two subnormal residue taps, ~1e-40, which this form drops). So
//   out[i][j] = S / 81,  S = sum_{r = 2..6} c[r] h(4i + r),  h(row) = sum_{k = 2..6} c[k] x[row][4j + k]
// Each h row serves two output rows. For u8 input h and S are exact integers (two dp4a per
// h), so the only rounding is the final scale.
__device__ __forceinline__ float hsum(const uint8_t* row, int j) {
  const uint32_t* r = reinterpret_cast<const uint32_t*>(row);
  // bytes of r[j]: columns 4j .. 4j+3 (weights 0, 0, 1, 2); r[j+1]: 4j+4 .. 4j+7 (3, 2, 1, 0)
  return static_cast<float>(__dp4a(r[j], 0x02010000u, __dp4a(r[j + 1], 0x00010203u, 0u)));
}
__device__ __forceinline__ float hsum(const float* row, int j) {
  const float4* r = reinterpret_cast<const float4*>(row);
  const float4 a = r[j], b = r[j + 1];  // columns 4j .. 4j+3 and 4j+4 .. 4j+7
  return (a.z + b.z) + 2.0f * (a.w + b.y) + 3.0f * b.x;
}
// h of rows 1..3 of a 4-row stage (rows 4s+2 .. 4s+4), carried to the next output row.
struct HCarry {
  float h1, h2, h3;
};
template <typename Tin, int kRow = 512>
__device__ __forceinline__ void hcarry_init(const Tin* st, int j, HCarry& c) {
  c.h1 = hsum(st + 1 * kRow, j);
  c.h2 = hsum(st + 2 * kRow, j);
  c.h3 = hsum(st + 3 * kRow, j);
}
// Output row i from the carried h of stage i and the new stage i+1 (rows 4i+5 .. 4i+8).
template <typename Tin, int kRow = 512>
__device__ __forceinline__ float compress_separable(const Tin* st1, int j, HCarry& c) {
  const float n0 = hsum(st1 + 0 * kRow, j), n1 = hsum(st1 + 1 * kRow, j);
  const float n2 = hsum(st1 + 2 * kRow, j), n3 = hsum(st1 + 3 * kRow, j);
  const float S = (c.h1 + n1) + 2.0f * (c.h2 + n0) + 3.0f * c.h3;
  c.h1 = n1;
  c.h2 = n2;
  c.h3 = n3;
  return S * (1.0f / 81.0f);
}

// ---------------------------------------------------------------- epilogue

__device__ __forceinline__ uint32_t f32_key(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_f32(uint32_t k) {
  uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  return __uint_as_float(u);
}

// Exact 128th-smallest (rank 127) of four 256-value sets held 8 per lane: MSB-first
// radix selection on order-preserving keys, one warp reduction per bit and set.
__device__ __forceinline__ void select_rank127_x4(const float (&v)[4][8], float (&out)[4]) {
  uint32_t key[4][8];
#pragma unroll
  for (int s = 0; s < 4; ++s)
#pragma unroll
    for (int e = 0; e < 8; ++e) key[s][e] = f32_key(v[s][e]);
  uint32_t prefix[4] = {0u, 0u, 0u, 0u};
  int rank[4] = {127, 127, 127, 127};
  uint32_t decided = 0u;
#pragma unroll 4
  for (int bit = 31; bit >= 0; --bit) {
    const uint32_t b = 1u << bit;
    const uint32_t m = decided | b;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      uint32_t c = 0;
#pragma unroll
      for (int e = 0; e < 8; ++e) c += ((key[s][e] & m) == prefix[s]) ? 1u : 0u;
      const int tot = static_cast<int>(__reduce_add_sync(0xffffffffu, c));
      if (rank[s] >= tot) {
        rank[s] -= tot;
        prefix[s] |= b;
      }
    }
    decided = m;
  }
#pragma unroll
  for (int s = 0; s < 4; ++s) out[s] = key_f32(prefix[s]);
}

// Slot s of the 8 outputs: value at (r, c) is sign * (s < 4 ? P[r][c] : P[c][r]).
// Row signs (row_mask) apply in slots 2, 3, 5, 6; column signs (col_mask) in 1, 2, 6, 7.
__device__ __forceinline__ bool slot_rows(int s) { return s == 2 || s == 3 || s == 5 || s == 6; }
__device__ __forceinline__ bool slot_cols(int s) { return s == 1 || s == 2 || s == 6 || s == 7; }

// Sum of gradients of slot s, summed sequentially in the reference order.
__device__ float slot_gradient(const float* P, int s, uint32_t rm, uint32_t cm) {
  const bool tr = s >= 4, ur = slot_rows(s), uc = slot_cols(s);
  auto val = [&](int r, int c) -> float {
    float x = tr ? P[c * 16 + r] : P[r * 16 + c];
    bool neg = (ur && ((rm >> r) & 1u)) != (uc && ((cm >> c) & 1u));
    return neg ? -x : x;
  };
  float g = 0.0f;
  float prev[16];
#pragma unroll
  for (int c = 0; c < 16; ++c) prev[c] = val(0, c);
#pragma unroll 1
  for (int r = 0; r < 15; ++r) {
    float nxt[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) nxt[c] = val(r + 1, c);
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      g = __fadd_rn(g, fabsf(__fsub_rn(prev[c], nxt[c])));
      prev[c] = nxt[c];
    }
  }
#pragma unroll 1
  for (int r = 0; r < 16; ++r) {
    float row[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) row[c] = val(r, c);
#pragma unroll
    for (int c = 0; c < 15; ++c) g = __fadd_rn(g, fabsf(__fsub_rn(row[c], row[c + 1])));
  }
  return g;
}

struct EpilogueOut {
  uint8_t* hashes;   // [8][32]
  float* quality;    // [8]
  float* thresholds; // [8]
  float* pdqf;       // [pdqf_slots][256]
  int pdqf_slots;
};

// One warp turns a PDQF held in shared memory into the 8 slot hashes, thresholds and
// qualities. With thr0_given the slot-0 threshold is taken from the caller.
__device__ void epilogue_warp(const float* P, bool thr0_given, float thr0_in, uint32_t rm,
                              uint32_t cm, int lane, const EpilogueOut& o) {
  // lane owns flat elements k = 8*lane + e, i.e. row i = lane/2, columns j0 .. j0+7
  const int i = lane >> 1, j0 = (lane & 1) << 3;
  const bool rneg = (rm >> i) & 1u;
  float x[8], xt[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    x[e] = P[i * 16 + j0 + e];
    xt[e] = P[(j0 + e) * 16 + i];
  }
  float v[8][8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const bool cneg = (cm >> (j0 + e)) & 1u;
    const float cx = cneg ? -x[e] : x[e];
    const float cxt = cneg ? -xt[e] : xt[e];
    v[0][e] = x[e];
    v[1][e] = cx;
    v[2][e] = rneg ? -cx : cx;
    v[3][e] = rneg ? -x[e] : x[e];
    v[4][e] = xt[e];
    v[5][e] = rneg ? -xt[e] : xt[e];
    v[6][e] = rneg ? -cxt : cxt;
    v[7][e] = cxt;
  }
  float med[4];
  {
    float sel[4][8];
#pragma unroll
    for (int s = 0; s < 4; ++s)
#pragma unroll
      for (int e = 0; e < 8; ++e) sel[s][e] = v[s][e];
    select_rank127_x4(sel, med);
  }
  float thr[8];
  thr[0] = thr0_given ? thr0_in : med[0];
  thr[1] = med[1];
  thr[2] = med[2];
  thr[3] = med[3];
  thr[4] = thr[0];
  thr[5] = thr[1];
  thr[6] = thr[2];
  thr[7] = thr[3];
  if (o.hashes) {
#pragma unroll
    for (int s = 0; s < 8; ++s) {
      uint32_t byte = 0;
#pragma unroll
      for (int e = 0; e < 8; ++e) byte |= (v[s][e] > thr[s] ? 1u : 0u) << e;
      o.hashes[s * 32 + 31 - lane] = static_cast<uint8_t>(byte);
    }
  }
  if (o.pdqf) {
    const int slots = o.pdqf_slots == 8 ? 8 : 1;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
      if (s < slots) {
        float4* dst = reinterpret_cast<float4*>(o.pdqf + s * 256 + lane * 8);
        dst[0] = make_float4(v[s][0], v[s][1], v[s][2], v[s][3]);
        dst[1] = make_float4(v[s][4], v[s][5], v[s][6], v[s][7]);
      }
    }
  }
  if (lane < 8) {
    float t = thr[0];
#pragma unroll
    for (int s = 1; s < 8; ++s)
      if (lane == s) t = thr[s];
    if (o.thresholds) o.thresholds[lane] = t;
    if (o.quality) {
      const float g = slot_gradient(P, lane, rm, cm);
      o.quality[lane] = fminf(__fdiv_rn(g, 180.0f), 1.0f);
    }
  }
}

// ------------------------------------------------------------------- kernel

// tcgen05 MMAs for the tensor-core DCT (M = 128, N = 16, f32 accumulate in TMEM).
__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
// D f32, A/B tf32 (format 2) or bf16 (format 1), K-major, M = 128, N = 16.
constexpr uint32_t kIdescTf32 = (1u << 4) | (2u << 7) | (2u << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);
constexpr uint32_t kIdescBf16 = (1u << 4) | (1u << 7) | (1u << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ void split_bf16(float x, uint16_t& hi, uint16_t& lo) {
  const __nv_bfloat16 h = __float2bfloat16_rn(x);
  const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
  hi = __bfloat16_as_ushort(h);
  lo = __bfloat16_as_ushort(l);
}
// split_bf16 of two values at once (packed conversions); a in the low halves.
__device__ __forceinline__ void split_bf16x2(float a, float b, uint32_t& hi, uint32_t& lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  const float2 hf = __bfloat1622float2(h);
  const __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}
// Byte offset of element e (of `esize` bytes) in row r of a 128B-swizzled K-major chunk.
__device__ __forceinline__ uint32_t sw128_offset(uint32_t r, uint32_t e, uint32_t esize) {
  const uint32_t byte = e * esize;
  return r * 128 + ((((byte >> 4) ^ (r & 7))) << 4) + (byte & 15);
}
// Byte offset of element e (of esize bytes) of row r in a 64-byte-swizzled K-major tile:
// rows of 64 B, 8-row atoms of 512 B, 16-byte chunk c stored at c ^ ((r >> 1) & 3).
__device__ __forceinline__ uint32_t sw64_offset(uint32_t r, uint32_t e, uint32_t esize) {
  const uint32_t byte = e * esize;
  return r * 64 + ((((byte >> 4) ^ ((r >> 1) & 3))) << 4) + (byte & 15);
}
// Operand descriptor of the tensor-core DCT's layout (TF32: 128 B swizzle, BF16: 64 B).
template <int kDct>
__device__ __forceinline__ uint64_t dct_desc(uint32_t saddr) {
  if constexpr (kDct == 1) return sw128_desc(saddr);
  else return sw64_desc(saddr);
}
// 16 consecutive TMEM columns of this warp's 32 lanes (valid after tmem_ld_wait).
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tmem_take16(uint32_t (&r)[16]) {
  asm volatile(""
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                 "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                 "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]));
}

// The compress input of global stage g: the ring slot itself, or (RGB) its luma slot.
// (for RGB: the calling warp's staging, which starts at input column 128 * warp, so the
// compress reads it at column index j - 32 * warp with rows kConvRow apart)
template <typename Tin, typename CT, int kNumStages, typename Smem>
__device__ __forceinline__ const CT* stage_ptr(Smem& sm, uint32_t g, int warp) {
  if constexpr (is_rgb<Tin>()) return sm.conv[warp][g % 3];
  else return reinterpret_cast<const CT*>(sm.ring[g % kNumStages]);
}

template <typename Tin, int kDct, bool kSep>
__global__ void __launch_bounds__(hash_threads<kDct>(), (hash_min_blocks<Tin, kDct>()))
    hash_kernel(const HashLaunch prm) {
  constexpr int kRowBytes = InputTraits<Tin>::kRowBytes;
  constexpr int kStageBytes = 4 * kRowBytes;
  constexpr int kNumStages = ring_stages<Tin, kDct>();
  constexpr int kThreads = hash_threads<kDct>();
  using Smem = HashSmem<kStageBytes, kNumStages, kDct, conv_slots<Tin>()>;
  constexpr bool kRgb = is_rgb<Tin>();
  using CT = typename CompressIn<Tin>::T;
  extern __shared__ unsigned char smem_raw[];
  // Align by offsetting the shared array itself so the compiler keeps the shared address
  // space (an integer round trip would turn every access into a generic one).
  Smem& sm = *reinterpret_cast<Smem*>(smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u));

  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;

  for (int idx = tid; idx < 16 * 127; idx += kThreads) {
    const int k = idx / 127, i = idx - k * 127;
    const float d = g_dct[idx];
    if constexpr (kDct == 0) sm.dt[i][k] = d;
    sm.dr[k][i] = d;
  }
  if constexpr (kDct == 0) {
    if (tid < 16) sm.dt[127][tid] = 0.0f;
  } else {
    // the DCT matrix as the MMA's B operand: N = 16 rows k, K = 128 (column 127 is zero)
    for (int idx = tid; idx < 16 * 128; idx += kThreads) {
      const int k = idx >> 7, i = idx & 127;
      const float d = i < 127 ? g_dct[k * 127 + i] : 0.0f;
      if constexpr (kDct == 1) {
        *reinterpret_cast<uint32_t*>(sm.dops + (i >> 5) * 2048 + sw128_offset(k, i & 31, 4)) = to_tf32(d);
      } else {
        uint16_t hi, lo;
        split_bf16(d, hi, lo);
        const uint32_t off = (i >> 5) * 1024 + sw64_offset(k, i & 31, 2);
        *reinterpret_cast<uint16_t*>(sm.dops + off) = hi;
        *reinterpret_cast<uint16_t*>(sm.dops + 4096 + off) = lo;
      }
    }
    fence_proxy_async_smem();
  }
  if (tid == 0) {
    for (int s = 0; s < kNumStages; ++s) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], kComputeThreads / 32);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sm.pfull[b], kComputeThreads / 32);
      mbar_init(&sm.pempty[b], 1);
      mbar_init(&sm.a_full[b], kComputeThreads / 32);
      mbar_init(&sm.a_empty[b], 1);
      mbar_init(&sm.acc_full[b], 1);
      mbar_init(&sm.acc_empty[b], kComputeThreads / 32);
    }
    mbar_init(&sm.tc_exit, kComputeThreads / 32);
    mbar_init(&sm.mma_done, 1);
    sm.abort_flag = 0;
    fence_mbar_init();
  }
  if constexpr (kDct != 0) {
    if (warp == kMmaWarpHash) {
      tmem_alloc(&sm.tmem_base, 32);  // two 16-column accumulators
      tmem_relinquish();
    }
    tc_fence_before();
  }
  __syncthreads();
  if constexpr (kDct != 0) tc_fence_after();

  volatile int* abort_flag = &sm.abort_flag;
  const int64_t n_images = prm.n_dev ? min(*prm.n_dev, prm.n) : prm.n;
  const unsigned char* images = static_cast<const unsigned char*>(prm.images);
  constexpr int64_t kImageBytes = 512ll * kRowBytes;

  if (warp == kProducerWarp) {
    if (lane != 0) return;
    const uint64_t policy = policy_evict_first();
    uint32_t g = 0;
    bool ok = true;
    for (int64_t n = blockIdx.x; n < n_images && ok; n += gridDim.x) {
      const unsigned char* img = images + n * kImageBytes;
      for (int s = 0; s < kStagesPerImage; ++s, ++g) {
        const uint32_t slot = g % kNumStages;
        if (!mbar_wait(&sm.empty[slot], ((g / kNumStages) & 1u) ^ 1u, abort_flag)) {
          ok = false;
          break;
        }
        const uint32_t bytes = (s < kStagesPerImage - 1) ? 4 * kRowBytes : 2 * kRowBytes;
        mbar_arrive_expect_tx(&sm.full[slot], bytes);
        bulk_g2s(sm.ring[slot], img + static_cast<int64_t>(4 * s + 1) * kRowBytes, bytes,
                 &sm.full[slot], policy);
      }
    }
    if (!ok) {
      *abort_flag = 1;
      atomicOr(prm.dev_err, kDevErrTimeout);
      // Let the copies already issued land before the CTA exits (bounded wait each).
      for (uint32_t k = 1; k <= kNumStages && k <= g; ++k) {
        const uint32_t gi = g - k;
        const uint64_t t0 = globaltimer_ns();
        while (!mbar_try_wait(&sm.full[gi % kNumStages], (gi / kNumStages) & 1u)) {
          if (globaltimer_ns() - t0 > kWaitLimitNs / 4) break;
        }
      }
    }
    return;
  }

  if (warp == kEpilogueWarp) {
    uint32_t it = 0;
    for (int64_t n = blockIdx.x; n < n_images; n += gridDim.x, ++it) {
      const int pb = it & 1;
      if (!mbar_wait(&sm.pfull[pb], (it >> 1) & 1u, abort_flag)) {
        *abort_flag = 1;
        if (lane == 0) atomicOr(prm.dev_err, kDevErrTimeout);
        return;
      }
      EpilogueOut o;
      o.hashes = prm.hashes ? prm.hashes + n * 256 : nullptr;
      o.quality = prm.quality ? prm.quality + n * 8 : nullptr;
      o.thresholds = prm.thresholds ? prm.thresholds + n * 8 : nullptr;
      o.pdqf_slots = prm.pdqf_slots;
      o.pdqf = prm.pdqf ? prm.pdqf + n * (prm.pdqf_slots == 8 ? 8 : 1) * 256 : nullptr;
      epilogue_warp(sm.p[pb], false, 0.0f, prm.row_mask, prm.col_mask, lane, o);
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.pempty[pb]);
    }
    return;
  }

  if constexpr (kDct != 0) {
    if (warp == kMmaWarpHash) {
      constexpr int kChunks = 128 / DctTraits<kDct>::kRowsPerChunk;
      const uint32_t tmem = sm.tmem_base;
      if (lane == 0) {
        bool ok = true;
        uint32_t gc = 0, it = 0;
        for (int64_t n = blockIdx.x; n < n_images && ok; n += gridDim.x, ++it) {
          const uint32_t acc = it & 1;
          if (!mbar_wait(&sm.acc_empty[acc], ((it >> 1) & 1u) ^ 1u, abort_flag)) {
            ok = false;
            break;
          }
          tc_fence_after();
          for (int c = 0; c < kChunks; ++c, ++gc) {
            const uint32_t buf = gc & 1;
            if (!mbar_wait(&sm.a_full[buf], (gc >> 1) & 1u, abort_flag)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t a = smem_u32(sm.ops[buf]);
            using TR = DctTraits<kDct>;
            const uint32_t d = smem_u32(sm.dops) + c * TR::kDChunkBytes;
#pragma unroll
            for (int ks = 0; ks < TR::kKSteps; ++ks) {
              const uint32_t accumulate = (c > 0 || ks > 0) ? 1u : 0u;
              if constexpr (kDct == 1) {
                mma_tf32(tmem + acc * 16, dct_desc<kDct>(a + ks * 32), dct_desc<kDct>(d + ks * 32),
                         kIdescTf32, accumulate);
              } else {
                // x * y ~ xh*yh + xh*yl + xl*yh   (x = A, y = D)
                mma_bf16(tmem + acc * 16, dct_desc<kDct>(a + ks * 32),
                         dct_desc<kDct>(d + ks * 32), kIdescBf16, accumulate);
                mma_bf16(tmem + acc * 16, dct_desc<kDct>(a + ks * 32),
                         dct_desc<kDct>(d + TR::kDLo + ks * 32), kIdescBf16, 1u);
                mma_bf16(tmem + acc * 16, dct_desc<kDct>(a + TR::kALo + ks * 32),
                         dct_desc<kDct>(d + ks * 32), kIdescBf16, 1u);
              }
            }
            mma_commit(&sm.a_empty[buf]);
          }
          if (ok) mma_commit(&sm.acc_full[acc]);
        }
        if (!ok) {
          *abort_flag = 1;
          atomicOr(prm.dev_err, kDevErrTimeout);
        }
        mma_commit(&sm.mma_done);
        const uint64_t t0 = globaltimer_ns();
        while (!mbar_try_wait(&sm.mma_done, 0))
          if (globaltimer_ns() - t0 > kWaitLimitNs) {
            // the MMAs did not drain: the results are not trustworthy, so flag the launch
            *abort_flag = 1;
            atomicOr(prm.dev_err, kDevErrTimeout);
            break;
          }
      }
      __syncwarp();
      const uint64_t t0 = globaltimer_ns();
      while (!mbar_try_wait(&sm.tc_exit, 0))
        if (globaltimer_ns() - t0 > kWaitLimitNs) {
          // the compute warps did not report that they stopped reading tensor memory
          if (lane == 0) {
            *abort_flag = 1;
            atomicOr(prm.dev_err, kDevErrTimeout);
          }
          break;
        }
      tc_fence_after();
      tmem_dealloc(tmem, 32);
      return;
    }
  }

  // ---- compute warps: thread j <-> compressed column j
  const int j = tid;
  const bool active = j < 127;
  // column index and row stride the compress reads with (RGB: the warp's own staging)
  const int jc = kRgb ? lane : j;
  constexpr int kCRow = kRgb ? kConvRow : 512;
  uint32_t it = 0;
  for (int64_t n = blockIdx.x; n < n_images; n += gridDim.x, ++it) {
    const uint32_t g0 = it * kStagesPerImage;
    if constexpr (kDct != 0) {
      // stage 1 on tensor cores: write the compressed column into the operand chunks
      constexpr int kR = DctTraits<kDct>::kRowsPerChunk;
      constexpr uint32_t kChunks = 128 / kR;
      const uint32_t gc0 = it * kChunks;
      if (!mbar_wait(&sm.full[g0 % kNumStages], (g0 / kNumStages) & 1u, abort_flag)) goto fail;
      if constexpr (kRgb) {
        // the first stage to luma; the barrier also orders this image's slot writes after
        // every thread's last read of the previous image
        convert_stage_warp<Tin>(sm.ring[g0 % kNumStages], sm.conv[warp][g0 % 3], warp, lane);
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.empty[g0 % kNumStages]);
      }
      HCarry hc{};
      CompressCarry cc{};
      if (kSep && active)
        hcarry_init<CT, kCRow>(stage_ptr<Tin, CT, kNumStages>(sm, g0, warp), jc, hc);
      for (int i0 = 0; i0 < 128; i0 += 4) {
        float b[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int i = i0 + r;
          b[r] = 0.0f;
          if (i < 127) {
            const uint32_t ga = g0 + i, gb = ga + 1;
            if (!mbar_wait(&sm.full[gb % kNumStages], (gb / kNumStages) & 1u, abort_flag))
              goto fail;
            if constexpr (kRgb) {
              convert_stage_warp<Tin>(sm.ring[gb % kNumStages], sm.conv[warp][gb % 3], warp, lane);
              __syncwarp();
              if (lane == 0) mbar_arrive(&sm.empty[gb % kNumStages]);
            }
            if (active) {
              const CT* st0 = stage_ptr<Tin, CT, kNumStages>(sm, ga, warp);
              const CT* st1 = stage_ptr<Tin, CT, kNumStages>(sm, gb, warp);
              b[r] = kSep ? compress_separable<CT, kCRow>(st1, jc, hc)
                          : compress_next<CT, kCRow>(st0, st1, jc, i == 0, cc);
              if (prm.buf1) prm.buf1[(n * 127 + i) * 128 + j] = b[r];
            }
            if constexpr (!kRgb) {
              __syncwarp();
              if (lane == 0) mbar_arrive(&sm.empty[ga % kNumStages]);
            }
          }
        }
        const uint32_t within = static_cast<uint32_t>(i0 % kR);
        const uint32_t chunk = gc0 + static_cast<uint32_t>(i0 / kR);
        const uint32_t buf = chunk & 1;
        if (within == 0 &&
            !mbar_wait(&sm.a_empty[buf], ((chunk >> 1) & 1u) ^ 1u, abort_flag))
          goto fail;
        if constexpr (kDct == 1) {
          const uint4 w = make_uint4(to_tf32(b[0]), to_tf32(b[1]), to_tf32(b[2]), to_tf32(b[3]));
          *reinterpret_cast<uint4*>(sm.ops[buf] + sw128_offset(j, within, 4)) = w;
        } else {
          uint32_t h01, l01, h23, l23;
          split_bf16x2(b[0], b[1], h01, l01);
          split_bf16x2(b[2], b[3], h23, l23);
          const uint32_t off = sw64_offset(j, within, 2);
          *reinterpret_cast<uint2*>(sm.ops[buf] + off) = make_uint2(h01, h23);
          *reinterpret_cast<uint2*>(sm.ops[buf] + DctTraits<kDct>::kALo + off) = make_uint2(l01, l23);
        }
        if (within + 4 == static_cast<uint32_t>(kR)) {
          fence_proxy_async_smem();
          __syncwarp();
          if (lane == 0) mbar_arrive(&sm.a_full[buf]);
        }
      }
      if constexpr (!kRgb) {
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.empty[(g0 + 127) % kNumStages]);
      }
      {
        const uint32_t acc = it & 1;
        if (!mbar_wait(&sm.acc_full[acc], (it >> 1) & 1u, abort_flag)) goto fail;
        tc_fence_after();
        uint32_t tr[16];
        tmem_ld16_nowait(sm.tmem_base + (static_cast<uint32_t>(warp * 32) << 16) + acc * 16, tr);
        tmem_ld_wait();
        tmem_take16(tr);
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&sm.acc_empty[acc]);
        if (active) {
#pragma unroll
          for (int k = 0; k < 16; ++k) sm.t[k][j] = __uint_as_float(tr[k]);
        }
      }
    } else {
    float acc[16][4];

#pragma unroll
    for (int k = 0; k < 16; ++k)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[k][r] = 0.0f;

    if (!mbar_wait(&sm.full[g0 % kNumStages], (g0 / kNumStages) & 1u, abort_flag)) goto fail;
    if constexpr (kRgb) {
      convert_stage_warp<Tin>(sm.ring[g0 % kNumStages], sm.conv[warp][g0 % 3], warp, lane);
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.empty[g0 % kNumStages]);
    }
    HCarry hc{};
    CompressCarry cc{};
    if (kSep && active)
      hcarry_init<CT, kCRow>(stage_ptr<Tin, CT, kNumStages>(sm, g0, warp), jc, hc);
    for (int i0 = 0; i0 < 128; i0 += 4) {
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int i = i0 + r;
        if (i < 127) {
          const uint32_t ga = g0 + i, gb = ga + 1;
          if (!mbar_wait(&sm.full[gb % kNumStages], (gb / kNumStages) & 1u, abort_flag))
            goto fail;
          if constexpr (kRgb) {
            convert_stage_warp<Tin>(sm.ring[gb % kNumStages], sm.conv[warp][gb % 3], warp, lane);
            __syncwarp();
            if (lane == 0) mbar_arrive(&sm.empty[gb % kNumStages]);
          }
          float b = 0.0f;
          if (active) {
            const CT* st0 = stage_ptr<Tin, CT, kNumStages>(sm, ga, warp);
            const CT* st1 = stage_ptr<Tin, CT, kNumStages>(sm, gb, warp);
            b = kSep ? compress_separable<CT, kCRow>(st1, jc, hc)
                     : compress_next<CT, kCRow>(st0, st1, jc, i == 0, cc);
            if (prm.buf1) prm.buf1[(n * 127 + i) * 128 + j] = b;
          }
          const float4* d4 = reinterpret_cast<const float4*>(&sm.dt[i][0]);
          const float4 da = d4[0], db = d4[1], dc = d4[2], dd = d4[3];
          const float d[16] = {da.x, da.y, da.z, da.w, db.x, db.y, db.z, db.w,
                               dc.x, dc.y, dc.z, dc.w, dd.x, dd.y, dd.z, dd.w};
#pragma unroll
          for (int k = 0; k < 16; ++k) acc[k][r] = __fadd_rn(acc[k][r], __fmul_rn(d[k], b));
          if constexpr (!kRgb) {
            __syncwarp();
            if (lane == 0) mbar_arrive(&sm.empty[ga % kNumStages]);
          }
        }
      }
    }
    if constexpr (!kRgb) {
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.empty[(g0 + 127) % kNumStages]);
    }

    if (active) {
#pragma unroll
      for (int k = 0; k < 16; ++k)
        sm.t[k][j] = __fadd_rn(__fadd_rn(__fadd_rn(acc[k][0], acc[k][1]), acc[k][2]), acc[k][3]);
    }
    }  // FP32 stage 1
    named_bar_sync(kComputeBarrier, kComputeThreads);
    {
      // stage 2: P[k][c] = sum_m T[k][m] * D[c][m]; thread -> (k, c0), (k, c0 + 1)
      const int k = tid >> 3, c0 = (tid & 7) * 2;
      float s0[4] = {0.f, 0.f, 0.f, 0.f}, s1[4] = {0.f, 0.f, 0.f, 0.f};
      for (int m0 = 0; m0 < 128; m0 += 4) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int m = m0 + r;
          if (m < 127) {
            const float tv = sm.t[k][m];
            s0[r] = __fadd_rn(s0[r], __fmul_rn(tv, sm.dr[c0][m]));
            s1[r] = __fadd_rn(s1[r], __fmul_rn(tv, sm.dr[c0 + 1][m]));
          }
        }
      }
      const float o0 = __fadd_rn(__fadd_rn(__fadd_rn(s0[0], s0[1]), s0[2]), s0[3]);
      const float o1 = __fadd_rn(__fadd_rn(__fadd_rn(s1[0], s1[1]), s1[2]), s1[3]);
      const int pb = it & 1;
      if (!mbar_wait(&sm.pempty[pb], ((it >> 1) & 1u) ^ 1u, abort_flag)) goto fail;
      sm.p[pb][k * 16 + c0] = o0;
      sm.p[pb][k * 16 + c0 + 1] = o1;
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.pfull[pb]);
    }
    named_bar_sync(kComputeBarrier, kComputeThreads);
  }
  if constexpr (kDct != 0) {
    tc_fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.tc_exit);
  }
  return;
fail:
  *abort_flag = 1;
  if (lane == 0) atomicOr(prm.dev_err, kDevErrTimeout);
  if constexpr (kDct != 0) {
    tc_fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.tc_exit);
  }
}

// Dihedrals of given PDQF matrices: one warp per matrix.
__global__ void __launch_bounds__(128) dihedral_kernel(const DihedralLaunch prm) {
  __shared__ __align__(16) float P[4][256];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t n = static_cast<int64_t>(blockIdx.x) * 4 + w;
  if (n >= prm.n) return;
  const float4* src = reinterpret_cast<const float4*>(prm.pdqf + n * 256);
  float4* dst = reinterpret_cast<float4*>(P[w]);
  dst[lane] = src[lane];
  dst[lane + 32] = src[lane + 32];
  __syncwarp();
  EpilogueOut o;
  o.hashes = prm.hashes ? prm.hashes + n * 256 : nullptr;
  o.quality = prm.quality ? prm.quality + n * 8 : nullptr;
  o.thresholds = prm.thresholds ? prm.thresholds + n * 8 : nullptr;
  o.pdqf = prm.pdqf_out ? prm.pdqf_out + n * 8 * 256 : nullptr;
  o.pdqf_slots = 8;
  const bool given = prm.thr_in != nullptr;
  epilogue_warp(P[w], given, given ? prm.thr_in[n] : 0.0f, prm.row_mask, prm.col_mask, lane, o);
}

// ------------------------------------------------------------------ host side

template <typename Tin, int kDct>
static size_t hash_smem_bytes() {
  return sizeof(HashSmem<4 * InputTraits<Tin>::kRowBytes, ring_stages<Tin, kDct>(), kDct,
                         conv_slots<Tin>()>) +
         1024;  // + base alignment
}

// Dynamic shared memory size, and the largest shared-memory carveout so that the
// occupancy query (and the grid) count the two CTAs per SM that fit.
template <typename Tin, int kDct, bool kSep>
static cudaError_t set_smem_attr_one() {
  cudaError_t e = cudaFuncSetAttribute(hash_kernel<Tin, kDct, kSep>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(hash_smem_bytes<Tin, kDct>()));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(hash_kernel<Tin, kDct, kSep>,
                              cudaFuncAttributePreferredSharedMemoryCarveout,
                              static_cast<int>(cudaSharedmemCarveoutMaxShared));
}



// Resident CTAs per SM. The runtime's occupancy query answers 1 for the tcgen05 variants
// although their registers and shared memory admit 2 (ncu's occupancy section agrees on 2),
// so the count is also derived from the per-SM limits and the larger answer is used.
template <typename Tin, int kDct, bool kSep>
static cudaError_t occupancy_of(int* ctas) {
  int api = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &api, hash_kernel<Tin, kDct, kSep>, hash_threads<kDct>(), hash_smem_bytes<Tin, kDct>());
  if (e != cudaSuccess) return e;
  cudaFuncAttributes fa{};
  int dev = 0, smem_sm = 0, reserved = 0, regs_sm = 0, threads_sm = 0;
  e = cudaFuncGetAttributes(&fa, hash_kernel<Tin, kDct, kSep>);
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
  if (e != cudaSuccess) return e;
  const int threads = hash_threads<kDct>();
  const size_t smem_block = hash_smem_bytes<Tin, kDct>() + fa.sharedSizeBytes + reserved;
  const int regs_warp = ((fa.numRegs * 32 + 255) / 256) * 256;  // allocation unit: 256
  const int by_smem = static_cast<int>(smem_sm / smem_block);
  const int by_regs = regs_sm / (regs_warp * (threads / 32));
  const int by_threads = threads_sm / threads;
  int derived = by_smem < by_regs ? by_smem : by_regs;
  if (by_threads < derived) derived = by_threads;
  *ctas = api > derived ? api : derived;
  return cudaSuccess;
}

cudaError_t hash_occupancy(int input_kind, int* ctas_per_sm) {
  return hash_occupancy_variant(input_kind, 0, 0, ctas_per_sm);
}

// Calls F<Tin, kDct, kSep>::run(args...) for the runtime (input kind, DCT, separable).
template <template <typename, int, bool> class F, typename... A>
static cudaError_t dispatch(int kind, int dct, int sep, A&&... args) {
#define YPDQ_CASE(K, T)                                                        \
  case K:                                                                      \
    switch (dct * 2 + (sep ? 1 : 0)) {                                         \
      case 0: return F<T, 0, false>::run(args...);                             \
      case 1: return F<T, 0, true>::run(args...);                              \
      case 2: return F<T, 1, false>::run(args...);                             \
      case 3: return F<T, 1, true>::run(args...);                              \
      case 4: return F<T, 2, false>::run(args...);                             \
      case 5: return F<T, 2, true>::run(args...);                              \
      default: return cudaErrorInvalidValue;                                   \
    }
  switch (kind) {
    YPDQ_CASE(YPDQ_INPUT_F32, float)
    YPDQ_CASE(YPDQ_INPUT_U8, uint8_t)
    YPDQ_CASE(YPDQ_INPUT_RGB8, rgb8_t)
    YPDQ_CASE(YPDQ_INPUT_RGBA8, rgba8_t)
    default: return cudaErrorInvalidValue;
  }
#undef YPDQ_CASE
}

template <typename Tin, int kDct, bool kSep>
struct OccupancyOf {
  static cudaError_t run(int* ctas) { return occupancy_of<Tin, kDct, kSep>(ctas); }
};
template <typename Tin, int kDct, bool kSep>
struct SetSmemAttr {
  static cudaError_t run() { return set_smem_attr_one<Tin, kDct, kSep>(); }
};
template <typename Tin, int kDct, bool kSep>
struct LaunchOne {
  static cudaError_t run(const HashLaunch& p, int64_t grid, cudaStream_t s) {
    hash_kernel<Tin, kDct, kSep><<<static_cast<int>(grid), hash_threads<kDct>(),
                                   hash_smem_bytes<Tin, kDct>(), s>>>(p);
    return cudaGetLastError();
  }
};

cudaError_t hash_occupancy_variant(int input_kind, int dct, int separable, int* ctas_per_sm) {
  return dispatch<OccupancyOf>(input_kind, dct, separable, ctas_per_sm);
}

cudaError_t launch_hash(const HashLaunch& p, int num_sms, int ctas_per_sm, cudaStream_t s) {
  if (p.n <= 0) return cudaSuccess;
  int64_t grid = static_cast<int64_t>(num_sms) * (ctas_per_sm > 0 ? ctas_per_sm : 1);
  if (grid > p.n) grid = p.n;
  return dispatch<LaunchOne>(p.input_kind, p.dct, p.separable, p, grid, s);
}

cudaError_t upload_constants() {
  float d[16 * 127];
  for (int i = 0; i < 16 * 127; ++i) {
    uint32_t b = YPDQ_DCT_F32_BITS[i];
    memcpy(&d[i], &b, 4);
  }
  cudaError_t e = cudaMemcpyToSymbol(g_dct, d, sizeof(d));
  for (int kind = 0; kind < 4 && e == cudaSuccess; ++kind)
    for (int dct = 0; dct < 3 && e == cudaSuccess; ++dct)
      for (int sep = 0; sep < 2 && e == cudaSuccess; ++sep) e = dispatch<SetSmemAttr>(kind, dct, sep);
  return e;
}

cudaError_t launch_dihedrals(const DihedralLaunch& p, cudaStream_t s) {
  if (p.n <= 0) return cudaSuccess;
  const int64_t grid = (p.n + 3) / 4;
  dihedral_kernel<<<static_cast<unsigned>(grid), 128, 0, s>>>(p);
  return cudaGetLastError();
}

}  // namespace ypdq
