// ReferenceKernel<f32> on the GPU (YPDQ_COMPRESS_JAROSZ): yume-pdq's pdqhash-faithful kernel.
//
// jarosz_compress (src/kernel/mod.rs:790-820) filters the whole 512x512 image with
// jarosz_filter_float (src/kernel/ref.rs): two repetitions of a box filter along rows, then
// along columns, with window ceil(512 / 254) = 3. Each line is filtered by a running sum in
// four phases (fill, grow, slide, shrink) with correctly rounded f32 divisions, so every
// output depends on the rounding of the whole prefix of its line; the kernels below replay
// that sum in the same order. The filtered image is sampled at ((2 o + 1) 512) / 254 and
// transformed by the reference kernel's DCT (one sequential accumulator per output,
// src/kernel/mod.rs:711-735).
// Median, packing, quality and dihedrals are the batched dihedral kernel's.
//
// Four launches per chunk of images, through two f32 planes (X, Y) per image. Every line is
// one thread's sequential running sum, so a chunk of 512 images puts 262,144 independent
// lines in flight per pass; each thread keeps the loads of its next 16 or 32 values in
// registers while it filters the current ones.
//   rows1      : Y = box along rows of the input (converted to f32 on load: u8 cast, or
//                BT.601 luma for RGB8/RGBA8). A warp owns 32 rows; 32x32 tiles transposed in
//                shared memory keep the global accesses coalesced.
//   cols1      : X = box along columns of Y (a thread owns a column; coalesced by construction)
//   rows2      : Yc = box along rows of X, keeping only the 127 sampled columns
//                (512 x 128 per image)
//   cols2+dct  : box along the columns of Yc, and at each of the 127 sampled rows the first
//                DCT stage takes the sample into its accumulators, in the reference's order;
//                the second DCT stage follows in shared memory.
// Only the sampled outputs of the second repetition are ever stored: 5.5 MB of HBM traffic
// per f32 image (4.75 MB per u8 image) instead of 10.5 MB for four full passes.
#include "ypdq_internal.cuh"
#include "ypdq_tables.h"

namespace ypdq {

__device__ float g_dct[16 * 127];  // the f32 DCT matrix D[i][k]

namespace {

constexpr int kN = 512;
constexpr size_t kPlane = static_cast<size_t>(kN) * kN;

// x / 3 correctly rounded (IEEE round to nearest even) without a division: Markstein's
// correction of the product by the reciprocal (P. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990).
// q0 = RN(x c) with c = RN(1/3); the remainder r = x - 3 q0 is exact in one FMA, and
// q = RN(q0 + r c). This equals x / 3 for every finite x: tests/test_div3.py compares all
// 2^31 non-negative patterns with IEEE division, and each step is odd in x. For x = +-inf
// the remainder is NaN and q0 (= x) is the quotient; NaN stays NaN.
__device__ __forceinline__ float div3_rn(float x) {
  const float c = 0x1.555556p-2f;  // RN(1/3)
  const float q0 = __fmul_rn(x, c);
  const float r = __fmaf_rn(-q0, 3.0f, x);
  return r == r ? __fmaf_rn(r, c, q0) : q0;
}

// The reference's running-sum box filter of window 3 over one line, one input at a time:
// fill takes in[0]; the value that grow2 / grow3 / slide take as in[ri] yields the output
// for position ri - 1; finish yields position 511. The reference divides by its running
// window count, which is 2 at positions 0 and 511 and 3 everywhere else: x / 2 is exactly
// RN(x * 0.5), and x / 3 is div3_rn. History holds in[ri-1], in[ri-2], in[ri-3].
struct Box3 {
  float sum = 0.0f;
  float h1 = 0.0f, h2 = 0.0f, h3 = 0.0f;
  __device__ __forceinline__ void shift(float v) {
    h3 = h2;
    h2 = h1;
    h1 = v;
  }
  __device__ __forceinline__ void fill(float v) {  // ri = 0 (half window - 1 = 1 value)
    sum = __fadd_rn(sum, v);
    shift(v);
  }
  __device__ __forceinline__ float grow2(float v) {  // ri = 1: position 0, window 2
    sum = __fadd_rn(sum, v);
    shift(v);
    return __fmul_rn(sum, 0.5f);
  }
  __device__ __forceinline__ float grow3(float v) {  // ri = 2: position 1, window 3
    sum = __fadd_rn(sum, v);
    shift(v);
    return div3_rn(sum);
  }
  __device__ __forceinline__ float slide(float v) {  // ri >= 3: position ri - 1, drop in[ri-3]
    sum = __fadd_rn(sum, v);
    sum = __fsub_rn(sum, h3);
    shift(v);
    return div3_rn(sum);
  }
  __device__ __forceinline__ float finish() {  // shrink: position 511 drops in[509] = h3
    sum = __fsub_rn(sum, h3);
    return __fmul_rn(sum, 0.5f);
  }
  // in[ri] for any ri; returns whether an output (for position ri - 1) was produced
  __device__ __forceinline__ bool push(int ri, float v, float& out) {
    if (ri == 0) {
      fill(v);
      return false;
    }
    out = ri == 1 ? grow2(v) : ri == 2 ? grow3(v) : slide(v);
    return true;
  }
};

__device__ __forceinline__ float byte_as_float(uint32_t b) { return static_cast<float>(b); }
__device__ __forceinline__ float luma601(uint32_t r, uint32_t g, uint32_t b) {
  return __fadd_rn(__fadd_rn(__fmul_rn(0.299f, byte_as_float(r)), __fmul_rn(0.587f, byte_as_float(g))),
                   __fmul_rn(0.114f, byte_as_float(b)));
}

constexpr size_t kCompactPlane = static_cast<size_t>(kN) * 128;  // rows2 output per image

__device__ __forceinline__ int sample_at(int o) { return ((2 * o + 1) * kN) / (127 * 2); }

// Four consecutive pixels (from pixel idx, a multiple of 4) of one image as raw words, and
// as f32: the reference's input buffer (u8 cast, or BT.601 luma for RGB8/RGBA8). The f32
// planes between the passes are read with kKind = YPDQ_INPUT_F32.
template <int kKind>
struct Px4;
template <>
struct Px4<YPDQ_INPUT_F32> {
  using Raw = float4;
  static __device__ __forceinline__ Raw load(const uint8_t* img, size_t idx) {
    return *reinterpret_cast<const float4*>(img + 4 * idx);
  }
  static __device__ __forceinline__ float4 cvt(Raw r) { return r; }
};
template <>
struct Px4<YPDQ_INPUT_U8> {
  using Raw = uint32_t;
  static __device__ __forceinline__ Raw load(const uint8_t* img, size_t idx) {
    return *reinterpret_cast<const uint32_t*>(img + idx);
  }
  static __device__ __forceinline__ float4 cvt(Raw r) {
    return make_float4(byte_as_float(r & 0xffu), byte_as_float((r >> 8) & 0xffu),
                       byte_as_float((r >> 16) & 0xffu), byte_as_float(r >> 24));
  }
};
template <>
struct Px4<YPDQ_INPUT_RGB8> {  // 12 bytes, 4-byte aligned: r0 g0 b0 r1 | g1 b1 r2 g2 | b2 r3 g3 b3
  using Raw = uint3;
  static __device__ __forceinline__ Raw load(const uint8_t* img, size_t idx) {
    const uint32_t* w = reinterpret_cast<const uint32_t*>(img + 3 * idx);
    return make_uint3(w[0], w[1], w[2]);
  }
  static __device__ __forceinline__ float4 cvt(Raw r) {
    return make_float4(luma601(r.x & 0xffu, (r.x >> 8) & 0xffu, (r.x >> 16) & 0xffu),
                       luma601(r.x >> 24, r.y & 0xffu, (r.y >> 8) & 0xffu),
                       luma601((r.y >> 16) & 0xffu, r.y >> 24, r.z & 0xffu),
                       luma601((r.z >> 8) & 0xffu, (r.z >> 16) & 0xffu, r.z >> 24));
  }
};
template <>
struct Px4<YPDQ_INPUT_RGBA8> {
  using Raw = uint4;
  static __device__ __forceinline__ Raw load(const uint8_t* img, size_t idx) {
    return *reinterpret_cast<const uint4*>(img + 4 * idx);
  }
  static __device__ __forceinline__ float rgba(uint32_t w) {
    return luma601(w & 0xffu, (w >> 8) & 0xffu, (w >> 16) & 0xffu);
  }
  static __device__ __forceinline__ float4 cvt(Raw r) {
    return make_float4(rgba(r.x), rgba(r.y), rgba(r.z), rgba(r.w));
  }
};

template <int kKind>
__host__ __device__ constexpr size_t bytes_per_px() {
  return kKind == YPDQ_INPUT_U8 ? 1 : kKind == YPDQ_INPUT_RGB8 ? 3 : 4;
}

constexpr int kTileStride = 36;  // floats per tile row: 16-byte rows, conflict-free float4

__device__ __forceinline__ void st4(float* p, float a, float b, float c, float d) {
  *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
}

// Box along rows: block = 4 warps; warp w of block b owns rows 32 (4 b + w) .. +31 of image
// blockIdx.y, in 16 tiles of 32 columns.
//   * Tile t is loaded with 16-byte accesses (lane l: rows l/8 + 4 i, columns 4 (l%8) .. +3;
//     each warp access covers four whole 128-byte rows) into one of two shared buffers,
//     while the loads of tile t+1 go out into registers.
//   * Lane l filters row l of the tile, four values per vector read. The output for position
//     p is produced by input p + 1, so outputs trail inputs by one: each float4 of outputs
//     (positions 4 g .. 4 g + 3) is written in place once input 4 g + 4 has been read, and
//     the last group of tile t - 1 is completed by the first input of tile t.
//   * Tile t - 1 (complete now) goes out with 16-byte stores; kCompact keeps the sampled
//     columns only: output column sample_at(j) goes to Yc[row][j].
// Images at or past *n_dev (graph replay with fewer images than the capture's bound; image
// blockIdx.y of the chunk is image i0 + blockIdx.y of the call) are skipped.
__device__ __forceinline__ bool past_count(const int64_t* n_dev, int64_t i0, unsigned img) {
  return n_dev && i0 + static_cast<int64_t>(img) >= *n_dev;
}

template <int kKind, bool kCompact>
__global__ void __launch_bounds__(128) rows_kernel(const uint8_t* __restrict__ in,
                                                   float* __restrict__ out,
                                                   const int64_t* n_dev, int64_t i0) {
  using P = Px4<kKind>;
  if (past_count(n_dev, i0, blockIdx.y)) return;
  __shared__ __align__(16) float tiles[4][2][32][kTileStride];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int lr = lane >> 3, lc = 4 * (lane & 7);
  const int r0 = 32 * (4 * blockIdx.x + w);
  const uint8_t* img = in + blockIdx.y * kPlane * bytes_per_px<kKind>();
  const size_t base = static_cast<size_t>(r0) * kN;
  float* dst = kCompact ? out + blockIdx.y * kCompactPlane + static_cast<size_t>(r0) * 128
                        : out + blockIdx.y * kPlane + base;
  typename P::Raw pre[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) pre[i] = P::load(img, base + (lr + 4 * i) * kN + lc);
  Box3 box;
  float h0 = 0.0f, h1 = 0.0f, h2 = 0.0f;  // outputs waiting for their group's last one
  int jlo = 0;                              // kCompact: first sampled column not yet stored

  // tile buffer b holds global columns c0 .. c0 + 31 of the warp's rows, all filtered
  auto store_tile = [&](float (*b)[kTileStride], int c0) {
    if constexpr (kCompact) {
      // n <= 8 sample columns fall in a tile (they are 4 or 5 apart); lane l stores sample
      // l % 8 of rows l / 8 + 4 i, so each store covers four rows' 32-byte runs of Yc
      const int jt = jlo + lane;
      const int n = __popc(__ballot_sync(0xffffffffu, jt < 127 && sample_at(jt) < c0 + 32));
      const int j = jlo + (lane & 7);
      const bool mine = (lane & 7) < n;
      const int pos = mine ? sample_at(j) - c0 : 0;
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (mine) dst[(lr + 4 * i) * 128 + j] = b[lr + 4 * i][pos];
      jlo += n;
    } else {
#pragma unroll
      for (int i = 0; i < 8; ++i)
        *reinterpret_cast<float4*>(dst + (lr + 4 * i) * kN + c0 + lc) =
            *reinterpret_cast<const float4*>(&b[lr + 4 * i][lc]);
    }
  };

  for (int t = 0; t < kN / 32; ++t) {
    float (*cur)[kTileStride] = tiles[w][t & 1];
    float (*prv)[kTileStride] = tiles[w][(t & 1) ^ 1];
#pragma unroll
    for (int i = 0; i < 8; ++i) *reinterpret_cast<float4*>(&cur[lr + 4 * i][lc]) = P::cvt(pre[i]);
    __syncwarp();
    if (t + 1 < kN / 32) {
#pragma unroll
      for (int i = 0; i < 8; ++i) pre[i] = P::load(img, base + (lr + 4 * i) * kN + 32 * (t + 1) + lc);
    }
    float* row = cur[lane];
    float4 x = *reinterpret_cast<const float4*>(row);
    if (t == 0) {
      box.fill(x.x);
    } else {
      const float o = box.slide(x.x);
      st4(prv[lane] + 28, h0, h1, h2, o);
    }
    h0 = t == 0 ? box.grow2(x.y) : box.slide(x.y);
    h1 = t == 0 ? box.grow3(x.z) : box.slide(x.z);
    h2 = box.slide(x.w);
#pragma unroll
    for (int g = 1; g < 8; ++g) {
      x = *reinterpret_cast<const float4*>(row + 4 * g);
      const float o = box.slide(x.x);
      st4(row + 4 * (g - 1), h0, h1, h2, o);
      h0 = box.slide(x.y);
      h1 = box.slide(x.z);
      h2 = box.slide(x.w);
    }
    __syncwarp();
    if (t > 0) store_tile(prv, 32 * (t - 1));
    __syncwarp();
  }
  float (*last)[kTileStride] = tiles[w][(kN / 32 - 1) & 1];
  st4(last[lane] + 28, h0, h1, h2, box.finish());
  __syncwarp();
  store_tile(last, kN - 32);
}

// Box along columns of full planes: thread c of block b owns column 128 b + c of image
// blockIdx.y, with the next 16 rows' loads in flight while it filters the current 16.
__global__ void __launch_bounds__(128) cols_kernel(const float* __restrict__ Y,
                                                   float* __restrict__ X,
                                                   const int64_t* n_dev, int64_t i0) {
  if (past_count(n_dev, i0, blockIdx.y)) return;
  const int col = 128 * blockIdx.x + threadIdx.x;
  const float* src = Y + blockIdx.y * kPlane + col;
  float* dst = X + blockIdx.y * kPlane + col;
  Box3 box;
  float cur[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) cur[q] = src[q * kN];
  for (int rb = 0; rb < kN / 16; ++rb) {
    float nxt[16];
    if (rb + 1 < kN / 16) {
#pragma unroll
      for (int q = 0; q < 16; ++q) nxt[q] = src[static_cast<size_t>(16 * (rb + 1) + q) * kN];
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int r = 16 * rb + q;
      float o;
      if (box.push(r, cur[q], o)) dst[static_cast<size_t>(r - 1) * kN] = o;
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) cur[q] = nxt[q];
  }
  dst[static_cast<size_t>(kN - 1) * kN] = box.finish();
}

// Box along the sampled columns of Yc and the reference kernel's DCT (one sequential
// accumulator per output, src/kernel/mod.rs:711-735), one CTA of 128 threads per image.
// Thread j filters sampled column j; at sampled row sample_at(k) its output is B[k][j], which
// enters T[i][j] = sum_k D[i][k] B[k][j] at step k (D column k read as four broadcast
// float4). Then P = T D^T from shared memory, k in order; rows padded to 129 floats keep the
// 16 different D rows of a warp in 16 banks. Thread 127 filters a copy of column 126 so
// that every thread reaches the barrier.
__global__ void __launch_bounds__(128) cols_dct_kernel(const float* __restrict__ Yc,
                                                       float* __restrict__ pdqf,
                                                       float* __restrict__ buf1,
                                                       const int64_t* n_dev, int64_t i0) {
  if (past_count(n_dev, i0, blockIdx.x)) return;  // the whole block: no barrier is split
  __shared__ float4 dk[127][4];  // dk[k][q] = D[4 q .. 4 q + 3][k]
  __shared__ float dj[16][129];  // D[i][k]
  __shared__ float t[16][129];   // T[i][j]
  const int j = threadIdx.x;
  for (int e = j; e < 16 * 127; e += 128) {
    const int i = e / 127, k = e % 127;
    const float d = g_dct[e];
    dj[i][k] = d;
    reinterpret_cast<float*>(&dk[k][i >> 2])[i & 3] = d;
  }
  const bool live = j < 127;
  const float* src = Yc + blockIdx.x * kCompactPlane + (live ? j : 126);
  float acc[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) acc[i] = 0.0f;
  int k = 0, next_row = sample_at(0);
  Box3 box;
  float cur[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) cur[q] = src[q * 128];
  __syncthreads();  // dk, dj
  for (int rb = 0; rb < kN / 16; ++rb) {
    float nxt[16];
    if (rb + 1 < kN / 16) {
#pragma unroll
      for (int q = 0; q < 16; ++q) nxt[q] = src[(16 * (rb + 1) + q) * 128];
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int r = 16 * rb + q;
      float b;
      if (box.push(r, cur[q], b) && r - 1 == next_row) {  // the same rows for every thread
        if (buf1 && live) buf1[(static_cast<size_t>(blockIdx.x) * 127 + k) * 128 + j] = b;
#pragma unroll
        for (int q4 = 0; q4 < 4; ++q4) {
          const float4 d = dk[k][q4];
          acc[4 * q4 + 0] = __fadd_rn(acc[4 * q4 + 0], __fmul_rn(d.x, b));
          acc[4 * q4 + 1] = __fadd_rn(acc[4 * q4 + 1], __fmul_rn(d.y, b));
          acc[4 * q4 + 2] = __fadd_rn(acc[4 * q4 + 2], __fmul_rn(d.z, b));
          acc[4 * q4 + 3] = __fadd_rn(acc[4 * q4 + 3], __fmul_rn(d.w, b));
        }
        ++k;
        next_row = k < 127 ? sample_at(k) : -1;
      }
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) cur[q] = nxt[q];
  }
#pragma unroll
  for (int i = 0; i < 16; ++i) t[i][j] = acc[i];
  __syncthreads();
  for (int o = j; o < 256; o += 128) {
    const int i = o >> 4, jj = o & 15;
    float s = 0.0f;
    for (int kk = 0; kk < 127; ++kk) s = __fadd_rn(s, __fmul_rn(t[i][kk], dj[jj][kk]));
    pdqf[static_cast<size_t>(blockIdx.x) * 256 + o] = s;
  }
}

template <int kKind>
void launch_rows1(const uint8_t* in, float* Y, dim3 grid, const int64_t* n_dev, int64_t i0,
                  cudaStream_t s) {
  rows_kernel<kKind, false><<<grid, 128, 0, s>>>(in, Y, n_dev, i0);
}

}  // namespace

cudaError_t jarosz_init() {
  float d[16 * 127];
  for (int i = 0; i < 16 * 127; ++i) {
    const uint32_t b = YPDQ_DCT_F32_BITS[i];
    memcpy(&d[i], &b, 4);
  }
  return cudaMemcpyToSymbol(g_dct, d, sizeof(d));
}

size_t jarosz_scratch_bytes(int64_t chunk) {
  return static_cast<size_t>(chunk) * (2 * kPlane * sizeof(float) + 256 * sizeof(float));
}

cudaError_t launch_hash_jarosz(const HashLaunch& p, void* scratch, int64_t chunk, cudaStream_t s) {
  if (p.n <= 0) return cudaSuccess;
  static const size_t kBytesPerPixel[4] = {4, 1, 3, 4};
  if (p.input_kind < 0 || p.input_kind > 3) return cudaErrorInvalidValue;
  float* X = static_cast<float*>(scratch);
  float* Y = X + chunk * kPlane;
  float* P = Y + chunk * kPlane;
  for (int64_t i0 = 0; i0 < p.n; i0 += chunk) {
    const int64_t m = p.n - i0 < chunk ? p.n - i0 : chunk;
    const uint8_t* in =
        static_cast<const uint8_t*>(p.images) + static_cast<size_t>(i0) * kPlane * kBytesPerPixel[p.input_kind];
    const dim3 grid(kN / 128, static_cast<unsigned>(m));
    const int64_t* nd = p.n_dev;
    switch (p.input_kind) {
      case YPDQ_INPUT_F32: launch_rows1<YPDQ_INPUT_F32>(in, Y, grid, nd, i0, s); break;
      case YPDQ_INPUT_U8: launch_rows1<YPDQ_INPUT_U8>(in, Y, grid, nd, i0, s); break;
      case YPDQ_INPUT_RGB8: launch_rows1<YPDQ_INPUT_RGB8>(in, Y, grid, nd, i0, s); break;
      default: launch_rows1<YPDQ_INPUT_RGBA8>(in, Y, grid, nd, i0, s); break;
    }
    cols_kernel<<<grid, 128, 0, s>>>(Y, X, nd, i0);
    rows_kernel<YPDQ_INPUT_F32, true><<<grid, 128, 0, s>>>(reinterpret_cast<const uint8_t*>(X), Y,
                                                           nd, i0);
    cols_dct_kernel<<<static_cast<unsigned>(m), 128, 0, s>>>(
        Y, P, p.buf1 ? p.buf1 + static_cast<size_t>(i0) * 127 * 128 : nullptr, nd, i0);
    DihedralLaunch d{};
    d.pdqf = P;
    d.thr_in = nullptr;
    d.n = m;
    d.row_mask = p.row_mask;
    d.col_mask = p.col_mask;
    d.hashes = p.hashes ? p.hashes + static_cast<size_t>(i0) * 256 : nullptr;
    d.quality = p.quality ? p.quality + static_cast<size_t>(i0) * 8 : nullptr;
    d.thresholds = p.thresholds ? p.thresholds + static_cast<size_t>(i0) * 8 : nullptr;
    // the dihedral kernel writes all 8 slots; with one slot requested, copy slot 0 instead
    d.pdqf_out = (p.pdqf && p.pdqf_slots == 8) ? p.pdqf + static_cast<size_t>(i0) * 8 * 256 : nullptr;
    cudaError_t e = launch_dihedrals(d, s);
    if (e == cudaSuccess && p.pdqf && p.pdqf_slots != 8)
      e = cudaMemcpyAsync(p.pdqf + static_cast<size_t>(i0) * 256, P, static_cast<size_t>(m) * 1024,
                          cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

}  // namespace ypdq
