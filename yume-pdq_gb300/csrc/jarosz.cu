// ReferenceKernel<f32> on the GPU (YPDQ_COMPRESS_JAROSZ): yume-pdq's pdqhash-faithful kernel.
//
// jarosz_compress (src/kernel/mod.rs:790-820) filters the whole 512x512 image with
// jarosz_filter_float (src/kernel/ref.rs): two repetitions of a box filter along rows, then
// along columns, with window ceil(512 / 254) = 3. Each line is filtered by a running sum in
// four phases (fill, grow, slide, shrink) with true f32 divisions, so every output depends on
// the rounding of the whole prefix of its line; the kernels below replay that sum in the same
// order. The filtered image is sampled at ((2 o + 1) 512) / 254 and transformed by the
// reference kernel's DCT (one sequential accumulator per output, src/kernel/mod.rs:711-735).
// Median, packing, quality and dihedrals are the batched dihedral kernel's.
//
// Passes over a chunk of images in two f32 planes (X, Y):
//   load   : X = input as f32 (u8 cast, or BT.601 luma for RGB8/RGBA8)
//   rows   : Y = box along rows of X    (a warp owns 32 rows; 32x32 tiles transposed in
//                                        shared memory keep the global accesses coalesced)
//   cols   : X = box along columns of Y (a thread owns a column; coalesced by construction)
//   rows, cols again; then dct: PDQF from the sampled X.
#include "ypdq_internal.cuh"
#include "ypdq_tables.h"

namespace ypdq {

__constant__ float c_dct[16 * 127];  // the f32 DCT matrix D[k][i]

namespace {

constexpr int kN = 512;
constexpr size_t kPlane = static_cast<size_t>(kN) * kN;

// The reference's running-sum box filter of window 3 over one line, fed one input at a
// time: after value ri it emits the output for position ri - 1 (from ri = 1 on); finish()
// emits position 511. History holds the inputs ri-1, ri-2, ri-3 for the slide phase.
struct Box3 {
  float sum = 0.0f, cws = 0.0f;
  float h1 = 0.0f, h2 = 0.0f, h3 = 0.0f;  // in[ri-1], in[ri-2], in[ri-3]
  __device__ __forceinline__ bool push(int ri, float v, float& out) {
    bool emit = true;
    if (ri == 0) {  // fill: half window - 1 = 1 value
      sum = __fadd_rn(sum, v);
      cws = __fadd_rn(cws, 1.0f);
      emit = false;
    } else if (ri < 3) {  // grow: positions 0 and 1
      sum = __fadd_rn(sum, v);
      cws = __fadd_rn(cws, 1.0f);
      out = __fdiv_rn(sum, cws);
    } else {  // slide: position ri-1, dropping in[ri-3]
      sum = __fadd_rn(sum, v);
      sum = __fsub_rn(sum, h3);  // in[ri-3]
      out = __fdiv_rn(sum, cws);
    }
    h3 = h2;
    h2 = h1;
    h1 = v;
    return emit;
  }
  // shrink: position 511 drops in[509], which is h3 after the last push (ri = 511)
  __device__ __forceinline__ float finish() {
    sum = __fsub_rn(sum, h3);
    cws = __fadd_rn(cws, -1.0f);
    return __fdiv_rn(sum, cws);
  }
};

__device__ __forceinline__ float byte_as_float(uint32_t b) { return static_cast<float>(b); }
__device__ __forceinline__ float luma601(uint32_t r, uint32_t g, uint32_t b) {
  return __fadd_rn(__fadd_rn(__fmul_rn(0.299f, byte_as_float(r)), __fmul_rn(0.587f, byte_as_float(g))),
                   __fmul_rn(0.114f, byte_as_float(b)));
}

// X[i] = pixel i of the chunk's images as f32 (the reference's input buffer)
__global__ void load_kernel(const uint8_t* in, int kind, float* X, uint64_t n_px) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n_px) return;
  float v;
  switch (kind) {
    case YPDQ_INPUT_F32: v = reinterpret_cast<const float*>(in)[i]; break;
    case YPDQ_INPUT_U8: v = byte_as_float(in[i]); break;
    case YPDQ_INPUT_RGB8: v = luma601(in[3 * i], in[3 * i + 1], in[3 * i + 2]); break;
    default: v = luma601(in[4 * i], in[4 * i + 1], in[4 * i + 2]); break;
  }
  X[i] = v;
}

// Box along rows: block = 4 warps; warp w of block b owns rows 32 (4 b + w) .. +31 of image
// blockIdx.y. Columns go by 32-wide tiles loaded row-coalesced into shared memory.
__global__ void __launch_bounds__(128) rows_kernel(const float* X, float* Y) {
  __shared__ float tin[4][32][33], tout[4][32][33];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r0 = 32 * (4 * blockIdx.x + w);
  const float* src = X + blockIdx.y * kPlane + static_cast<size_t>(r0) * kN;
  float* dst = Y + blockIdx.y * kPlane + static_cast<size_t>(r0) * kN;
  Box3 box;
  for (int t = 0; t < kN / 32; ++t) {
#pragma unroll 8
    for (int k = 0; k < 32; ++k) tin[w][k][lane] = src[k * kN + 32 * t + lane];
    __syncwarp();
    // lane filters its row over the tile's 32 columns; tout[w][lane][c] = output column 32t+c-1
    for (int c = 0; c < 32; ++c) {
      float o;
      if (box.push(32 * t + c, tin[w][lane][c], o)) tout[w][lane][c] = o;
    }
    __syncwarp();
#pragma unroll 8
    for (int k = 0; k < 32; ++k) {
      const int col = 32 * t - 1 + lane;
      if (col >= 0) dst[k * kN + col] = tout[w][k][lane];
    }
    __syncwarp();
  }
  dst[lane * kN + (kN - 1)] = box.finish();
}

// Box along columns: thread c of block b owns column 128 b + c of image blockIdx.y.
__global__ void __launch_bounds__(128) cols_kernel(const float* Y, float* X) {
  const int col = 128 * blockIdx.x + threadIdx.x;
  const float* src = Y + blockIdx.y * kPlane + col;
  float* dst = X + blockIdx.y * kPlane + col;
  Box3 box;
  for (int r = 0; r < kN; ++r) {
    float o;
    if (box.push(r, src[static_cast<size_t>(r) * kN], o)) dst[static_cast<size_t>(r - 1) * kN] = o;
  }
  dst[static_cast<size_t>(kN - 1) * kN] = box.finish();
}

__device__ __forceinline__ int sample_at(int o) { return ((2 * o + 1) * kN) / (127 * 2); }

// PDQF of the sampled image (one CTA of 128 threads per image): T = D B row by row with one
// accumulator per (i, j) summed over k in order, then P = T D^T the same way.
__global__ void __launch_bounds__(128) dct_kernel(const float* X, float* pdqf, float* buf1) {
  __shared__ float t[16][128];
  const float* img = X + blockIdx.x * kPlane;
  const int j = threadIdx.x;
  if (j < 127) {
    float acc[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) acc[i] = 0.0f;
    const int col = sample_at(j);
    for (int k = 0; k < 127; ++k) {
      const float b = img[static_cast<size_t>(sample_at(k)) * kN + col];
      if (buf1) buf1[(static_cast<size_t>(blockIdx.x) * 127 + k) * 128 + j] = b;
#pragma unroll
      for (int i = 0; i < 16; ++i) acc[i] = __fadd_rn(acc[i], __fmul_rn(c_dct[i * 127 + k], b));
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) t[i][j] = acc[i];
  }
  __syncthreads();
  for (int o = j; o < 256; o += 128) {
    const int i = o >> 4, jj = o & 15;
    float s = 0.0f;
    for (int k = 0; k < 127; ++k) s = __fadd_rn(s, __fmul_rn(t[i][k], c_dct[jj * 127 + k]));
    pdqf[static_cast<size_t>(blockIdx.x) * 256 + o] = s;
  }
}

}  // namespace

cudaError_t jarosz_init() {
  float d[16 * 127];
  for (int i = 0; i < 16 * 127; ++i) {
    const uint32_t b = YPDQ_DCT_F32_BITS[i];
    memcpy(&d[i], &b, 4);
  }
  return cudaMemcpyToSymbol(c_dct, d, sizeof(d));
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
    const uint64_t px = static_cast<uint64_t>(m) * kPlane;
    load_kernel<<<static_cast<unsigned>((px + 255) / 256), 256, 0, s>>>(in, p.input_kind, X, px);
    const dim3 grid(kN / 128, static_cast<unsigned>(m));
    for (int rep = 0; rep < 2; ++rep) {
      rows_kernel<<<grid, 128, 0, s>>>(X, Y);
      cols_kernel<<<grid, 128, 0, s>>>(Y, X);
    }
    dct_kernel<<<static_cast<unsigned>(m), 128, 0, s>>>(
        X, P, p.buf1 ? p.buf1 + static_cast<size_t>(i0) * 127 * 128 : nullptr);
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
