// Per-stage kernels of the Kernel trait surface, batched: each entry point applies one of
// yume-pdq's per-image Kernel methods (src/kernel/mod.rs:268-497) to n items on the device,
// bit for bit with the reference's f32 implementation. The fused hash kernel (hash.cu) is
// the fast path; these serve callers that drive the stages one by one, as the reference's
// pipeline functions (src/lib.rs:427-455) and its tests do.
//
//   dct2d_kernel       Kernel::dct2d              DefaultKernel dct2d_impl, mod.rs:543-574
//   gradients_kernel   Kernel::sum_of_gradients   mod.rs:617-642
//   pdqf_op_kernel     Kernel::pdqf_t / pdqf_negate_alt_cols / pdqf_negate_alt_rows /
//                      pdqf_negate_off_diagonals  mod.rs:345-427, with the overrides of
//                      Avx2F32Kernel (x86.rs:285-436) and Avx512F32Kernel (x86.rs:989-1079)
//   luma_kernel        Kernel::cvt_rgb8_to_luma8f / cvt_rgba8_to_luma8f   mod.rs:303-340
//
// Every product and sum is rounded separately (__fmul_rn / __fadd_rn): Rust never contracts
// a * b + c into a fused multiply-add, so neither may these kernels.
#include "ypdq_internal.cuh"
#include "ypdq_tables.h"

namespace ypdq {

namespace {

__constant__ float c_dct[16 * 127];  // D[k][i] = sqrt(2/127) cos(pi (k+1) (2i+1) / 254), f32

constexpr int kDctThreads = 128;

// One CTA per buffer. Stage 1, T[k][j] = sum_i D[k][i] B[i][j]: thread j keeps the four
// partial sums of all 16 k (the reference's sumks[i % 4], added in i order) while it walks
// column j of B from i = 0 to 126, so each (k, j) sees exactly the reference's additions.
// Stage 2, P[k][l] = sum_m T[k][m] D[l][m], is the same four-way split over m; T and D sit
// in shared memory (D rows padded to 129 floats so the threads of a warp hit different banks).
__global__ void __launch_bounds__(kDctThreads) dct2d_kernel(const float* __restrict__ buf,
                                                            int64_t n, int stride,
                                                            float* __restrict__ pdqf) {
  __shared__ float t[16][128];
  __shared__ float d[16][129];
  const int tid = threadIdx.x;
  for (int i = tid; i < 16 * 127; i += kDctThreads) d[i / 127][i % 127] = c_dct[i];
  for (int64_t img = blockIdx.x; img < n; img += gridDim.x) {
    const float* b = buf + img * 127 * static_cast<int64_t>(stride);
    if (tid < 127) {
      float s[16][4];
#pragma unroll
      for (int k = 0; k < 16; ++k) s[k][0] = s[k][1] = s[k][2] = s[k][3] = 0.0f;
      for (int i = 0; i < 124; i += 4) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const float x = b[(i + u) * static_cast<int64_t>(stride) + tid];
#pragma unroll
          for (int k = 0; k < 16; ++k)
            s[k][u] = __fadd_rn(s[k][u], __fmul_rn(c_dct[k * 127 + i + u], x));
        }
      }
#pragma unroll
      for (int u = 0; u < 3; ++u) {  // i = 124, 125, 126
        const float x = b[(124 + u) * static_cast<int64_t>(stride) + tid];
#pragma unroll
        for (int k = 0; k < 16; ++k)
          s[k][u] = __fadd_rn(s[k][u], __fmul_rn(c_dct[k * 127 + 124 + u], x));
      }
#pragma unroll
      for (int k = 0; k < 16; ++k)
        t[k][tid] = __fadd_rn(__fadd_rn(__fadd_rn(s[k][0], s[k][1]), s[k][2]), s[k][3]);
    }
    __syncthreads();
    for (int o = tid; o < 256; o += kDctThreads) {
      const int k = o >> 4, l = o & 15;
      float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
      for (int m = 0; m < 124; m += 4) {
        s0 = __fadd_rn(s0, __fmul_rn(t[k][m], d[l][m]));
        s1 = __fadd_rn(s1, __fmul_rn(t[k][m + 1], d[l][m + 1]));
        s2 = __fadd_rn(s2, __fmul_rn(t[k][m + 2], d[l][m + 2]));
        s3 = __fadd_rn(s3, __fmul_rn(t[k][m + 3], d[l][m + 3]));
      }
      s0 = __fadd_rn(s0, __fmul_rn(t[k][124], d[l][124]));
      s1 = __fadd_rn(s1, __fmul_rn(t[k][125], d[l][125]));
      s2 = __fadd_rn(s2, __fmul_rn(t[k][126], d[l][126]));
      pdqf[img * 256 + o] = __fadd_rn(__fadd_rn(__fadd_rn(s0, s1), s2), s3);
    }
    __syncthreads();
  }
}

// One thread per matrix: the reference's single accumulator, vertical differences first
// (rows i, i+1 for i < 15, all columns), then horizontal ones (columns j, j+1).
__global__ void gradients_kernel(const float* __restrict__ pdqf, int64_t n,
                                 float* __restrict__ out) {
  const int64_t m = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (m >= n) return;
  const float* p = pdqf + m * 256;
  float g = 0.0f;
  for (int i = 0; i < 15; ++i)
    for (int j = 0; j < 16; ++j)
      g = __fadd_rn(g, fabsf(__fsub_rn(p[i * 16 + j], p[(i + 1) * 16 + j])));
  for (int i = 0; i < 16; ++i)
    for (int j = 0; j < 15; ++j)
      g = __fadd_rn(g, fabsf(__fsub_rn(p[i * 16 + j], p[i * 16 + j + 1])));
  out[m] = g;
}

// One CTA of 256 threads per matrix, one thread per element. YPDQ_PDQF_T transposes;
// the other ops negate element (i, j) when i + j is odd (off-diagonals) or when bit i of
// row_mask and bit j of col_mask are both set (alternate rows / columns).
__global__ void __launch_bounds__(256) pdqf_op_kernel(float* __restrict__ pdqf, int64_t n, int op,
                                                      uint32_t row_mask, uint32_t col_mask) {
  const int e = threadIdx.x, i = e >> 4, j = e & 15;
  for (int64_t m = blockIdx.x; m < n; m += gridDim.x) {
    float* p = pdqf + m * 256;
    float v = p[e];
    if (op == YPDQ_PDQF_T) {  // uniform over the block
      v = p[j * 16 + i];
      __syncthreads();        // every element read before any is written
    } else if (op == YPDQ_PDQF_NEGATE_OFF_DIAGONALS) {
      if ((i + j) & 1) v = -v;
    } else if (((row_mask >> i) & 1u) && ((col_mask >> j) & 1u)) {
      v = -v;
    }
    p[e] = v;
    __syncthreads();
  }
}

// One thread per pixel: (r_coeff r + g_coeff g) + b_coeff b, each step rounded to f32.
template <int kChannels>
__global__ void luma_kernel(const uint8_t* __restrict__ px, int64_t n, float rc, float gc,
                            float bc, float* __restrict__ out) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n;
       k += stride) {
    const uint8_t* q = px + k * kChannels;
    const float r = static_cast<float>(q[0]), g = static_cast<float>(q[1]),
                b = static_cast<float>(q[2]);
    out[k] = __fadd_rn(__fadd_rn(__fmul_rn(rc, r), __fmul_rn(gc, g)), __fmul_rn(bc, b));
  }
}

unsigned grid_for(int64_t items, int64_t per_block, int num_sms, int blocks_per_sm) {
  int64_t g = (items + per_block - 1) / per_block;
  const int64_t cap = static_cast<int64_t>(num_sms) * blocks_per_sm;
  if (g > cap) g = cap;
  return static_cast<unsigned>(g < 1 ? 1 : g);
}

}  // namespace

cudaError_t stages_init() {
  return cudaMemcpyToSymbol(c_dct, YPDQ_DCT_F32_BITS, sizeof(YPDQ_DCT_F32_BITS));
}

cudaError_t launch_dct2d(const float* buf, int64_t n, int stride, float* pdqf, int num_sms,
                         cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  dct2d_kernel<<<grid_for(n, 1, num_sms, 16), kDctThreads, 0, s>>>(buf, n, stride, pdqf);
  return cudaGetLastError();
}

cudaError_t launch_gradients(const float* pdqf, int64_t n, float* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  gradients_kernel<<<static_cast<unsigned>((n + 127) / 128), 128, 0, s>>>(pdqf, n, out);
  return cudaGetLastError();
}

cudaError_t launch_pdqf_op(float* pdqf, int64_t n, int op, uint32_t row_mask, uint32_t col_mask,
                           int num_sms, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  pdqf_op_kernel<<<grid_for(n, 1, num_sms, 8), 256, 0, s>>>(pdqf, n, op, row_mask, col_mask);
  return cudaGetLastError();
}

cudaError_t launch_luma(const uint8_t* px, int64_t n, int channels, float rc, float gc, float bc,
                        float* out, int num_sms, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const unsigned g = grid_for(n, 256, num_sms, 8);
  if (channels == 3)
    luma_kernel<3><<<g, 256, 0, s>>>(px, n, rc, gc, bc, out);
  else
    luma_kernel<4><<<g, 256, 0, s>>>(px, n, rc, gc, bc, out);
  return cudaGetLastError();
}

}  // namespace ypdq
