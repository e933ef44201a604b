// Internal C++ view of the C ABI's opaque handles, shared by the translation units that
// implement include/ypdq.h.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "ypdq.h"

struct ypdq_ctx {
  int device = 0;
  int num_sms = 0;
  int hash_ctas_f32 = 1;
  int hash_ctas_u8 = 1;
  int hash_ctas[4][3][2] = {};  // [input kind][dct precision][separable compress]
  int* d_err = nullptr;
  cudaStream_t stream = nullptr;       // compute stream of the blocking _host calls
  cudaStream_t copy_stream = nullptr;  // host->device copies that overlap that compute
  static constexpr int kMaxChunks = 32;
  cudaEvent_t chunk_copied[kMaxChunks] = {};
  std::mutex mu;                  // guards the scratch buffers below
  void* scratch[8] = {};
  size_t scratch_bytes[8] = {};
  // page-locked host staging of ypdq_screen_host's results (count, error word, hits), so
  // its device-to-host copies never take the driver's path for pageable memory
  void* h_stage = nullptr;
  size_t h_stage_bytes = 0;
  void* jarosz_scratch = nullptr;  // YPDQ_COMPRESS_JAROSZ filter planes
  size_t jarosz_bytes = 0;
  cudaEvent_t jarosz_done = nullptr;  // recorded after the last work that used it
};

struct ypdq_db {
  ypdq_ctx* ctx;
  const uint8_t* d_rows;
  uint64_t n_rows;
  bool owned;
};

namespace ypdq {

// Bytes of one 512x512 image of an input kind, 0 for an unknown kind.
inline size_t image_bytes_of(int kind) {
  switch (kind) {
    case YPDQ_INPUT_F32: return 4u * 512u * 512u;
    case YPDQ_INPUT_U8: return 512u * 512u;
    case YPDQ_INPUT_RGB8: return 3u * 512u * 512u;
    case YPDQ_INPUT_RGBA8: return 4u * 512u * 512u;
    default: return 0;
  }
}

// Record a formatted message for ypdq_last_error() on the calling thread; returns st.
ypdq_status fail(ypdq_status st, const char* fmt, ...);
// Map a CUDA error to YPDQ_ERR_NOMEM or YPDQ_ERR_CUDA with its text.
ypdq_status cuda_fail(cudaError_t e, const char* what);
// Row and column sign masks of the dihedral derivation for a ypdq_dihedral_semantics.
void semantics_masks(int sem, uint32_t* rm, uint32_t* cm);
// Splits a dct_precision argument into the DCT variant (0..2) and the
// YPDQ_COMPRESS_SEPARABLE flag; false if it holds anything else.
inline bool parse_precision(int v, int* dct, int* separable) {
  const int d = v & 0xFF;
  if ((v & ~(0xFF | YPDQ_COMPRESS_SEPARABLE)) != 0 || d < YPDQ_DCT_FP32 || d > YPDQ_DCT_BF16X3)
    return false;
  *dct = d;
  *separable = (v & YPDQ_COMPRESS_SEPARABLE) ? 1 : 0;
  return true;
}

}  // namespace ypdq

#define CK(call, what)                                           \
  do {                                                           \
    cudaError_t e_ = (call);                                     \
    if (e_ != cudaSuccess) return ::ypdq::cuda_fail(e_, what);   \
  } while (0)
