// C ABI of libyumepdq_gb300: the batched device API (include/ypdq.h) and the drop-in
// symbols of yume-pdq's C header (include/yume_pdq.h).
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "capi_internal.h"
#include "ypdq_internal.cuh"
#include "ypdq_tables.h"
#include "yume_pdq.h"

using namespace ypdq;

namespace {
thread_local std::string g_last_error;
}  // namespace

namespace ypdq {

ypdq_status fail(ypdq_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return st;
}

ypdq_status cuda_fail(cudaError_t e, const char* what) {
  if (e == cudaErrorMemoryAllocation)
    return fail(YPDQ_ERR_NOMEM, "%s: %s", what, cudaGetErrorString(e));
  return fail(YPDQ_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

void semantics_masks(int sem, uint32_t* rm, uint32_t* cm) {
  switch (sem) {
    case YPDQ_DIHEDRAL_AVX2:
      *rm = 0x5555u;
      *cm = 0x0055u;
      break;
    case YPDQ_DIHEDRAL_SCALAR:
      *rm = 0xAAAAu;
      *cm = 0x5555u;
      break;
    default:
      *rm = 0x5555u;
      *cm = 0x5555u;
      break;
  }
}

}  // namespace ypdq

namespace {

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Grow-only scratch buffer `slot` of ctx to at least `bytes`. Caller holds ctx->mu.
ypdq_status scratch(ypdq_ctx* ctx, int slot, size_t bytes, void** out) {
  if (ctx->scratch_bytes[slot] < bytes) {
    if (ctx->scratch[slot]) cudaFree(ctx->scratch[slot]);
    ctx->scratch[slot] = nullptr;
    ctx->scratch_bytes[slot] = 0;
    size_t want = bytes < 4096 ? 4096 : bytes;
    CK(cudaMalloc(&ctx->scratch[slot], want), "cudaMalloc(scratch)");
    ctx->scratch_bytes[slot] = want;
  }
  *out = ctx->scratch[slot];
  return YPDQ_OK;
}

// The context's page-locked staging buffer, at least `bytes` long (under ctx->mu).
ypdq_status host_stage(ypdq_ctx* ctx, size_t bytes, uint8_t** out) {
  if (ctx->h_stage_bytes < bytes) {
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    ctx->h_stage = nullptr;
    ctx->h_stage_bytes = 0;
    const size_t want = bytes < 65536 ? 65536 : bytes;
    CK(cudaMallocHost(&ctx->h_stage, want), "cudaMallocHost(staging)");
    ctx->h_stage_bytes = want;
  }
  *out = static_cast<uint8_t*>(ctx->h_stage);
  return YPDQ_OK;
}

ypdq_status check_ctx(ypdq_ctx* ctx) {
  if (!ctx) return fail(YPDQ_ERR_INVALID, "ctx is NULL");
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  return YPDQ_OK;
}

ypdq_status read_device_errors(ypdq_ctx* ctx) {
  int err = 0;
  CK(cudaMemcpy(&err, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost), "read device errors");
  if (err) {
    CK(cudaMemset(ctx->d_err, 0, sizeof(int)), "clear device errors");
    if (err & kDevErrTimeout)
      return fail(YPDQ_ERR_TIMEOUT, "a kernel wait exceeded its time limit and gave up");
    return fail(YPDQ_ERR_CUDA, "device error flags 0x%x", err);
  }
  return YPDQ_OK;
}

}  // namespace

namespace ypdq {
void set_last_error_text(const char* text) { g_last_error = text; }
}  // namespace ypdq

namespace {

// YPDQ_COMPRESS_JAROSZ: the filter passes need two f32 planes per image in flight, in a
// context-owned scratch for chunks of up to 2,048 images (4 GiB). Each pass runs one thread
// per line, 512 per image, so a chunk is about nine rounds of the GPU's resident warps and
// the last, partly filled round costs little. Calls on different streams take turns on it
// (under ctx->mu): each waits for the previous user's completion event (jarosz_done) and
// records its own.
int64_t jarosz_chunk(int64_t n) { return n < 2048 ? (n > 0 ? n : 1) : 2048; }

// Chunk bounds for ypdq_screen_host. The copy of chunk c+1 (copy stream) runs while chunk c
// is hashed and scanned (compute stream). The copies run back to back, so with u the copy
// time per image and v s + h the compute time of a chunk of s images, chunk c+1 arrives in
// time when its end S_{c+1} (images counted from the start) satisfies
// S_{c+1} u <= S_1 u + S_c v + c h, i.e. S_{c+1} <= S_1 + (v / u) S_c + c (h / u): chunks
// grow geometrically by the compute/copy ratio, and only the first chunk's copy is exposed.
// `ratio` is v / u and `chunk_images` h / u. Chunks are whole multiples of `granule` images
// (whole scan passes: 32 images = 256 queries, or 90 = one pass of 720 queries taken in
// triples); the first is one granule unless more than `max_chunks` chunks would be needed.
// When copying is the longer stage (v / u <= 1) chunks still grow by h / u each, since a
// chunk's fixed cost is then all its compute, and a remainder smaller than a granule stays
// the last chunk: its compute after the last copy is exposed, so it should be small. When
// computing is the longer stage the remainder joins the last chunk instead.
int plan_screen_chunks(int64_t n, double ratio, double chunk_images, int max_chunks,
                       int64_t granule, int64_t* bounds) {
  const double r = std::min(2.0, std::max(1.0, ratio));
  const double h = std::min(256.0, std::max(0.0, chunk_images));
  bounds[0] = 0;
  if (n <= 0) return 0;
  for (int64_t first = granule;; first *= 2) {
    int nch = 0;
    int64_t end = n < first + granule ? n : first;
    bounds[++nch] = end;
    while (end < n && nch < max_chunks) {
      const double limit = static_cast<double>(first) + r * static_cast<double>(end) + nch * h;
      int64_t next =
          std::max<int64_t>(end + granule, static_cast<int64_t>(limit) / granule * granule);
      if (next >= n || (next + granule > n && ratio > 1.0)) next = n;
      end = next;
      bounds[++nch] = end;
    }
    if (end == n) return nch;
  }
}

// Estimated device time of one ypdq_screen_host chunk on a GB300 (152 SMs), in
// microseconds: fixed_us + per_image_us x images.
struct ChunkCost {
  double fixed_us, per_image_us;
};
ChunkCost screen_chunk_cost(int input_kind, bool jarosz, uint64_t n_rows, uint32_t threshold) {
  // the tensor-core scan: 21.5 T (row, query) pairs/s in passes of 720 queries taken in
  // triples (FP4, the 126-bit prefix bound), 9.5 T with the 192-bit bound, 8.3 T with all
  // 256 bits; 8 queries per image
  const double pairs_per_us = threshold <= 36 ? 21.5e6 : threshold <= 62 ? 9.5e6 : 8.3e6;
  const double scan_us = 8.0 * static_cast<double>(n_rows) / pairs_per_us;
  // the Jarosz filter: four passes, each at least one line's sequential replay (512
  // dependent steps, ~5 us) however few images the chunk holds, plus the DCT
  if (jarosz) return {30.0, (input_kind == YPDQ_INPUT_U8 ? 0.95 : 1.1) + scan_us};
  // hash_kernel runs one image per CTA, two CTAs per SM: a chunk of up to 304 images takes
  // one image's time on a CTA, 304 x the per-image rate
  const double hash_us = input_kind == YPDQ_INPUT_U8 ? 0.135 : input_kind == YPDQ_INPUT_F32 ? 0.18 : 0.28;
  return {304.0 * hash_us, hash_us + scan_us};
}

// The chunk plan of ypdq_screen_host (and ypdq_screen_plan).
int screen_chunks(int64_t n, int input_kind, int dct_precision, uint64_t n_rows,
                  uint32_t threshold, int64_t* bounds) {
  // host memory reaches the device at ~211 GB/s on a GB300 host link, for copy-engine copies
  // and SM loads from mapped or pageable memory alike
  const double copy_us = static_cast<double>(image_bytes_of(input_kind)) / 2.11e5;
  const ChunkCost cost =
      screen_chunk_cost(input_kind, dct_precision == YPDQ_COMPRESS_JAROSZ, n_rows, threshold);
  // at t <= 36 chunks of 90 images fill whole passes of the triple scan (720 queries)
  const int64_t granule = threshold <= 36 ? 90 : 32;
  return plan_screen_chunks(n, 0.95 * cost.per_image_us / copy_us, 0.95 * cost.fixed_us / copy_us,
                            ypdq_ctx::kMaxChunks, granule, bounds);
}

ypdq_status ensure_jarosz_scratch(ypdq_ctx* ctx, int64_t chunk) {
  const size_t need = jarosz_scratch_bytes(chunk);
  if (ctx->jarosz_bytes >= need) return YPDQ_OK;
  // the previous user may still be running on another stream
  CK(cudaEventSynchronize(ctx->jarosz_done), "wait jarosz scratch");
  if (ctx->jarosz_scratch) CK(cudaFree(ctx->jarosz_scratch), "cudaFree(jarosz scratch)");
  ctx->jarosz_scratch = nullptr;
  ctx->jarosz_bytes = 0;
  CK(cudaMalloc(&ctx->jarosz_scratch, need), "cudaMalloc(jarosz scratch)");
  ctx->jarosz_bytes = need;
  return YPDQ_OK;
}

}  // namespace

extern "C" {

// ----------------------------------------------------------------- context

const char* ypdq_last_error(void) { return g_last_error.c_str(); }

ypdq_status ypdq_ctx_create(int device, ypdq_ctx** out) {
  if (!out) return fail(YPDQ_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int count = 0;
  CK(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
  if (device < 0 || device >= count)
    return fail(YPDQ_ERR_INVALID, "device %d out of range (%d devices)", device, count);
  CK(cudaSetDevice(device), "cudaSetDevice");
  ypdq_ctx* ctx = new ypdq_ctx();
  ctx->device = device;
  cudaError_t e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = upload_constants();
  if (e == cudaSuccess) e = scan_init();
  if (e == cudaSuccess) e = jarosz_init();
  if (e == cudaSuccess) e = stages_init();
  if (e == cudaSuccess) e = hash_occupancy(0, &ctx->hash_ctas_f32);
  if (e == cudaSuccess) e = hash_occupancy(1, &ctx->hash_ctas_u8);
  for (int u = 0; u < 4 && e == cudaSuccess; ++u)
    for (int d = 0; d < 3 && e == cudaSuccess; ++d)
      for (int sp = 0; sp < 2 && e == cudaSuccess; ++sp)
        e = hash_occupancy_variant(u, d, sp, &ctx->hash_ctas[u][d][sp]);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(ctx->d_err, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->jarosz_done, cudaEventDisableTiming);
  for (int i = 0; i < ypdq_ctx::kMaxChunks && e == cudaSuccess; ++i)
    e = cudaEventCreateWithFlags(&ctx->chunk_copied[i], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    if (ctx->d_err) cudaFree(ctx->d_err);
    delete ctx;
    return cuda_fail(e, "ypdq_ctx_create");
  }
  if (ctx->hash_ctas_f32 < 1 || ctx->hash_ctas_u8 < 1) {
    cudaFree(ctx->d_err);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return fail(YPDQ_ERR_UNSUPPORTED, "hash kernel does not fit on this device");
  }
  *out = ctx;
  return YPDQ_OK;
}

ypdq_status ypdq_ctx_destroy(ypdq_ctx* ctx) {
  if (!ctx) return YPDQ_OK;
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  for (int i = 0; i < 8; ++i)
    if (ctx->scratch[i]) cudaFree(ctx->scratch[i]);
  if (ctx->jarosz_scratch) cudaFree(ctx->jarosz_scratch);
  if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
  if (ctx->jarosz_done) cudaEventDestroy(ctx->jarosz_done);
  if (ctx->d_err) cudaFree(ctx->d_err);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  for (int i = 0; i < ypdq_ctx::kMaxChunks; ++i)
    if (ctx->chunk_copied[i]) cudaEventDestroy(ctx->chunk_copied[i]);
  delete ctx;
  return YPDQ_OK;
}

ypdq_status ypdq_check_device_errors(ypdq_ctx* ctx) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  CK(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
  return read_device_errors(ctx);
}

ypdq_status ypdq_hash_occupancy(ypdq_ctx* ctx, int input_kind, int dct_precision,
                                int* ctas_per_sm) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (!ctas_per_sm) return fail(YPDQ_ERR_INVALID, "ctas_per_sm is NULL");
  if (image_bytes_of(input_kind) == 0)
    return fail(YPDQ_ERR_INVALID, "input_kind %d", input_kind);
  int dct = 0, sep = 0;
  if (!parse_precision(dct_precision, &dct, &sep))
    return fail(YPDQ_ERR_INVALID, "dct_precision %d", dct_precision);
  *ctas_per_sm = ctx->hash_ctas[input_kind][dct][sep];
  return YPDQ_OK;
}

ypdq_status ypdq_device_info(ypdq_ctx* ctx, int* num_sms, int* hash_ctas_per_sm) {
  if (!ctx) return fail(YPDQ_ERR_INVALID, "ctx is NULL");
  if (num_sms) *num_sms = ctx->num_sms;
  if (hash_ctas_per_sm) *hash_ctas_per_sm = ctx->hash_ctas_f32;
  return YPDQ_OK;
}

ypdq_status ypdq_constants(float* h_dct, float* h_tent) {
  if (h_dct) memcpy(h_dct, YPDQ_DCT_F32_BITS, sizeof(YPDQ_DCT_F32_BITS));
  if (h_tent) memcpy(h_tent, YPDQ_TENT_F32_BITS, sizeof(YPDQ_TENT_F32_BITS));
  return YPDQ_OK;
}

// ----------------------------------------------------------------- hashing

ypdq_status ypdq_hash_batch(ypdq_ctx* ctx, const void* d_images, int64_t n, int input_kind,
                            int dct_precision, int semantics, uint8_t* d_hashes,
                            float* d_quality, float* d_thresholds, float* d_pdqf,
                            int pdqf_slots, float* d_buf1, ypdq_stream_t stream) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (n < 0) return fail(YPDQ_ERR_INVALID, "n < 0");
  if (n > 0 && !d_images) return fail(YPDQ_ERR_INVALID, "d_images is NULL");
  if (image_bytes_of(input_kind) == 0)
    return fail(YPDQ_ERR_INVALID, "input_kind %d", input_kind);
  if (semantics < YPDQ_DIHEDRAL_EXACT || semantics > YPDQ_DIHEDRAL_SCALAR)
    return fail(YPDQ_ERR_INVALID, "semantics %d", semantics);
  const bool jarosz = dct_precision == YPDQ_COMPRESS_JAROSZ;
  int dct = 0, sep = 0;
  if (!jarosz && !parse_precision(dct_precision, &dct, &sep))
    return fail(YPDQ_ERR_INVALID, "dct_precision %d", dct_precision);
  if (d_pdqf && pdqf_slots != 1 && pdqf_slots != 8)
    return fail(YPDQ_ERR_INVALID, "pdqf_slots must be 1 or 8");
  if (!aligned16(d_images)) return fail(YPDQ_ERR_ALIGN, "d_images must be 16-byte aligned");
  if (d_pdqf && !aligned16(d_pdqf)) return fail(YPDQ_ERR_ALIGN, "d_pdqf must be 16-byte aligned");
  HashLaunch p{};
  p.images = d_images;
  p.n = n;
  p.input_kind = input_kind;
  semantics_masks(semantics, &p.row_mask, &p.col_mask);
  p.hashes = d_hashes;
  p.quality = d_quality;
  p.thresholds = d_thresholds;
  p.pdqf = d_pdqf;
  p.pdqf_slots = pdqf_slots;
  p.buf1 = d_buf1;
  p.dev_err = ctx->d_err;
  p.dct = dct;
  p.separable = sep;
  if (jarosz) {
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int64_t chunk = jarosz_chunk(n);
    if ((st = ensure_jarosz_scratch(ctx, chunk))) return st;
    CK(cudaStreamWaitEvent(s, ctx->jarosz_done, 0), "wait jarosz scratch");
    CK(launch_hash_jarosz(p, ctx->jarosz_scratch, chunk, s), "jarosz launch");
    CK(cudaEventRecord(ctx->jarosz_done, s), "record jarosz scratch");
    return YPDQ_OK;
  }
  CK(launch_hash(p, ctx->num_sms, ctx->hash_ctas[p.input_kind][dct][sep],
                 reinterpret_cast<cudaStream_t>(stream)),
     "hash kernel launch");
  return YPDQ_OK;
}

ypdq_status ypdq_dct2d_batch(ypdq_ctx* ctx, const float* d_buf1, int64_t n, int stride,
                             float* d_pdqf, ypdq_stream_t stream) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (n < 0) return fail(YPDQ_ERR_INVALID, "n < 0");
  if (stride < 127) return fail(YPDQ_ERR_INVALID, "stride %d < 127", stride);
  if (n > 0 && (!d_buf1 || !d_pdqf)) return fail(YPDQ_ERR_INVALID, "NULL buffer");
  if (!aligned16(d_buf1) || !aligned16(d_pdqf))
    return fail(YPDQ_ERR_ALIGN, "buffers must be 16-byte aligned");
  CK(launch_dct2d(d_buf1, n, stride, d_pdqf, ctx->num_sms, reinterpret_cast<cudaStream_t>(stream)),
     "dct2d launch");
  return YPDQ_OK;
}

ypdq_status ypdq_sum_of_gradients_batch(ypdq_ctx* ctx, const float* d_pdqf, int64_t n,
                                        float* d_out, ypdq_stream_t stream) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (n < 0) return fail(YPDQ_ERR_INVALID, "n < 0");
  if (n > 0 && (!d_pdqf || !d_out)) return fail(YPDQ_ERR_INVALID, "NULL buffer");
  if (!aligned16(d_pdqf)) return fail(YPDQ_ERR_ALIGN, "d_pdqf must be 16-byte aligned");
  CK(launch_gradients(d_pdqf, n, d_out, reinterpret_cast<cudaStream_t>(stream)),
     "gradients launch");
  return YPDQ_OK;
}

ypdq_status ypdq_pdqf_transform_batch(ypdq_ctx* ctx, float* d_pdqf, int64_t n, int op,
                                      int negate, int semantics, ypdq_stream_t stream) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (n < 0) return fail(YPDQ_ERR_INVALID, "n < 0");
  if (n > 0 && !d_pdqf) return fail(YPDQ_ERR_INVALID, "d_pdqf is NULL");
  if (op < YPDQ_PDQF_T || op > YPDQ_PDQF_NEGATE_OFF_DIAGONALS)
    return fail(YPDQ_ERR_INVALID, "op %d", op);
  if (semantics < YPDQ_DIHEDRAL_EXACT || semantics > YPDQ_DIHEDRAL_SCALAR)
    return fail(YPDQ_ERR_INVALID, "semantics %d", semantics);
  if (!aligned16(d_pdqf)) return fail(YPDQ_ERR_ALIGN, "d_pdqf must be 16-byte aligned");
  const bool neg = negate != 0;
  // bit i: row / column i negated
  uint32_t rows = 0xFFFFu, cols = 0xFFFFu;
  if (op == YPDQ_PDQF_NEGATE_ALT_ROWS)
    rows = (semantics == YPDQ_DIHEDRAL_SCALAR) == neg ? 0xAAAAu : 0x5555u;
  if (op == YPDQ_PDQF_NEGATE_ALT_COLS)
    cols = (neg ? 0xAAAAu : 0x5555u) & (semantics == YPDQ_DIHEDRAL_AVX2 ? 0x00FFu : 0xFFFFu);
  CK(launch_pdqf_op(d_pdqf, n, op, rows, cols, ctx->num_sms,
                    reinterpret_cast<cudaStream_t>(stream)),
     "pdqf transform launch");
  return YPDQ_OK;
}

ypdq_status ypdq_cvt_luma8f(ypdq_ctx* ctx, const uint8_t* d_pixels, int64_t n_pixels,
                            int channels, float r_coeff, float g_coeff, float b_coeff,
                            float* d_out, ypdq_stream_t stream) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (n_pixels < 0) return fail(YPDQ_ERR_INVALID, "n_pixels < 0");
  if (channels != 3 && channels != 4) return fail(YPDQ_ERR_INVALID, "channels %d", channels);
  if (n_pixels > 0 && (!d_pixels || !d_out)) return fail(YPDQ_ERR_INVALID, "NULL buffer");
  CK(launch_luma(d_pixels, n_pixels, channels, r_coeff, g_coeff, b_coeff, d_out, ctx->num_sms,
                 reinterpret_cast<cudaStream_t>(stream)),
     "luma launch");
  return YPDQ_OK;
}

ypdq_status ypdq_dihedrals_batch(ypdq_ctx* ctx, const float* d_pdqf, const float* d_thr,
                                 int64_t n, int semantics, uint8_t* d_hashes, float* d_quality,
                                 float* d_thr_out, float* d_pdqf_out, ypdq_stream_t stream) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (n < 0) return fail(YPDQ_ERR_INVALID, "n < 0");
  if (n > 0 && !d_pdqf) return fail(YPDQ_ERR_INVALID, "d_pdqf is NULL");
  if (semantics < YPDQ_DIHEDRAL_EXACT || semantics > YPDQ_DIHEDRAL_SCALAR)
    return fail(YPDQ_ERR_INVALID, "semantics %d", semantics);
  if (!aligned16(d_pdqf) || (d_pdqf_out && !aligned16(d_pdqf_out)))
    return fail(YPDQ_ERR_ALIGN, "PDQF buffers must be 16-byte aligned");
  DihedralLaunch p{};
  p.pdqf = d_pdqf;
  p.thr_in = d_thr;
  p.n = n;
  semantics_masks(semantics, &p.row_mask, &p.col_mask);
  p.hashes = d_hashes;
  p.quality = d_quality;
  p.thresholds = d_thr_out;
  p.pdqf_out = d_pdqf_out;
  CK(launch_dihedrals(p, reinterpret_cast<cudaStream_t>(stream)), "dihedral kernel launch");
  return YPDQ_OK;
}

// ----------------------------------------------------------------- matching

ypdq_status ypdq_scan(ypdq_ctx* ctx, const uint8_t* d_rows, uint64_t n_rows,
                      const uint8_t* d_queries, uint32_t n_queries, uint32_t threshold,
                      ypdq_hit* d_hits, uint64_t capacity, uint64_t* d_count, int algo,
                      ypdq_stream_t stream) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (!d_count) return fail(YPDQ_ERR_INVALID, "d_count is NULL");
  if (n_rows > 0 && !d_rows) return fail(YPDQ_ERR_INVALID, "d_rows is NULL");
  if (n_queries > 0 && !d_queries) return fail(YPDQ_ERR_INVALID, "d_queries is NULL");
  if (capacity > 0 && !d_hits) return fail(YPDQ_ERR_INVALID, "d_hits is NULL");
  if (threshold > 256) return fail(YPDQ_ERR_INVALID, "threshold %u > 256", threshold);
  if (algo < YPDQ_SCAN_AUTO || algo > YPDQ_SCAN_TC_FP8)
    return fail(YPDQ_ERR_INVALID, "algo %d", algo);
  if (!aligned16(d_rows) || !aligned16(d_queries))
    return fail(YPDQ_ERR_ALIGN, "rows and queries must be 16-byte aligned");
  ScanLaunch p{};
  p.rows = d_rows;
  p.n_rows = n_rows;
  p.queries = d_queries;
  p.n_queries = n_queries;
  p.threshold = threshold;
  p.hits = d_hits;
  p.capacity = capacity;
  p.count = reinterpret_cast<unsigned long long*>(d_count);
  p.dev_err = ctx->d_err;
  CK(launch_scan(p, algo, ctx->num_sms, reinterpret_cast<cudaStream_t>(stream)), "scan launch");
  return YPDQ_OK;
}

ypdq_status ypdq_sort_hits(ypdq_ctx* ctx, ypdq_hit* d_hits, uint64_t n, ypdq_stream_t stream) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (n > 0 && !d_hits) return fail(YPDQ_ERR_INVALID, "d_hits is NULL");
  CK(launch_sort_hits(d_hits, n, reinterpret_cast<cudaStream_t>(stream)), "sort launch");
  return YPDQ_OK;
}

// ----------------------------------------------------------------- database

ypdq_status ypdq_db_create(ypdq_ctx* ctx, const uint8_t* h_rows, uint64_t n_rows, ypdq_db** out) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (!out || (n_rows > 0 && !h_rows)) return fail(YPDQ_ERR_INVALID, "NULL argument");
  void* d = nullptr;
  if (n_rows > 0) {
    CK(cudaMalloc(&d, n_rows * 32), "cudaMalloc(db)");
    cudaError_t e = cudaMemcpy(d, h_rows, n_rows * 32, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(d);
      return cuda_fail(e, "db upload");
    }
  }
  *out = new ypdq_db{ctx, static_cast<const uint8_t*>(d), n_rows, true};
  return YPDQ_OK;
}

ypdq_status ypdq_db_wrap(ypdq_ctx* ctx, const uint8_t* d_rows, uint64_t n_rows, ypdq_db** out) {
  if (!ctx || !out || (n_rows > 0 && !d_rows)) return fail(YPDQ_ERR_INVALID, "NULL argument");
  if (!aligned16(d_rows)) return fail(YPDQ_ERR_ALIGN, "d_rows must be 16-byte aligned");
  *out = new ypdq_db{ctx, d_rows, n_rows, false};
  return YPDQ_OK;
}

ypdq_status ypdq_db_destroy(ypdq_db* db) {
  if (!db) return YPDQ_OK;
  if (db->owned && db->d_rows) {
    cudaSetDevice(db->ctx->device);
    cudaFree(const_cast<uint8_t*>(db->d_rows));
  }
  delete db;
  return YPDQ_OK;
}

ypdq_status ypdq_db_info(ypdq_db* db, const uint8_t** d_rows, uint64_t* n_rows) {
  if (!db) return fail(YPDQ_ERR_INVALID, "db is NULL");
  if (d_rows) *d_rows = db->d_rows;
  if (n_rows) *n_rows = db->n_rows;
  return YPDQ_OK;
}

ypdq_status ypdq_screen_host(ypdq_ctx* ctx, ypdq_db* db, const void* h_images, int64_t n,
                             int input_kind, int dct_precision, int semantics,
                             uint32_t threshold, ypdq_hit* h_hits, uint64_t capacity,
                             uint64_t* n_hits, uint8_t* h_hashes, float* h_quality) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (!db || !n_hits || (n > 0 && !h_images) || (capacity > 0 && !h_hits))
    return fail(YPDQ_ERR_INVALID, "NULL argument");
  if (n < 0 || n * 8 > 0xffffffffll) return fail(YPDQ_ERR_INVALID, "n out of range");
  if (image_bytes_of(input_kind) == 0)
    return fail(YPDQ_ERR_INVALID, "input_kind %d", input_kind);
  if (threshold > 256) return fail(YPDQ_ERR_INVALID, "threshold %u > 256", threshold);
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaStream_t s = ctx->stream;
  const size_t img_bytes = image_bytes_of(input_kind);
  void *d_img, *d_hash, *d_q, *d_hits, *d_cnt;
  if ((st = scratch(ctx, 0, img_bytes * (n > 0 ? n : 1), &d_img))) return st;
  if ((st = scratch(ctx, 1, 256 * (n > 0 ? n : 1), &d_hash))) return st;
  if ((st = scratch(ctx, 2, 32 * (n > 0 ? n : 1), &d_q))) return st;
  if ((st = scratch(ctx, 3, sizeof(ypdq_hit) * (capacity > 0 ? capacity : 1), &d_hits))) return st;
  if ((st = scratch(ctx, 4, 64, &d_cnt))) return st;
  CK(cudaMemsetAsync(d_cnt, 0, sizeof(uint64_t), s), "clear count");
  // Chunks whose copies (copy stream) overlap the hash and scan of the chunk before
  // (compute stream). Every chunk's scan appends to one hit list.
  int64_t bounds[ypdq_ctx::kMaxChunks + 1];
  const int nch = screen_chunks(n, input_kind, dct_precision, db->n_rows, threshold, bounds);
  uint32_t rm, cm;
  semantics_masks(semantics, &rm, &cm);
  const bool jarosz = dct_precision == YPDQ_COMPRESS_JAROSZ;
  int dct = 0, sep = 0;
  if (!jarosz && !parse_precision(dct_precision, &dct, &sep))
    return fail(YPDQ_ERR_INVALID, "dct_precision %d", dct_precision);
  int64_t jchunk = 1;
  if (jarosz && n > 0) {
    for (int c = 0; c < nch; ++c)
      jchunk = std::max<int64_t>(jchunk, jarosz_chunk(bounds[c + 1] - bounds[c]));
    if ((st = ensure_jarosz_scratch(ctx, jchunk))) return st;
    CK(cudaStreamWaitEvent(s, ctx->jarosz_done, 0), "wait jarosz scratch");
  }
  for (int c = 0; c < nch && n > 0; ++c) {
    const int64_t i0 = bounds[c], i1 = bounds[c + 1];
    const uint8_t* src = static_cast<const uint8_t*>(h_images) + i0 * img_bytes;
    uint8_t* dst = static_cast<uint8_t*>(d_img) + i0 * img_bytes;
    CK(cudaMemcpyAsync(dst, src, (i1 - i0) * img_bytes, cudaMemcpyHostToDevice, ctx->copy_stream),
       "H2D images");
    CK(cudaEventRecord(ctx->chunk_copied[c], ctx->copy_stream), "record copy");
    CK(cudaStreamWaitEvent(s, ctx->chunk_copied[c], 0), "wait copy");
    HashLaunch hp{};
    hp.images = dst;
    hp.n = i1 - i0;
    hp.input_kind = input_kind;
    hp.row_mask = rm;
    hp.col_mask = cm;
    hp.hashes = static_cast<uint8_t*>(d_hash) + i0 * 256;
    hp.quality = static_cast<float*>(d_q) + i0 * 8;
    hp.pdqf_slots = 1;
    hp.dev_err = ctx->d_err;
    hp.dct = dct;
    hp.separable = sep;
    if (jarosz)
      CK(launch_hash_jarosz(hp, ctx->jarosz_scratch, jchunk, s), "jarosz launch");
    else
      CK(launch_hash(hp, ctx->num_sms, ctx->hash_ctas[hp.input_kind][dct][sep], s),
         "hash launch");
    ScanLaunch sp{};
    sp.rows = db->d_rows;
    sp.n_rows = db->n_rows;
    sp.queries = static_cast<uint8_t*>(d_hash) + i0 * 256;
    sp.n_queries = static_cast<uint32_t>((i1 - i0) * 8);
    sp.threshold = threshold;
    sp.hits = static_cast<ypdq_hit*>(d_hits);
    sp.capacity = capacity;
    sp.count = static_cast<unsigned long long*>(d_cnt);
    sp.dev_err = ctx->d_err;
    sp.append = 1;
    sp.query_base = static_cast<uint32_t>(i0 * 8);
    CK(launch_scan(sp, YPDQ_SCAN_AUTO, ctx->num_sms, s), "scan launch");
  }
  if (jarosz && n > 0) CK(cudaEventRecord(ctx->jarosz_done, s), "record jarosz scratch");
  // results come back through the page-locked staging buffer: [count][error word][hits]
  uint8_t* stage = nullptr;
  if ((st = host_stage(ctx, 64 + sizeof(ypdq_hit) * capacity, &stage))) return st;
  CK(cudaMemcpyAsync(stage, d_cnt, sizeof(uint64_t), cudaMemcpyDeviceToHost, s), "D2H count");
  CK(cudaMemcpyAsync(stage + 8, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, s), "D2H error word");
  CK(cudaStreamSynchronize(s), "screen sync");
  uint64_t total = 0;
  memcpy(&total, stage, sizeof(total));
  const uint64_t m = total < capacity ? total : capacity;
  CK(launch_sort_hits(static_cast<ypdq_hit*>(d_hits), m, s), "sort launch");
  if (m > 0) CK(cudaMemcpyAsync(stage + 64, d_hits, m * sizeof(ypdq_hit), cudaMemcpyDeviceToHost, s), "D2H hits");
  if (h_hashes && n > 0) CK(cudaMemcpyAsync(h_hashes, d_hash, 256 * n, cudaMemcpyDeviceToHost, s), "D2H hashes");
  if (h_quality && n > 0) CK(cudaMemcpyAsync(h_quality, d_q, 32 * n, cudaMemcpyDeviceToHost, s), "D2H quality");
  CK(cudaStreamSynchronize(s), "screen sync");
  if (m > 0) memcpy(h_hits, stage + 64, m * sizeof(ypdq_hit));
  int dev_err = 0;
  memcpy(&dev_err, stage + 8, sizeof(dev_err));
  if (dev_err && (st = read_device_errors(ctx))) return st;
  *n_hits = total;
  if (total > capacity) return fail(YPDQ_ERR_OVERFLOW, "%llu hits > capacity %llu",
                                    (unsigned long long)total, (unsigned long long)capacity);
  return YPDQ_OK;
}

ypdq_status ypdq_screen_plan(int64_t n, int input_kind, int dct_precision, uint64_t n_rows,
                             uint32_t threshold, int64_t* bounds, int* n_chunks) {
  static_assert(ypdq_ctx::kMaxChunks == YPDQ_MAX_SCREEN_CHUNKS, "chunk bound");
  if (!bounds || !n_chunks) return fail(YPDQ_ERR_INVALID, "NULL argument");
  if (n < 0) return fail(YPDQ_ERR_INVALID, "n out of range");
  if (image_bytes_of(input_kind) == 0)
    return fail(YPDQ_ERR_INVALID, "input_kind %d", input_kind);
  *n_chunks = screen_chunks(n, input_kind, dct_precision, n_rows, threshold, bounds);
  return YPDQ_OK;
}

// --------------------------------------------------------- memory utilities

ypdq_status ypdq_malloc_device(ypdq_ctx* ctx, size_t bytes, void** d_ptr) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (!d_ptr) return fail(YPDQ_ERR_INVALID, "d_ptr is NULL");
  CK(cudaMalloc(d_ptr, bytes ? bytes : 1), "cudaMalloc");
  return YPDQ_OK;
}
ypdq_status ypdq_free_device(ypdq_ctx* ctx, void* d_ptr) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  CK(cudaFree(d_ptr), "cudaFree");
  return YPDQ_OK;
}
ypdq_status ypdq_malloc_host(ypdq_ctx* ctx, size_t bytes, void** h_ptr) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (!h_ptr) return fail(YPDQ_ERR_INVALID, "h_ptr is NULL");
  CK(cudaMallocHost(h_ptr, bytes ? bytes : 1), "cudaMallocHost");
  return YPDQ_OK;
}
ypdq_status ypdq_free_host(ypdq_ctx* ctx, void* h_ptr) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  CK(cudaFreeHost(h_ptr), "cudaFreeHost");
  return YPDQ_OK;
}
ypdq_status ypdq_memcpy(ypdq_ctx* ctx, void* dst, const void* src, size_t bytes, int kind,
                        ypdq_stream_t stream) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  cudaMemcpyKind k = kind == 0   ? cudaMemcpyHostToDevice
                     : kind == 1 ? cudaMemcpyDeviceToHost
                     : kind == 2 ? cudaMemcpyDeviceToDevice
                                 : cudaMemcpyDefault;
  if (kind < 0 || kind > 2) return fail(YPDQ_ERR_INVALID, "memcpy kind %d", kind);
  CK(cudaMemcpyAsync(dst, src, bytes, k, reinterpret_cast<cudaStream_t>(stream)), "cudaMemcpyAsync");
  return YPDQ_OK;
}
ypdq_status ypdq_memset(ypdq_ctx* ctx, void* d_ptr, int value, size_t bytes, ypdq_stream_t stream) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  CK(cudaMemsetAsync(d_ptr, value, bytes, reinterpret_cast<cudaStream_t>(stream)), "cudaMemsetAsync");
  return YPDQ_OK;
}
ypdq_status ypdq_stream_create(ypdq_ctx* ctx, ypdq_stream_t* out) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (!out) return fail(YPDQ_ERR_INVALID, "out is NULL");
  cudaStream_t s;
  CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
  *out = reinterpret_cast<ypdq_stream_t>(s);
  return YPDQ_OK;
}
ypdq_status ypdq_stream_destroy(ypdq_ctx* ctx, ypdq_stream_t stream) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  CK(cudaStreamDestroy(reinterpret_cast<cudaStream_t>(stream)), "cudaStreamDestroy");
  return YPDQ_OK;
}
ypdq_status ypdq_stream_sync(ypdq_ctx* ctx, ypdq_stream_t stream) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  CK(cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream)), "cudaStreamSynchronize");
  return read_device_errors(ctx);
}
ypdq_status ypdq_event_create(ypdq_ctx* ctx, ypdq_event_t* out) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (!out) return fail(YPDQ_ERR_INVALID, "out is NULL");
  cudaEvent_t ev;
  CK(cudaEventCreate(&ev), "cudaEventCreate");
  *out = reinterpret_cast<ypdq_event_t>(ev);
  return YPDQ_OK;
}
ypdq_status ypdq_event_destroy(ypdq_ctx* ctx, ypdq_event_t ev) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  CK(cudaEventDestroy(reinterpret_cast<cudaEvent_t>(ev)), "cudaEventDestroy");
  return YPDQ_OK;
}
ypdq_status ypdq_event_record(ypdq_ctx* ctx, ypdq_event_t ev, ypdq_stream_t stream) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  CK(cudaEventRecord(reinterpret_cast<cudaEvent_t>(ev), reinterpret_cast<cudaStream_t>(stream)),
     "cudaEventRecord");
  return YPDQ_OK;
}
ypdq_status ypdq_event_elapsed_ms(ypdq_ctx* ctx, ypdq_event_t a, ypdq_event_t b, float* ms) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (!ms) return fail(YPDQ_ERR_INVALID, "ms is NULL");
  CK(cudaEventSynchronize(reinterpret_cast<cudaEvent_t>(b)), "cudaEventSynchronize");
  CK(cudaEventElapsedTime(ms, reinterpret_cast<cudaEvent_t>(a), reinterpret_cast<cudaEvent_t>(b)),
     "cudaEventElapsedTime");
  return YPDQ_OK;
}

ypdq_status ypdq_synth_rows(ypdq_ctx* ctx, uint8_t* d_rows, uint64_t n_rows, uint64_t first_row,
                            uint64_t seed, ypdq_stream_t stream) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (n_rows > 0 && !d_rows) return fail(YPDQ_ERR_INVALID, "d_rows is NULL");
  if (!aligned16(d_rows)) return fail(YPDQ_ERR_ALIGN, "d_rows must be 16-byte aligned");
  CK(launch_synth_rows(d_rows, n_rows, first_row, seed, reinterpret_cast<cudaStream_t>(stream)),
     "synth launch");
  return YPDQ_OK;
}

ypdq_status ypdq_synth_clustered_rows(ypdq_ctx* ctx, uint8_t* d_rows, uint64_t n_rows,
                                      uint64_t first_row, uint64_t members_per_centre,
                                      uint32_t flip_trials, uint64_t seed, ypdq_stream_t stream) {
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  if (n_rows > 0 && !d_rows) return fail(YPDQ_ERR_INVALID, "d_rows is NULL");
  if (!aligned16(d_rows)) return fail(YPDQ_ERR_ALIGN, "d_rows must be 16-byte aligned");
  if (members_per_centre == 0) return fail(YPDQ_ERR_INVALID, "members_per_centre is 0");
  if (flip_trials > 64) return fail(YPDQ_ERR_INVALID, "flip_trials %u > 64", flip_trials);
  CK(launch_synth_clustered(d_rows, n_rows, first_row, members_per_centre, flip_trials, seed,
                            reinterpret_cast<cudaStream_t>(stream)),
     "synth launch");
  return YPDQ_OK;
}

// ------------------------------------------------------------ drop-in ABI

__attribute__((visibility("default"))) const uint32_t YUME_PDQ_VERSION_MAJOR = 1;
__attribute__((visibility("default"))) const uint32_t YUME_PDQ_VERSION_MINOR = 1;
__attribute__((visibility("default"))) const uint32_t YUME_PDQ_VERSION_PATCH = 0;
__attribute__((visibility("default"))) const char YUME_PDQ_VERSION_STRING[] = "1.1.0";

// Dihedrals::from_tuples packs ((xx, xy), (yx, yy)) as big-endian i8 bytes (src/lib.rs:97-104).
#define YPDQ_PACK(a, b, c, d)                                                             \
  ((static_cast<uint32_t>(static_cast<uint8_t>(a)) << 24) |                               \
   (static_cast<uint32_t>(static_cast<uint8_t>(b)) << 16) |                               \
   (static_cast<uint32_t>(static_cast<uint8_t>(c)) << 8) | static_cast<uint32_t>(static_cast<uint8_t>(d)))
__attribute__((visibility("default"))) const YumePDQ_Dihedrals YUME_PDQ_DIHEDRAL_NORMAL = {YPDQ_PACK(1, 0, 0, 1)};
__attribute__((visibility("default"))) const YumePDQ_Dihedrals YUME_PDQ_DIHEDRAL_FLIPPED = {YPDQ_PACK(1, 0, 0, -1)};
__attribute__((visibility("default"))) const YumePDQ_Dihedrals YUME_PDQ_DIHEDRAL_FLOPPED = {YPDQ_PACK(-1, 0, 0, 1)};
__attribute__((visibility("default"))) const YumePDQ_Dihedrals YUME_PDQ_DIHEDRAL_ROTATED_180 = {YPDQ_PACK(-1, 0, 0, -1)};
__attribute__((visibility("default"))) const YumePDQ_Dihedrals YUME_PDQ_DIHEDRAL_ROTATED_90 = {YPDQ_PACK(0, 1, -1, 0)};
__attribute__((visibility("default"))) const YumePDQ_Dihedrals YUME_PDQ_DIHEDRAL_ROTATED_270 = {YPDQ_PACK(0, 1, 1, 0)};
__attribute__((visibility("default"))) const YumePDQ_Dihedrals YUME_PDQ_DIHEDRAL_ROTATED_90_FLOPPED = {YPDQ_PACK(0, -1, -1, 0)};
__attribute__((visibility("default"))) const YumePDQ_Dihedrals YUME_PDQ_DIHEDRAL_FLOPPED_ROTATED_270 = {YPDQ_PACK(0, -1, 1, 0)};

}  // extern "C"

namespace {

std::once_flag g_dropin_once, g_dropin_sem_once;
ypdq_ctx* g_dropin_ctx = nullptr;
int g_dropin_semantics = YPDQ_DIHEDRAL_SCALAR;

// The dihedral sign convention of the drop-in symbols: the one yume-pdq's smart_kernel()
// computes on this host (src/kernel/mod.rs:79-176) in its default build (without the
// non-default `avx512` feature). On x86_64 with AVX2 and FMA that is Avx2F32Kernel (the
// router's runtime check); on any other host the trait-default DefaultKernel. The
// environment variable YUME_PDQ_DIHEDRAL_SEMANTICS = exact | avx2 | scalar overrides it
// (exact = Avx512F32Kernel, what a build with `avx512` computes on an AVX-512 host).
int dropin_semantics() {
  std::call_once(g_dropin_sem_once, [] {
    int sem = YPDQ_DIHEDRAL_SCALAR;
#if defined(__x86_64__)
    if (__builtin_cpu_supports("avx2") && __builtin_cpu_supports("fma")) sem = YPDQ_DIHEDRAL_AVX2;
#endif
    const char* env = getenv("YUME_PDQ_DIHEDRAL_SEMANTICS");
    if (env && !strcmp(env, "exact")) sem = YPDQ_DIHEDRAL_EXACT;
    if (env && !strcmp(env, "avx2")) sem = YPDQ_DIHEDRAL_AVX2;
    if (env && !strcmp(env, "scalar")) sem = YPDQ_DIHEDRAL_SCALAR;
    g_dropin_semantics = sem;
  });
  return g_dropin_semantics;
}

// The drop-in symbols use one library-owned context on device 0.
ypdq_ctx* dropin_ctx() {
  dropin_semantics();
  std::call_once(g_dropin_once, [] {
    ypdq_ctx* c = nullptr;
    if (ypdq_ctx_create(0, &c) == YPDQ_OK) g_dropin_ctx = c;
    else fprintf(stderr, "yume_pdq (gb300): %s\n", ypdq_last_error());
  });
  return g_dropin_ctx;
}

const uint32_t kSlotDihedral[8] = {
    YPDQ_PACK(1, 0, 0, 1),   YPDQ_PACK(-1, 0, 0, 1), YPDQ_PACK(-1, 0, 0, -1), YPDQ_PACK(1, 0, 0, -1),
    YPDQ_PACK(0, -1, -1, 0), YPDQ_PACK(0, 1, 1, 0),  YPDQ_PACK(0, -1, 1, 0),  YPDQ_PACK(0, 1, -1, 0)};

ypdq_status dropin_hash(ypdq_ctx* ctx, const float* input, float* threshold, uint8_t* output,
                        float* buf1, float* pdqf, float* quality) {
  std::lock_guard<std::mutex> lock(ctx->mu);
  ypdq_status st = check_ctx(ctx);
  if (st) return st;
  cudaStream_t s = ctx->stream;
  void *d_img, *d_out, *d_buf1;
  if ((st = scratch(ctx, 0, 512 * 512 * 4, &d_img))) return st;
  if ((st = scratch(ctx, 5, 256 + 32 + 32 + 1024, &d_out))) return st;
  if ((st = scratch(ctx, 6, 127 * 128 * 4, &d_buf1))) return st;
  uint8_t* d_hash = static_cast<uint8_t*>(d_out);
  float* d_q = reinterpret_cast<float*>(d_hash + 256);
  float* d_t = d_q + 8;
  float* d_p = d_t + 8;
  CK(cudaMemcpyAsync(d_img, input, 512 * 512 * 4, cudaMemcpyHostToDevice, s), "H2D image");
  HashLaunch p{};
  p.images = d_img;
  p.n = 1;
  p.input_kind = YPDQ_INPUT_F32;
  semantics_masks(g_dropin_semantics, &p.row_mask, &p.col_mask);
  p.hashes = d_hash;
  p.quality = d_q;
  p.thresholds = d_t;
  p.pdqf = d_p;
  p.pdqf_slots = 1;
  p.buf1 = buf1 ? static_cast<float*>(d_buf1) : nullptr;
  p.dev_err = ctx->d_err;
  CK(launch_hash(p, ctx->num_sms, ctx->hash_ctas_f32, s), "hash launch");
  uint8_t out[256 + 32 + 32 + 1024];
  CK(cudaMemcpyAsync(out, d_out, sizeof(out), cudaMemcpyDeviceToHost, s), "D2H results");
  if (buf1)
    CK(cudaMemcpy2DAsync(buf1, 128 * 4, d_buf1, 128 * 4, 127 * 4, 127, cudaMemcpyDeviceToHost, s),
       "D2H buf1");
  CK(cudaStreamSynchronize(s), "sync");
  if ((st = read_device_errors(ctx))) return st;
  memcpy(output, out, 32);
  float q, t;
  memcpy(&q, out + 256, 4);
  memcpy(&t, out + 256 + 32, 4);
  if (threshold) *threshold = t;
  if (pdqf) memcpy(pdqf, out + 256 + 64, 1024);
  *quality = q;
  return YPDQ_OK;
}

}  // namespace

extern "C" {

__attribute__((visibility("default"))) float yume_pdq_hash_smart_kernel(
    const float* input, float* threshold, uint8_t* output, float* buf1, float* tmp, float* pdqf) {
  (void)tmp;
  ypdq_ctx* ctx = dropin_ctx();
  if (!ctx || !input || !output) {
    fprintf(stderr, "yume_pdq_hash_smart_kernel: %s\n",
            ctx ? "NULL input/output" : "no CUDA context");
    return -1.0f;
  }
  float q = -1.0f;
  if (dropin_hash(ctx, input, threshold, output, buf1, pdqf, &q) != YPDQ_OK) {
    fprintf(stderr, "yume_pdq_hash_smart_kernel: %s\n", ypdq_last_error());
    return -1.0f;
  }
  return q;
}

__attribute__((visibility("default"))) bool yume_pdq_visit_dihedrals_smart_kernel(
    void* cb_ctx, float threshold, uint8_t* output, float* pdqf, DihedralCallback callback) {
  ypdq_ctx* ctx = dropin_ctx();
  if (!ctx || !output || !pdqf || !callback) {
    fprintf(stderr, "yume_pdq_visit_dihedrals_smart_kernel: %s\n",
            ctx ? "NULL argument" : "no CUDA context");
    return false;
  }
  uint8_t res[256 + 32 + 32 + 8 * 1024];
  {
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (check_ctx(ctx) != YPDQ_OK) return false;
    cudaStream_t s = ctx->stream;
    void *d_in, *d_out;
    if (scratch(ctx, 5, 1024 + 16, &d_in) != YPDQ_OK ||
        scratch(ctx, 7, sizeof(res), &d_out) != YPDQ_OK) {
      fprintf(stderr, "yume_pdq_visit_dihedrals_smart_kernel: %s\n", ypdq_last_error());
      return false;
    }
    float* d_p = static_cast<float*>(d_in);
    float* d_thr = d_p + 256;
    uint8_t* d_hash = static_cast<uint8_t*>(d_out);
    float* d_q = reinterpret_cast<float*>(d_hash + 256);
    float* d_t = d_q + 8;
    float* d_pv = d_t + 8;
    cudaError_t e = cudaMemcpyAsync(d_p, pdqf, 1024, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_thr, &threshold, 4, cudaMemcpyHostToDevice, s);
    DihedralLaunch p{};
    p.pdqf = d_p;
    p.thr_in = d_thr;
    p.n = 1;
    semantics_masks(g_dropin_semantics, &p.row_mask, &p.col_mask);
    p.hashes = d_hash;
    p.quality = d_q;
    p.thresholds = d_t;
    p.pdqf_out = d_pv;
    if (e == cudaSuccess) e = launch_dihedrals(p, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(res, d_out, sizeof(res), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      fprintf(stderr, "yume_pdq_visit_dihedrals_smart_kernel: %s\n", cudaGetErrorString(e));
      return false;
    }
  }
  const float* q = reinterpret_cast<const float*>(res + 256);
  const float* pv = reinterpret_cast<const float*>(res + 256 + 64);
  for (int v = 1; v < 8; ++v) {
    memcpy(output, res + v * 32, 32);
    memcpy(pdqf, pv + v * 256, 1024);
    if (!callback(cb_ctx, kSlotDihedral[v], threshold, q[v])) return false;
  }
  return true;
}

ypdq_status ypdq_dropin_semantics(int* semantics) {
  if (!semantics) return YPDQ_ERR_INVALID;
  *semantics = dropin_semantics();
  return YPDQ_OK;
}

}  // extern "C"
