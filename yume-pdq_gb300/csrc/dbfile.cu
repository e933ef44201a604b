// Database files: ypdq_db_load_file / ypdq_db_save_file of include/ypdq.h.
//
// The format is yume-pdq's in-memory database: consecutive 32-byte rows (four little-endian
// u64), no header. The reference batches rows in whole 2,048-row chunks and pads the last
// one by repeating the final row (examples/end_to_end.rs:52-53); such a file loads as-is,
// padding included, so a scan over it reports what the reference's matcher reports over the
// same rows. Files of any size (beyond 4 GB) stream through two pinned staging buffers: the
// read of chunk c+1 overlaps the device copy of chunk c.
#define _FILE_OFFSET_BITS 64
#include <cstdio>

#include "capi_internal.h"
#include "ypdq_internal.cuh"

using namespace ypdq;

namespace {

constexpr size_t kDefaultChunk = 64ull << 20;

struct FileCloser {
  FILE* f;
  ~FileCloser() {
    if (f) fclose(f);
  }
};

struct Staging {
  void* buf[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  ~Staging() {
    for (int i = 0; i < 2; ++i) {
      if (done[i]) cudaEventDestroy(done[i]);
      if (buf[i]) cudaFreeHost(buf[i]);
    }
  }
};

size_t chunk_of(uint64_t chunk_bytes) {
  size_t c = chunk_bytes ? static_cast<size_t>(chunk_bytes) : kDefaultChunk;
  c -= c % 32;
  return c < 32 ? 32 : c;
}

}  // namespace

extern "C" {

ypdq_status ypdq_db_load_file(ypdq_ctx* ctx, const char* path, uint64_t chunk_bytes,
                              ypdq_db** out) {
  if (!ctx || !path || !out) return fail(YPDQ_ERR_INVALID, "NULL argument");
  *out = nullptr;
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  FileCloser fc{fopen(path, "rb")};
  if (!fc.f) return fail(YPDQ_ERR_INVALID, "cannot open %s", path);
  if (fseeko(fc.f, 0, SEEK_END) != 0) return fail(YPDQ_ERR_INVALID, "cannot seek %s", path);
  const off_t size = ftello(fc.f);
  if (size < 0 || fseeko(fc.f, 0, SEEK_SET) != 0)
    return fail(YPDQ_ERR_INVALID, "cannot size %s", path);
  if (size % 32 != 0)
    return fail(YPDQ_ERR_INVALID, "%s: %lld bytes is not a whole number of 32-byte rows", path,
                static_cast<long long>(size));
  const uint64_t n_rows = static_cast<uint64_t>(size) / 32;
  const size_t chunk = chunk_of(chunk_bytes);
  void* d = nullptr;
  if (n_rows > 0) CK(cudaMalloc(&d, static_cast<size_t>(size)), "cudaMalloc(db)");
  Staging stg;
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
    e = cudaMallocHost(&stg.buf[i], chunk);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&stg.done[i], cudaEventDisableTiming);
  }
  uint64_t off = 0;
  int k = 0;
  while (e == cudaSuccess && off < static_cast<uint64_t>(size)) {
    const size_t len = static_cast<size_t>(
        static_cast<uint64_t>(size) - off < chunk ? static_cast<uint64_t>(size) - off : chunk);
    e = cudaEventSynchronize(stg.done[k]);  // the copy that last used this buffer
    if (e != cudaSuccess) break;
    if (fread(stg.buf[k], 1, len, fc.f) != len) {
      cudaStreamSynchronize(ctx->copy_stream);
      cudaFree(d);
      return fail(YPDQ_ERR_INVALID, "%s: short read at byte %llu", path,
                  static_cast<unsigned long long>(off));
    }
    e = cudaMemcpyAsync(static_cast<uint8_t*>(d) + off, stg.buf[k], len, cudaMemcpyHostToDevice,
                        ctx->copy_stream);
    if (e == cudaSuccess) e = cudaEventRecord(stg.done[k], ctx->copy_stream);
    off += len;
    k ^= 1;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->copy_stream);
  if (e != cudaSuccess) {
    cudaFree(d);
    return cuda_fail(e, "db file upload");
  }
  *out = new ypdq_db{ctx, static_cast<const uint8_t*>(d), n_rows, true};
  return YPDQ_OK;
}

ypdq_status ypdq_db_save_file(ypdq_db* db, const char* path, uint64_t chunk_bytes) {
  if (!db || !path) return fail(YPDQ_ERR_INVALID, "NULL argument");
  CK(cudaSetDevice(db->ctx->device), "cudaSetDevice");
  FileCloser fc{fopen(path, "wb")};
  if (!fc.f) return fail(YPDQ_ERR_INVALID, "cannot create %s", path);
  const uint64_t size = db->n_rows * 32;
  const size_t chunk = chunk_of(chunk_bytes);
  Staging stg;
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
    e = cudaMallocHost(&stg.buf[i], chunk);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&stg.done[i], cudaEventDisableTiming);
  }
  // copy chunk c+1 to the host while chunk c is written to the file
  uint64_t issued = 0, written = 0;
  size_t len[2] = {0, 0};
  int k = 0;
  if (e == cudaSuccess && size > 0) {
    len[0] = static_cast<size_t>(size < chunk ? size : chunk);
    e = cudaMemcpyAsync(stg.buf[0], db->d_rows, len[0], cudaMemcpyDeviceToHost, db->ctx->copy_stream);
    if (e == cudaSuccess) e = cudaEventRecord(stg.done[0], db->ctx->copy_stream);
    issued = len[0];
  }
  while (e == cudaSuccess && written < size) {
    if (issued < size) {
      const int nk = k ^ 1;
      len[nk] = static_cast<size_t>(size - issued < chunk ? size - issued : chunk);
      e = cudaMemcpyAsync(stg.buf[nk], db->d_rows + issued, len[nk], cudaMemcpyDeviceToHost,
                          db->ctx->copy_stream);
      if (e == cudaSuccess) e = cudaEventRecord(stg.done[nk], db->ctx->copy_stream);
      issued += len[nk];
    }
    if (e == cudaSuccess) e = cudaEventSynchronize(stg.done[k]);
    if (e != cudaSuccess) break;
    if (fwrite(stg.buf[k], 1, len[k], fc.f) != len[k]) {
      cudaStreamSynchronize(db->ctx->copy_stream);
      return fail(YPDQ_ERR_INVALID, "%s: short write at byte %llu", path,
                  static_cast<unsigned long long>(written));
    }
    written += len[k];
    k ^= 1;
  }
  if (e != cudaSuccess) {
    cudaStreamSynchronize(db->ctx->copy_stream);
    return cuda_fail(e, "db file download");
  }
  if (fflush(fc.f) != 0) return fail(YPDQ_ERR_INVALID, "%s: flush failed", path);
  return YPDQ_OK;
}

}  // extern "C"
