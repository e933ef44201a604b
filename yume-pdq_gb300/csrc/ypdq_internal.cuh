// Internal declarations shared by the CUDA translation units of libyumepdq_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ypdq.h"

namespace ypdq {

// Device-side error bits, OR-ed into the context's error word by a kernel that gives up.
constexpr int kDevErrTimeout = 1;

// Accumulator columns per pass of the FP4 scan (pair_n of its launches): three queries each.
constexpr uint32_t kPairFp4N = 240;

// Longest time a device-side wait spins before the kernel reports a timeout and returns.
constexpr uint64_t kWaitLimitNs = 4ull * 1000 * 1000 * 1000;

// ----------------------------------------------------------------- PTX helpers

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// mbar_try_wait that may suspend the thread until the phase completes or about hint_ns pass
// (the suspend-time hint of mbarrier.try_wait), instead of the hardware's short default.
__device__ __forceinline__ bool mbar_try_wait_hint(uint64_t* bar, uint32_t parity,
                                                   uint32_t hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}

// Wait for the phase with the given parity. Gives up (returns false) when *abort_flag is
// set by another warp or when limit_ns passes; the caller then raises the error. Between
// checks the thread sleeps in try_wait (up to 20 us a time) rather than spinning: a spinning
// waiter takes issue slots from the warps that share its scheduler, which in the tensor-core
// scans are the expanders and the epilogue on the critical path.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          const volatile int* abort_flag,
                                          uint64_t limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  for (;;) {
    if (mbar_try_wait_hint(bar, parity, 20000u)) return true;
    if (*abort_flag) return false;
    if (globaltimer_ns() - t0 > limit_ns) return false;
  }
}

// 1-D bulk copy global -> shared, completing `bytes` transactions on `bar`.
// Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* smem_dst, const void* gsrc, uint32_t bytes,
                                         uint64_t* bar, uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint "
      "[%0], [%1], %2, [%3], %4;" ::"r"(smem_u32(smem_dst)),
      "l"(gsrc), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
      : "memory");
}

__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}

__device__ __forceinline__ void named_bar_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ------------------------------------------------------------- tcgen05 helpers

__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  return static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4) |
         (static_cast<uint64_t>(1) << 16) |              // leading byte offset (unused here)
         (static_cast<uint64_t>(1024 >> 4) << 32) |      // stride byte offset
         (static_cast<uint64_t>(1) << 46) |              // descriptor version (tcgen05)
         (static_cast<uint64_t>(2) << 61);               // swizzle: 128 B
}

// The same for a 64-byte-swizzled K-major operand: rows of 64 B, 8-row atoms of 512 B.
__device__ __forceinline__ uint64_t sw64_desc(uint32_t saddr) {
  return static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4) |
         (static_cast<uint64_t>(1) << 16) |              // leading byte offset (unused here)
         (static_cast<uint64_t>(512 >> 4) << 32) |       // stride byte offset
         (static_cast<uint64_t>(1) << 46) |              // descriptor version (tcgen05)
         (static_cast<uint64_t>(4) << 61);               // swizzle: 64 B
}

// ------------------------------------------------------------- launch plumbing

struct HashLaunch {
  const void* images;
  int64_t n;
  int input_kind;  // ypdq_input_kind: 0 f32, 1 u8, 2 RGB8, 3 RGBA8
  uint32_t row_mask, col_mask;
  uint8_t* hashes;
  float* quality;
  float* thresholds;
  float* pdqf;
  int pdqf_slots;
  float* buf1;
  int* dev_err;
  int dct;  // 0 FP32 SIMT (bit-exact), 1 TF32, 2 BF16x3 tensor cores
  int separable;  // nonzero: separable compress (YPDQ_COMPRESS_SEPARABLE) instead of the
                  // reference's tap order
  const int64_t* n_dev;  // if set, the image count is read from here (graph replay); n is the bound
};

struct DihedralLaunch {
  const float* pdqf;
  const float* thr_in;
  int64_t n;
  uint32_t row_mask, col_mask;
  uint8_t* hashes;
  float* quality;
  float* thresholds;
  float* pdqf_out;
};

struct ScanLaunch {
  const uint8_t* rows;
  uint64_t n_rows;
  const uint8_t* queries;
  uint32_t n_queries;
  uint32_t threshold;
  ypdq_hit* hits;
  uint64_t capacity;
  unsigned long long* count;
  int* dev_err;
  int append;            // nonzero: add to *count instead of resetting it first
  uint32_t query_base;   // added to every reported query number
  const uint32_t* nq_dev;  // if set, the query count is read from here when the kernel runs
                           // (graph replay); n_queries is then its upper bound
  uint32_t n_tile;         // tensor-core scan: queries per pass (multiple of 64, <= 256);
                           // 0 picks min(256, n_queries rounded up to 64)
  uint32_t pair_n;         // tensor-core scan at t <= 36: 256 = passes of 256 query pairs,
                           // two per accumulator column (FP8 operands); kPairFp4N = passes of
                           // that many triples of queries, three per column, with block-scaled
                           // FP4 operands; with n_tile and pair_n both 0 the launcher picks
                           // past 256 queries
};

// hash.cu
cudaError_t upload_constants();
cudaError_t hash_occupancy(int input_kind, int* ctas_per_sm);
cudaError_t hash_occupancy_variant(int input_kind, int dct, int separable, int* ctas_per_sm);
cudaError_t launch_hash(const HashLaunch& p, int num_sms, int ctas_per_sm, cudaStream_t s);
cudaError_t launch_dihedrals(const DihedralLaunch& p, cudaStream_t s);

// jarosz.cu: ReferenceKernel<f32> (full Jarosz compress, sequential DCT) over p.n images in
// chunks of `chunk`, using `scratch` (jarosz_scratch_bytes(chunk) bytes).
cudaError_t jarosz_init();
size_t jarosz_scratch_bytes(int64_t chunk);
cudaError_t launch_hash_jarosz(const HashLaunch& p, void* scratch, int64_t chunk, cudaStream_t s);

// scan.cu
cudaError_t scan_init();
cudaError_t launch_scan(const ScanLaunch& p, int algo, int num_sms, cudaStream_t s);
// the algorithm YPDQ_SCAN_AUTO runs for n_queries queries at threshold t
int auto_scan_algo(uint32_t n_queries, uint32_t threshold);
cudaError_t launch_sort_hits(ypdq_hit* hits, uint64_t n, cudaStream_t s);

// scan_tc.cu
cudaError_t scan_tc_init();
// Wait limit of the tensor-core scan kernels and the number of their next launches whose
// producer issues nothing (ypdq_set_scan_wait_limit, ypdq_debug_stall_scans)
uint64_t scan_wait_limit_ns();
bool take_scan_stall();
cudaError_t launch_scan_tc(const ScanLaunch& p, int num_sms, cudaStream_t s);

// stages.cu: the Kernel trait's per-stage methods on n items
cudaError_t stages_init();
cudaError_t launch_dct2d(const float* buf, int64_t n, int stride, float* pdqf, int num_sms,
                         cudaStream_t s);
cudaError_t launch_gradients(const float* pdqf, int64_t n, float* out, cudaStream_t s);
cudaError_t launch_pdqf_op(float* pdqf, int64_t n, int op, uint32_t row_mask, uint32_t col_mask,
                           int num_sms, cudaStream_t s);
cudaError_t launch_luma(const uint8_t* px, int64_t n, int channels, float rc, float gc, float bc,
                        float* out, int num_sms, cudaStream_t s);

// synth.cu
cudaError_t launch_synth_rows(uint8_t* rows, uint64_t n, uint64_t first, uint64_t seed,
                              cudaStream_t s);
cudaError_t launch_synth_clustered(uint8_t* rows, uint64_t n, uint64_t first, uint64_t members,
                                   uint32_t trials, uint64_t seed, cudaStream_t s);

}  // namespace ypdq
