// ypdq_screen_noalloc: screening (hash + 8 dihedrals + exact scan) with no allocation.
//
// Some callers cannot call cudaMalloc: code running inside a host framework that owns
// all device memory through its own pool, or code that screens from a real-time path
// where an allocation (which may synchronise the device) is not allowed. This entry point
// lets them screen images they already hold on the device. It keeps the one piece of
// working memory the screen path needs, the 8 hashes per image that the scan reads as its
// queries, in a fixed file-scope device array instead of allocating it.
//
// Limits and behaviour:
//   * at most kMaxImages = 4096 images per call (1 MiB of hashes); larger n is rejected
//     with YPDQ_ERR_INVALID before anything is launched;
//   * the array is in every GPU's memory for as long as the library is loaded;
//   * all calls share the array, so calls that overlap on the GPU (different streams or
//     threads without ordering) race and corrupt each other's results; order them;
//   * the first call on a device does a one-time set-up there: it resolves the array's
//     device address (cudaGetSymbolAddress), uploads the DCT table and sets kernel
//     attributes. Make that first call before any stream capture. The set-up belongs to
//     the device's CUDA context: after cudaDeviceReset the next call (in the new context)
//     does it again;
//   * no cudaMalloc, cudaFree or allocating library routine is called.
#include <cstdio>
#include <mutex>

#include "capi_internal.h"
#include "ypdq_internal.cuh"

namespace ypdq {

void set_last_error_text(const char* text);

namespace noalloc {

constexpr int64_t kMaxImages = 4096;
constexpr size_t kHashBytes = static_cast<size_t>(kMaxImages) * 8 * 32;
constexpr size_t kScratchBytes = kHashBytes + 256;  // hashes, then the device error word
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct DeviceState {
  bool ready = false;
  unsigned long long context_id = 0;  // the CUDA context the set-up was done in
  uint8_t* hashes = nullptr;  // device address of g_noalloc_scratch on this device
  int* err = nullptr;
  int num_sms = 0;
  int ctas_f32 = 1;
  int ctas_u8 = 1;
};

static std::mutex g_mu;
static DeviceState g_state[kMaxDevices];

static ypdq_status fail_with(ypdq_status st, const char* msg, const char* detail = nullptr) {
  char buf[256];
  if (detail)
    snprintf(buf, sizeof(buf), "%s: %s", msg, detail);
  else
    snprintf(buf, sizeof(buf), "%s", msg);
  set_last_error_text(buf);
  return st;
}

// Unique id of the calling thread's current CUDA context (driver cuCtxGetCurrent and
// cuCtxGetId, reached through the runtime's entry-point query so the library needs no
// libcuda link), or 0 when it cannot be read. A context that cudaDeviceReset destroyed and
// the runtime created again has a new id.
static unsigned long long current_context_id() {
  using GetCurrent = int (*)(void**);
  using GetId = int (*)(void*, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault,
                                         nullptr) == cudaSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, nullptr) ==
        cudaSuccess)
      get_id = reinterpret_cast<GetId>(f);
  });
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

// Set-up on the current device, once per CUDA context; host code may not use the array's
// name as an address, so the device address comes from cudaGetSymbolAddress with that
// device current.
static ypdq_status setup(int dev, DeviceState** out) {
  std::lock_guard<std::mutex> lock(g_mu);
  DeviceState& s = g_state[dev];
  // a new context (the device was reset) needs its own set-up; when the context cannot be
  // identified, every call redoes it
  const unsigned long long cid = current_context_id();
  if (s.ready && (cid == 0 || cid != s.context_id)) s.ready = false;
  if (!s.ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return fail_with(YPDQ_ERR_CUDA, "cudaGetSymbolAddress", cudaGetErrorString(e));
    if ((e = upload_constants()) != cudaSuccess || (e = scan_init()) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&s.num_sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
        (e = hash_occupancy(0, &s.ctas_f32)) != cudaSuccess ||
        (e = hash_occupancy(1, &s.ctas_u8)) != cudaSuccess)
      return fail_with(YPDQ_ERR_CUDA, "no-alloc set-up", cudaGetErrorString(e));
    s.hashes = static_cast<uint8_t*>(p);
    s.err = reinterpret_cast<int*>(static_cast<uint8_t*>(p) + kHashBytes);
    s.context_id = current_context_id();
    s.ready = true;
  }
  *out = &s;
  return YPDQ_OK;
}

// A device-side timeout during the call turns the hit count into UINT64_MAX.
__global__ void report_kernel(const int* err, unsigned long long* count) {
  if (*err) *count = ~0ull;
}

}  // namespace noalloc
}  // namespace ypdq

extern "C" ypdq_status ypdq_screen_noalloc(const void* d_images, int64_t n, int input_kind,
                                           int semantics, const uint8_t* d_rows,
                                           uint64_t n_rows, uint32_t threshold,
                                           ypdq_hit* d_hits, uint64_t capacity,
                                           uint64_t* d_count, ypdq_stream_t stream) {
  using namespace ypdq;
  using namespace ypdq::noalloc;
  if (n < 0 || n > kMaxImages)
    return fail_with(YPDQ_ERR_INVALID, "n out of range: ypdq_screen_noalloc takes 0..4096 images");
  if (input_kind != YPDQ_INPUT_F32 && input_kind != YPDQ_INPUT_U8)
    return fail_with(YPDQ_ERR_INVALID, "input_kind must be YPDQ_INPUT_F32 or YPDQ_INPUT_U8");
  if (semantics < YPDQ_DIHEDRAL_EXACT || semantics > YPDQ_DIHEDRAL_SCALAR)
    return fail_with(YPDQ_ERR_INVALID, "unknown dihedral semantics");
  if (threshold > 256) return fail_with(YPDQ_ERR_INVALID, "threshold > 256");
  if (!d_count || (n > 0 && !d_images) || (n_rows > 0 && !d_rows) || (capacity > 0 && !d_hits))
    return fail_with(YPDQ_ERR_INVALID, "NULL argument");
  if ((reinterpret_cast<uintptr_t>(d_images) & 15u) || (reinterpret_cast<uintptr_t>(d_rows) & 15u))
    return fail_with(YPDQ_ERR_ALIGN, "images and rows must be 16-byte aligned");
  // the count takes 64-bit atomics and a memset; hits are stored as 16-byte records
  if ((reinterpret_cast<uintptr_t>(d_count) & 7u) ||
      (reinterpret_cast<uintptr_t>(d_hits) % alignof(ypdq_hit)))
    return fail_with(YPDQ_ERR_ALIGN, "d_count and d_hits must be 8-byte aligned");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail_with(YPDQ_ERR_CUDA, "cudaGetDevice", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail_with(YPDQ_ERR_UNSUPPORTED, "device ordinal too large");
  DeviceState* s = nullptr;
  ypdq_status st = setup(dev, &s);
  if (st != YPDQ_OK) return st;
  cudaStream_t cs = reinterpret_cast<cudaStream_t>(stream);

  // The array keeps the previous call's contents: the error word must start at zero. The
  // hashes are overwritten in full before the scan reads them; the count is reset by the scan.
  e = cudaMemsetAsync(s->err, 0, sizeof(int), cs);
  if (e == cudaSuccess) {
    HashLaunch hp{};
    hp.images = d_images;
    hp.n = n;
    hp.input_kind = input_kind;
    semantics_masks(semantics, &hp.row_mask, &hp.col_mask);
    hp.hashes = s->hashes;
    hp.pdqf_slots = 1;
    hp.dev_err = s->err;
    e = launch_hash(hp, s->num_sms, input_kind == YPDQ_INPUT_U8 ? s->ctas_u8 : s->ctas_f32, cs);
  }
  if (e == cudaSuccess) {
    ScanLaunch sp{};
    sp.rows = d_rows;
    sp.n_rows = n_rows;
    sp.queries = s->hashes;
    sp.n_queries = static_cast<uint32_t>(n * 8);
    sp.threshold = threshold;
    sp.hits = d_hits;
    sp.capacity = capacity;
    sp.count = reinterpret_cast<unsigned long long*>(d_count);
    sp.dev_err = s->err;
    e = launch_scan(sp, YPDQ_SCAN_AUTO, s->num_sms, cs);
  }
  if (e == cudaSuccess) {
    report_kernel<<<1, 1, 0, cs>>>(s->err, reinterpret_cast<unsigned long long*>(d_count));
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return fail_with(YPDQ_ERR_CUDA, "ypdq_screen_noalloc", cudaGetErrorString(e));
  return YPDQ_OK;
}
