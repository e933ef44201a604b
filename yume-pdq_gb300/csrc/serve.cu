// Continuous-batching screening service: ypdq_server_* of include/ypdq.h.
//
// The reference's only serving pattern is the CLI `pipe` loop (src/main.rs:391-836): two
// threads ping-pong one frame at a time between reading and hashing. Here a worker thread
// packs whole requests of any image count into device steps and keeps up to `slots` steps
// on the GPU at once, each in its own stream with its own device memory:
//
//   submit() -> host queue (bounded in images) -> free slot -> per-request H2D copies
//            -> graph replay of the step's batch bucket [header H2D, clear count, hash,
//               scan, D2H of count / hit prefix / hashes / quality] -> event
//   worker: event done -> (rare: copy the rest of the hits, or re-scan exactly past the
//            step's hit capacity) -> split hits per request, sort, write outputs -> post
//
// The graph of a bucket reads the step's image and query counts from device memory (the
// kernels take a device-side count bounded by the bucket), so one capture per bucket and
// slot serves every step size.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "capi_internal.h"
#include "ypdq_internal.cuh"

using namespace ypdq;
using Clock = std::chrono::steady_clock;

namespace {

constexpr uint64_t kHitPrefix = 8192;  // hits every step's graph copies back
constexpr uint32_t kDefaultStepImages = 1024;
constexpr uint32_t kDefaultSlots = 3;
constexpr uint64_t kDefaultStepHits = 1ull << 20;

// Per-step control block; the device copy is read by the kernels, the pinned host copy is
// written by the worker before a replay and receives count and error flags after it.
struct StepHeader {
  int64_t n_images;
  uint32_t n_queries;
  uint32_t pad0;
  unsigned long long count;  // hits found by the scan
  int err;                   // kernel error flags of this step
  int pad1;
};
static_assert(sizeof(StepHeader) == 32, "header layout");

struct Request {
  uint64_t id = 0, tag = 0;
  const uint8_t* images = nullptr;
  uint32_t n = 0;
  ypdq_hit* hits = nullptr;
  uint64_t cap = 0;
  uint8_t* hashes = nullptr;
  float* quality = nullptr;
  Clock::time_point t_submit;
};

struct Bucket {
  uint32_t images = 0;
  int algo = YPDQ_SCAN_TC;
  uint32_t n_tile = 0;   // tensor-core scan: queries per pass, one per accumulator column
  uint32_t pair_n = 0;   // or query pairs per pass, two per column (t <= 36)
  float ms = 0.0f;
  uint64_t steps = 0;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  uint8_t* d_images = nullptr;
  uint8_t* d_hashes = nullptr;
  float* d_quality = nullptr;
  ypdq_hit* d_hits = nullptr;
  void* d_jarosz = nullptr;  // YPDQ_COMPRESS_JAROSZ: the filter planes of a whole step
  StepHeader* d_hdr = nullptr;
  StepHeader* h_hdr = nullptr;  // pinned
  ypdq_hit* h_hits = nullptr;   // pinned, step_hit_capacity entries
  uint8_t* h_hashes = nullptr;  // pinned, max_step_images x 256 B
  float* h_quality = nullptr;   // pinned, max_step_images x 8 floats
  std::vector<cudaGraphExec_t> exec;  // one per bucket
  std::vector<Request> reqs;
  uint64_t step = 0;
  int bucket = 0;
  uint32_t n_images = 0;
  ypdq_status launch_status = YPDQ_OK;
};

bool hit_order(const ypdq_hit& a, const ypdq_hit& b) {
  return a.index < b.index || (a.index == b.index && a.query < b.query);
}

}  // namespace

struct ypdq_server {
  ypdq_ctx* ctx = nullptr;
  ypdq_db* db = nullptr;
  ypdq_server_config cfg{};
  size_t image_bytes = 0;
  uint32_t row_mask = 0, col_mask = 0;
  uint32_t max_step = 0;  // images per step after tuning
  std::vector<Bucket> buckets;
  std::vector<Slot> slots;

  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request> pending;
  uint64_t pending_images = 0;
  std::vector<int> free_slots;
  std::deque<int> inflight;
  std::deque<ypdq_completion> completions;
  bool stop = false;
  std::thread worker;
  std::atomic<uint64_t> arrivals{0};  // submissions, read by the worker's spin loop
  uint64_t next_id = 1, next_step = 0;
  uint64_t outstanding = 0;  // accepted, not yet posted

  // statistics window
  uint64_t submitted = 0, rejected = 0, completed = 0, images_completed = 0;
  uint64_t hits_completed = 0, steps = 0, rescans = 0, step_images = 0;
  std::vector<double> latencies;
  Clock::time_point window_start;
};

namespace {

ypdq_status capture_bucket(ypdq_server* S, Slot& sl, const Bucket& b, cudaGraphExec_t* out) {
  cudaStream_t s = sl.stream;
  const uint32_t nb = b.images;
  const int kind = S->cfg.input_kind;
  CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
  HashLaunch hp{};
  hp.images = sl.d_images;
  hp.n = nb;
  hp.n_dev = &sl.d_hdr->n_images;
  hp.input_kind = kind;
  hp.row_mask = S->row_mask;
  hp.col_mask = S->col_mask;
  hp.hashes = sl.d_hashes;
  hp.quality = sl.d_quality;
  hp.pdqf_slots = 1;
  hp.dev_err = &sl.d_hdr->err;
  const bool jarosz = S->cfg.dct_precision == YPDQ_COMPRESS_JAROSZ;
  if (!jarosz) parse_precision(S->cfg.dct_precision, &hp.dct, &hp.separable);
  ScanLaunch sp{};
  sp.rows = S->db->d_rows;
  sp.n_rows = S->db->n_rows;
  sp.queries = sl.d_hashes;
  sp.n_queries = 8 * nb;
  sp.nq_dev = &sl.d_hdr->n_queries;
  sp.n_tile = b.algo == YPDQ_SCAN_TC ? b.n_tile : 0;
  sp.pair_n = b.algo == YPDQ_SCAN_TC ? b.pair_n : 0;
  sp.threshold = S->cfg.threshold;
  sp.hits = sl.d_hits;
  sp.capacity = S->cfg.step_hit_capacity;
  sp.count = &sl.d_hdr->count;
  sp.dev_err = &sl.d_hdr->err;
  sp.append = 1;
  const uint64_t prefix = std::min<uint64_t>(kHitPrefix, S->cfg.step_hit_capacity);
  cudaError_t e = cudaMemcpyAsync(sl.d_hdr, sl.h_hdr, 16, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(&sl.d_hdr->count, 0, 16, s);
  if (e == cudaSuccess)
    e = jarosz ? launch_hash_jarosz(hp, sl.d_jarosz, nb, s)
               : launch_hash(hp, S->ctx->num_sms, S->ctx->hash_ctas[kind][hp.dct][hp.separable], s);
  if (e == cudaSuccess) e = launch_scan(sp, b.algo, S->ctx->num_sms, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&sl.h_hdr->count, &sl.d_hdr->count, 16, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(sl.h_hits, sl.d_hits, prefix * sizeof(ypdq_hit), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(sl.h_hashes, sl.d_hashes, size_t(nb) * 256, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(sl.h_quality, sl.d_quality, size_t(nb) * 32, cudaMemcpyDeviceToHost, s);
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(s, &g);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
  if (g) cudaGraphDestroy(g);
  CK(e, "capture step graph");
  return YPDQ_OK;
}

// Copies the step's images, writes its header and replays the bucket graph.
ypdq_status launch_step(ypdq_server* S, Slot& sl) {
  size_t off = 0;
  for (const Request& r : sl.reqs) {
    CK(cudaMemcpyAsync(sl.d_images + off, r.images, size_t(r.n) * S->image_bytes,
                       cudaMemcpyHostToDevice, sl.stream),
       "H2D request images");
    off += size_t(r.n) * S->image_bytes;
  }
  sl.h_hdr->n_images = sl.n_images;
  sl.h_hdr->n_queries = 8 * sl.n_images;
  CK(cudaGraphLaunch(sl.exec[sl.bucket], sl.stream), "graph launch");
  CK(cudaEventRecord(sl.done, sl.stream), "record step");
  return YPDQ_OK;
}

// Exact re-scan of a step whose hits overflowed its device buffer: the hashes are still on
// the device, and the count of the first scan is exact, so one buffer of that size holds all.
ypdq_status rescan_step(ypdq_server* S, Slot& sl, uint64_t total, std::vector<ypdq_hit>& out) {
  ypdq_hit* d_big = nullptr;
  CK(cudaMalloc(&d_big, total * sizeof(ypdq_hit)), "cudaMalloc(rescan hits)");
  ScanLaunch sp{};
  sp.rows = S->db->d_rows;
  sp.n_rows = S->db->n_rows;
  sp.queries = sl.d_hashes;
  sp.n_queries = 8 * sl.n_images;
  sp.threshold = S->cfg.threshold;
  sp.hits = d_big;
  sp.capacity = total;
  sp.count = &sl.d_hdr->count;
  sp.dev_err = &sl.d_hdr->err;
  cudaError_t e = launch_scan(sp, YPDQ_SCAN_AUTO, S->ctx->num_sms, sl.stream);
  unsigned long long again = 0;
  out.resize(total);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&again, &sl.d_hdr->count, 8, cudaMemcpyDeviceToHost, sl.stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out.data(), d_big, total * sizeof(ypdq_hit), cudaMemcpyDeviceToHost,
                        sl.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(sl.stream);
  cudaFree(d_big);
  CK(e, "re-scan");
  if (again != total) return fail(YPDQ_ERR_CUDA, "re-scan found %llu hits, first scan %llu",
                                  again, (unsigned long long)total);
  return YPDQ_OK;
}

// Reads a finished step back, splits its hits per request and posts the completions.
void finish_step(ypdq_server* S, Slot& sl, cudaError_t q) {
  thread_local std::vector<ypdq_hit> big, sorted;
  thread_local std::vector<uint32_t> img_req, counts, starts;
  ypdq_status st = sl.launch_status;
  if (st == YPDQ_OK && q != cudaSuccess) st = cuda_fail(q, "step");
  uint64_t total = 0;
  const ypdq_hit* hits = sl.h_hits;
  if (st == YPDQ_OK) {
    total = sl.h_hdr->count;
    if (sl.h_hdr->err) st = (sl.h_hdr->err & kDevErrTimeout) ? YPDQ_ERR_TIMEOUT : YPDQ_ERR_CUDA;
  }
  bool rescanned = false;
  if (st == YPDQ_OK && total > S->cfg.step_hit_capacity) {
    st = rescan_step(S, sl, total, big);
    hits = big.data();
    rescanned = true;
  } else if (st == YPDQ_OK && total > kHitPrefix) {
    cudaError_t e = cudaMemcpyAsync(sl.h_hits + kHitPrefix, sl.d_hits + kHitPrefix,
                                    (total - kHitPrefix) * sizeof(ypdq_hit),
                                    cudaMemcpyDeviceToHost, sl.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(sl.stream);
    if (e != cudaSuccess) st = cuda_fail(e, "D2H step hits");
  }
  const size_t nr = sl.reqs.size();
  counts.assign(nr, 0);
  starts.assign(nr + 1, 0);
  if (st == YPDQ_OK) {
    // image -> request, then a counting sort of the hits by request
    img_req.resize(sl.n_images);
    uint32_t o = 0;
    for (size_t r = 0; r < nr; ++r) {
      starts[r] = o;
      for (uint32_t i = 0; i < sl.reqs[r].n; ++i) img_req[o + i] = static_cast<uint32_t>(r);
      o += sl.reqs[r].n;
    }
    // every hit names one of this step's 8 n queries; anything else is a device fault
    for (uint64_t h = 0; h < total; ++h)
      if (hits[h].query >= 8u * sl.n_images) st = YPDQ_ERR_CUDA;
  }
  if (st == YPDQ_OK) {
    for (uint64_t h = 0; h < total; ++h) ++counts[img_req[hits[h].query >> 3]];
    std::vector<uint64_t> pos(nr + 1, 0);
    for (size_t r = 0; r < nr; ++r) pos[r + 1] = pos[r] + counts[r];
    sorted.resize(total);
    std::vector<uint64_t> fill(pos.begin(), pos.end() - 1);
    for (uint64_t h = 0; h < total; ++h) {
      const uint32_t r = img_req[hits[h].query >> 3];
      ypdq_hit x = hits[h];
      x.query -= 8 * starts[r];
      sorted[fill[r]++] = x;
    }
    for (size_t r = 0; r < nr; ++r) {
      Request& rq = sl.reqs[r];
      ypdq_hit* b = sorted.data() + pos[r];
      std::sort(b, b + counts[r], hit_order);
      const uint64_t m = std::min<uint64_t>(counts[r], rq.cap);
      if (m) std::memcpy(rq.hits, b, m * sizeof(ypdq_hit));
      if (rq.hashes) std::memcpy(rq.hashes, sl.h_hashes + size_t(starts[r]) * 256, size_t(rq.n) * 256);
      if (rq.quality) std::memcpy(rq.quality, sl.h_quality + size_t(starts[r]) * 8, size_t(rq.n) * 32);
    }
  }
  const Clock::time_point now = Clock::now();
  std::lock_guard<std::mutex> lk(S->mu);
  for (size_t r = 0; r < nr; ++r) {
    const Request& rq = sl.reqs[r];
    ypdq_completion c{};
    c.request_id = rq.id;
    c.user_tag = rq.tag;
    c.n_images = rq.n;
    c.step = sl.step;
    c.n_hits = counts[r];
    c.status = st != YPDQ_OK ? st : (counts[r] > rq.cap ? YPDQ_ERR_OVERFLOW : YPDQ_OK);
    c.latency_us = std::chrono::duration<double, std::micro>(now - rq.t_submit).count();
    S->completions.push_back(c);
    S->latencies.push_back(c.latency_us);
    ++S->completed;
    S->images_completed += rq.n;
    S->hits_completed += counts[r];
    --S->outstanding;
  }
  if (rescanned) ++S->rescans;
  S->cv_done.notify_all();
}

void worker_main(ypdq_server* S) {
  cudaSetDevice(S->ctx->device);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    // admit waiting requests into every free slot, oldest first
    while (!S->free_slots.empty() && !S->pending.empty()) {
      const int si = S->free_slots.back();
      S->free_slots.pop_back();
      Slot& sl = S->slots[si];
      sl.reqs.clear();
      uint32_t n = 0;
      while (!S->pending.empty() && n + S->pending.front().n <= S->max_step) {
        n += S->pending.front().n;
        sl.reqs.push_back(S->pending.front());
        S->pending.pop_front();
      }
      S->pending_images -= n;
      sl.n_images = n;
      sl.step = S->next_step++;
      sl.bucket = 0;
      while (S->buckets[sl.bucket].images < n) ++sl.bucket;
      ++S->buckets[sl.bucket].steps;
      ++S->steps;
      S->step_images += n;
      S->inflight.push_back(si);
      lk.unlock();
      sl.launch_status = launch_step(S, sl);
      lk.lock();
    }
    if (!S->inflight.empty()) {
      const int si = S->inflight.front();
      Slot& sl = S->slots[si];
      const bool slot_free = !S->free_slots.empty();
      lk.unlock();
      cudaError_t q = sl.launch_status == YPDQ_OK ? cudaEventQuery(sl.done) : cudaSuccess;
      if (q == cudaErrorNotReady) {
        if (!slot_free) {
          q = cudaEventSynchronize(sl.done);
        } else {
          // a slot is free: watch for both the step and new arrivals
          const uint64_t seen = S->arrivals.load(std::memory_order_acquire);
          const Clock::time_point t0 = Clock::now();
          while ((q = cudaEventQuery(sl.done)) == cudaErrorNotReady &&
                 S->arrivals.load(std::memory_order_acquire) == seen &&
                 Clock::now() - t0 < std::chrono::microseconds(500))
            std::this_thread::yield();
        }
      }
      if (q == cudaErrorNotReady) {
        lk.lock();
        continue;
      }
      finish_step(S, sl, q);
      lk.lock();
      S->inflight.pop_front();
      S->free_slots.push_back(si);
      continue;
    }
    if (S->stop && S->pending.empty()) break;
    S->cv_work.wait(lk, [S] { return S->stop || !S->pending.empty(); });
  }
}

void release(ypdq_server* S) {
  for (Slot& sl : S->slots) {
    for (cudaGraphExec_t g : sl.exec)
      if (g) cudaGraphExecDestroy(g);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.stream) cudaStreamDestroy(sl.stream);
    cudaFree(sl.d_images);
    cudaFree(sl.d_hashes);
    cudaFree(sl.d_quality);
    cudaFree(sl.d_hits);
    cudaFree(sl.d_jarosz);
    cudaFree(sl.d_hdr);
    cudaFreeHost(sl.h_hdr);
    cudaFreeHost(sl.h_hits);
    cudaFreeHost(sl.h_hashes);
    cudaFreeHost(sl.h_quality);
  }
  delete S;
}

ypdq_status alloc_slot(ypdq_server* S, Slot& sl) {
  const uint32_t B = S->cfg.max_step_images;
  CK(cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking), "slot stream");
  CK(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming), "slot event");
  CK(cudaMalloc(&sl.d_images, size_t(B) * S->image_bytes), "cudaMalloc(slot images)");
  CK(cudaMalloc(&sl.d_hashes, size_t(B) * 256), "cudaMalloc(slot hashes)");
  CK(cudaMalloc(&sl.d_quality, size_t(B) * 32), "cudaMalloc(slot quality)");
  CK(cudaMalloc(&sl.d_hits, S->cfg.step_hit_capacity * sizeof(ypdq_hit)), "cudaMalloc(slot hits)");
  if (S->cfg.dct_precision == YPDQ_COMPRESS_JAROSZ)
    CK(cudaMalloc(&sl.d_jarosz, jarosz_scratch_bytes(B)), "cudaMalloc(slot jarosz planes)");
  CK(cudaMalloc(&sl.d_hdr, sizeof(StepHeader)), "cudaMalloc(slot header)");
  CK(cudaMallocHost(&sl.h_hdr, sizeof(StepHeader)), "cudaMallocHost(slot header)");
  CK(cudaMallocHost(&sl.h_hits, S->cfg.step_hit_capacity * sizeof(ypdq_hit)), "cudaMallocHost(slot hits)");
  CK(cudaMallocHost(&sl.h_hashes, size_t(B) * 256), "cudaMallocHost(slot hashes)");
  CK(cudaMallocHost(&sl.h_quality, size_t(B) * 32), "cudaMallocHost(slot quality)");
  std::memset(sl.h_hdr, 0, sizeof(StepHeader));
  // defined pixels for the autotuner's replays (any content times the same)
  CK(cudaMemsetAsync(sl.d_images, 0, size_t(B) * S->image_bytes, sl.stream), "clear slot images");
  CK(cudaMemsetAsync(sl.d_hdr, 0, sizeof(StepHeader), sl.stream), "clear slot header");
  CK(cudaStreamSynchronize(sl.stream), "slot setup");
  sl.exec.assign(S->buckets.size(), nullptr);
  return YPDQ_OK;
}

// Median time of `reps` replays of one bucket with a full batch, on slot 0.
ypdq_status time_bucket(ypdq_server* S, const Bucket& b, float* ms) {
  Slot& sl = S->slots[0];
  cudaGraphExec_t g = nullptr;
  ypdq_status st = capture_bucket(S, sl, b, &g);
  if (st) return st;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  sl.h_hdr->n_images = b.images;
  sl.h_hdr->n_queries = 8 * b.images;
  std::vector<float> t;
  cudaError_t e = cudaGraphLaunch(g, sl.stream);  // warm-up
  for (int r = 0; r < 3 && e == cudaSuccess; ++r) {
    e = cudaEventRecord(e0, sl.stream);
    if (e == cudaSuccess) e = cudaGraphLaunch(g, sl.stream);
    if (e == cudaSuccess) e = cudaEventRecord(e1, sl.stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float x = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&x, e0, e1);
    t.push_back(x);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(sl.stream);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaGraphExecDestroy(g);
  CK(e, "autotune replay");
  if (sl.h_hdr->err) return fail(YPDQ_ERR_TIMEOUT, "autotune: a kernel wait gave up");
  std::sort(t.begin(), t.end());
  *ms = t[t.size() / 2];
  return YPDQ_OK;
}

// Picks the scan kernel and pass width per bucket by timing, then the largest bucket kept.
ypdq_status autotune(ypdq_server* S) {
  for (Bucket& b : S->buckets) {
    std::vector<Bucket> cand;
    const uint32_t nq = 8 * b.images;
    if (nq <= 64) cand.push_back(Bucket{b.images, YPDQ_SCAN_SIMT, 0, 0, 0.0f, 0});
    // the launcher's choice: at t <= 36 queries as A with three database rows per column (FP4,
    // one launch per 128 queries) up to 512 queries and FP4 triple passes of 720 past that;
    // above t = 36 queries as A (FP8) up to 128 queries, then one query per column
    cand.push_back(Bucket{b.images, YPDQ_SCAN_TC, 0, 0, 0.0f, 0});
    const uint32_t nq64 = (nq + 63u) & ~63u;
    for (uint32_t nt = 64; nt <= 256; nt *= 2)
      if (nt <= nq64 || nt == 64) cand.push_back(Bucket{b.images, YPDQ_SCAN_TC, nt, 0, 0.0f, 0});
    // FP8 pairs, passes of 512 queries (t <= 36)
    if (S->cfg.threshold <= 36 && nq > 128)
      cand.push_back(Bucket{b.images, YPDQ_SCAN_TC, 0, 256, 0.0f, 0});
    float best = 0.0f;
    for (Bucket& c : cand) {
      ypdq_status st = time_bucket(S, c, &c.ms);
      if (st) return st;
      if (best == 0.0f || c.ms < best) {
        best = c.ms;
        b.algo = c.algo;
        b.n_tile = c.n_tile;
        b.pair_n = c.pair_n;
        b.ms = c.ms;
      }
    }
  }
  if (S->cfg.target_step_ms > 0.0) {
    size_t keep = 1;
    for (size_t i = 1; i < S->buckets.size(); ++i)
      if (S->buckets[i].ms <= S->cfg.target_step_ms) keep = i + 1;
    S->buckets.resize(keep);
  }
  S->max_step = S->buckets.back().images;
  return YPDQ_OK;
}

}  // namespace

extern "C" {

ypdq_status ypdq_server_config_default(ypdq_server_config* cfg) {
  if (!cfg) return fail(YPDQ_ERR_INVALID, "cfg is NULL");
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->input_kind = YPDQ_INPUT_F32;
  cfg->dct_precision = YPDQ_DCT_FP32;
  cfg->semantics = YPDQ_DIHEDRAL_EXACT;
  cfg->threshold = 31;
  cfg->max_step_images = kDefaultStepImages;
  cfg->slots = kDefaultSlots;
  cfg->step_hit_capacity = kDefaultStepHits;
  return YPDQ_OK;
}

ypdq_status ypdq_server_create(ypdq_ctx* ctx, ypdq_db* db, const ypdq_server_config* cfg_in,
                               ypdq_server** out) {
  if (!ctx || !db || !cfg_in || !out) return fail(YPDQ_ERR_INVALID, "NULL argument");
  *out = nullptr;
  ypdq_server_config cfg = *cfg_in;
  if (image_bytes_of(cfg.input_kind) == 0)
    return fail(YPDQ_ERR_INVALID, "input_kind %d", cfg.input_kind);
  int dct_v = 0, sep_v = 0;
  if (cfg.dct_precision != YPDQ_COMPRESS_JAROSZ &&
      !parse_precision(cfg.dct_precision, &dct_v, &sep_v))
    return fail(YPDQ_ERR_INVALID, "dct_precision %d", cfg.dct_precision);
  if (cfg.semantics < YPDQ_DIHEDRAL_EXACT || cfg.semantics > YPDQ_DIHEDRAL_SCALAR)
    return fail(YPDQ_ERR_INVALID, "semantics %d", cfg.semantics);
  if (cfg.threshold > 256) return fail(YPDQ_ERR_INVALID, "threshold %u > 256", cfg.threshold);
  if (cfg.max_step_images == 0) cfg.max_step_images = kDefaultStepImages;
  if (cfg.max_step_images & (cfg.max_step_images - 1) || cfg.max_step_images > 32768)
    return fail(YPDQ_ERR_INVALID, "max_step_images %u: a power of two <= 32768",
                cfg.max_step_images);
  if (cfg.slots == 0) cfg.slots = kDefaultSlots;
  if (cfg.slots > 16) return fail(YPDQ_ERR_INVALID, "slots %u > 16", cfg.slots);
  if (cfg.step_hit_capacity == 0) cfg.step_hit_capacity = kDefaultStepHits;
  if (cfg.max_queued_images == 0) cfg.max_queued_images = 4ull * cfg.max_step_images;
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");

  ypdq_server* S = new ypdq_server();
  S->ctx = ctx;
  S->db = db;
  S->cfg = cfg;
  S->image_bytes = image_bytes_of(cfg.input_kind);
  semantics_masks(cfg.semantics, &S->row_mask, &S->col_mask);
  for (uint32_t b = 1; b <= cfg.max_step_images; b *= 2) {
    Bucket k;
    k.images = b;
    k.algo = auto_scan_algo(8 * b, cfg.threshold);  // the ypdq_scan AUTO rule
    S->buckets.push_back(k);
  }
  S->max_step = cfg.max_step_images;

  // admission by memory: as many slots as the budget holds, at most cfg.slots
  size_t free_b = 0, total_b = 0;
  cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
  if (e != cudaSuccess) {
    delete S;
    return cuda_fail(e, "cudaMemGetInfo");
  }
  const uint64_t budget = cfg.device_bytes ? cfg.device_bytes : free_b / 2;
  const uint64_t slot_bytes =
      uint64_t(cfg.max_step_images) * (S->image_bytes + 256 + 32) +
      cfg.step_hit_capacity * sizeof(ypdq_hit) + sizeof(StepHeader) +
      (cfg.dct_precision == YPDQ_COMPRESS_JAROSZ ? jarosz_scratch_bytes(cfg.max_step_images) : 0);
  const uint64_t fit = budget / slot_bytes;
  const uint32_t n_slots = static_cast<uint32_t>(std::min<uint64_t>(fit, cfg.slots));
  if (n_slots == 0) {
    delete S;
    return fail(YPDQ_ERR_NOMEM, "device budget %llu B holds no step slot of %llu B",
                (unsigned long long)budget, (unsigned long long)slot_bytes);
  }
  S->slots.resize(n_slots);
  ypdq_status st = YPDQ_OK;
  for (Slot& sl : S->slots)
    if ((st = alloc_slot(S, sl))) break;
  if (!st && cfg.autotune) st = autotune(S);
  for (Slot& sl : S->slots) {
    if (st) break;
    sl.exec.assign(S->buckets.size(), nullptr);
    for (size_t b = 0; b < S->buckets.size() && !st; ++b)
      st = capture_bucket(S, sl, S->buckets[b], &sl.exec[b]);
  }
  if (st) {
    release(S);
    return st;
  }
  for (int i = static_cast<int>(n_slots) - 1; i >= 0; --i) S->free_slots.push_back(i);
  S->window_start = Clock::now();
  S->worker = std::thread(worker_main, S);
  *out = S;
  return YPDQ_OK;
}

ypdq_status ypdq_server_submit(ypdq_server* S, const void* h_images, uint32_t n_images,
                               ypdq_hit* h_hits, uint64_t hit_capacity, uint8_t* h_hashes,
                               float* h_quality, uint64_t user_tag, uint64_t* request_id) {
  if (!S || !h_images || (hit_capacity && !h_hits)) return fail(YPDQ_ERR_INVALID, "NULL argument");
  Request r;
  r.images = static_cast<const uint8_t*>(h_images);
  r.n = n_images;
  r.hits = h_hits;
  r.cap = hit_capacity;
  r.hashes = h_hashes;
  r.quality = h_quality;
  r.tag = user_tag;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (n_images == 0 || n_images > S->max_step)
      return fail(YPDQ_ERR_INVALID, "n_images %u outside 1..%u", n_images, S->max_step);
    if (S->stop) return fail(YPDQ_ERR_INVALID, "server is stopping");
    ++S->submitted;
    if (S->pending_images + n_images > S->cfg.max_queued_images) {
      ++S->rejected;
      return fail(YPDQ_ERR_BUSY, "queue holds %llu images; limit %llu",
                  (unsigned long long)S->pending_images,
                  (unsigned long long)S->cfg.max_queued_images);
    }
    r.id = S->next_id++;
    r.t_submit = Clock::now();
    S->pending.push_back(r);
    S->pending_images += n_images;
    ++S->outstanding;
    if (request_id) *request_id = r.id;
  }
  S->arrivals.fetch_add(1, std::memory_order_release);
  S->cv_work.notify_one();
  return YPDQ_OK;
}

ypdq_status ypdq_server_poll(ypdq_server* S, ypdq_completion* out, uint32_t max, uint32_t* n_out,
                             int64_t timeout_us) {
  if (!S || !n_out || (max && !out)) return fail(YPDQ_ERR_INVALID, "NULL argument");
  std::unique_lock<std::mutex> lk(S->mu);
  auto ready = [S] { return !S->completions.empty() || S->outstanding == 0; };
  if (timeout_us < 0)
    S->cv_done.wait(lk, ready);
  else if (timeout_us > 0)
    S->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), ready);
  uint32_t n = 0;
  while (n < max && !S->completions.empty()) {
    out[n++] = S->completions.front();
    S->completions.pop_front();
  }
  *n_out = n;
  return YPDQ_OK;
}

ypdq_status ypdq_server_replay(ypdq_server* S, const void* h_pool, uint32_t pool_images,
                               const uint32_t* first, const uint32_t* n_images,
                               const uint64_t* arrival_ns, uint32_t n_requests,
                               uint64_t duration_ns, ypdq_hit* h_hits, uint64_t hit_capacity,
                               uint64_t* n_hits, uint64_t* n_submitted, uint64_t* n_rejected) {
  if (!S || !h_pool || !first || !n_images || !n_submitted || !n_rejected ||
      (hit_capacity && !h_hits))
    return fail(YPDQ_ERR_INVALID, "NULL argument");
  for (uint32_t i = 0; i < n_requests; ++i)
    if (n_images[i] == 0 || first[i] > pool_images || n_images[i] > pool_images - first[i])
      return fail(YPDQ_ERR_INVALID, "request %u: images %u..%u outside the pool of %u", i,
                  first[i], first[i] + n_images[i], pool_images);
  const uint8_t* pool = static_cast<const uint8_t*>(h_pool);
  std::vector<ypdq_completion> comp(256);
  uint64_t submitted = 0, rejected = 0, done = 0;
  const Clock::time_point t0 = Clock::now();
  auto elapsed_ns = [&] {
    return static_cast<uint64_t>(
        std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t0).count());
  };
  auto take = [&](int64_t timeout_us) -> ypdq_status {
    uint32_t got = 0;
    const ypdq_status st = ypdq_server_poll(S, comp.data(), static_cast<uint32_t>(comp.size()),
                                            &got, timeout_us);
    for (uint32_t c = 0; c < got; ++c)
      if (n_hits && comp[c].user_tag < n_requests) n_hits[comp[c].user_tag] = comp[c].n_hits;
    done += got;
    return st;
  };
  uint32_t i = 0;
  while (i < n_requests) {
    const uint64_t now = elapsed_ns();
    if (now >= duration_ns) break;
    if (arrival_ns && now < arrival_ns[i]) {
      // spin until the next arrival, taking completions meanwhile
      if (ypdq_status st = take(0)) return st;
      continue;
    }
    ypdq_hit* hits = hit_capacity ? h_hits + static_cast<uint64_t>(i) * hit_capacity : nullptr;
    const ypdq_status st =
        ypdq_server_submit(S, pool + static_cast<uint64_t>(first[i]) * S->image_bytes,
                           n_images[i], hits, hit_capacity, nullptr, nullptr, i, nullptr);
    if (st == YPDQ_OK) {
      ++submitted;
      ++i;
    } else if (st == YPDQ_ERR_BUSY) {
      ++rejected;
      if (arrival_ns) {
        ++i;  // an open-loop arrival that finds the queue full is lost
      } else if (ypdq_status st2 = take(200)) {  // closed loop: wait for room, then retry
        return st2;
      }
    } else {
      return st;
    }
    if (ypdq_status st2 = take(0)) return st2;
  }
  while (done < submitted)
    if (ypdq_status st = take(-1)) return st;
  *n_submitted = submitted;
  *n_rejected = rejected;
  return YPDQ_OK;
}

ypdq_status ypdq_server_get_stats(ypdq_server* S, ypdq_server_stats* o, int reset) {
  if (!S || !o) return fail(YPDQ_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lk(S->mu);
  std::memset(o, 0, sizeof(*o));
  o->submitted = S->submitted;
  o->rejected = S->rejected;
  o->completed = S->completed;
  o->images_completed = S->images_completed;
  o->hits_completed = S->hits_completed;
  o->steps = S->steps;
  o->rescans = S->rescans;
  o->queued_requests = static_cast<uint32_t>(S->pending.size());
  o->queued_images = static_cast<uint32_t>(S->pending_images);
  o->inflight_steps = static_cast<uint32_t>(S->inflight.size());
  o->slots = static_cast<uint32_t>(S->slots.size());
  o->max_step_images = S->max_step;
  o->mean_step_images = S->steps ? double(S->step_images) / double(S->steps) : 0.0;
  o->elapsed_s = std::chrono::duration<double>(Clock::now() - S->window_start).count();
  if (!S->latencies.empty()) {
    std::vector<double> v(S->latencies);
    std::sort(v.begin(), v.end());
    auto pct = [&v](double p) {
      size_t i = static_cast<size_t>(p * double(v.size() - 1) + 0.5);
      return v[std::min(i, v.size() - 1)];
    };
    o->p50_us = pct(0.50);
    o->p99_us = pct(0.99);
    o->max_us = v.back();
    double s = 0;
    for (double x : v) s += x;
    o->mean_us = s / double(v.size());
  }
  o->n_buckets = static_cast<uint32_t>(std::min<size_t>(S->buckets.size(), YPDQ_SERVER_MAX_BUCKETS));
  for (uint32_t i = 0; i < o->n_buckets; ++i) {
    o->bucket_images[i] = S->buckets[i].images;
    o->bucket_algo[i] = S->buckets[i].algo;
    const Bucket& b = S->buckets[i];
    const bool tc = b.algo == YPDQ_SCAN_TC;
    // tensor-core kernel: 0 one query per column, 1 FP8 pairs, 2 queries as A (FP8), 3 FP4
    // triples, 4 queries as A with three database rows per column (FP4); bucket_n_tile the
    // queries per pass or launch
    const uint32_t nq = 8 * b.images;
    const bool low_t = S->cfg.threshold <= 36;
    uint32_t kern = 0, width = 0;
    if (tc) {
      if (b.n_tile) {
        kern = 0, width = b.n_tile;
      } else if (b.pair_n == 256) {
        kern = 1, width = 512;
      } else if (low_t) {
        kern = nq <= 512 ? 4 : 3, width = nq <= 512 ? 128 : 3 * kPairFp4N;
      } else if (nq <= 128) {
        kern = 2, width = 128;
      } else {
        kern = 0, width = std::min(256u, (nq + 63u) & ~63u);
      }
    }
    o->bucket_kernel[i] = kern;
    o->bucket_n_tile[i] = width;
    o->bucket_ms[i] = S->buckets[i].ms;
    o->bucket_steps[i] = S->buckets[i].steps;
  }
  if (reset) {
    S->submitted = S->rejected = S->completed = S->images_completed = 0;
    S->hits_completed = S->steps = S->rescans = S->step_images = 0;
    S->latencies.clear();
    for (Bucket& b : S->buckets) b.steps = 0;
    S->window_start = Clock::now();
  }
  return YPDQ_OK;
}

ypdq_status ypdq_server_destroy(ypdq_server* S) {
  if (!S) return fail(YPDQ_ERR_INVALID, "server is NULL");
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  if (S->worker.joinable()) S->worker.join();
  cudaSetDevice(S->ctx->device);
  release(S);
  return YPDQ_OK;
}

}  // extern "C"
