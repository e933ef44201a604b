/*
 * ypdq.h -- batched, device-resident C interface of the GB300 PDQ library.
 *
 * Plain pointers and sizes only. Device pointers are marked d_*; host pointers h_*.
 * Every call takes a CUDA stream (ypdq_stream_t is layout-compatible with cudaStream_t;
 * NULL means the legacy default stream). Calls are asynchronous on that stream unless
 * their comment says otherwise. Every call returns a ypdq_status. The _host calls are
 * the exceptions: they copy from and to host memory and block until the result is there.
 *
 * The reference (yume-pdq) has no batched or device API. Each entry point below replaces
 * a per-image or per-batch reference item, cited beside it:
 *
 *   ypdq_hash_batch   Kernel::{jarosz_compress,dct2d,sum_of_gradients,quantize} driven by
 *                     hash_get_threshold (src/lib.rs:427-455), plus visit_dihedrals
 *                     (src/lib.rs:358-420), over n images per launch.
 *   ypdq_dihedrals_batch  visit_dihedrals (src/lib.rs:358-420) on given PDQF matrices.
 *   ypdq_scan         PDQMatcher::find of CpuMatcher (src/matching/mod.rs:336-362) and of
 *                     VulkanMatcher (src/matching/vulkan.rs:408-472), returning every hit
 *                     with its distance instead of a callback or the first hit.
 *                     With capacity 0 it is PDQMatcher::scan (src/matching/mod.rs:94-102,
 *                     232-257): the count alone says whether any row matched.
 *   ypdq_db_*         VulkanVectorDatabase (src/matching/vulkan.rs:40-65).
 *   ypdq_screen_host  the hash + 8-dihedral match loop of examples/end_to_end.rs:68-140,
 *                     as one call from host buffers.
 *   ypdq_server_*     the CLI's two-thread read -> hash -> write loop (`pipe`,
 *                     src/main.rs:391-836, 1091-1304), as a continuous-batching service
 *                     that hashes and matches requests of any image count.
 */
#ifndef YPDQ_GB300_H
#define YPDQ_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *ypdq_stream_t;
typedef struct ypdq_ctx ypdq_ctx;
typedef struct ypdq_db ypdq_db;

typedef enum {
  YPDQ_OK = 0,
  YPDQ_ERR_INVALID = 1,   /* bad argument: NULL where not allowed, size or enum out of range */
  YPDQ_ERR_ALIGN = 2,     /* a pointer is not 16-byte aligned where the call requires it */
  YPDQ_ERR_CUDA = 3,      /* a CUDA runtime call failed; ypdq_last_error() has the text */
  YPDQ_ERR_NOMEM = 4,     /* device or pinned-host allocation failed */
  YPDQ_ERR_OVERFLOW = 5,  /* more hits than capacity; the count holds the true total */
  YPDQ_ERR_TIMEOUT = 6,   /* a device-side wait ran past its limit and the kernel gave up */
  YPDQ_ERR_UNSUPPORTED = 7,
  YPDQ_ERR_BUSY = 8       /* the server's request queue is full; submit again later */
} ypdq_status;

/*
 * Input pixel format of 512x512 images, row-major, values 0..255. RGB8 (3 bytes per pixel)
 * and RGBA8 (4 bytes; alpha ignored) are converted to luma inside the hash kernel exactly as
 * yume-pdq's Kernel::cvt_rgb8_to_luma8f / cvt_rgba8_to_luma8f do (src/kernel/mod.rs:303-340,
 * ITU-R BT.601, src/kernel/constants.rs:23), the conversion the CLI applies to rgb8/rgba8
 * frames (src/main.rs:517-606).
 */
typedef enum {
  YPDQ_INPUT_F32 = 0,
  YPDQ_INPUT_U8 = 1,
  YPDQ_INPUT_RGB8 = 2,
  YPDQ_INPUT_RGBA8 = 3
} ypdq_input_kind;

/* DCT arithmetic. FP32 reproduces yume-pdq's scalar f32 kernel bit for bit. */
typedef enum {
  YPDQ_DCT_FP32 = 0,      /* SIMT f32, no fused multiply-add, reference operation order */
  YPDQ_DCT_TF32 = 1,      /* tensor cores, TF32 inputs, f32 accumulate */
  YPDQ_DCT_BF16X3 = 2     /* tensor cores, split bf16 (hi*hi + hi*lo + lo*hi), f32 accumulate */
} ypdq_dct_precision;

/*
 * OR'd into a dct_precision argument: compute the 512 -> 127 compress separably,
 * out = (c^T X c) / 81 with c = (0,1,2,3,2,1,0), instead of the reference's 27-tap order.
 * Exact integer sums for u8 input (one rounding, the final scale); it drops the reference
 * table's two subnormal taps (~1e-40). Not bit-exact with yume-pdq; a fast path for callers
 * within the stated coefficient tolerance.
 */
#define YPDQ_COMPRESS_SEPARABLE 0x100

/*
 * Passed as the whole dct_precision of ypdq_hash_batch: yume-pdq's ReferenceKernel<f32>, the
 * pdqhash-faithful kernel (src/kernel/mod.rs:690-820, src/kernel/ref.rs). Its compress runs
 * the full Jarosz filter (two box passes of window 3 along rows and columns of the whole
 * 512x512 image, running sums in f32) and samples it; its DCT sums each output in one
 * sequential accumulator. Bit-exact with that kernel for finite inputs. Slower (four passes
 * over the image through two f32 planes per image; the context keeps up to 4 GiB of
 * scratch for chunks of 2,048 images, and each server slot 2 MiB per image of its step).
 * Accepted by ypdq_hash_batch, ypdq_screen_host and ypdq_server_config.dct_precision.
 */
#define YPDQ_COMPRESS_JAROSZ 0x200

/*
 * Sign conventions of the dihedral derivation. yume-pdq's kernels disagree:
 *   EXACT  = Avx512F32Kernel: negate rows 0,2,..,14 and columns 0,2,..,14, which is the
 *            sign pattern of a real flip/flop of the image (src/kernel/x86.rs:989-1079).
 *   AVX2   = Avx2F32Kernel: rows 0,2,..,14 but columns 0,2,4,6 only
 *            (src/kernel/x86.rs:285-378).
 *   SCALAR = trait default used by DefaultKernel / ReferenceKernel: rows 1,3,..,15,
 *            columns 0,2,..,14 (src/kernel/mod.rs:345-406).
 */
typedef enum {
  YPDQ_DIHEDRAL_EXACT = 0,
  YPDQ_DIHEDRAL_AVX2 = 1,
  YPDQ_DIHEDRAL_SCALAR = 2
} ypdq_dihedral_semantics;

/* The order of the 8 hashes per image in every batched output: slot 0 is the image,
 * slots 1..7 the derived dihedrals in yume-pdq's visit order (src/lib.rs:391-419). */
#define YPDQ_SLOT_NORMAL 0
#define YPDQ_SLOT_FLOPPED 1
#define YPDQ_SLOT_ROTATED_180 2
#define YPDQ_SLOT_FLIPPED 3
#define YPDQ_SLOT_ROTATED_90_FLOPPED 4
#define YPDQ_SLOT_ROTATED_270 5
#define YPDQ_SLOT_FLOPPED_ROTATED_270 6
#define YPDQ_SLOT_ROTATED_90 7

/* One match: database row, query number and Hamming distance. 16 bytes. */
typedef struct {
  uint64_t index;
  uint32_t query;
  uint32_t distance;
} ypdq_hit;

/* Scan algorithms (all exact, all return the same hit set). */
typedef enum {
  YPDQ_SCAN_AUTO = 0,   /* pick by query count */
  YPDQ_SCAN_SIMT = 1,   /* XOR + popcount, one row per thread */
  YPDQ_SCAN_B1MMA = 2,  /* legacy binary MMA (mma.sync .b1 .xor.popc) */
  YPDQ_SCAN_TC = 3,     /* tcgen05 tensor cores on +-1 vectors: at threshold <= 36 block-scaled
                           FP4 (e2m1) on the first 126 bits, up to 512 queries with three
                           database rows per accumulator column (launches of 128 queries),
                           past that three queries per column (passes of 720); above 36 FP8
                           (dot = 256 - 2 d) */
  YPDQ_SCAN_TC_FP4 = 4, /* the FP4 forms of YPDQ_SCAN_TC at threshold <= 36 (the same choice
                           between them); above that the same as YPDQ_SCAN_TC */
  YPDQ_SCAN_TC_FP8 = 5  /* tcgen05 with FP8 operands at every threshold: at threshold <= 36
                           two queries per accumulator column (passes of 512) past 256
                           queries and one per column (passes of up to 256) otherwise; above
                           36 the same as YPDQ_SCAN_TC */
} ypdq_scan_algo;

/* ------------------------------------------------------------------ context */

/* Create a context on CUDA device `device` (it becomes current on the calling thread). */
ypdq_status ypdq_ctx_create(int device, ypdq_ctx **out);
ypdq_status ypdq_ctx_destroy(ypdq_ctx *ctx);
/* Text of the last error on this thread. */
const char *ypdq_last_error(void);
/* Sticky device-side error flags (timeouts) raised by kernels of this context; clears them.
 * Blocks until the device is idle. */
ypdq_status ypdq_check_device_errors(ypdq_ctx *ctx);
/*
 * Longest time a barrier wait inside the tensor-core scan kernels may take (default 4 s;
 * 0 restores the default; at most 60 s), for scans launched afterwards by any context and
 * by ypdq_screen_noalloc. A kernel whose wait runs out stops, sets the context's sticky
 * timeout flag and returns; ypdq_stream_sync / ypdq_check_device_errors then report
 * YPDQ_ERR_TIMEOUT (ypdq_screen_noalloc: *d_count = UINT64_MAX) and the context stays usable.
 */
ypdq_status ypdq_set_scan_wait_limit(uint64_t ns);
/*
 * Testing the timeout path: the next n tensor-core scan launches (any context) issue no
 * database copies, so their other roles wait until the wait limit and give up as above.
 * Nothing faults and no wait is unbounded. 0 cancels.
 */
ypdq_status ypdq_debug_stall_scans(int n);

/* Number of SMs and the hash kernel's resident CTAs per SM (for sizing batches). */
ypdq_status ypdq_device_info(ypdq_ctx *ctx, int *num_sms, int *hash_ctas_per_sm);
/* CTAs per SM the hash kernel of this input kind and DCT precision runs with (its grid is
 * that many per SM, persistent over the images). */
ypdq_status ypdq_hash_occupancy(ypdq_ctx *ctx, int input_kind, int dct_precision,
                                int *ctas_per_sm);

/* ------------------------------------------------------------------ hashing */

/*
 * Hash n images and derive their dihedrals.
 *   d_images      n * 512 * 512 f32 or u8, 16-byte aligned.
 *   d_hashes      n * 8 * 32 bytes (slot order above), or NULL.
 *   d_quality     n * 8 f32, or NULL.
 *   d_thresholds  n * 8 f32 (slot 0: the median; others as yume-pdq passes them), or NULL.
 *   d_pdqf        n * pdqf_slots * 256 f32, or NULL. pdqf_slots is 1 (the image's PDQF)
 *                 or 8 (every slot's matrix as the reference's buffer holds it).
 *   d_buf1        n * 127 * 128 f32 compressed images (row stride 128), or NULL.
 */
ypdq_status ypdq_hash_batch(ypdq_ctx *ctx, const void *d_images, int64_t n, int input_kind,
                            int dct_precision, int semantics, uint8_t *d_hashes,
                            float *d_quality, float *d_thresholds, float *d_pdqf,
                            int pdqf_slots, float *d_buf1, ypdq_stream_t stream);

/*
 * Dihedrals of n given PDQF matrices (n * 256 f32) with their thresholds (n f32, the
 * value passed to visit_dihedrals). Outputs as in ypdq_hash_batch, 8 slots per matrix;
 * slot 0 is the input quantized at the given threshold. With d_thresholds NULL, slot 0
 * uses the exact median, which makes slot 0 the reference's Kernel::quantize
 * (src/kernel/mod.rs:595-608).
 */
ypdq_status ypdq_dihedrals_batch(ypdq_ctx *ctx, const float *d_pdqf, const float *d_thresholds,
                                 int64_t n, int semantics, uint8_t *d_hashes, float *d_quality,
                                 float *d_thresholds_out, float *d_pdqf_out,
                                 ypdq_stream_t stream);

/* --------------------------------------------------------- per-stage calls */

/*
 * The Kernel trait's per-image methods (src/kernel/mod.rs:268-497) on n items per call, on
 * the device, bit for bit with yume-pdq's f32 implementations. ypdq_hash_batch fuses these
 * stages; the calls below serve callers that run them one at a time, as the reference's
 * pipeline functions (src/lib.rs:427-455) do. Kernel::quantize is ypdq_dihedrals_batch with
 * d_thresholds NULL (slot 0); Kernel::jarosz_compress is ypdq_hash_batch's d_buf1 output.
 */

/* Kernel::dct2d (src/kernel/mod.rs:484; DefaultKernel::dct2d_impl :543-574): n compressed
 * buffers of 127 rows of `stride` f32 each (the first 127 columns are read; stride >= 127,
 * 128 for the reference's padded Buffer1), consecutive, -> n x 16 x 16 f32 PDQF. */
ypdq_status ypdq_dct2d_batch(ypdq_ctx *ctx, const float *d_buf1, int64_t n, int stride,
                             float *d_pdqf, ypdq_stream_t stream);

/* Kernel::sum_of_gradients (src/kernel/mod.rs:469; DefaultKernel :617-642): the quality
 * numerator of n PDQF matrices (n x 256 f32) -> n f32. Kernel::adjust_quality is then
 * min(x / 180, 1). */
ypdq_status ypdq_sum_of_gradients_batch(ypdq_ctx *ctx, const float *d_pdqf, int64_t n,
                                        float *d_out, ypdq_stream_t stream);

typedef enum {
  YPDQ_PDQF_T = 0,                    /* Kernel::pdqf_t (src/kernel/mod.rs:345-361) */
  YPDQ_PDQF_NEGATE_ALT_COLS = 1,      /* Kernel::pdqf_negate_alt_cols::<NEGATE> (:368-383) */
  YPDQ_PDQF_NEGATE_ALT_ROWS = 2,      /* Kernel::pdqf_negate_alt_rows::<NEGATE> (:391-406) */
  YPDQ_PDQF_NEGATE_OFF_DIAGONALS = 3  /* Kernel::pdqf_negate_off_diagonals (:413-427) */
} ypdq_pdqf_op;

/*
 * A PDQF transform, in place on n matrices (n x 256 f32), as the kernel of `semantics`
 * implements it; `negate` is the method's NEGATE parameter. yume-pdq's kernels differ:
 *   NEGATE_ALT_ROWS  SCALAR (trait default): rows 0,2,..,14 (negate 0) or 1,3,..,15
 *                    (negate 1); AVX2 and EXACT (x86.rs:285-327, 989-1024): the other rows.
 *   NEGATE_ALT_COLS  SCALAR and EXACT (x86.rs:1026-1079): columns 0,2,..,14 (negate 0) or
 *                    1,3,..,15; AVX2 (x86.rs:330-378): the same among columns 0..7 only.
 *   T and NEGATE_OFF_DIAGONALS are the same in every kernel; negate is ignored.
 */
ypdq_status ypdq_pdqf_transform_batch(ypdq_ctx *ctx, float *d_pdqf, int64_t n, int op,
                                      int negate, int semantics, ypdq_stream_t stream);

/* Kernel::cvt_rgb8_to_luma8f / cvt_rgba8_to_luma8f (src/kernel/mod.rs:303-340): n pixels
 * of `channels` bytes (3: RGB8, 4: RGBA8, alpha ignored) -> n f32 luma values
 * (r_coeff r + g_coeff g) + b_coeff b, each product and sum rounded to f32. The reference
 * passes the BT.601 coefficients (src/kernel/constants.rs:23). */
ypdq_status ypdq_cvt_luma8f(ypdq_ctx *ctx, const uint8_t *d_pixels, int64_t n_pixels,
                            int channels, float r_coeff, float g_coeff, float b_coeff,
                            float *d_out, ypdq_stream_t stream);

/* ----------------------------------------------------------------- matching */

/*
 * Exact linear scan: every (row, query) with popcount(row ^ query) <= threshold.
 *   d_rows     n_rows * 32 bytes (four little-endian u64 per row), 16-byte aligned.
 *   d_queries  n_queries * 32 bytes, 16-byte aligned.
 *   d_hits     capacity entries; hits land in no particular order.
 *   d_count    one u64, set (not added to) by the call: the total number of hits, which
 *              can exceed capacity; then only `capacity` hits are stored.
 * The call does not synchronise; read d_count after the stream completes.
 */
ypdq_status ypdq_scan(ypdq_ctx *ctx, const uint8_t *d_rows, uint64_t n_rows,
                      const uint8_t *d_queries, uint32_t n_queries, uint32_t threshold,
                      ypdq_hit *d_hits, uint64_t capacity, uint64_t *d_count, int algo,
                      ypdq_stream_t stream);

/* Sort n hits in place into the scalar matcher's visit order: index, then query. */
ypdq_status ypdq_sort_hits(ypdq_ctx *ctx, ypdq_hit *d_hits, uint64_t n, ypdq_stream_t stream);

/* ------------------------------------------------------------------ database */

/* Copy n_rows * 32 bytes of host rows into a device-resident database owned by ctx. */
ypdq_status ypdq_db_create(ypdq_ctx *ctx, const uint8_t *h_rows, uint64_t n_rows, ypdq_db **out);
/* Wrap caller-owned device rows (not copied, not freed). */
ypdq_status ypdq_db_wrap(ypdq_ctx *ctx, const uint8_t *d_rows, uint64_t n_rows, ypdq_db **out);
ypdq_status ypdq_db_destroy(ypdq_db *db);
ypdq_status ypdq_db_info(ypdq_db *db, const uint8_t **d_rows, uint64_t *n_rows);
/*
 * Database files: consecutive 32-byte rows, no header (yume-pdq's in-memory layout; its CPU
 * matcher's files pad the last 2,048-row batch by repeating the final row,
 * examples/end_to_end.rs:52-53, and load as-is). Any size, streamed through two pinned
 * staging buffers of chunk_bytes (0 -> 64 MiB) so that reading and copying overlap. The
 * load creates an owned database; YPDQ_ERR_INVALID if the file cannot be read or its size
 * is not a multiple of 32. Blocking.
 */
ypdq_status ypdq_db_load_file(ypdq_ctx *ctx, const char *path, uint64_t chunk_bytes,
                              ypdq_db **out);
ypdq_status ypdq_db_save_file(ypdq_db *db, const char *path, uint64_t chunk_bytes);

/*
 * Screen n host images against db: hash, derive 8 dihedrals, scan all 8n hashes at
 * `threshold`. Queries are numbered image * 8 + slot. Hits come back sorted by
 * (index, query), as the scalar matcher reports them. Copies images in and results out
 * inside the call and blocks until done.
 *   h_images     n * 512 * 512 f32 or u8 (pinned memory is fastest; any host memory works).
 *   h_hits       capacity entries; *n_hits gets the total (YPDQ_ERR_OVERFLOW if > capacity).
 *   h_hashes     n * 8 * 32 bytes, or NULL.  h_quality  n * 8 f32, or NULL.
 */
ypdq_status ypdq_screen_host(ypdq_ctx *ctx, ypdq_db *db, const void *h_images, int64_t n,
                             int input_kind, int dct_precision, int semantics,
                             uint32_t threshold, ypdq_hit *h_hits, uint64_t capacity,
                             uint64_t *n_hits, uint8_t *h_hashes, float *h_quality);

/*
 * The chunks ypdq_screen_host cuts n images into (host-only; no device or context needed).
 * The copy of each chunk overlaps the hash and scan of the one before. Chunks grow from one
 * granule of whole scan passes (64 images at threshold <= 36, where passes hold 512
 * queries; 32 images otherwise), in whole granules, as fast as the copies stay ahead of the compute
 * (estimated for a GB300 from the input kind, the hash kernel's fixed cost per chunk and
 * the scan of 8 queries per image against n_rows rows at `threshold`). Writes
 * bounds[0] = 0 < bounds[1] < ... < bounds[*n_chunks] = n (at most
 * YPDQ_MAX_SCREEN_CHUNKS + 1 entries).
 */
#define YPDQ_MAX_SCREEN_CHUNKS 32
ypdq_status ypdq_screen_plan(int64_t n, int input_kind, int dct_precision, uint64_t n_rows,
                             uint32_t threshold, int64_t *bounds, int *n_chunks);

/* --------------------------------------------------------- memory utilities */

ypdq_status ypdq_malloc_device(ypdq_ctx *ctx, size_t bytes, void **d_ptr);
ypdq_status ypdq_free_device(ypdq_ctx *ctx, void *d_ptr);
ypdq_status ypdq_malloc_host(ypdq_ctx *ctx, size_t bytes, void **h_ptr); /* pinned */
ypdq_status ypdq_free_host(ypdq_ctx *ctx, void *h_ptr);
/* kind: 0 host->device, 1 device->host, 2 device->device. Asynchronous on stream. */
ypdq_status ypdq_memcpy(ypdq_ctx *ctx, void *dst, const void *src, size_t bytes, int kind,
                        ypdq_stream_t stream);
ypdq_status ypdq_memset(ypdq_ctx *ctx, void *d_ptr, int value, size_t bytes, ypdq_stream_t stream);
ypdq_status ypdq_stream_create(ypdq_ctx *ctx, ypdq_stream_t *out);
ypdq_status ypdq_stream_destroy(ypdq_ctx *ctx, ypdq_stream_t stream);
ypdq_status ypdq_stream_sync(ypdq_ctx *ctx, ypdq_stream_t stream);

/* Events for timing on a stream (milliseconds between two recorded events). */
typedef struct CUevent_st *ypdq_event_t;
ypdq_status ypdq_event_create(ypdq_ctx *ctx, ypdq_event_t *out);
ypdq_status ypdq_event_destroy(ypdq_ctx *ctx, ypdq_event_t ev);
ypdq_status ypdq_event_record(ypdq_ctx *ctx, ypdq_event_t ev, ypdq_stream_t stream);
ypdq_status ypdq_event_elapsed_ms(ypdq_ctx *ctx, ypdq_event_t start, ypdq_event_t end, float *ms);

/* ------------------------------------------------- screening without allocation */

/*
 * Screen n device-resident images against device-resident rows without allocating.
 * This entry point has no counterpart in the reference. It is for callers that cannot call
 * cudaMalloc, such as code inside a framework that owns all device memory through its own
 * pool, or a latency-critical path where an allocation (which can synchronise the device)
 * is not allowed. It hashes the images (FP32, bit-exact), derives the 8 dihedrals, and
 * scans the 8n hashes (queries numbered image * 8 + slot) at `threshold`. Hits are
 * unsorted; *d_count gets the total, or UINT64_MAX if a device-side wait timed out.
 * The 8n hashes live in a fixed 1 MiB device array inside the library, so n is at most
 * 4096 (larger n returns YPDQ_ERR_INVALID) and every GPU that loads the library holds
 * that array until exit. All calls share the array: calls that overlap on the GPU race,
 * so order them. The first call on a device sets it up there (symbol address, DCT table,
 * kernel attributes); make that call before any stream capture. After cudaDeviceReset the
 * next call sets it up again in the new context. d_images and d_rows must be 16-byte
 * aligned, d_hits and d_count 8-byte aligned (YPDQ_ERR_ALIGN). Asynchronous on stream.
 */
ypdq_status ypdq_screen_noalloc(const void *d_images, int64_t n, int input_kind, int semantics,
                                const uint8_t *d_rows, uint64_t n_rows, uint32_t threshold,
                                ypdq_hit *d_hits, uint64_t capacity, uint64_t *d_count,
                                ypdq_stream_t stream);

/* ------------------------------------------------------------ serving loop */

/*
 * A continuous-batching screening service over one device-resident database. Each request
 * carries 1..max_step_images images; the server hashes them (8 dihedrals each) and matches
 * every hash exactly against the database, like ypdq_screen_host on that request alone.
 *
 * Device steps. A worker thread packs waiting requests, oldest first, into a device step
 * of at most max_step_images images and launches it as soon as a step slot is free. Each
 * slot owns the device memory of one step (images, hashes, hits) and its own stream, so
 * up to `slots` steps are on the device at once: the image copy of one step overlaps the
 * hash and scan of another. A step replays a CUDA graph captured for the smallest batch
 * bucket (a power of two) that holds its images; the graph reads the step's image count
 * from device memory, so one graph serves every count up to its bucket.
 *
 * Admission by memory. The slots are sized at creation from the device memory the server
 * may take (device_bytes), so requests join the device exactly as slots and their memory
 * free up. Requests wait in a host queue before that; the queue holds at most
 * max_queued_images images, and a submit beyond that returns YPDQ_ERR_BUSY.
 *
 * Results. A request's hits are sorted by (database index, query) with query numbers local
 * to the request (image i, slot s -> 8 i + s) and are identical to those of the same images
 * screened alone. Hits past the step's device capacity are recovered by an exact re-scan.
 */
typedef struct ypdq_server ypdq_server;

typedef struct {
  int input_kind;              /* ypdq_input_kind */
  int dct_precision;           /* ypdq_dct_precision */
  int semantics;               /* ypdq_dihedral_semantics */
  uint32_t threshold;          /* Hamming distance bound, <= 256 */
  uint32_t max_step_images;    /* largest batch bucket, a power of two; 0 -> 1024 */
  uint32_t slots;              /* device steps in flight at most; 0 -> 3 */
  uint64_t step_hit_capacity;  /* hits a step keeps on the device; 0 -> 1 << 20 */
  uint64_t device_bytes;       /* device memory for all slots; 0 -> half the free memory */
  uint64_t max_queued_images;  /* host queue bound in images; 0 -> 4 x max_step_images */
  int autotune;                /* nonzero: time each bucket's scan variants at creation
                                  and keep the fastest per bucket */
  double target_step_ms;       /* with autotune: largest bucket kept is the biggest whose
                                  step takes at most this long; 0 -> no bound */
} ypdq_server_config;

typedef struct {
  uint64_t request_id;
  uint64_t user_tag;
  int32_t status;      /* YPDQ_OK, YPDQ_ERR_OVERFLOW (more hits than hit_capacity: the first
                          hit_capacity in order were written), or the step's error */
  uint32_t n_images;
  uint64_t n_hits;     /* the request's true number of hits */
  uint64_t step;       /* sequence number of the device step that carried the request */
  double latency_us;   /* from ypdq_server_submit to the completion being posted */
} ypdq_completion;

#define YPDQ_SERVER_MAX_BUCKETS 16

typedef struct {
  uint64_t submitted, rejected, completed;
  uint64_t images_completed, hits_completed, steps, rescans;
  uint32_t queued_requests, queued_images, inflight_steps, slots;
  uint32_t max_step_images;
  double p50_us, p99_us, mean_us, max_us;  /* latency of the requests completed since reset */
  double mean_step_images;
  double elapsed_s;                         /* since creation or the last reset */
  uint32_t n_buckets;
  uint32_t bucket_images[YPDQ_SERVER_MAX_BUCKETS];
  int32_t bucket_algo[YPDQ_SERVER_MAX_BUCKETS];     /* ypdq_scan_algo the bucket's graph uses */
  uint32_t bucket_n_tile[YPDQ_SERVER_MAX_BUCKETS];  /* tensor-core queries per pass or launch
                                                       (0: SIMT) */
  float bucket_ms[YPDQ_SERVER_MAX_BUCKETS];         /* step time measured by the autotuner */
  uint64_t bucket_steps[YPDQ_SERVER_MAX_BUCKETS];   /* steps launched per bucket */
  uint32_t bucket_kernel[YPDQ_SERVER_MAX_BUCKETS];  /* tensor-core scan form: 0 one query per
                                                       accumulator column, 1 two per column,
                                                       2 queries as the MMA's A operand,
                                                       3 three per column, FP4 operands,
                                                       4 queries as A with three database
                                                       rows per column, FP4 operands */
} ypdq_server_stats;

/* Fills cfg with the defaults above (threshold 31, f32 input, FP32 DCT, exact semantics). */
ypdq_status ypdq_server_config_default(ypdq_server_config *cfg);
/* Creates the slots, captures the bucket graphs and starts the worker thread. The database
 * must outlive the server. */
ypdq_status ypdq_server_create(ypdq_ctx *ctx, ypdq_db *db, const ypdq_server_config *cfg,
                               ypdq_server **out);
/*
 * Queues one request. h_images (n_images x 512 x 512 of the configured input kind; pinned
 * memory copies fastest) must stay valid until the completion is polled. h_hits (hit_capacity
 * entries), h_hashes (n_images x 8 x 32 bytes) and h_quality (n_images x 8 floats) are written
 * before the completion is posted; each may be NULL. Returns YPDQ_ERR_BUSY (and counts a
 * rejection) when the queue is full, YPDQ_ERR_INVALID for n_images outside
 * 1..max_step_images. Thread-safe.
 */
ypdq_status ypdq_server_submit(ypdq_server *srv, const void *h_images, uint32_t n_images,
                               ypdq_hit *h_hits, uint64_t hit_capacity, uint8_t *h_hashes,
                               float *h_quality, uint64_t user_tag, uint64_t *request_id);
/* Takes up to max completions, waiting up to timeout_us (0: no wait, < 0: until at least one
 * is there or nothing is pending). Thread-safe. */
ypdq_status ypdq_server_poll(ypdq_server *srv, ypdq_completion *out, uint32_t max,
                             uint32_t *n_out, int64_t timeout_us);
/*
 * Load generator for measurement: submits requests from the calling thread (native, so no
 * interpreter pause of a caller delays an arrival) and takes their completions meanwhile.
 * Request i is images first[i] .. first[i] + n_images[i] - 1 of h_pool (pool_images images
 * of the configured input kind; pinned memory copies fastest). Requests go in index order,
 * request i arrival_ns[i] ns after the call starts (non-decreasing times; open loop: an
 * arrival that finds the queue full is lost and counted in *n_rejected), or,
 * with arrival_ns NULL, as soon as the queue has room (closed loop: a full queue is waited
 * for and counted). Submission stops after n_requests requests or duration_ns ns; the call
 * returns once every submitted request has completed. Request i's hits go to h_hits +
 * i * hit_capacity (NULL with hit_capacity 0: counts only) and its true hit count to
 * n_hits[i] (may be NULL). No other request of the server may be in flight meanwhile. The
 * server's statistics window (ypdq_server_get_stats) covers the replay.
 */
ypdq_status ypdq_server_replay(ypdq_server *srv, const void *h_pool, uint32_t pool_images,
                               const uint32_t *first, const uint32_t *n_images,
                               const uint64_t *arrival_ns, uint32_t n_requests,
                               uint64_t duration_ns, ypdq_hit *h_hits, uint64_t hit_capacity,
                               uint64_t *n_hits, uint64_t *n_submitted, uint64_t *n_rejected);
/* Latency percentiles, counters and the bucket table; reset != 0 starts a new window. */
ypdq_status ypdq_server_get_stats(ypdq_server *srv, ypdq_server_stats *out, int reset);
/* Finishes every queued and in-flight request, stops the worker and frees the slots.
 * Completions not yet polled are dropped. */
ypdq_status ypdq_server_destroy(ypdq_server *srv);

/* -------------------------------------------------------- synthetic workloads */

/*
 * Fill d_rows with n_rows pseudo-random 256-bit rows, each with exactly 128 set bits.
 * Row r depends only on (seed, first_row + r). Workload generator for benchmarks and
 * tests; it is not part of the hashing or matching path.
 */
ypdq_status ypdq_synth_rows(ypdq_ctx *ctx, uint8_t *d_rows, uint64_t n_rows, uint64_t first_row,
                            uint64_t seed, ypdq_stream_t stream);

/*
 * Clustered rows: global row g = first_row + r is a member of centre c = g /
 * members_per_centre, where centre c is row c of ypdq_synth_rows for the same seed (128 set
 * bits). The member flips d distinct bits of its centre, d ~ Binomial(flip_trials, 1/2)
 * (flip_trials <= 64; 40 gives a distance around 20). Row g depends only on (seed, g,
 * members_per_centre, flip_trials).
 */
ypdq_status ypdq_synth_clustered_rows(ypdq_ctx *ctx, uint8_t *d_rows, uint64_t n_rows,
                                      uint64_t first_row, uint64_t members_per_centre,
                                      uint32_t flip_trials, uint64_t seed, ypdq_stream_t stream);

/*
 * The dihedral sign convention (ypdq_dihedral_semantics) that the drop-in symbols of
 * yume_pdq.h use: what yume-pdq's smart_kernel() computes on this host in its default build
 * (src/kernel/mod.rs:79-176), i.e. AVX2 on an x86_64 CPU with AVX2 and FMA, SCALAR on any
 * other host, unless the environment variable YUME_PDQ_DIHEDRAL_SEMANTICS (exact | avx2 |
 * scalar) overrides it. Read once per process. Host-only; needs no device.
 */
ypdq_status ypdq_dropin_semantics(int *semantics);

/* The f32 DCT matrix (16 x 127) and tent weights (7 x 7) compiled into the library. */
ypdq_status ypdq_constants(float *h_dct16x127, float *h_tent7x7);

#ifdef __cplusplus
}
#endif

#endif /* YPDQ_GB300_H */
