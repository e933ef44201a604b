/*
 * ypdq_oracle.c -- CPU oracle for the yume-pdq hot path.
 *
 * TEST INFRASTRUCTURE ONLY. The tests and the CPU baseline of the benchmark load
 * this code as the reference for results. The product library never calls, links or
 * executes it.
 *
 * It is a plain-C restatement of yume-pdq's scalar path. Citations point into the
 * yume-pdq sources:
 *   - jarosz_compress   : DefaultKernel::jarosz_compress  src/kernel/mod.rs:644-666
 *   - dct2d             : DefaultKernel::dct2d_impl       src/kernel/mod.rs:543-574
 *   - sum_of_gradients  : DefaultKernel::sum_of_gradients src/kernel/mod.rs:617-642
 *   - adjust_quality    : DefaultKernel::adjust_quality   src/kernel/mod.rs:611-615 (divisor :257)
 *   - torben_median     : src/kernel/mod.rs:212-253
 *   - quantize          : DefaultKernel::quantize         src/kernel/mod.rs:595-608
 *   - threshold_2d_f32  : src/kernel/threshold.rs:37-119
 *   - hash_get_threshold: src/lib.rs:427-455
 *   - visit_dihedrals   : src/lib.rs:358-420; sign conventions src/kernel/mod.rs:345-427
 *                         (trait default), src/kernel/x86.rs:285-378 (AVX2),
 *                         src/kernel/x86.rs:989-1079 (AVX-512)
 *   - dct2d f64 twin    : ReferenceKernel<f64>::dct2d     src/kernel/mod.rs:838-864
 *   - scalar matcher    : CpuMatcher::find (u64 scalar)   src/matching/mod.rs:336-362
 *   - Avx2F32Kernel     : jarosz_compress_avx2 src/kernel/x86.rs:626-682, dct2d_impl
 *                         :100-281, quantize_impl :440-621, sign patterns :285-436;
 *                         restated lane by lane with fmaf for every fused multiply-add
 *
 * The f32 arithmetic keeps the reference's operation order: a multiply and then an
 * add, each rounded, with no fused multiply-add, because Rust does not contract a*b+c
 * (the Avx2F32Kernel restatement calls fmaf exactly where that kernel fuses).
 * Build this file with -ffp-contract=off.
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "ypdq_constants.h"

#define YPDQO_EXPORT __attribute__((visibility("default")))

static float DCT32[16 * 127];
static double DCT64[16 * 127];
static float TENT[49];
static int CONSTANTS_READY = 0;

static void init_constants(void) {
  if (CONSTANTS_READY) return;
  for (int i = 0; i < 16 * 127; i++) {
    uint32_t b = YPDQO_DCT_F32_BITS[i];
    uint64_t d = YPDQO_DCT_F64_BITS[i];
    memcpy(&DCT32[i], &b, 4);
    memcpy(&DCT64[i], &d, 8);
  }
  for (int i = 0; i < 49; i++) {
    uint32_t b = YPDQO_TENT_F32_BITS[i];
    memcpy(&TENT[i], &b, 4);
  }
  CONSTANTS_READY = 1;
}

YPDQO_EXPORT void ypdqo_init(void) { init_constants(); }

YPDQO_EXPORT void ypdqo_dct_matrix_f32(float* out) {
  init_constants();
  memcpy(out, DCT32, sizeof(DCT32));
}
YPDQO_EXPORT void ypdqo_dct_matrix_f64(double* out) {
  init_constants();
  memcpy(out, DCT64, sizeof(DCT64));
}
YPDQO_EXPORT void ypdqo_tent_weights(float* out) {
  init_constants();
  memcpy(out, TENT, sizeof(TENT));
}

/* 512x512 -> 127x127, all 7x7 taps in the reference order (di outer, dj inner). */
YPDQO_EXPORT void ypdqo_compress(const float* img, float* out /* 127*127 */) {
  init_constants();
  for (int oi = 0; oi < 127; oi++) {
    int in_i = YPDQO_CONV_OFFSET[oi] - YPDQO_TENT_OFFSET;
    for (int oj = 0; oj < 127; oj++) {
      int in_j = YPDQO_CONV_OFFSET[oj] - YPDQO_TENT_OFFSET;
      float sum = 0.0f;
      for (int di = 0; di < 7; di++)
        for (int dj = 0; dj < 7; dj++) {
          float p = TENT[di * 7 + dj] * img[(in_i + di) * 512 + (in_j + dj)];
          sum = sum + p;
        }
      out[oi * 127 + oj] = sum;
    }
  }
}

/* 127x127 -> 16x16 with four interleaved partial sums, as dct2d_impl does, for a given
 * 16 x 127 matrix D (the reference's tests also run it on test matrices). */
static void dct2d_with(const float* DCT32, const float* buf, float* pdqf) {
  float tmp[127];
  for (int k = 0; k < 16; k++) {
    for (int j = 0; j < 127; j++) {
      float s[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      for (int k2 = 0; k2 < 127; k2++) {
        float p = DCT32[k * 127 + k2] * buf[k2 * 127 + j];
        s[k2 & 3] = s[k2 & 3] + p;
      }
      tmp[j] = ((s[0] + s[1]) + s[2]) + s[3];
    }
    for (int j = 0; j < 16; j++) {
      float s[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      for (int m = 0; m < 127; m++) {
        float p = tmp[m] * DCT32[j * 127 + m];
        s[m & 3] = s[m & 3] + p;
      }
      pdqf[k * 16 + j] = ((s[0] + s[1]) + s[2]) + s[3];
    }
  }
}

YPDQO_EXPORT void ypdqo_dct2d(const float* buf /* 127*127 */, float* pdqf /* 256 */) {
  init_constants();
  dct2d_with(DCT32, buf, pdqf);
}
YPDQO_EXPORT void ypdqo_dct2d_matrix(const float* D /* 16*127 */, const float* buf /* 127*127 */,
                                     float* pdqf /* 256 */) {
  dct2d_with(D, buf, pdqf);
}

/* FP64 DCT (straight sums) on the f32 compress output, for coefficient-error reports. */
YPDQO_EXPORT void ypdqo_dct2d_f64(const float* buf /* 127*127 */, double* pdqf /* 256 */) {
  init_constants();
  double tmp[127];
  for (int i = 0; i < 16; i++) {
    for (int j = 0; j < 127; j++) {
      double s = 0.0;
      for (int k = 0; k < 127; k++) s += DCT64[i * 127 + k] * (double)buf[k * 127 + j];
      tmp[j] = s;
    }
    for (int j = 0; j < 16; j++) {
      double s = 0.0;
      for (int k = 0; k < 127; k++) s += tmp[k] * DCT64[j * 127 + k];
      pdqf[i * 16 + j] = s;
    }
  }
}

YPDQO_EXPORT float ypdqo_sum_of_gradients(const float* p) {
  float g = 0.0f;
  for (int i = 0; i < 15; i++)
    for (int j = 0; j < 16; j++) {
      float d = p[i * 16 + j] - p[(i + 1) * 16 + j];
      g = g + fabsf(d);
    }
  for (int i = 0; i < 16; i++)
    for (int j = 0; j < 15; j++) {
      float d = p[i * 16 + j] - p[i * 16 + j + 1];
      g = g + fabsf(d);
    }
  return g;
}

YPDQO_EXPORT float ypdqo_adjust_quality(float g) {
  float scaled = g / 180.0f;
  return scaled < 1.0f ? scaled : 1.0f;
}

/* Torben's median selection (returns the 128th smallest of 256 for finite inputs). */
YPDQO_EXPORT float ypdqo_torben_median(const float* m) {
  float mn = m[0], mx = m[0];
  for (int i = 1; i < 256; i++) {
    mn = fminf(mn, m[i]);
    mx = fmaxf(mx, m[i]);
  }
  const int half = (256 + 1) / 2;
  for (;;) {
    float guess = (mn + mx) / 2.0f;
    int less = 0, greater = 0, equal = 0;
    float maxlt = mn, mingt = mx;
    for (int i = 0; i < 256; i++) {
      float v = m[i];
      if (v < guess) {
        less++;
        if (v > maxlt) maxlt = v;
      } else if (v > guess) {
        greater++;
        if (v < mingt) mingt = v;
      } else {
        equal++;
      }
    }
    if (less <= half && greater <= half) {
      if (less >= half) return maxlt;
      if (less + equal >= half) return guess;
      return mingt;
    } else if (less > greater) {
      mx = maxlt;
    } else {
      mn = mingt;
    }
  }
}

/* Element k = 16*i + j goes to byte 31 - k/8, bit k%8 (src/kernel/mod.rs:605-606). */
YPDQO_EXPORT void ypdqo_threshold_2d(const float* p, uint8_t* out, float thr) {
  memset(out, 0, 32);
  for (int k = 0; k < 256; k++)
    if (p[k] > thr) out[31 - k / 8] |= (uint8_t)(1u << (k % 8));
}

YPDQO_EXPORT void ypdqo_quantize(const float* p, float* thr, uint8_t* out) {
  float med = ypdqo_torben_median(p);
  *thr = med;
  ypdqo_threshold_2d(p, out, med);
}

/* Whole single-image pipeline (src/lib.rs:427-455). buf127 and pdqf may be NULL. */
YPDQO_EXPORT float ypdqo_hash_get_threshold(const float* img, float* thr, uint8_t* out,
                                            float* buf127, float* pdqf) {
  float b[127 * 127];
  float p[256];
  ypdqo_compress(img, b);
  ypdqo_dct2d(b, p);
  float q = ypdqo_adjust_quality(ypdqo_sum_of_gradients(p));
  float t;
  ypdqo_quantize(p, &t, out);
  if (thr) *thr = t;
  if (buf127) memcpy(buf127, b, sizeof(b));
  if (pdqf) memcpy(pdqf, p, sizeof(p));
  return q;
}

/*
 * visit_dihedrals with parameterised sign conventions.
 *
 * row_mask bit i set: pdqf_negate_alt_rows::<true> negates row i.
 * col_mask bit j set: pdqf_negate_alt_cols::<false> negates column j.
 *   trait default (DefaultKernel, ReferenceKernel): rows 0xAAAA, cols 0x5555
 *   Avx2F32Kernel                                 : rows 0x5555, cols 0x0055
 *   Avx512F32Kernel (the true flip/flop pattern)  : rows 0x5555, cols 0x5555
 *
 * The seven variants come out in visit order: FLOPPED, ROTATED_180, FLIPPED,
 * ROTATED_90_FLOPPED, ROTATED_270, FLOPPED_ROTATED_270, ROTATED_90.
 * out_pdqf (may be NULL) receives each variant's matrix as the reference's buffer
 * holds it at the callback.
 */
static void neg_rows(float* p, uint32_t mask) {
  for (int i = 0; i < 16; i++)
    if (mask >> i & 1)
      for (int j = 0; j < 16; j++) p[i * 16 + j] = -p[i * 16 + j];
}
static void neg_cols(float* p, uint32_t mask) {
  for (int i = 0; i < 16; i++)
    for (int j = 0; j < 16; j++)
      if (mask >> j & 1) p[i * 16 + j] = -p[i * 16 + j];
}
static void transpose16(float* p) {
  for (int i = 0; i < 16; i++)
    for (int j = i + 1; j < 16; j++) {
      float t = p[i * 16 + j];
      p[i * 16 + j] = p[j * 16 + i];
      p[j * 16 + i] = t;
    }
}

typedef void (*quantize_fn)(const float* p, float* thr, uint8_t* out);

static void dihedrals_with(const float* pdqf_in, float threshold, uint32_t row_mask,
                           uint32_t col_mask, uint8_t* out_hashes, float* out_thr,
                           float* out_quality, float* out_pdqf, quantize_fn ypdqo_quantize) {
  float p[256];
  memcpy(p, pdqf_in, sizeof(p));
  float t_cols = threshold, t_rows = threshold, t_diag = threshold;
  int v = 0;
#define EMIT(thr)                                                   \
  do {                                                              \
    out_thr[v] = (thr);                                             \
    out_quality[v] = ypdqo_adjust_quality(ypdqo_sum_of_gradients(p)); \
    if (out_pdqf) memcpy(out_pdqf + v * 256, p, sizeof(p));          \
    v++;                                                            \
  } while (0)
  neg_cols(p, col_mask);
  ypdqo_quantize(p, &t_cols, out_hashes + v * 32);
  EMIT(t_cols); /* FLOPPED */
  neg_rows(p, row_mask);
  ypdqo_quantize(p, &t_diag, out_hashes + v * 32);
  EMIT(t_diag); /* ROTATED_180 */
  neg_cols(p, col_mask);
  ypdqo_quantize(p, &t_rows, out_hashes + v * 32);
  EMIT(t_rows); /* FLIPPED */
  neg_rows(p, row_mask);
  transpose16(p);
  ypdqo_threshold_2d(p, out_hashes + v * 32, threshold);
  EMIT(threshold); /* ROTATED_90_FLOPPED */
  neg_rows(p, row_mask);
  ypdqo_threshold_2d(p, out_hashes + v * 32, t_cols);
  EMIT(t_cols); /* ROTATED_270 */
  neg_cols(p, col_mask);
  ypdqo_threshold_2d(p, out_hashes + v * 32, t_diag);
  EMIT(t_diag); /* FLOPPED_ROTATED_270 */
  neg_rows(p, row_mask);
  ypdqo_threshold_2d(p, out_hashes + v * 32, t_rows);
  EMIT(t_rows); /* ROTATED_90 */
#undef EMIT
}

YPDQO_EXPORT void ypdqo_dihedrals(const float* pdqf_in, float threshold, uint32_t row_mask,
                                  uint32_t col_mask, uint8_t* out_hashes /* 7*32 */,
                                  float* out_thr /* 7 */, float* out_quality /* 7 */,
                                  float* out_pdqf /* 7*256 or NULL */) {
  dihedrals_with(pdqf_in, threshold, row_mask, col_mask, out_hashes, out_thr, out_quality,
                 out_pdqf, ypdqo_quantize);
}

/* ------------------------------------------------------------------ threads */

typedef void (*range_fn)(void* ctx, int64_t begin, int64_t end);
typedef struct {
  range_fn fn;
  void* ctx;
  int64_t begin, end;
} range_job;

static void* range_thread(void* arg) {
  range_job* j = (range_job*)arg;
  j->fn(j->ctx, j->begin, j->end);
  return NULL;
}

static void parallel_ranges(range_fn fn, void* ctx, int64_t n, int nthreads) {
  if (nthreads <= 1 || n <= 1) {
    fn(ctx, 0, n);
    return;
  }
  if (nthreads > 256) nthreads = 256;
  if ((int64_t)nthreads > n) nthreads = (int)n;
  pthread_t th[256];
  range_job jobs[256];
  for (int t = 0; t < nthreads; t++) {
    jobs[t].fn = fn;
    jobs[t].ctx = ctx;
    jobs[t].begin = n * t / nthreads;
    jobs[t].end = n * (t + 1) / nthreads;
  }
  for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, range_thread, &jobs[t]);
  range_thread(&jobs[0]);
  for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
}

/* ------------------------------------------------ batched hashing (baseline) */

typedef struct {
  const void* imgs;
  int is_u8;
  uint32_t row_mask, col_mask;
  uint8_t* hashes;   /* n * 8 * 32 */
  float* quality;    /* n * 8 */
  float* thresholds; /* n * 8 */
  float* pdqf;       /* n * 256 or NULL */
} hash_batch_ctx;

static void hash_batch_range(void* vctx, int64_t b, int64_t e) {
  hash_batch_ctx* c = (hash_batch_ctx*)vctx;
  float* img = NULL;
  if (c->is_u8) img = (float*)malloc(512 * 512 * sizeof(float));
  for (int64_t n = b; n < e; n++) {
    const float* src;
    if (c->is_u8) {
      const uint8_t* u = (const uint8_t*)c->imgs + n * 512 * 512;
      for (int i = 0; i < 512 * 512; i++) img[i] = (float)u[i];
      src = img;
    } else {
      src = (const float*)c->imgs + n * 512 * 512;
    }
    float p[256], t;
    float q = ypdqo_hash_get_threshold(src, &t, c->hashes + n * 256, NULL, p);
    c->quality[n * 8] = q;
    c->thresholds[n * 8] = t;
    if (c->pdqf) memcpy(c->pdqf + n * 256, p, sizeof(p));
    ypdqo_dihedrals(p, t, c->row_mask, c->col_mask, c->hashes + n * 256 + 32,
                    c->thresholds + n * 8 + 1, c->quality + n * 8 + 1, NULL);
  }
  free(img);
}

/* Hash n images and derive the seven dihedrals of each (slot 0 = the image itself). */
YPDQO_EXPORT void ypdqo_hash_batch(const void* imgs, int64_t n, int is_u8, uint32_t row_mask,
                                   uint32_t col_mask, uint8_t* hashes, float* quality,
                                   float* thresholds, float* pdqf, int nthreads) {
  init_constants();
  hash_batch_ctx c = {imgs, is_u8, row_mask, col_mask, hashes, quality, thresholds, pdqf};
  parallel_ranges(hash_batch_range, &c, n, nthreads);
}

/* ------------------------------------------------------------ scalar matcher */

typedef struct {
  uint64_t index;
  uint32_t query;
  uint32_t distance;
} ypdqo_hit;

static inline uint32_t dist256(const uint64_t* a, const uint64_t* b) {
  return (uint32_t)(__builtin_popcountll(a[0] ^ b[0]) + __builtin_popcountll(a[1] ^ b[1]) +
                    __builtin_popcountll(a[2] ^ b[2]) + __builtin_popcountll(a[3] ^ b[3]));
}

typedef struct {
  const uint64_t* db;
  const uint64_t* needles;
  int n_needles;
  uint32_t threshold;
  int nthreads;
  int64_t n_rows;
  ypdqo_hit** bufs;
  int64_t* counts;
  int64_t* caps;
} find_ctx;

static void push_hit(ypdqo_hit** buf, int64_t* cnt, int64_t* cap, int64_t r, int q,
                     uint32_t d) {
  if (*cnt == *cap) {
    *cap *= 2;
    *buf = (ypdqo_hit*)realloc(*buf, *cap * sizeof(ypdqo_hit));
  }
  (*buf)[*cnt].index = (uint64_t)r;
  (*buf)[*cnt].query = (uint32_t)q;
  (*buf)[*cnt].distance = d;
  (*cnt)++;
}

/* The scalar matcher's loop (src/matching/mod.rs:336-362): rows in order, each row loaded
 * once and compared with the needles in order, 8 at a time without branches; the rare
 * block holding a hit is then visited needle by needle, so hits come out in (row, needle)
 * order. */
static void find_range(void* vctx, int64_t b, int64_t e) {
  find_ctx* c = (find_ctx*)vctx;
  const int full = c->n_needles / 8 * 8;
  const uint32_t t_max = c->threshold;
  for (int64_t t = b; t < e; t++) {
    int64_t r0 = c->n_rows * t / c->nthreads, r1 = c->n_rows * (t + 1) / c->nthreads;
    int64_t cnt = 0, cap = 64;
    ypdqo_hit* buf = (ypdqo_hit*)malloc(cap * sizeof(ypdqo_hit));
    for (int64_t r = r0; r < r1; r++) {
      const uint64_t* row = c->db + r * 4;
      const uint64_t a0 = row[0], a1 = row[1], a2 = row[2], a3 = row[3];
      for (int q = 0; q < full; q += 8) {
        const uint64_t* n = c->needles + q * 4;
        uint32_t d[8], any = 0;
        for (int k = 0; k < 8; k++) {
          d[k] = (uint32_t)(__builtin_popcountll(a0 ^ n[4 * k]) +
                            __builtin_popcountll(a1 ^ n[4 * k + 1]) +
                            __builtin_popcountll(a2 ^ n[4 * k + 2]) +
                            __builtin_popcountll(a3 ^ n[4 * k + 3]));
          any |= (uint32_t)(d[k] <= t_max) << k;
        }
        if (any)
          for (int k = 0; k < 8; k++)
            if ((any >> k) & 1u) push_hit(&buf, &cnt, &cap, r, q + k, d[k]);
      }
      for (int q = full; q < c->n_needles; q++) {
        const uint32_t d = dist256(row, c->needles + q * 4);
        if (d <= t_max) push_hit(&buf, &cnt, &cap, r, q, d);
      }
    }
    c->bufs[t] = buf;
    c->counts[t] = cnt;
  }
}

/*
 * All (row, needle, distance) with popcount(row ^ needle) <= threshold, in the order
 * the scalar CpuMatcher::find visits them: rows ascending, then needles ascending.
 * Returns the total number of hits; writes at most cap of them.
 */
YPDQO_EXPORT int64_t ypdqo_find_all(const uint8_t* db, int64_t n_rows, const uint8_t* needles,
                                    int n_needles, uint32_t threshold, ypdqo_hit* out,
                                    int64_t cap, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  ypdqo_hit* bufs[256];
  int64_t counts[256];
  find_ctx c = {(const uint64_t*)db, (const uint64_t*)needles, n_needles, threshold,
                nthreads, n_rows, bufs, counts, NULL};
  parallel_ranges(find_range, &c, nthreads, nthreads);
  int64_t total = 0;
  for (int t = 0; t < nthreads; t++) {
    for (int64_t k = 0; k < counts[t]; k++) {
      if (total + k < cap) out[total + k] = bufs[t][k];
    }
    total += counts[t];
    free(bufs[t]);
  }
  return total;
}

/* Number of hits only (no storage), for timing the matcher without a callback. */
typedef struct {
  const uint64_t* db;
  const uint64_t* needles;
  int n_needles;
  uint32_t threshold;
  int64_t n_rows;
  int nthreads;
  int64_t* counts;
} count_ctx;

/* The scalar CpuMatcher's inner loop (src/matching/mod.rs:231-257): each database row is
 * loaded once and compared with the needles in fixed blocks of 8 (the matcher's batch of
 * needles, unrolled at compile time there as here), counting without branches. */
static inline int64_t count_block8(uint64_t a0, uint64_t a1, uint64_t a2, uint64_t a3,
                                   const uint64_t* n, uint32_t t) {
  int64_t c = 0;
  for (int k = 0; k < 8; k++) {
    const uint32_t d = (uint32_t)(__builtin_popcountll(a0 ^ n[4 * k]) +
                                  __builtin_popcountll(a1 ^ n[4 * k + 1]) +
                                  __builtin_popcountll(a2 ^ n[4 * k + 2]) +
                                  __builtin_popcountll(a3 ^ n[4 * k + 3]));
    c += d <= t;
  }
  return c;
}

static void count_range(void* vctx, int64_t b, int64_t e) {
  count_ctx* c = (count_ctx*)vctx;
  const int full = c->n_needles / 8 * 8;
  for (int64_t t = b; t < e; t++) {
    int64_t r0 = c->n_rows * t / c->nthreads, r1 = c->n_rows * (t + 1) / c->nthreads;
    int64_t cnt = 0;
    for (int64_t r = r0; r < r1; r++) {
      const uint64_t* row = c->db + r * 4;
      const uint64_t a0 = row[0], a1 = row[1], a2 = row[2], a3 = row[3];
      for (int q = 0; q < full; q += 8)
        cnt += count_block8(a0, a1, a2, a3, c->needles + q * 4, c->threshold);
      for (int q = full; q < c->n_needles; q++)
        cnt += dist256(row, c->needles + q * 4) <= c->threshold;
    }
    c->counts[t] = cnt;
  }
}

YPDQO_EXPORT int64_t ypdqo_count_all(const uint8_t* db, int64_t n_rows, const uint8_t* needles,
                                     int n_needles, uint32_t threshold, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  int64_t counts[256];
  count_ctx c = {(const uint64_t*)db, (const uint64_t*)needles, n_needles, threshold,
                 n_rows, nthreads, counts};
  parallel_ranges(count_range, &c, nthreads, nthreads);
  int64_t total = 0;
  for (int t = 0; t < nthreads; t++) total += counts[t];
  return total;
}

/* README "API Usage" known-answer input: a horizontal FM sine, generated in f32 with the
 * C library's sinf, in the same operation order as the README's Rust snippet
 * (README.md:305-330). */
YPDQO_EXPORT void ypdqo_fm_sine_image(float* out /* 512*512 */) {
  const float pi = 3.14159265358979323846f;
  float frequency = 4.0f;
  const float modulation = frequency / 512.0f;
  for (int i = 0; i < 512; i++)
    for (int j = 0; j < 512; j++) {
      frequency = frequency + modulation;
      float a = (float)j * 2.0f;
      a = a * pi;
      a = a * frequency;
      a = a / 512.0f;
      float v = sinf(a);
      float s = v * 127.0f;
      out[i * 512 + j] = s + 128.0f;
    }
}

/* ----------------------------------------------- synthetic rows (CPU twin) */

/* Same construction as the library's workload generator: a splitmix64 stream per row
 * (seeded by seed and row number), then bits cleared or set at uniformly drawn positions
 * until exactly 128 remain. Used to give the CPU baseline the same database. */
static inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

typedef struct {
  uint64_t* out;
  uint64_t first, seed;
} synth_ctx;

static void synth_range(void* vctx, int64_t b, int64_t e) {
  synth_ctx* c = (synth_ctx*)vctx;
  for (int64_t r = b; r < e; r++) {
    uint64_t state = mix64(c->seed ^ mix64(c->first + (uint64_t)r + 0x9E3779B97F4A7C15ull));
    uint64_t w[4];
    for (int k = 0; k < 4; k++) {
      state += 0x9E3779B97F4A7C15ull;
      w[k] = mix64(state);
    }
    int pc = __builtin_popcountll(w[0]) + __builtin_popcountll(w[1]) +
             __builtin_popcountll(w[2]) + __builtin_popcountll(w[3]);
    while (pc != 128) {
      state += 0x9E3779B97F4A7C15ull;
      uint32_t pos = (uint32_t)(mix64(state) & 255u);
      uint64_t bit = 1ull << (pos & 63);
      uint64_t* word = &w[pos >> 6];
      if (pc > 128 && (*word & bit)) {
        *word &= ~bit;
        pc--;
      } else if (pc < 128 && !(*word & bit)) {
        *word |= bit;
        pc++;
      }
    }
    memcpy(c->out + r * 4, w, 32);
  }
}

YPDQO_EXPORT void ypdqo_synth_rows(uint8_t* out, int64_t n, uint64_t first, uint64_t seed,
                                   int nthreads) {
  synth_ctx c = {(uint64_t*)out, first, seed};
  parallel_ranges(synth_range, &c, n, nthreads);
}

/* Clustered rows (CPU twin of ypdq_synth_clustered_rows): global row g is centre
 * g / members (row g / members of the generator above) with d distinct bits flipped,
 * d = popcount of `trials` bits of a second splitmix64 stream, positions from the same
 * stream, duplicates redrawn. */
typedef struct {
  uint64_t* out;
  uint64_t first, members, seed;
  uint32_t trials;
} clustered_ctx;

static void clustered_range(void* vctx, int64_t b, int64_t e) {
  clustered_ctx* c = (clustered_ctx*)vctx;
  for (int64_t r = b; r < e; r++) {
    const uint64_t g = c->first + (uint64_t)r;
    uint64_t w[4];
    synth_ctx one = {w, g / c->members, c->seed};
    synth_range(&one, 0, 1);
    uint64_t state = mix64((c->seed ^ 0xC13FA9A902A6328Full) ^ mix64(g + 0x632BE59BD9B4E019ull));
    state += 0x9E3779B97F4A7C15ull;
    const uint64_t mask = c->trials >= 64 ? ~0ull : ((1ull << c->trials) - 1);
    const int d = __builtin_popcountll(mix64(state) & mask);
    uint64_t f[4] = {0, 0, 0, 0};
    for (int k = 0; k < d;) {
      state += 0x9E3779B97F4A7C15ull;
      const uint32_t pos = (uint32_t)(mix64(state) & 255u);
      const uint64_t bit = 1ull << (pos & 63);
      if (!(f[pos >> 6] & bit)) {
        f[pos >> 6] |= bit;
        k++;
      }
    }
    for (int k = 0; k < 4; k++) w[k] ^= f[k];
    memcpy(c->out + r * 4, w, 32);
  }
}

YPDQO_EXPORT void ypdqo_synth_clustered(uint8_t* out, int64_t n, uint64_t first, uint64_t members,
                                        uint32_t trials, uint64_t seed, int nthreads) {
  clustered_ctx c = {(uint64_t*)out, first, members, seed, trials};
  parallel_ranges(clustered_range, &c, n, nthreads);
}

/* ------------------------------------------------------ RGB8 / RGBA8 to luma */

/* Kernel::cvt_rgb8_to_luma8f / cvt_rgba8_to_luma8f (src/kernel/mod.rs:303-340) with the
 * ITU-R BT.601 table of src/kernel/constants.rs:23, the conversion the CLI applies to rgb8
 * and rgba8 frames (src/main.rs:517-606): luma = (0.299 r + 0.587 g) + 0.114 b evaluated left
 * to right in f32 (no contraction: this file builds with -ffp-contract=off). */
YPDQO_EXPORT void ypdqo_luma(const uint8_t* px, int64_t n_pixels, int channels, float* out) {
  const float kr = 0.299f, kg = 0.587f, kb = 0.114f;
  for (int64_t i = 0; i < n_pixels; i++) {
    const uint8_t* p = px + i * channels;
    const float r = kr * (float)p[0];
    const float g = kg * (float)p[1];
    const float b = kb * (float)p[2];
    out[i] = (r + g) + b;
  }
}

/* ------------------------------------- ReferenceKernel<f32>: full Jarosz compress */

/* compute_jarosz_filter_window_size (src/kernel/ref.rs): ceil(old / (2 new)); 3 for 512 -> 127. */
static int jarosz_window(int old_dim, int new_dim) {
  return (old_dim + 2 * new_dim - 1) / (2 * new_dim);
}

/* box_one_d_float (src/kernel/ref.rs): a running-sum box filter of one line in four phases
 * (fill, grow, slide, shrink), all in f32 with true divisions by the current window size. */
static void box_one_d(const float* in, int64_t start, float* out, int len, int64_t stride,
                      int w) {
  const int half = (w + 2) / 2;
  const int64_t oi_off = (int64_t)(half - 1) * stride, li_off = (int64_t)(w - half + 1) * stride;
  float sum = 0.0f, cws = 0.0f;
  const int64_t p1_end = oi_off + start;
  for (int64_t ri = start; ri < p1_end; ri += stride) {
    sum += in[ri];
    cws += 1.0f;
  }
  const int64_t p2_end = (int64_t)w * stride + start;
  for (int64_t ri = p1_end; ri < p2_end; ri += stride) {
    sum += in[ri];
    cws += 1.0f;
    out[ri - oi_off] = sum / cws;
  }
  const int64_t p3_end = (int64_t)len * stride + start;
  for (int64_t ri = p2_end; ri < p3_end; ri += stride) {
    const int64_t oi = ri - oi_off;
    sum += in[ri];
    sum -= in[oi - li_off];
    out[oi] = sum / cws;
  }
  const int64_t p4_start = (int64_t)(len - half + 1) * stride + start;
  for (int64_t oi = p4_start; oi < p3_end; oi += stride) {
    sum -= in[oi - li_off];
    cws += -1.0f;
    out[oi] = sum / cws;
  }
}

/* ReferenceKernel<f32>::jarosz_compress (src/kernel/mod.rs:790-820): jarosz_filter_float
 * (two repetitions of a box filter along rows then along columns, src/kernel/ref.rs) on the
 * whole 512x512 image, then samples ((2 o + 1) 512) / 254 in each dimension. */
YPDQO_EXPORT void ypdqo_jarosz_compress(const float* img, float* out /* 127*127 */) {
  const int w = jarosz_window(512, 127);
  float* buf = (float*)malloc(512 * 512 * sizeof(float));
  float* tmp = (float*)malloc(512 * 512 * sizeof(float));
  memcpy(buf, img, 512 * 512 * sizeof(float));
  for (int rep = 0; rep < 2; rep++) {
    for (int i = 0; i < 512; i++) box_one_d(buf, (int64_t)i * 512, tmp, 512, 1, w);
    for (int j = 0; j < 512; j++) box_one_d(tmp, j, buf, 512, 512, w);
  }
  for (int oi = 0; oi < 127; oi++) {
    const int ini = ((oi * 2 + 1) * 512) / (127 * 2);
    for (int oj = 0; oj < 127; oj++) {
      const int inj = ((oj * 2 + 1) * 512) / (127 * 2);
      out[oi * 127 + oj] = buf[ini * 512 + inj];
    }
  }
  free(tmp);
  free(buf);
}

/* ReferenceKernel<f32>::dct2d (src/kernel/mod.rs:711-735): one sequential accumulator per
 * output, row pass then column pass. */
YPDQO_EXPORT void ypdqo_dct2d_reference(const float* buf /* 127*127 */, float* pdqf /* 256 */) {
  init_constants();
  float tmp[127];
  for (int i = 0; i < 16; i++) {
    for (int j = 0; j < 127; j++) {
      float s = 0.0f;
      for (int k = 0; k < 127; k++) s += DCT32[i * 127 + k] * buf[k * 127 + j];
      tmp[j] = s;
    }
    for (int j = 0; j < 16; j++) {
      float s = 0.0f;
      for (int k = 0; k < 127; k++) s += tmp[k] * DCT32[j * 127 + k];
      pdqf[i * 16 + j] = s;
    }
  }
}

typedef struct {
  const void* imgs;
  int is_u8;
  uint32_t row_mask, col_mask;
  uint8_t* hashes;
  float *quality, *thresholds, *pdqf, *buf127;
} ref_batch_ctx;

static void ref_batch_range(void* vctx, int64_t b, int64_t e) {
  ref_batch_ctx* c = (ref_batch_ctx*)vctx;
  float* img = (float*)malloc(512 * 512 * sizeof(float));
  float* bb = (float*)malloc(127 * 127 * sizeof(float));
  for (int64_t n = b; n < e; n++) {
    if (c->is_u8) {
      const uint8_t* u = (const uint8_t*)c->imgs + n * 512 * 512;
      for (int i = 0; i < 512 * 512; i++) img[i] = (float)u[i];
    } else {
      memcpy(img, (const float*)c->imgs + n * 512 * 512, 512 * 512 * sizeof(float));
    }
    float p[256], t;
    ypdqo_jarosz_compress(img, bb);
    ypdqo_dct2d_reference(bb, p);
    c->quality[n * 8] = ypdqo_adjust_quality(ypdqo_sum_of_gradients(p));
    ypdqo_quantize(p, &t, c->hashes + n * 256);
    c->thresholds[n * 8] = t;
    if (c->pdqf) memcpy(c->pdqf + n * 256, p, sizeof(p));
    if (c->buf127) memcpy(c->buf127 + n * 127 * 127, bb, 127 * 127 * sizeof(float));
    ypdqo_dihedrals(p, t, c->row_mask, c->col_mask, c->hashes + n * 256 + 32,
                    c->thresholds + n * 8 + 1, c->quality + n * 8 + 1, NULL);
  }
  free(bb);
  free(img);
}

/* ReferenceKernel<f32> (the pdqhash-faithful kernel) over n images, with the dihedrals. */
YPDQO_EXPORT void ypdqo_hash_batch_reference(const void* imgs, int64_t n, int is_u8,
                                             uint32_t row_mask, uint32_t col_mask,
                                             uint8_t* hashes, float* quality, float* thresholds,
                                             float* pdqf, float* buf127, int nthreads) {
  init_constants();
  ref_batch_ctx c = {imgs, is_u8, row_mask, col_mask, hashes, quality, thresholds, pdqf, buf127};
  parallel_ranges(ref_batch_range, &c, n, nthreads);
}

/* ----------------------------------------------- Avx2F32Kernel (x86.rs), restated */

/* The sum of the 8 lanes as the kernel's permute-and-add reduction forms it:
 * ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7)). */
static float hsum8(const float* a) {
  return ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
}

/* jarosz_compress_avx2 (src/kernel/x86.rs:626-682): per output, 8 lanes l accumulate
 * fma(img[in_i + di][in_j + l], W8[di][l], .) over di (W8 = the 7 tent weights of a row
 * and a 0), reduced by two hadds as ((l0 + l1) + (l2 + l3)) + ((l4 + l5) + (l6 + l7)).
 * Lane 7 reads the next pixel in memory (weight 0); for the last output of the last row
 * it reads in_j + 6 again (the kernel's rewind-and-permute), staying inside the image.
 * out is 128 x 128 with a zero last row and column, as the kernel's buffer. */
static void avx2_compress(const float* img, float* out) {
  memset(out, 0, 128 * 128 * sizeof(float));
  for (int oi = 0; oi < 127; oi++) {
    const int in_i = YPDQO_CONV_OFFSET[oi] - YPDQO_TENT_OFFSET;
    for (int oj = 0; oj < 127; oj++) {
      const int in_j = YPDQO_CONV_OFFSET[oj] - YPDQO_TENT_OFFSET;
      float lane[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (int di = 0; di < 7; di++) {
        const int64_t row = (int64_t)(in_i + di) * 512 + in_j;
        for (int l = 0; l < 8; l++) {
          int64_t idx = row + l;
          if (l == 7 && di == 6 && oi == 126 && oj == 126) idx = row + 6;
          const float w = l < 7 ? TENT[di * 7 + l] : 0.0f;
          lane[l] = fmaf(img[idx], w, lane[l]);
        }
      }
      /* _mm256_hadd_ps twice with zero, then element 0 + element 4 */
      const float h0 = (lane[0] + lane[1]) + (lane[2] + lane[3]);
      const float h4 = (lane[4] + lane[5]) + (lane[6] + lane[7]);
      out[oi * 128 + oj] = h0 + h4;
    }
  }
}

/* A 16 x 127 DCT matrix as the kernel reads it: row-major followed by zero padding, so
 * element (k, 127) is element (k + 1, 0), and (15, 127) is 0. */
static float dct_padded(const float* D, int k, int c) {
  const int idx = k * 127 + c;
  return idx < 16 * 127 ? D[idx] : 0.0f;
}

/* Avx2F32Kernel::dct2d_impl (src/kernel/x86.rs:100-281). Stage 1: for each frequency k and
 * column j, two accumulators take the products of rows k2 = 0..127 (the padding row
 * included) by fma in the pattern 1, 0, 0, 1, 1, 0, 0, 1 per 8 rows; a NaN sum becomes 0;
 * tmp[j] = sum0 + sum1. Stage 2: per output j, two 8-lane accumulators take 8-column
 * blocks in the pattern 1, 0, 0, 1; their lane sums are added and reduced by hsum8. */
static void avx2_dct2d(const float* D, const float* buf /* 128*128 */, float* pdqf /* 256 */) {
  static const int pat8[8] = {1, 0, 0, 1, 1, 0, 0, 1};
  float tmp[128];
  for (int k = 0; k < 16; k++) {
    for (int j = 0; j < 128; j++) {
      float acc[2] = {0.0f, 0.0f};
      for (int k2 = 0; k2 < 128; k2++)
        acc[pat8[k2 & 7]] = fmaf(buf[k2 * 128 + j], dct_padded(D, k, k2), acc[pat8[k2 & 7]]);
      const float s0 = isnan(acc[0]) ? 0.0f : acc[0];
      const float s1 = isnan(acc[1]) ? 0.0f : acc[1];
      tmp[j] = s0 + s1;
    }
    for (int j = 0; j < 16; j++) {
      float acc[2][8];
      memset(acc, 0, sizeof(acc));
      for (int blk = 0; blk < 16; blk++) {
        const int t = pat8[blk & 3];
        for (int l = 0; l < 8; l++)
          acc[t][l] = fmaf(tmp[blk * 8 + l], dct_padded(D, j, blk * 8 + l), acc[t][l]);
      }
      float sum[8];
      for (int l = 0; l < 8; l++) sum[l] = acc[0][l] + acc[1][l];
      pdqf[k * 16 + j] = hsum8(sum);
    }
  }
}

/* Avx2F32Kernel::quantize_impl (src/kernel/x86.rs:440-621): a search for the threshold by
 * the mean of the residual elements beyond the guess, at most 32 rounds. Each round writes
 * the bits x > guess (byte 31 - c for elements 8c .. 8c + 7); 8-lane residual sums are
 * reduced by hsum8 and divided by their counts. */
/* _mm256_min_ps / _mm256_max_ps per lane: the first operand if it compares less /
 * greater, else the second (so ties and NaNs take the second). */
static float vmin(float a, float b) { return a < b ? a : b; }
static float vmax(float a, float b) { return a > b ? a : b; }
/* The kernel's horizontal min / max: op(a[i], a[i+1]), then op(.[i], .[i+2]), then
 * op(.[0], .[4]), indices mod 8 (permutevar8x32 rotations). */
static float htree(const float* a, float (*op)(float, float)) {
  float pw[8], e4[8];
  for (int i = 0; i < 8; i++) pw[i] = op(a[i], a[(i + 1) & 7]);
  for (int i = 0; i < 8; i++) e4[i] = op(pw[i], pw[(i + 2) & 7]);
  return op(e4[0], e4[4]);
}

static void avx2_quantize(const float* p, float* thr, uint8_t* out) {
  float lmin[8], lmax[8];
  for (int l = 0; l < 8; l++) {
    lmin[l] = FLT_MAX;
    lmax[l] = -FLT_MAX;
  }
  for (int c = 0; c < 32; c++)
    for (int l = 0; l < 8; l++) {
      const float x = p[8 * c + l];
      lmin[l] = vmin(lmin[l], x);
      lmax[l] = vmax(lmax[l], x);
    }
  float mx = htree(lmax, vmax), mn = htree(lmin, vmin);
  const uint32_t half = 128;
  float guess = (mn + mx) * 0.5f;
  uint32_t num_over = 0, num_under = 0;
  for (int iter = 0; iter < 32; iter++) {
    float rgt[8] = {0, 0, 0, 0, 0, 0, 0, 0}, rlt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    uint32_t gt_count = 0, lt_count = 0;
    for (int c = 0; c < 32; c++) {
      uint8_t bits = 0;
      for (int l = 0; l < 8; l++) {
        const float x = p[8 * c + l];
        const int gt = x > guess, lt = x < guess;
        if (gt) bits |= (uint8_t)(1u << l);
        const int mgt = gt && x <= mx, mlt = lt && x >= mn;
        gt_count += (uint32_t)mgt;
        lt_count += (uint32_t)mlt;
        rgt[l] = rgt[l] + (mgt ? x : 0.0f);  /* and_ps(mask, x): x or +0 */
        rlt[l] = rlt[l] + (mlt ? x : 0.0f);
      }
      out[31 - c] = bits;
    }
    if (gt_count + num_over > half) {
      num_under += lt_count;
      mn = guess;
      guess = hsum8(rgt) / (float)gt_count;
    } else if (lt_count + num_under > half) {
      num_over += gt_count;
      mx = guess;
      guess = hsum8(rlt) / (float)lt_count;
    } else {
      break;
    }
  }
  *thr = guess;
}

/* u8 -> f32 is exact in both kernels; quality is the trait's sum of gradients over the
 * kernel's PDQF (same loop order) and the same adjustment. */
typedef struct {
  const void* imgs;
  int is_u8;
  uint8_t* hashes;
  float *quality, *thresholds, *pdqf;
} avx2_batch_ctx;

static void avx2_batch_range(void* vctx, int64_t b, int64_t e) {
  avx2_batch_ctx* c = (avx2_batch_ctx*)vctx;
  float* img = (float*)malloc(512 * 512 * sizeof(float));
  float* bb = (float*)malloc(128 * 128 * sizeof(float));
  for (int64_t n = b; n < e; n++) {
    if (c->is_u8) {
      const uint8_t* u = (const uint8_t*)c->imgs + n * 512 * 512;
      for (int i = 0; i < 512 * 512; i++) img[i] = (float)u[i];
    } else {
      memcpy(img, (const float*)c->imgs + n * 512 * 512, 512 * 512 * sizeof(float));
    }
    float p[256], t;
    avx2_compress(img, bb);
    avx2_dct2d(DCT32, bb, p);
    c->quality[n * 8] = ypdqo_adjust_quality(ypdqo_sum_of_gradients(p));
    avx2_quantize(p, &t, c->hashes + n * 256);
    c->thresholds[n * 8] = t;
    if (c->pdqf) memcpy(c->pdqf + n * 256, p, sizeof(p));
    /* Avx2F32Kernel sign patterns: rows 0, 2, .., 14; columns 0, 2, 4, 6 */
    dihedrals_with(p, t, 0x5555u, 0x0055u, c->hashes + n * 256 + 32, c->thresholds + n * 8 + 1,
                   c->quality + n * 8 + 1, NULL, avx2_quantize);
  }
  free(bb);
  free(img);
}

/* yume-pdq's Avx2F32Kernel (smart_kernel on AVX2 + FMA hosts) over n images, with its
 * dihedrals: hashes n x 8 x 32, quality and thresholds n x 8, pdqf n x 256 (or NULL). */
YPDQO_EXPORT void ypdqo_hash_batch_avx2(const void* imgs, int64_t n, int is_u8, uint8_t* hashes,
                                        float* quality, float* thresholds, float* pdqf,
                                        int nthreads) {
  init_constants();
  avx2_batch_ctx c = {imgs, is_u8, hashes, quality, thresholds, pdqf};
  parallel_ranges(avx2_batch_range, &c, n, nthreads);
}

/* The Avx2F32Kernel DCT alone on a 128 x 128 zero-padded buffer and a given matrix (the
 * reference's AVX2-equivalence test, src/kernel/mod.rs:1249-1345). */
YPDQO_EXPORT void ypdqo_dct2d_avx2_matrix(const float* D /* 16*127 */,
                                          const float* buf /* 128*128 */, float* pdqf /* 256 */) {
  avx2_dct2d(D, buf, pdqf);
}
