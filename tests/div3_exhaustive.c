/* Exhaustive check of the division-free x / 3 used by the GPU's Jarosz running sums
 * (div3_rn in yume-pdq_gb300/csrc/jarosz.cu): Markstein's remainder correction
 *   q0 = RN(x c), r = fma(-q0, 3, x), q = r is NaN ? q0 : fma(r, c, q0),  c = RN(1/3)
 * against IEEE x / 3 for every non-negative float bit pattern (NaN inputs only need a NaN
 * result). Each step is odd in x, so negative inputs follow by symmetry. Prints the number of
 * mismatches and the first one; built with -ffp-contract=off so that only the written FMAs
 * are fused. */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

enum { kThreads = 8 };

typedef struct {
  uint64_t lo, hi, bad;
  uint32_t first;
} job;

static float as_float(uint32_t b) {
  float x;
  memcpy(&x, &b, 4);
  return x;
}
static uint32_t bits_of(float x) {
  uint32_t b;
  memcpy(&b, &x, 4);
  return b;
}

static float div3_markstein(float x) {
  const float c = 0x1.555556p-2f; /* RN(1/3) */
  const float q0 = x * c;
  const float r = fmaf(-q0, 3.0f, x);
  return r == r ? fmaf(r, c, q0) : q0;
}

static void* run(void* p) {
  job* j = (job*)p;
  j->first = 0xffffffffu;
  for (uint64_t b = j->lo; b < j->hi; b++) {
    const float x = as_float((uint32_t)b);
    const float want = x / 3.0f, got = div3_markstein(x);
    const int ok = isnan(x) ? isnan(got) : bits_of(got) == bits_of(want);
    if (!ok) {
      if (!j->bad) j->first = (uint32_t)b;
      j->bad++;
    }
  }
  return NULL;
}

int main(void) {
  if (1.0f / 3.0f != 0x1.555556p-2f) {
    printf("RN(1/3) constant wrong\n");
    return 2;
  }
  const uint64_t n = 1ull << 31;
  pthread_t th[kThreads];
  job js[kThreads];
  for (int i = 0; i < kThreads; i++) {
    js[i].lo = n * i / kThreads;
    js[i].hi = n * (i + 1) / kThreads;
    js[i].bad = 0;
    pthread_create(&th[i], NULL, run, &js[i]);
  }
  uint64_t bad = 0;
  uint32_t first = 0xffffffffu;
  for (int i = 0; i < kThreads; i++) {
    pthread_join(th[i], NULL);
    if (js[i].bad && first == 0xffffffffu) first = js[i].first;
    bad += js[i].bad;
  }
  printf("checked %llu mismatches %llu first %08x\n", (unsigned long long)n,
         (unsigned long long)bad, first);
  return bad ? 1 : 0;
}
