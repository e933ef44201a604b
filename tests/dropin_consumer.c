/*
 * A plain C consumer of the drop-in interface (include/yume_pdq.h), built by the tests with
 * gcc and linked against libyumepdq_gb300.so: it hashes two ramp images the way yume-pdq's
 * own C example does (pixel i holds i, then i + 1), visits the dihedrals of the second
 * through a C callback that asks to stop after `stop_after` variants (0: never), and prints
 * everything with enough digits to compare bit for bit.
 *
 * usage: dropin_consumer [stop_after]
 */
#include <stdio.h>
#include <stdlib.h>

#include "yume_pdq.h"

struct visit_state {
  const uint8_t *hash;
  const float *pdqf;
  int seen;
  int stop_after;
};

static void print_hash(const uint8_t *h) {
  for (int i = 0; i < 32; i++) printf("%02x", h[i]);
}

static bool on_variant(void *ctx, uint32_t dihedral, float threshold, float quality) {
  struct visit_state *st = (struct visit_state *)ctx;
  printf("variant %d dihedral %08x threshold %.9g quality %.9g pdqf0 %.9g hash ", st->seen,
         (unsigned)dihedral, threshold, quality, st->pdqf[0]);
  print_hash(st->hash);
  printf("\n");
  st->seen++;
  return st->stop_after <= 0 || st->seen < st->stop_after;
}

int main(int argc, char **argv) {
  float *input = (float *)malloc(512 * 512 * sizeof(float));
  float *buf1 = (float *)malloc(128 * 128 * sizeof(float));
  float *tmp = (float *)malloc(128 * sizeof(float));
  float *pdqf = (float *)malloc(256 * sizeof(float));
  uint8_t hash[32];
  float threshold = 0.0f;
  if (!input || !buf1 || !tmp || !pdqf) return 2;
  for (int k = 0; k < 2; k++) {
    for (int i = 0; i < 512 * 512; i++) input[i] = (float)(i + k);
    const float quality = yume_pdq_hash_smart_kernel(input, &threshold, hash, buf1, tmp, pdqf);
    printf("image %d quality %.9g threshold %.9g buf1_0 %.9g pdqf0 %.9g hash ", k, quality,
           threshold, buf1[0], pdqf[0]);
    print_hash(hash);
    printf("\n");
  }
  struct visit_state st = {hash, pdqf, 0, argc > 1 ? atoi(argv[1]) : 0};
  const bool done = yume_pdq_visit_dihedrals_smart_kernel(&st, threshold, hash, pdqf, on_variant);
  printf("visited %d completed %d\n", st.seen, done ? 1 : 0);
  printf("version %u.%u.%u %s\n", (unsigned)YUME_PDQ_VERSION_MAJOR,
         (unsigned)YUME_PDQ_VERSION_MINOR, (unsigned)YUME_PDQ_VERSION_PATCH,
         YUME_PDQ_VERSION_STRING);
  printf("flipped %08x rotated_90 %08x\n", (unsigned)YUME_PDQ_DIHEDRAL_FLIPPED.packed,
         (unsigned)YUME_PDQ_DIHEDRAL_ROTATED_90.packed);
  free(input);
  free(buf1);
  free(tmp);
  free(pdqf);
  return 0;
}
