/*
 * yume_pdq.h -- drop-in C interface of the GB300 library.
 *
 * libyumepdq_gb300.so exports the symbols of yume-pdq's C header with the same
 * signatures and semantics, so an existing consumer (C, or Python ctypes as in
 * yume-pdq's integration/hash.py) can load this library in place of libyume_pdq.so.
 * Each entry point replaces the reference item cited beside it:
 *
 *   yume_pdq_hash_smart_kernel            include/yume_pdq.h:122-137, src/lib.rs:234-283
 *   yume_pdq_visit_dihedrals_smart_kernel include/yume_pdq.h:139-150, src/lib.rs:187-232
 *   DihedralCallback                      include/yume_pdq.h:40-49,   src/lib.rs:180-185
 *   YumePDQ_Dihedrals, YUME_PDQ_DIHEDRAL_* include/yume_pdq.h:51-109, src/lib.rs:85-172
 *   YUME_PDQ_VERSION_*                    include/yume_pdq.h:22-25,   build.rs:389-429
 *
 * The work runs on CUDA device 0 through a library-owned context that the first call
 * creates. Calls are synchronous and thread-safe, like the reference's. The reference
 * returns no error for these symbols, so a CUDA failure here prints a message to stderr
 * and returns quality -1.0f (hash) or false (visit).
 *
 * Dihedral signs. yume-pdq's CPU kernels derive ROTATED_180, FLIPPED and three transposed
 * variants with different sign patterns, and smart_kernel() picks the kernel by host
 * (src/kernel/mod.rs:79-176): Avx2F32Kernel on x86_64 with AVX2 and FMA, the trait-default
 * DefaultKernel elsewhere (an aarch64 host, for one). The visit symbol follows the same
 * choice, so it returns what the replaced library returns on the same host. The
 * environment variable YUME_PDQ_DIHEDRAL_SEMANTICS = exact | avx2 | scalar overrides it
 * (exact is Avx512F32Kernel's pattern, the sign pattern of a true flip); the batched API in
 * ypdq.h takes the convention as an argument and ypdq_dropin_semantics() reports this one.
 */
#ifndef YUME_PDQ_GB300_DROPIN_H
#define YUME_PDQ_GB300_DROPIN_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

extern const uint32_t YUME_PDQ_VERSION_MAJOR;
extern const uint32_t YUME_PDQ_VERSION_MINOR;
extern const uint32_t YUME_PDQ_VERSION_PATCH;
extern const char YUME_PDQ_VERSION_STRING[];

/* Return true to continue, false to stop (src/lib.rs:180-185). The buffers passed to the
 * visit call hold the current variant only until the callback returns. */
typedef bool (*DihedralCallback)(void *ctx, uint32_t dihedral, float threshold, float quality);

/* A dihedral transform: big-endian packed i8 matrix (x->x, x->y, y->x, y->y). */
typedef struct YumePDQ_Dihedrals {
  uint32_t packed;
} YumePDQ_Dihedrals;

extern const struct YumePDQ_Dihedrals YUME_PDQ_DIHEDRAL_NORMAL;
extern const struct YumePDQ_Dihedrals YUME_PDQ_DIHEDRAL_FLIPPED;
extern const struct YumePDQ_Dihedrals YUME_PDQ_DIHEDRAL_FLOPPED;
extern const struct YumePDQ_Dihedrals YUME_PDQ_DIHEDRAL_ROTATED_180;
extern const struct YumePDQ_Dihedrals YUME_PDQ_DIHEDRAL_ROTATED_90;
extern const struct YumePDQ_Dihedrals YUME_PDQ_DIHEDRAL_ROTATED_270;
extern const struct YumePDQ_Dihedrals YUME_PDQ_DIHEDRAL_ROTATED_90_FLOPPED;
extern const struct YumePDQ_Dihedrals YUME_PDQ_DIHEDRAL_FLOPPED_ROTATED_270;

/*
 * Hash one 512x512 f32 grayscale image (row-major) on the GPU.
 * threshold: out, may be NULL. output: 32-byte hash. buf1: 128x128 f32 that receives the
 * 127x127 compressed image in its top-left corner (row stride 128, padding untouched).
 * tmp: 128 f32 of scratch, left untouched. pdqf: 16x16 f32 unquantized hash.
 * Returns the quality in [0, 1].
 */
float yume_pdq_hash_smart_kernel(const float *input, float *threshold, uint8_t *output,
                                 float *buf1, float *tmp, float *pdqf);

/*
 * Visit the seven derived dihedrals of a PDQF in the reference order. For each, output
 * and pdqf hold that variant's hash and matrix when the callback runs. The callback gets
 * the threshold argument of this call, not the variant's own (the reference's behaviour,
 * src/lib.rs:224). Returns false if a callback returned false.
 */
bool yume_pdq_visit_dihedrals_smart_kernel(void *ctx, float threshold, uint8_t *output,
                                           float *pdqf, DihedralCallback callback);

#ifdef __cplusplus
}
#endif

#endif /* YUME_PDQ_GB300_DROPIN_H */
