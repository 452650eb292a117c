/* CPU restatement of OpenZL's numeric codec-graph path (the test oracle).
 *
 * Test infrastructure only: the tests, the smoke check and the benchmark's
 * CPU-baseline leg call it as the checker. The GPU library never links it.
 *
 * Parity is pinned two ways: against the compiled reference library
 * (oracle/ref.mk) on seeded inputs, and against golden frames committed
 * under tests/golden/ that the reference produced.
 */
#ifndef OZL_ORACLE_H
#define OZL_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes returned (negated) by the oracle. */
enum {
    OZO_ERR_GENERIC     = 1,
    OZO_ERR_SRC_SIZE    = 2,
    OZO_ERR_CORRUPTION  = 3,
    OZO_ERR_VERSION     = 4,
    OZO_ERR_UNSUPPORTED = 5,
    OZO_ERR_DST_SIZE    = 6,
    OZO_ERR_CHECKSUM    = 7,
    OZO_ERR_ALLOC       = 8,
};

/* XXH3-64 with seed 0 and the default secret. */
uint64_t ozo_xxh3_64(const void* src, size_t len);

/* Decodes a single-output frame into dst. On success returns the number of
 * bytes written and sets *outType (1 serial, 2 struct, 4 numeric) and
 * *outEltWidth. Returns a negative OZO_ERR_* on failure. */
int64_t ozo_decompress(const void* src, size_t srcSize, void* dst, size_t dstCap,
                       int* outType, int* outEltWidth);

/* Decodes a frame of any number of outputs; outs[o] and strLens[o] (the
 * 4-byte string lengths of a string output, nbStrings[o] of them) are
 * malloc'ed (free them with ozo_free). Returns the number of outputs or a
 * negative error. */
int64_t ozo_decompress_multi(const void* src, size_t srcSize, size_t maxOut, void** outs, size_t* lens, int* types,
                             int* widths, void** strLens, size_t* nbStrings);
void ozo_free(void* p);

/* Decompressed size recorded in a single-output frame header, or < 0. */
int64_t ozo_decompressed_size(const void* src, size_t srcSize);

/* Compresses nbElts elements (eltWidth 0 = serial bytes) with one of the
 * numeric graph recipes (same numbering as oracle/ref_driver.c). Returns the
 * frame size or a negative error. */
int64_t ozo_compress(int recipe, const void* src, size_t nbElts, int eltWidth,
                     void* dst, size_t dstCap, int checksums);

size_t ozo_compress_bound(size_t srcSize);

/* Test entry points (known-answer vectors): one decoder on caller streams
 * (inputs in the decoder's order; returns output bytes), and the tokenize
 * node alone (returns the alphabet size). */
int64_t ozo_decode_transform(unsigned id, const uint8_t* hdr, size_t hsz, size_t nbIn, const int* types,
                             const size_t* widths, const size_t* counts, const uint8_t* const* data, void* out,
                             size_t outCap, int* outType, size_t* outW, size_t* outN);
int64_t ozo_tokenize(const void* src, size_t n, int w, int sorted, void* alphaOut, void* idxOut, int* iwOut);
/* Test entry point: the largest FSE table log the encoder may pick, 11 (the
 * reference encoder's) or 12 (the decoders' limit). Not thread-safe. */
void ozo_test_set_fse_max_tablelog(unsigned tl);
void ozo_test_set_huf_max_tablelog(unsigned tl);

#ifdef __cplusplus
}
#endif
#endif
