/* openzl_gb300: GB300-native (sm_103a) implementation of OpenZL's numeric
 * codec-graph hot path, exposed through OpenZL's own C entry points.
 *
 * Everything here is plain C: pointers, sizes and opaque handles. The
 * ZL_* functions keep the names, argument meaning and error behaviour of the
 * reference declarations cited beside each one, so that a caller written
 * against OpenZL's C API (and the C++/Python bindings layered on it) reaches
 * the GPU path unchanged. The ozl_gpu_* functions are additions for callers
 * that hold their data on the device (batched and serving paths).
 *
 * Frames are OpenZL wire format 21-23 (chunked block format). Older frames
 * and codecs outside the numeric path are rejected with an error; there is
 * no CPU fallback.
 */
#ifndef OPENZL_GB300_H
#define OPENZL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* ------------------------------------------------------------------ */
/* Errors: same layout and codes as the reference's ZL_Report
 * (include/openzl/zl_errors.h:206-207, zl_errors_types.h:38-120):
 * a 4-byte code followed by an 8-byte value. */
typedef enum {
    ZL_ErrorCode_no_error = 0,
    ZL_ErrorCode_GENERIC = 1,
    ZL_ErrorCode_srcSize_tooSmall = 3,
    ZL_ErrorCode_srcSize_tooLarge = 4,
    ZL_ErrorCode_dstCapacity_tooSmall = 5,
    ZL_ErrorCode_header_unknown = 10,
    ZL_ErrorCode_frameParameter_unsupported = 11,
    ZL_ErrorCode_corruption = 12,
    ZL_ErrorCode_compressedChecksumWrong = 13,
    ZL_ErrorCode_contentChecksumWrong = 14,
    ZL_ErrorCode_parameter_invalid = 21,
    ZL_ErrorCode_invalidRequest_singleOutputFrameOnly = 23,
    ZL_ErrorCode_graph_invalid = 30,
    ZL_ErrorCode_invalidTransform = 32,
    ZL_ErrorCode_formatVersion_unsupported = 60,
    ZL_ErrorCode_formatVersion_notSet = 61,
    ZL_ErrorCode_allocation = 70,
    ZL_ErrorCode_logicError = 80,
    ZL_ErrorCode_temporaryLibraryLimitation = 81,
} ZL_ErrorCode;

typedef struct {
    ZL_ErrorCode _code;
    size_t _value;
} ZL_Report;

/* include/openzl/zl_errors.h:216-235 */
int ZL_isError(ZL_Report report);
size_t ZL_validResult(ZL_Report report);
ZL_ErrorCode ZL_errorCode(ZL_Report report);
const char* ZL_ErrorCode_toString(ZL_ErrorCode code);

/* ------------------------------------------------------------------ */
/* Types (include/openzl/zl_data.h:35-40). */
typedef enum {
    ZL_Type_serial = 1,
    ZL_Type_struct = 2,
    ZL_Type_numeric = 4,
    ZL_Type_string = 8,
} ZL_Type;

/* ------------------------------------------------------------------ */
/* Frame inspection (include/openzl/zl_decompress.h:47, :64). */
ZL_Report ZL_getDecompressedSize(const void* compressed, size_t cSize);
ZL_Report ZL_getCompressedSize(const void* compressed, size_t cSize);

/* ------------------------------------------------------------------ */
/* Decompression context (include/openzl/zl_decompress.h:80-230). */
typedef struct ZL_DCtx_s ZL_DCtx;

typedef enum {
    ZL_DParam_stickyParameters = 1,
    ZL_DParam_checkCompressedChecksum = 2,
    ZL_DParam_checkContentChecksum = 3,
} ZL_DParam;

typedef enum {
    ZL_TernaryParam_auto = 0,
    ZL_TernaryParam_enable = 1,
    ZL_TernaryParam_disable = 2,
} ZL_TernaryParam;

/* zl_decompress.h:80 */
ZL_DCtx* ZL_DCtx_create(void);
/* zl_decompress.h:87 */
void ZL_DCtx_free(ZL_DCtx* dctx);
/* zl_decompress.h:140 */
ZL_Report ZL_DCtx_setParameter(ZL_DCtx* dctx, ZL_DParam param, int value);
/* zl_decompress.h:188 */
const char* ZL_DCtx_getErrorContextString(const ZL_DCtx* dctx, ZL_Report report);
/* zl_decompress.h:230: host buffers in and out; decoding runs on cuda:0. */
ZL_Report ZL_DCtx_decompress(ZL_DCtx* dctx, void* dst, size_t dstCapacity,
                             const void* compressed, size_t cSize);
/* zl_decompress.h:32: one-shot variant with an internal context. */
ZL_Report ZL_decompress(void* dst, size_t dstCapacity, const void* compressed, size_t cSize);

/* ------------------------------------------------------------------ */
/* GPU additions (no counterpart in the reference; the reference has no
 * device path). Pointers prefixed d_ are device pointers on the current
 * CUDA device; `stream` is a cudaStream_t (NULL = default stream). */

/* Decodes one frame whose bytes are already on the device. `h_frame` is a
 * host copy of the same frame, read for header planning only. Output goes to
 * d_dst. Enqueued on `stream`; errors detected on the device are reported by
 * the return value after the call synchronizes the stream. */
ZL_Report ozl_gpu_decompress(ZL_DCtx* dctx, void* d_dst, size_t dstCapacity,
                             const void* h_frame, const void* d_frame, size_t cSize,
                             void* stream);

/* Batched decode: many frames, one plan, one CUDA graph launch per run. */
typedef struct OZL_GpuBatch_s OZL_GpuBatch;
OZL_GpuBatch* ozl_gpu_batch_create(void);
void ozl_gpu_batch_free(OZL_GpuBatch* b);
/* Sets a DParam for subsequent plans (same meaning as ZL_DCtx_setParameter). */
ZL_Report ozl_gpu_batch_setParameter(OZL_GpuBatch* b, ZL_DParam param, int value);
/* Plans the decode of nbFrames frames. h_frames[i]: host copy (planning);
 * d_frames[i]: device copy; d_dsts[i]/dstCapacities[i]: device outputs.
 * Returns the total decompressed size. Allocates device scratch sized for
 * the plan; reuses it across runs. */
ZL_Report ozl_gpu_batch_plan(OZL_GpuBatch* b, size_t nbFrames,
                             const void* const* h_frames, const size_t* frameSizes,
                             const void* const* d_frames, void* const* d_dsts,
                             const size_t* dstCapacities);
/* Launches the planned decode on `stream` (a CUDA graph when useGraph != 0). */
ZL_Report ozl_gpu_batch_run(OZL_GpuBatch* b, void* stream, int useGraph);
/* Synchronizes `stream` and reports device-detected errors of the last run
 * (corruption, checksum mismatch). Returns the total decompressed size. */
ZL_Report ozl_gpu_batch_check(OZL_GpuBatch* b, void* stream);
/* Runs the planned decode launch by launch on `stream`, bracketing each with
 * CUDA events. For launch i, writes its duration in milliseconds to
 * ms[i], its codec family to kinds[i] (see ozl_gpu_kind_name) and the bytes
 * it must read plus write to bytes[i], for i < capacity. Returns the number
 * of launches. Synchronizes `stream`. */
ZL_Report ozl_gpu_batch_profile(OZL_GpuBatch* b, void* stream, float* ms, int* kinds,
                                uint64_t* bytes, size_t capacity);
/* Name of a codec family reported by ozl_gpu_batch_profile. */
const char* ozl_gpu_kind_name(int kind);
/* Host-buffer run of a planned batch whose device frames sit back to back
 * from d_frames[0] and whose outputs sit back to back from d_dsts[0] (as
 * passed to ozl_gpu_batch_plan): copies h_in (inBytes) to the device, runs
 * the decode, copies the outputs to h_out (outBytes) and synchronizes.
 * Returns the total decompressed size. */
ZL_Report ozl_gpu_batch_run_host(OZL_GpuBatch* b, const void* h_in, size_t inBytes, void* h_out,
                                 size_t outBytes, void* stream, int useGraph);
/* Number of kernel launches one run issues. */
size_t ozl_gpu_batch_launches(const OZL_GpuBatch* b);
/* Per-frame decoded sizes of the last plan (array of nbFrames). */
const size_t* ozl_gpu_batch_sizes(const OZL_GpuBatch* b);
/* Message describing the last error of this batch ("" when none). */
const char* ozl_gpu_batch_error(const OZL_GpuBatch* b);

/* Batched compression (no counterpart in the reference: the reference
 * compresses one frame per call on the CPU). Each frame i compresses
 * nbElts[i] elements of eltWidths[i] bytes (0 = serial bytes) at device
 * address d_srcs[i] with the numeric graph recipes[i] (OZL_GRAPH_*) into
 * d_dsts[i] (capacity dstCapacities[i], see ozl_gpu_compress_bound), format
 * version 23. The frames are byte-identical to what the reference's
 * ZL_CCtx_compressTypedRef emits for the same graph and parameters.
 * frameSizes[i] receives each frame's size. Synchronizes `stream`. */
typedef enum {
    OZL_GRAPH_STORE = 0,            /* ZL_GRAPH_STORE */
    OZL_GRAPH_DZ_TSPLIT_FSE = 1,    /* delta -> zigzag -> to-struct -> transpose-split(ZL_GRAPH_FSE) */
    OZL_GRAPH_DZ_BITPACK_HUF = 2,   /* delta -> zigzag -> bitpack_int -> ZL_GRAPH_HUFFMAN */
    OZL_GRAPH_D_TSPLIT_FSE = 3,     /* delta -> to-struct -> transpose-split(ZL_GRAPH_FSE) */
    OZL_GRAPH_D_BITPACK_HUF = 4,    /* delta -> bitpack_int -> ZL_GRAPH_HUFFMAN */
    OZL_GRAPH_FSE = 7,              /* ZL_GRAPH_FSE */
    OZL_GRAPH_HUFFMAN = 8,          /* ZL_GRAPH_HUFFMAN */
    OZL_GRAPH_DELTA_STORE = 9,      /* delta -> store */
    OZL_GRAPH_ZIGZAG_STORE = 10,    /* zigzag -> store */
    OZL_GRAPH_BITPACK_STORE = 11,   /* bitpack_int -> store */
    OZL_GRAPH_TSPLIT_STORE = 12,    /* to-struct -> transpose-split(store) */
    OZL_GRAPH_CONSTANT = 13,        /* ZL_GRAPH_CONSTANT */
    OZL_GRAPH_FLATPACK = 14,        /* ZL_GRAPH_FLATPACK */
    OZL_GRAPH_BITPACK = 15,         /* ZL_GRAPH_BITPACK */
} OZL_GraphRecipe;

typedef struct OZL_GpuEncoder_s OZL_GpuEncoder;
OZL_GpuEncoder* ozl_gpu_encoder_create(void);
void ozl_gpu_encoder_free(OZL_GpuEncoder* e);
size_t ozl_gpu_compress_bound(size_t srcBytes);
ZL_Report ozl_gpu_compress_batch(OZL_GpuEncoder* e, size_t nbFrames, const void* const* d_srcs,
                                 const size_t* nbElts, const int* eltWidths, const int* recipes,
                                 void* const* d_dsts, const size_t* dstCapacities, size_t* frameSizes,
                                 int checksums, void* stream);
/* Message describing the encoder's last error ("" when none). */
const char* ozl_gpu_encoder_error(const OZL_GpuEncoder* e);

/* XXH3-64 (seed 0), the hash behind OpenZL's checksums, of `len` bytes of
 * device memory; computed on the GPU. Returns the hash in the report value. */
ZL_Report ozl_gpu_xxh3_64(const void* d_data, size_t len, void* stream);

/* Allocation-free variant of ozl_gpu_xxh3_64 (no counterpart in the
 * reference), for callers that cannot call cudaMalloc: the same hash and
 * kernels, with their scratch (task, block list, per-1 KiB block sums and the
 * result) in one fixed file-scope device array of OZL_XXH3_STATIC_SCRATCH
 * bytes per device instead of a per-call allocation. Accepts at most
 * OZL_XXH3_STATIC_MAX_LEN bytes; longer inputs return
 * ZL_ErrorCode_srcSize_tooLarge without touching the device. Calls no
 * allocating routine. Every call on a device shares that array: calls whose
 * work overlaps on the GPU (other streams, other host threads) race and must
 * be serialized by the caller. Synchronizes `stream`; returns the hash in the
 * report value. */
#define OZL_XXH3_STATIC_MAX_LEN ((size_t)32 << 20)
#define OZL_XXH3_STATIC_SCRATCH ((size_t)256 + ((size_t)32 << 10) * 72)
ZL_Report ozl_gpu_xxh3_64_static(const void* d_data, size_t len, void* stream);

/* Library build identification (for load checks). */
const char* ozl_gpu_version(void);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif
#endif
