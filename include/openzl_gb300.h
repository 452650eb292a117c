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
 * Frames of OpenZL wire format versions 8-23 decode; the encoder writes
 * version 23. Codecs outside the numeric path (and the deprecated entropy
 * codecs of versions 8-14) are rejected with an error; there is no CPU
 * fallback.
 */
#ifndef OPENZL_GB300_H
#define OPENZL_GB300_H

#include <stdbool.h>
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
    ZL_ErrorCode_userBuffers_invalidNum = 8,
    ZL_ErrorCode_header_unknown = 10,
    ZL_ErrorCode_frameParameter_unsupported = 11,
    ZL_ErrorCode_corruption = 12,
    ZL_ErrorCode_compressedChecksumWrong = 13,
    ZL_ErrorCode_contentChecksumWrong = 14,
    ZL_ErrorCode_compressionParameter_invalid = 20,
    ZL_ErrorCode_parameter_invalid = 21,
    ZL_ErrorCode_outputID_invalid = 22,
    ZL_ErrorCode_invalidRequest_singleOutputFrameOnly = 23,
    ZL_ErrorCode_graph_invalid = 30,
    ZL_ErrorCode_invalidTransform = 32,
    ZL_ErrorCode_node_unexpected_input_type = 54,
    ZL_ErrorCode_node_invalid = 56,
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
    /* batch API only (no counterpart in the reference): the frames decoded
     * through Huffman and the others each split into this many runs of
     * contiguous frames, decoded as parallel branches at stream priorities
     * that fall with the run (1..8). Default: 2 for batches that decode at
     * least 512 MiB, else 1. */
    OZL_DParam_partsPerKind = 1000,
    /* batch API only: the FSE decoder of the plan's launches until the
     * autotuner chooses: 0 the library's default shapes, 1 one lane per
     * stream, 2 one lane per decoder state (four lanes per stream). The
     * bytes decoded are the same. */
    OZL_DParam_fseKernel = 1001,
    /* batch API only: frames holding an FSE stream of at least this many
     * symbols (one lane decodes such a stream serially: the batch's longest
     * chains) decode as their own branch, ahead of the runs in stream
     * priority; 0 turns it off. Default: 16000 for batches that decode at
     * least 512 MiB, else off. */
    OZL_DParam_criticalSymbols = 1002,
    /* batch API only: stream priorities of the branches. 0: a branch's
     * launches share its rank (critical part first, then each kind's runs in
     * order); 1: every element-wise launch ahead of all entropy decoding. */
    OZL_DParam_schedule = 1003,
    /* batch API only: rounds of contiguous frames of about equal decoded
     * bytes in ozl_gpu_batch_run_host (1..16, default 16); each round's
     * outputs go down as soon as it is decoded. */
    OZL_DParam_hostRounds = 1004,
    /* batch API only: rounds of ozl_gpu_batch_run_host that decode at once
     * (round r starts after round r - depth has decoded; 0 = all at once;
     * default 6) */
    OZL_DParam_hostDepth = 1005,
} ZL_DParam;

typedef enum {
    ZL_TernaryParam_auto = 0,
    ZL_TernaryParam_enable = 1,
    ZL_TernaryParam_disable = 2,
} ZL_TernaryParam;

/* zl_decompress.h:80. A DCtx is bound to the CUDA device current when it is
 * created: its calls decode there whatever device is current at the call,
 * and give the caller's current device back. */
ZL_DCtx* ZL_DCtx_create(void);
/* zl_decompress.h:87 */
void ZL_DCtx_free(ZL_DCtx* dctx);
/* zl_decompress.h:140 */
ZL_Report ZL_DCtx_setParameter(ZL_DCtx* dctx, ZL_DParam param, int value);
/* zl_decompress.h:149: the value set, 0 when unset */
int ZL_DCtx_getParameter(const ZL_DCtx* dctx, ZL_DParam param);
/* zl_decompress.h:159: every parameter back to its default */
ZL_Report ZL_DCtx_resetParameters(ZL_DCtx* dctx);
/* zl_decompress.h:188 */
const char* ZL_DCtx_getErrorContextString(const ZL_DCtx* dctx, ZL_Report report);
/* zl_decompress.h:230: host buffers in and out; decoding runs on cuda:0. */
ZL_Report ZL_DCtx_decompress(ZL_DCtx* dctx, void* dst, size_t dstCapacity,
                             const void* compressed, size_t cSize);
/* zl_decompress.h:32: one-shot variant with an internal context. */
ZL_Report ZL_decompress(void* dst, size_t dstCapacity, const void* compressed, size_t cSize);

/* ------------------------------------------------------------------ */
/* Typed decompression (include/openzl/zl_decompress.h:358-599). */
typedef struct {
    ZL_Type type;                  /* type of the output */
    uint32_t fixedWidth;           /* element width in bytes */
    uint64_t decompressedByteSize; /* decompressed size in bytes */
    uint64_t numElts;              /* number of elements */
} ZL_OutputInfo;

/* zl_decompress.h:388: single typed output into a caller buffer. */
ZL_Report ZL_DCtx_decompressTyped(ZL_DCtx* dctx, ZL_OutputInfo* outputInfo, void* dst, size_t dstByteCapacity,
                                  const void* compressed, size_t cSize);

typedef struct ZL_TypedBuffer_s ZL_TypedBuffer;
/* zl_decompress.h:418-599 */
ZL_TypedBuffer* ZL_TypedBuffer_create(void);
void ZL_TypedBuffer_free(ZL_TypedBuffer* tbuffer);
ZL_TypedBuffer* ZL_TypedBuffer_createWrapSerial(void* buffer, size_t bufferCapacity);
ZL_TypedBuffer* ZL_TypedBuffer_createWrapStruct(void* structBuffer, size_t structWidth, size_t numStructs);
ZL_TypedBuffer* ZL_TypedBuffer_createWrapNumeric(void* numArray, size_t numWidth, size_t numCapacity);
ZL_Type ZL_TypedBuffer_type(const ZL_TypedBuffer* tbuffer);
size_t ZL_TypedBuffer_byteSize(const ZL_TypedBuffer* tbuffer);
const void* ZL_TypedBuffer_rPtr(const ZL_TypedBuffer* tbuffer);
size_t ZL_TypedBuffer_numElts(const ZL_TypedBuffer* tbuffer);
size_t ZL_TypedBuffer_eltWidth(const ZL_TypedBuffer* tbuffer);
/* zl_decompress.h:590-599: a string output's lengths, numElts of them */
const uint32_t* ZL_TypedBuffer_rStringLens(const ZL_TypedBuffer* tbuffer);
/* zl_decompress.h:505 */
ZL_Report ZL_DCtx_decompressTBuffer(ZL_DCtx* dctx, ZL_TypedBuffer* output, const void* compressed, size_t cSize);
/* zl_decompress.h:527: nbOutputs must equal the frame's output count
 * (userBuffers_invalidNum otherwise); returns the number of outputs. */
ZL_Report ZL_DCtx_decompressMultiTBuffer(ZL_DCtx* dctx, ZL_TypedBuffer* outputs[], size_t nbOutputs,
                                         const void* compressed, size_t cSize);

typedef struct ZL_FrameInfo_s ZL_FrameInfo;
/* zl_decompress.h:290-342 */
ZL_FrameInfo* ZL_FrameInfo_create(const void* compressed, size_t cSize);
void ZL_FrameInfo_free(ZL_FrameInfo* fi);
ZL_Report ZL_FrameInfo_getFormatVersion(const ZL_FrameInfo* fi);
ZL_Report ZL_FrameInfo_getNumOutputs(const ZL_FrameInfo* fi);
ZL_Report ZL_FrameInfo_getOutputType(const ZL_FrameInfo* fi, int outputID);
ZL_Report ZL_FrameInfo_getDecompressedSize(const ZL_FrameInfo* fi, int outputID);
ZL_Report ZL_FrameInfo_getNumElts(const ZL_FrameInfo* fi, int outputID);

/* ------------------------------------------------------------------ */
/* Graph building and compression (include/openzl/zl_compressor.h,
 * zl_compress.h, zl_opaque_types.h, zl_nodes.h, zl_graphs.h). Node and
 * graph identifiers keep the reference's numeric values, so code written
 * against the reference's headers runs unchanged. Compression runs on the
 * GPU; a graph the GPU encoder does not implement is rejected with
 * ZL_ErrorCode_graph_invalid (there is no CPU path). Frames are format
 * version 23. */
typedef unsigned ZL_IDType;
typedef struct { ZL_IDType nid; } ZL_NodeID;   /* zl_opaque_types.h:28-30 */
typedef struct { ZL_IDType gid; } ZL_GraphID;  /* zl_opaque_types.h:32-34 */
#if defined(__cplusplus)
#define ZL_MAKE_NODE_ID(id) (ZL_NodeID{ (id) })
#define ZL_MAKE_GRAPH_ID(id) (ZL_GraphID{ (id) })
#else
#define ZL_MAKE_NODE_ID(id) ((ZL_NodeID){ .nid = (id) })
#define ZL_MAKE_GRAPH_ID(id) ((ZL_GraphID){ .gid = (id) })
#endif
/* standard nodes (zl_nodes.h, codecs/zl_*.h, compress/private_nodes.h) */
#define ZL_NODE_DELTA_INT ZL_MAKE_NODE_ID(2)
#define ZL_NODE_TRANSPOSE_SPLIT ZL_MAKE_NODE_ID(3)
#define ZL_NODE_ZIGZAG ZL_MAKE_NODE_ID(4)
#define ZL_NODE_BFLOAT16_DECONSTRUCT ZL_MAKE_NODE_ID(7)
#define ZL_NODE_CONVERT_TOKEN_TO_SERIAL ZL_MAKE_NODE_ID(10)
#define ZL_NODE_CONVERT_NUM_TO_TOKEN ZL_MAKE_NODE_ID(11)
#define ZL_NODE_CONVERT_NUM_TO_SERIAL ZL_MAKE_NODE_ID(12)
#define ZL_NODE_BITPACK_INT ZL_MAKE_NODE_ID(53)
/* standard graphs (zl_graphs.h, codecs/zl_*.h) */
#define ZL_GRAPH_ILLEGAL ZL_MAKE_GRAPH_ID(0)
#define ZL_GRAPH_STORE ZL_MAKE_GRAPH_ID(2)
#define ZL_GRAPH_FSE ZL_MAKE_GRAPH_ID(3)
#define ZL_GRAPH_HUFFMAN ZL_MAKE_GRAPH_ID(4)
#define ZL_GRAPH_ENTROPY ZL_MAKE_GRAPH_ID(5)
#define ZL_GRAPH_CONSTANT ZL_MAKE_GRAPH_ID(6)
#define ZL_GRAPH_BITPACK ZL_MAKE_GRAPH_ID(8)
#define ZL_GRAPH_FLATPACK ZL_MAKE_GRAPH_ID(9)

/* zl_compress.h:64-150 */
typedef enum {
    ZL_CParam_stickyParameters = 1,
    ZL_CParam_compressionLevel = 2,
    ZL_CParam_decompressionLevel = 3,
    ZL_CParam_formatVersion = 4,
    ZL_CParam_permissiveCompression = 5,
    ZL_CParam_compressedChecksum = 6,
    ZL_CParam_contentChecksum = 7,
    ZL_CParam_minStreamSize = 11,
} ZL_CParam;

typedef struct ZL_Compressor_s ZL_Compressor;
typedef struct ZL_CCtx_s ZL_CCtx;
typedef struct ZL_TypedRef_s ZL_TypedRef;

/* zl_compressor.h:69, :78 */
ZL_Compressor* ZL_Compressor_create(void);
void ZL_Compressor_free(ZL_Compressor* compressor);
/* zl_compressor.h:151, :162 */
ZL_Report ZL_Compressor_setParameter(ZL_Compressor* compressor, ZL_CParam gcparam, int value);
int ZL_Compressor_getParameter(const ZL_Compressor* compressor, ZL_CParam gcparam);
/* zl_compressor.h:232, :249, :281 */
ZL_GraphID ZL_Compressor_registerStaticGraph_fromNode1o(ZL_Compressor* compressor, ZL_NodeID headNode,
                                                        ZL_GraphID dstGraph);
ZL_GraphID ZL_Compressor_registerStaticGraph_fromPipelineNodes1o(ZL_Compressor* compressor, const ZL_NodeID* nodes,
                                                                 size_t nbNodes, ZL_GraphID dstGraph);
ZL_GraphID ZL_Compressor_registerStaticGraph_fromNode(ZL_Compressor* compressor, ZL_NodeID headNode,
                                                      const ZL_GraphID* dstGraphs, size_t nbDstGraphs);
/* codecs/zl_transpose.h:43 */
ZL_GraphID ZL_Compressor_registerTransposeSplitGraph(ZL_Compressor* cgraph, ZL_GraphID successor);
/* codecs/zl_tokenize.h:67 */
ZL_GraphID ZL_Compressor_registerTokenizeGraph(ZL_Compressor* compressor, ZL_Type inputType, bool sort,
                                               ZL_GraphID alphabetGraph, ZL_GraphID indicesGraph);
/* zl_compressor.h:555 */
ZL_Report ZL_Compressor_selectStartingGraphID(ZL_Compressor* compressor, ZL_GraphID graph);
/* zl_graph_api.h:125: nonzero unless ZL_GRAPH_ILLEGAL */
int ZL_GraphID_isValid(ZL_GraphID graphid);
/* zl_compressor.h:105 */
const char* ZL_Compressor_getErrorContextString(const ZL_Compressor* compressor, ZL_Report report);

/* Custom codecs (zl_ctransform.h:134-359, zl_dtransform.h:79-217). A custom
 * codec runs the caller's host functions and writes a custom transform ID,
 * so it has no GPU form and cannot give the standard codecs' frames. These
 * entry points exist so that callers built against the reference's headers
 * link. Each refuses the registration: the encoders return ZL_NODE_ILLEGAL
 * (reason in ZL_Compressor_getErrorContextString), the decoders
 * ZL_ErrorCode_temporaryLibraryLimitation. As in the reference, the
 * descriptor's opaque pointer is owned by the library even when registration
 * fails, so its free function is called once. The descriptors have the
 * reference's layout; they are opaque here because nothing else reads them. */
#define ZL_NODE_ILLEGAL ZL_MAKE_NODE_ID(0)
typedef struct ZL_TypedEncoderDesc_s ZL_TypedEncoderDesc;
typedef struct ZL_VOEncoderDesc_s ZL_VOEncoderDesc;
typedef struct ZL_MIEncoderDesc_s ZL_MIEncoderDesc;
typedef struct ZL_TypedDecoderDesc_s ZL_TypedDecoderDesc;
typedef struct ZL_VODecoderDesc_s ZL_VODecoderDesc;
typedef struct ZL_MIDecoderDesc_s ZL_MIDecoderDesc;
/* zl_ctransform.h:170, :287, :359 */
ZL_NodeID ZL_Compressor_registerTypedEncoder(ZL_Compressor* cgraph, const ZL_TypedEncoderDesc* ctd);
ZL_NodeID ZL_Compressor_registerVOEncoder(ZL_Compressor* cgraph, const ZL_VOEncoderDesc* ctd);
ZL_NodeID ZL_Compressor_registerMIEncoder(ZL_Compressor* cgraph, const ZL_MIEncoderDesc* ctd);
/* zl_dtransform.h:97, :177, :217 */
ZL_Report ZL_DCtx_registerTypedDecoder(ZL_DCtx* dctx, const ZL_TypedDecoderDesc* dtd);
ZL_Report ZL_DCtx_registerVODecoder(ZL_DCtx* dctx, const ZL_VODecoderDesc* dtd);
ZL_Report ZL_DCtx_registerMIDecoder(ZL_DCtx* dctx, const ZL_MIDecoderDesc* dtd);

/* zl_compress.h:39-53 */
#define ZL_COMPRESSBOUND(s) (((s) * 2) + 512 + 8)
size_t ZL_compressBound(size_t totalSrcSize);
/* zl_compress.h:60-61. A CCtx is bound to the CUDA device current when it is
 * created, like a DCtx. */
ZL_CCtx* ZL_CCtx_create(void);
void ZL_CCtx_free(ZL_CCtx* cctx);
/* zl_compress.h:152, :161, :168 */
ZL_Report ZL_CCtx_setParameter(ZL_CCtx* cctx, ZL_CParam gcparam, int value);
int ZL_CCtx_getParameter(const ZL_CCtx* cctx, ZL_CParam gcparam);
ZL_Report ZL_CCtx_resetParameters(ZL_CCtx* cctx);
/* zl_compressor.h:597 */
ZL_Report ZL_CCtx_refCompressor(ZL_CCtx* cctx, const ZL_Compressor* compressor);
/* zl_compress.h:194: serial input */
ZL_Report ZL_CCtx_compress(ZL_CCtx* cctx, void* dst, size_t dstCapacity, const void* src, size_t srcSize);
/* zl_compress.h:213 */
const char* ZL_CCtx_getErrorContextString(const ZL_CCtx* cctx, ZL_Report report);
/* zl_compress.h:274 */
ZL_Report ZL_CCtx_compressTypedRef(ZL_CCtx* cctx, void* dst, size_t dstCapacity, const ZL_TypedRef* input);
/* zl_compress.h:295: one input per frame here. Several inputs need a
 * function graph (ZL_Compressor_registerFunctionGraph, a host callback that
 * routes each input), which the GPU encoder has no form of; nbInputs > 1
 * returns ZL_ErrorCode_temporaryLibraryLimitation. Frames of several
 * outputs decode (ZL_DCtx_decompressMultiTBuffer). */
ZL_Report ZL_CCtx_compressMultiTypedRef(ZL_CCtx* cctx, void* dst, size_t dstCapacity, const ZL_TypedRef* inputs[],
                                        size_t nbInputs);
/* zl_compress.h:313-394 */
ZL_TypedRef* ZL_TypedRef_createSerial(const void* src, size_t srcSize);
ZL_TypedRef* ZL_TypedRef_createStruct(const void* start, size_t structWidth, size_t structCount);
ZL_TypedRef* ZL_TypedRef_createNumeric(const void* start, size_t numWidth, size_t numCount);
void ZL_TypedRef_free(ZL_TypedRef* tref);

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
/* Frame header summary (no counterpart in the reference; the fields its
 * ZL_FrameInfo and ZL_getDecompressedSize give, src/openzl/decompress/
 * decode_frameheader.c:58-370, plus what the batch API needs to place the
 * outputs). status is 0 or the ZL error code of the header parse. */
typedef struct {
    int32_t status;
    uint32_t formatVersion;
    uint32_t nbOutputs;
    uint32_t flags;          /* bit 0 content checksum, bit 1 compressed checksum, bit 2 header checksum byte */
    uint64_t headerBytes;    /* offset of the first block */
    uint64_t output0Bytes;   /* decompressed bytes of output 0 (a string output: its content) */
    uint64_t extent;         /* destination bytes of the batch API: every output at a 16-byte-aligned
                                offset, a string output's 4-byte lengths after its content */
    int32_t output0Type;     /* ZL_Type of output 0 */
    uint32_t reserved;
} OZL_FrameInfo;
/* The summary of one frame in host memory, parsed on the host. */
ZL_Report ozl_frame_info(const void* frame, size_t frameSize, OZL_FrameInfo* info);
/* The summaries of n frames in device memory, parsed on the device (one
 * thread per frame): d_frames[i] (a device array of device pointers) holds
 * d_frameSizes[i] bytes (a device array); the records go to d_info[i]
 * (device memory). Enqueued on `stream`; nothing is read back. Equal to
 * ozl_frame_info on the same bytes. Returns n. */
ZL_Report ozl_gpu_frame_info(const void* const* d_frames, const uint64_t* d_frameSizes, size_t n,
                             OZL_FrameInfo* d_info, void* stream);

typedef struct OZL_GpuBatch_s OZL_GpuBatch;
OZL_GpuBatch* ozl_gpu_batch_create(void);
void ozl_gpu_batch_free(OZL_GpuBatch* b);
/* Output layout of one frame for the batch API (no counterpart in the
 * reference; its ZL_FrameInfo gives counts, types and sizes but not element
 * widths, which sit in the block headers). Plans the frame on the host and
 * writes, for the first `capacity` outputs, the offset in the destination,
 * the size in bytes (a string output: its content), the type, the element
 * width (1 for serial and string outputs), the number of elements (strings
 * for a string output) and, for a string output, the offset of its 4-byte
 * lengths (0 otherwise); any array may be NULL. Returns the number of
 * outputs and writes the destination bytes needed to *extent. */
ZL_Report ozl_frame_outputs(const void* frame, size_t frameSize, size_t capacity, uint64_t* offsets,
                            uint64_t* sizes, int* types, uint32_t* widths, uint64_t* counts,
                            uint64_t* lensOffsets, uint64_t* extent);
/* Sets a DParam for subsequent plans (same meaning as ZL_DCtx_setParameter). */
ZL_Report ozl_gpu_batch_setParameter(OZL_GpuBatch* b, ZL_DParam param, int value);
/* Plans the decode of nbFrames frames. h_frames[i]: host copy (planning);
 * d_frames[i]: device copy; d_dsts[i]/dstCapacities[i]: device outputs.
 * A frame with several outputs writes them one after another into its
 * destination, each at a 16-byte-aligned offset (ozl_frame_outputs gives the
 * layout). Returns the total destination bytes. Allocates device scratch
 * sized for the plan; reuses it across runs. */
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
/* Concurrency timeline: runs the planned batch once without a graph, its
 * parallel branches as ozl_gpu_batch_run does, with a timing event before
 * and after every launch on its branch's stream. Writes 5 floats per launch
 * (part order) to rows[5 i ..]: branch, codec family, dependency level, the
 * ms from the run's start at which its stream reached the launch, and the ms
 * at which the launch ended; for i < capacity. Returns the number of
 * launches. Synchronizes `stream`. */
ZL_Report ozl_gpu_batch_timeline(OZL_GpuBatch* b, void* stream, float* rows, size_t capacity);
/* Host-buffer timeline: one ozl_gpu_batch_run_host run without a graph, with
 * timing events. Writes 3 floats per round to rows[3 r ..] (r < capacity):
 * the ms from the run's start at which round r's frames were in, its decode
 * ended and its outputs were out. Returns the number of rounds (0 when the
 * frames are not laid out in order and the run is not split into rounds).
 * Synchronizes `stream`. */
ZL_Report ozl_gpu_batch_host_timeline(OZL_GpuBatch* b, const void* h_in, size_t inBytes, void* h_out,
                                      size_t outBytes, void* stream, float* rows, size_t capacity);
/* Name of a codec family reported by ozl_gpu_batch_profile. */
const char* ozl_gpu_kind_name(int kind);
/* Autotuner: times the candidate launch shapes (chunks per CTA of the FSE
 * and Huffman launches) of the planned batch on `stream`, best of `reps`,
 * after one full run; keeps the fastest per launch for the following runs
 * (the next graph run recaptures). Writes the chosen shape of launch i to
 * shapes[i] (0 = not tunable) for i < capacity. Returns the number of
 * planned launches. Results do not depend on the shapes. */
ZL_Report ozl_gpu_batch_autotune(OZL_GpuBatch* b, void* stream, int reps, uint32_t* shapes, size_t capacity);
/* Host-buffer run of a planned batch whose device frames sit back to back
 * from d_frames[0] and whose outputs sit back to back from d_dsts[0] (as
 * passed to ozl_gpu_batch_plan): copies h_in (inBytes) to the device, runs
 * the decode, copies the outputs to h_out (outBytes) and synchronizes.
 * When both images hold the frames in increasing order, the copies in, the
 * decode and the copies out overlap in rounds of contiguous frames (pinned
 * h_in / h_out make the copies asynchronous); otherwise they run one after
 * another. Returns the total decompressed size. */
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
    OZL_GRAPH_ENTROPY = 17,         /* ZL_GRAPH_ENTROPY (FSE or Huffman per chunk) */
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
/* Batches of 64 MiB or more are encoded in `parts` (1..16, default 8) runs of
 * contiguous frames of about equal bytes, each on its own host thread and
 * CUDA stream, so that one part's host work overlaps another's kernels; each
 * part's parallel host phases use its share of the cores (-parts: all of
 * them). The frames do not depend on it. */
ZL_Report ozl_gpu_encoder_setParts(OZL_GpuEncoder* e, int parts);
/* Wall-clock milliseconds of the last ozl_gpu_compress_batch's phases, in
 * order: front end (GPU), graph discovery (host), histograms (GPU), codec
 * decisions and coding tables, entropy bitstreams (GPU), graph replay
 * (host), frame assembly and checksums (GPU); a phase that ends in a stream
 * synchronize includes its device work. Writes ms[i] for i < capacity and
 * returns the number of phases (7). */
ZL_Report ozl_gpu_encoder_phases(const OZL_GpuEncoder* e, float* ms, size_t capacity);

/* XXH3-64 (seed 0), the hash behind OpenZL's checksums, of `len` bytes of
 * device memory; computed on the GPU. Returns the hash in the report value. */
ZL_Report ozl_gpu_xxh3_64(const void* d_data, size_t len, void* stream);

/* Allocation-free variant of ozl_gpu_xxh3_64 (no counterpart in the
 * reference), for callers that cannot call cudaMalloc: code whose device
 * memory is owned by another allocator (a framework's caching pool with a
 * fixed budget), or that runs where cudaMalloc's implicit synchronization and
 * possible failure are not allowed (a latency-bound request path). The same
 * hash and kernels, with their scratch (task, block list, per-1 KiB block
 * sums and the result) in one fixed file-scope device array of
 * OZL_XXH3_STATIC_SCRATCH bytes per device instead of a per-call allocation;
 * every GPU that loads the library holds that array until the process exits.
 * Accepts at most OZL_XXH3_STATIC_MAX_LEN bytes; longer inputs return
 * ZL_ErrorCode_srcSize_tooLarge without touching the device. Calls no
 * allocating routine: each call looks up the array's device address in the
 * current device's context (cudaGetSymbolAddress), so the entry point stays
 * valid across a cudaDeviceReset. Every call on a device shares the
 * array and the array keeps the last call's contents (what must start at
 * zero is cleared by each call): calls whose work overlaps on the GPU (other
 * streams, other host threads) race and must be serialized by the caller.
 * Synchronizes `stream`; returns the hash in the report value. */
#define OZL_XXH3_STATIC_MAX_LEN ((size_t)32 << 20)
#define OZL_XXH3_STATIC_SCRATCH ((size_t)256 + ((size_t)32 << 10) * 72)
ZL_Report ozl_gpu_xxh3_64_static(const void* d_data, size_t len, void* stream);

/* Serving loop (no counterpart in the reference): continuous batching of
 * decompress and compress requests with host buffers on the current device.
 * `hbmBudget` bytes of device memory are allocated once as a pool shared by
 * the workers, and hold each batch's inputs and outputs. A free worker (its
 * own CUDA stream) admits the oldest queued request as soon as a block of its
 * size is free in the pool, with the next queued requests of the same kind
 * that fit the same block (a batch is at most hbmBudget / nbWorkers unless
 * its first request alone is larger), and runs them as one batch, so batches
 * of different workers overlap on the GPU. `checksums` selects whether frames
 * carry (compress) and have verified (decompress) both checksums. Host
 * buffers must stay valid until the request completes. A request needs its
 * input plus its output (decoded size, or ZL_compressBound of the input) in
 * the pool; one larger than hbmBudget completes with
 * ZL_ErrorCode_srcSize_tooLarge. Returns NULL if the pool cannot be
 * allocated. */
typedef struct OZL_Server_s OZL_Server;
OZL_Server* ozl_server_create(size_t hbmBudget, int nbWorkers, int checksums);
/* Drains the queue, then stops the workers. */
void ozl_server_free(OZL_Server* server);
/* Returns the request id (> 0), or 0 when the arguments are invalid. */
uint64_t ozl_server_submit_decompress(OZL_Server* server, const void* frame, size_t frameSize, void* dst,
                                      size_t dstCapacity);
/* eltWidth 0 = serial bytes; recipe: OZL_GRAPH_* */
uint64_t ozl_server_submit_compress(OZL_Server* server, const void* src, size_t nbElts, int eltWidth, int recipe,
                                    void* dst, size_t dstCapacity);
/* Completed requests, oldest first: up to `max` ids, results (decoded or
 * frame size, or an error) and latencies from submission in microseconds.
 * Waits up to waitMs for a first completion. Returns the count. */
size_t ozl_server_poll(OZL_Server* server, uint64_t* ids, ZL_Report* results, double* latencyUs, size_t max,
                       int waitMs);
/* Cumulative worker statistics since the server was created, summed over
 * its workers: decode batches, decode requests, seconds planning decode
 * batches on the host, seconds running them (launch to completion, copies
 * out included), encode batches, encode requests, seconds encoding, and
 * seconds workers waited for a request or for free memory. Writes
 * out[i] for i < capacity; returns the number of values (8). */
size_t ozl_server_stats(OZL_Server* server, double* out, size_t capacity);
/* Requests submitted and not yet returned by ozl_server_poll. */
size_t ozl_server_in_flight(OZL_Server* server);

/* Library build identification (for load checks). */
const char* ozl_gpu_version(void);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif
#endif
