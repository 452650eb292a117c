/* A C program written against the reference's own public headers (the
 * include/openzl headers). It is linked twice: against libopenzl_gb300.so and,
 * where it was built, against the reference library, and the two runs must
 * print the same results for every call both libraries implement alike.
 *
 * It uses only entry points that need no GPU: frame inspection, ZL_Report
 * handling through the headers' inline accessors, context parameters,
 * host-side refusals, graph building. Each result is printed as one line,
 * "<call>: err=<0|1> code=<error code> value=<value>". Lines after
 * "-- custom codecs" differ by design: the reference registers custom codecs,
 * this library refuses them (and still releases the opaque pointer).
 *
 *   ref_header_caller <frame.zl>
 */
#include "openzl/codecs/zl_transpose.h"
#include "openzl/zl_compress.h"
#include "openzl/zl_compressor.h"
#include "openzl/zl_ctransform.h"
#include "openzl/zl_decompress.h"
#include "openzl/zl_dtransform.h"
#include "openzl/zl_graph_api.h"

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

static void show(const char* what, ZL_Report r)
{
    printf("%s: err=%d code=%d value=%zu\n", what, ZL_isError(r), (int)ZL_errorCode(r),
           ZL_isError(r) ? (size_t)0 : ZL_validResult(r));
}

static void showInt(const char* what, long v) { printf("%s: %ld\n", what, v); }

static int freed;
static void free_opaque(void* freeOpaquePtr, void* ptr)
{
    (void)freeOpaquePtr;
    freed += ptr == (void*)&freed ? 1 : 100;
}

static ZL_Report dec_fn(ZL_Decoder* d, const ZL_Input* src[])
{
    (void)d;
    (void)src;
    return ZL_returnSuccess();
}

static ZL_Report enc_fn(ZL_Encoder* e, const ZL_Input* in)
{
    (void)e;
    (void)in;
    return ZL_returnSuccess();
}

int main(int argc, char** argv)
{
    if (argc != 2) return 2;
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    static uint8_t frame[1 << 21];
    size_t const n = fread(frame, 1, sizeof(frame), f);
    fclose(f);

    /* frame inspection */
    show("getDecompressedSize", ZL_getDecompressedSize(frame, n));
    show("getCompressedSize", ZL_getCompressedSize(frame, n));
    show("getCompressedSize(truncated)", ZL_getCompressedSize(frame, 100));
    ZL_FrameInfo* fi = ZL_FrameInfo_create(frame, n);
    showInt("FrameInfo_create", fi != NULL);
    if (fi) {
        show("FrameInfo_getFormatVersion", ZL_FrameInfo_getFormatVersion(fi));
        show("FrameInfo_getNumOutputs", ZL_FrameInfo_getNumOutputs(fi));
        show("FrameInfo_getOutputType", ZL_FrameInfo_getOutputType(fi, 0));
        show("FrameInfo_getDecompressedSize", ZL_FrameInfo_getDecompressedSize(fi, 0));
        ZL_FrameInfo_free(fi);
    }
    static const uint8_t junk[16] = { 0 };
    ZL_Report r = ZL_getDecompressedSize(junk, sizeof junk);
    printf("getDecompressedSize(junk): err=%d\n", ZL_isError(r));
    showInt("toString(junk) set", ZL_ErrorCode_toString(ZL_errorCode(r)) != NULL);

    /* decompression context */
    ZL_DCtx* d = ZL_DCtx_create();
    showInt("DCtx_create", d != NULL);
    show("DCtx_setParameter(sticky)", ZL_DCtx_setParameter(d, ZL_DParam_stickyParameters, 1));
    show("DCtx_setParameter(contentChecksum)",
         ZL_DCtx_setParameter(d, ZL_DParam_checkContentChecksum, ZL_TernaryParam_disable));
    showInt("DCtx_getParameter(sticky)", ZL_DCtx_getParameter(d, ZL_DParam_stickyParameters));
    showInt("DCtx_getParameter(contentChecksum)", ZL_DCtx_getParameter(d, ZL_DParam_checkContentChecksum));
    show("DCtx_resetParameters", ZL_DCtx_resetParameters(d));
    showInt("DCtx_getParameter(sticky) after reset", ZL_DCtx_getParameter(d, ZL_DParam_stickyParameters));
    showInt("DCtx_getParameter(contentChecksum) after reset",
            ZL_DCtx_getParameter(d, ZL_DParam_checkContentChecksum));
    char small[8];
    r = ZL_DCtx_decompress(d, small, sizeof small, frame, n);
    show("DCtx_decompress(8-byte dst)", r);
    showInt("DCtx_getErrorContextString set", ZL_DCtx_getErrorContextString(d, r) != NULL);

    /* graph building with the reference's identifiers */
    ZL_Compressor* c = ZL_Compressor_create();
    showInt("Compressor_create", c != NULL);
    ZL_GraphID const ts = ZL_Compressor_registerTransposeSplitGraph(c, ZL_GRAPH_FSE);
    showInt("registerTransposeSplitGraph valid", ZL_GraphID_isValid(ts));
    ZL_NodeID const nodes[3] = { ZL_NODE_DELTA_INT, ZL_NODE_ZIGZAG, ZL_NODE_CONVERT_NUM_TO_TOKEN };
    ZL_GraphID const g = ZL_Compressor_registerStaticGraph_fromPipelineNodes1o(c, nodes, 3, ts);
    showInt("registerStaticGraph_fromPipelineNodes1o valid", ZL_GraphID_isValid(g));
    showInt("GraphID_isValid(ILLEGAL)", ZL_GraphID_isValid(ZL_GRAPH_ILLEGAL));
    show("Compressor_selectStartingGraphID", ZL_Compressor_selectStartingGraphID(c, g));

    /* compression refuses a missing format version before any work */
    ZL_CCtx* cc = ZL_CCtx_create();
    showInt("CCtx_create", cc != NULL);
    show("CCtx_refCompressor", ZL_CCtx_refCompressor(cc, c));
    static uint32_t vals[1000];
    for (int i = 0; i < 1000; i++) vals[i] = 1000000u + (uint32_t)i * 3u;
    ZL_TypedRef* in = ZL_TypedRef_createNumeric(vals, sizeof vals[0], 1000);
    showInt("TypedRef_createNumeric", in != NULL);
    size_t const cap = ZL_compressBound(sizeof vals);
    showInt("compressBound(4000) >= 4000", cap >= sizeof vals);
    void* dst = malloc(cap);
    r = ZL_CCtx_compressTypedRef(cc, dst, cap, in);
    show("CCtx_compressTypedRef(no formatVersion)", r);
    showInt("CCtx_getErrorContextString set", ZL_CCtx_getErrorContextString(cc, r) != NULL);
    show("CCtx_setParameter(formatVersion)", ZL_CCtx_setParameter(cc, ZL_CParam_formatVersion, 23));
    showInt("CCtx_getParameter(formatVersion)", ZL_CCtx_getParameter(cc, ZL_CParam_formatVersion));
    free(dst);
    ZL_TypedRef_free(in);
    ZL_CCtx_free(cc);

    /* custom codecs: registration results differ by design; the opaque
     * pointer is released exactly once by this library (at once, since it
     * refuses) and by the reference (when the context is freed) */
    printf("-- custom codecs\n");
    static const ZL_Type serial = ZL_Type_serial;
    ZL_TypedDecoderDesc dd = { .gd = { .CTid = 7, .inStreamType = ZL_Type_serial, .outStreamTypes = &serial,
                                       .nbOutStreams = 1 },
                               .transform_f = dec_fn, .name = "custom",
                               .opaque = { .ptr = &freed, .freeOpaquePtr = NULL, .freeFn = free_opaque } };
    show("DCtx_registerTypedDecoder", ZL_DCtx_registerTypedDecoder(d, &dd));
    ZL_TypedEncoderDesc ed = { .gd = { .CTid = 7, .inStreamType = ZL_Type_serial, .outStreamTypes = &serial,
                                       .nbOutStreams = 1 },
                               .transform_f = enc_fn, .name = "custom",
                               .opaque = { .ptr = &freed, .freeFn = free_opaque } };
    ZL_NodeID const nid = ZL_Compressor_registerTypedEncoder(c, &ed);
    showInt("Compressor_registerTypedEncoder illegal", nid.nid == ZL_NODE_ILLEGAL.nid);
    showInt("Compressor_getErrorContextString set", ZL_Compressor_getErrorContextString(c, r) != NULL);
    showInt("opaque released before free", freed);
    ZL_DCtx_free(d);
    ZL_Compressor_free(c);
    showInt("opaque released after free", freed);
    return 0;
}
