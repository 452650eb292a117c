/* Thin ctypes-facing driver over the reference OpenZL library built by
 * oracle/ref.mk. Test infrastructure only: fixture generators and parity
 * tests call it to make reference frames and to decode frames with the
 * reference's universal decoder. It is never linked into the product.
 *
 * Graph "recipes" (numbers below) name the codec graphs the numeric path
 * uses; each is built with the reference's public graph API exactly as a
 * user of the reference would build it.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "openzl/codecs/zl_bitpack.h"
#include "openzl/codecs/zl_conversion.h"
#include "openzl/codecs/zl_delta.h"
#include "openzl/codecs/zl_entropy.h"
#include "openzl/codecs/zl_float_deconstruct.h"
#include "openzl/codecs/zl_store.h"
#include "openzl/codecs/zl_tokenize.h"
#include "openzl/codecs/zl_transpose.h"
#include "openzl/codecs/zl_zigzag.h"
#include "openzl/compress/private_nodes.h"
#include "openzl/openzl.h"
#include "openzl/zl_compressor.h"
#include "openzl/zl_reflection.h"

enum {
    R_STORE            = 0,  /* store */
    R_DZ_TSPLIT_FSE    = 1,  /* delta -> zigzag -> num_to_token -> tsplit(FSE) */
    R_DZ_BITPACK_HUF   = 2,  /* delta -> zigzag -> bitpack_int -> HUFFMAN */
    R_D_TSPLIT_FSE     = 3,  /* delta -> num_to_token -> tsplit(FSE) */
    R_D_BITPACK_HUF    = 4,  /* delta -> bitpack_int -> HUFFMAN */
    R_TOKENIZE         = 5,  /* tokenize(numeric) alphabet->STORE, idx->bitpack->HUF */
    R_BF16             = 6,  /* bf16 deconstruct: signfrac->STORE, exponent->FSE */
    R_FSE              = 7,  /* FSE graph directly */
    R_HUFFMAN          = 8,  /* HUFFMAN graph directly */
    R_DELTA_STORE      = 9,  /* delta -> store */
    R_ZIGZAG_STORE     = 10, /* zigzag -> store */
    R_BITPACK_STORE    = 11, /* bitpack_int -> store */
    R_TSPLIT_STORE     = 12, /* num_to_token -> tsplit(STORE) */
    R_CONSTANT         = 13, /* constant graph */
    R_FLATPACK         = 14, /* flatpack graph */
    R_BITPACK_GRAPH    = 15, /* public bitpack graph */
    R_TOKENIZE_SORTED  = 16, /* tokenize(numeric, sorted) alphabet->STORE, idx->bitpack->HUF */
    R_ENTROPY          = 17, /* ENTROPY graph directly (FSE or Huffman per chunk) */
};

static ZL_GraphID build(ZL_Compressor* c, int recipe, int eltWidth)
{
    (void)eltWidth;
    switch (recipe) {
        case R_STORE:
            return ZL_GRAPH_STORE;
        case R_DZ_TSPLIT_FSE: {
            ZL_GraphID ts = ZL_Compressor_registerTransposeSplitGraph(c, ZL_GRAPH_FSE);
            ZL_NodeID n[3] = { ZL_NODE_DELTA_INT, ZL_NODE_ZIGZAG, ZL_NODE_CONVERT_NUM_TO_TOKEN };
            return ZL_Compressor_registerStaticGraph_fromPipelineNodes1o(c, n, 3, ts);
        }
        case R_DZ_BITPACK_HUF: {
            ZL_GraphID bp = ZL_Compressor_registerStaticGraph_fromNode1o(
                    c, ZL_NODE_BITPACK_INT, ZL_GRAPH_HUFFMAN);
            ZL_NodeID n[2] = { ZL_NODE_DELTA_INT, ZL_NODE_ZIGZAG };
            return ZL_Compressor_registerStaticGraph_fromPipelineNodes1o(c, n, 2, bp);
        }
        case R_D_TSPLIT_FSE: {
            ZL_GraphID ts = ZL_Compressor_registerTransposeSplitGraph(c, ZL_GRAPH_FSE);
            ZL_NodeID n[2] = { ZL_NODE_DELTA_INT, ZL_NODE_CONVERT_NUM_TO_TOKEN };
            return ZL_Compressor_registerStaticGraph_fromPipelineNodes1o(c, n, 2, ts);
        }
        case R_D_BITPACK_HUF: {
            ZL_GraphID bp = ZL_Compressor_registerStaticGraph_fromNode1o(
                    c, ZL_NODE_BITPACK_INT, ZL_GRAPH_HUFFMAN);
            return ZL_Compressor_registerStaticGraph_fromNode1o(c, ZL_NODE_DELTA_INT, bp);
        }
        case R_TOKENIZE:
        case R_TOKENIZE_SORTED: {
            ZL_GraphID bp = ZL_Compressor_registerStaticGraph_fromNode1o(
                    c, ZL_NODE_BITPACK_INT, ZL_GRAPH_HUFFMAN);
            return ZL_Compressor_registerTokenizeGraph(
                    c, ZL_Type_numeric, recipe == R_TOKENIZE_SORTED, ZL_GRAPH_STORE, bp);
        }
        case R_BF16: {
            ZL_GraphID succ[2] = { ZL_GRAPH_STORE, ZL_GRAPH_FSE };
            return ZL_Compressor_registerStaticGraph_fromNode(
                    c, ZL_NODE_BFLOAT16_DECONSTRUCT, succ, 2);
        }
        case R_FSE:
            return ZL_GRAPH_FSE;
        case R_HUFFMAN:
            return ZL_GRAPH_HUFFMAN;
        case R_ENTROPY:
            return ZL_GRAPH_ENTROPY;
        case R_DELTA_STORE:
            return ZL_Compressor_registerStaticGraph_fromNode1o(c, ZL_NODE_DELTA_INT, ZL_GRAPH_STORE);
        case R_ZIGZAG_STORE:
            return ZL_Compressor_registerStaticGraph_fromNode1o(c, ZL_NODE_ZIGZAG, ZL_GRAPH_STORE);
        case R_BITPACK_STORE:
            return ZL_Compressor_registerStaticGraph_fromNode1o(c, ZL_NODE_BITPACK_INT, ZL_GRAPH_STORE);
        case R_TSPLIT_STORE: {
            ZL_GraphID ts = ZL_Compressor_registerTransposeSplitGraph(c, ZL_GRAPH_STORE);
            return ZL_Compressor_registerStaticGraph_fromNode1o(c, ZL_NODE_CONVERT_NUM_TO_TOKEN, ts);
        }
        case R_CONSTANT:
            return ZL_GRAPH_CONSTANT;
        case R_FLATPACK:
            return ZL_GRAPH_FLATPACK;
        case R_BITPACK_GRAPH:
            return ZL_GRAPH_BITPACK;
        default:
            return ZL_GRAPH_ILLEGAL;
    }
}

size_t ref_compressBound(size_t n) { return ZL_compressBound(n); }

/* eltWidth 0 => serial input; 1/2/4/8 => numeric. Returns compressed size,
 * or -(error code) on failure. */
int64_t ref_compress(int recipe, const void* src, size_t nbElts, int eltWidth,
                     void* dst, size_t dstCap, int checksums, int formatVersion)
{
    ZL_Compressor* c = ZL_Compressor_create();
    if (!c) return -1;
    if (formatVersion <= 0) formatVersion = ZL_MAX_FORMAT_VERSION;
    ZL_Compressor_setParameter(c, ZL_CParam_formatVersion, formatVersion);
    if (!checksums) {
        ZL_Compressor_setParameter(c, ZL_CParam_contentChecksum, ZL_TernaryParam_disable);
        ZL_Compressor_setParameter(c, ZL_CParam_compressedChecksum, ZL_TernaryParam_disable);
    }
    ZL_GraphID g = build(c, recipe, eltWidth);
    if (!ZL_GraphID_isValid(g)) { ZL_Compressor_free(c); return -2; }
    ZL_Report r = ZL_Compressor_selectStartingGraphID(c, g);
    if (ZL_isError(r)) { ZL_Compressor_free(c); return -3; }
    ZL_CCtx* cc = ZL_CCtx_create();
    ZL_CCtx_refCompressor(cc, c);
    ZL_TypedRef* tr = eltWidth == 0 ? ZL_TypedRef_createSerial(src, nbElts)
                                    : ZL_TypedRef_createNumeric(src, (size_t)eltWidth, nbElts);
    r = ZL_CCtx_compressTypedRef(cc, dst, dstCap, tr);
    int64_t ret = ZL_isError(r) ? -(int64_t)ZL_errorCode(r) - 1000 : (int64_t)ZL_validResult(r);
    ZL_TypedRef_free(tr);
    ZL_CCtx_free(cc);
    ZL_Compressor_free(c);
    return ret;
}

/* Multi-input frames: a function graph sends input i to the graph of
 * recipe i, each registered as one of its custom graphs. */
static ZL_Report multi_graph(ZL_Graph* g, ZL_Edge* inputs[], size_t nbInputs)
{
    ZL_GraphIDList const cg = ZL_Graph_getCustomGraphs(g);
    if (cg.nbGraphIDs < nbInputs) return ZL_returnError(ZL_ErrorCode_graph_invalid);
    for (size_t i = 0; i < nbInputs; i++) {
        ZL_Report const r = ZL_Edge_setDestination(inputs[i], cg.graphids[i]);
        if (ZL_isError(r)) return r;
    }
    return ZL_returnSuccess();
}

/* nb inputs (eltWidths[i] 0 => serial), compressed together into one frame
 * whose outputs come back in input order. Returns the frame size or
 * -(error code). */
int64_t ref_compress_multi(int nb, const int* recipes, const void* const* srcs, const size_t* nbElts,
                           const int* eltWidths, void* dst, size_t dstCap, int checksums, int formatVersion)
{
    if (nb <= 0 || nb > 64) return -1;
    ZL_Compressor* c = ZL_Compressor_create();
    if (!c) return -1;
    if (formatVersion <= 0) formatVersion = ZL_MAX_FORMAT_VERSION;
    ZL_Compressor_setParameter(c, ZL_CParam_formatVersion, formatVersion);
    if (!checksums) {
        ZL_Compressor_setParameter(c, ZL_CParam_contentChecksum, ZL_TernaryParam_disable);
        ZL_Compressor_setParameter(c, ZL_CParam_compressedChecksum, ZL_TernaryParam_disable);
    }
    ZL_GraphID gids[64];
    ZL_Type masks[64];
    for (int i = 0; i < nb; i++) {
        gids[i] = build(c, recipes[i], eltWidths[i]);
        if (!ZL_GraphID_isValid(gids[i])) { ZL_Compressor_free(c); return -2; }
        masks[i] = ZL_Type_serial | ZL_Type_numeric | ZL_Type_struct;
    }
    ZL_FunctionGraphDesc const d = {
        .name = "per_input",
        .graph_f = multi_graph,
        .inputTypeMasks = masks,
        .nbInputs = (size_t)nb,
        .customGraphs = gids,
        .nbCustomGraphs = (size_t)nb,
    };
    ZL_GraphID const g = ZL_Compressor_registerFunctionGraph(c, &d);
    ZL_Report r = ZL_Compressor_selectStartingGraphID(c, g);
    if (ZL_isError(r)) { ZL_Compressor_free(c); return -3; }
    ZL_CCtx* cc = ZL_CCtx_create();
    ZL_CCtx_refCompressor(cc, c);
    ZL_TypedRef* trs[64];
    for (int i = 0; i < nb; i++)
        trs[i] = eltWidths[i] == 0 ? ZL_TypedRef_createSerial(srcs[i], nbElts[i])
                                   : ZL_TypedRef_createNumeric(srcs[i], (size_t)eltWidths[i], nbElts[i]);
    r = ZL_CCtx_compressMultiTypedRef(cc, dst, dstCap, (const ZL_TypedRef**)trs, (size_t)nb);
    int64_t ret = ZL_isError(r) ? -(int64_t)ZL_errorCode(r) - 1000 : (int64_t)ZL_validResult(r);
    for (int i = 0; i < nb; i++) ZL_TypedRef_free(trs[i]);
    ZL_CCtx_free(cc);
    ZL_Compressor_free(c);
    return ret;
}

/* One string input (nbStrings lengths over `content`) through recipe
 * 100 + k: 100 store, 101 separate_string_components -> (content: FSE,
 * lengths: store), 102 separate components -> (content: Huffman, lengths:
 * delta -> bitpack -> Huffman). Returns the frame size or -(error code). */
int64_t ref_compress_string(int recipe, const void* content, size_t contentSize, const uint32_t* lens,
                            size_t nbStrings, void* dst, size_t dstCap, int checksums, int formatVersion)
{
    ZL_Compressor* c = ZL_Compressor_create();
    if (!c) return -1;
    if (formatVersion <= 0) formatVersion = ZL_MAX_FORMAT_VERSION;
    ZL_Compressor_setParameter(c, ZL_CParam_formatVersion, formatVersion);
    if (!checksums) {
        ZL_Compressor_setParameter(c, ZL_CParam_contentChecksum, ZL_TernaryParam_disable);
        ZL_Compressor_setParameter(c, ZL_CParam_compressedChecksum, ZL_TernaryParam_disable);
    }
    ZL_GraphID g = ZL_GRAPH_STORE;
    if (recipe == 101 || recipe == 102) {
        ZL_GraphID const lensGraph = recipe == 101 ? ZL_GRAPH_STORE : build(c, R_D_BITPACK_HUF, 4);
        ZL_GraphID const succ[2] = { recipe == 101 ? ZL_GRAPH_FSE : ZL_GRAPH_HUFFMAN, lensGraph };
        g = ZL_Compressor_registerStaticGraph_fromNode(c, ZL_NODE_SEPARATE_STRING_COMPONENTS, succ, 2);
    } else if (recipe != 100) {
        ZL_Compressor_free(c);
        return -2;
    }
    ZL_Report r = ZL_Compressor_selectStartingGraphID(c, g);
    if (ZL_isError(r)) { ZL_Compressor_free(c); return -3; }
    ZL_CCtx* cc = ZL_CCtx_create();
    ZL_CCtx_refCompressor(cc, c);
    ZL_TypedRef* tr = ZL_TypedRef_createString(content, contentSize, lens, nbStrings);
    r = ZL_CCtx_compressTypedRef(cc, dst, dstCap, tr);
    int64_t ret = ZL_isError(r) ? -(int64_t)ZL_errorCode(r) - 1000 : (int64_t)ZL_validResult(r);
    ZL_TypedRef_free(tr);
    ZL_CCtx_free(cc);
    ZL_Compressor_free(c);
    return ret;
}

/* Decodes one single-output frame into dst. Writes the output's element
 * width (1 for serial) and type. Returns the decoded byte count or -(code). */
int64_t ref_decompress(const void* src, size_t srcSize, void* dst, size_t dstCap,
                       int* eltWidthOut, int* typeOut)
{
    ZL_DCtx* dc = ZL_DCtx_create();
    ZL_TypedBuffer* tb = ZL_TypedBuffer_create();
    ZL_Report r = ZL_DCtx_decompressTBuffer(dc, tb, src, srcSize);
    int64_t ret;
    if (ZL_isError(r)) {
        ret = -(int64_t)ZL_errorCode(r) - 1000;
    } else {
        size_t bytes = ZL_TypedBuffer_byteSize(tb);
        if (bytes > dstCap) {
            ret = -4;
        } else {
            memcpy(dst, ZL_TypedBuffer_rPtr(tb), bytes);
            if (eltWidthOut) *eltWidthOut = (int)ZL_TypedBuffer_eltWidth(tb);
            if (typeOut) *typeOut = (int)ZL_TypedBuffer_type(tb);
            ret = (int64_t)bytes;
        }
    }
    ZL_TypedBuffer_free(tb);
    ZL_DCtx_free(dc);
    return ret;
}

/* Decodes a frame into a caller buffer repeatedly (timing helper). Returns
 * the decoded byte count of the last call or -(code). */
int64_t ref_decompress_into(const void* src, size_t srcSize, void* dst, size_t dstCap, int reps)
{
    ZL_DCtx* dc = ZL_DCtx_create();
    int64_t ret = -1;
    for (int i = 0; i < reps; i++) {
        ZL_OutputInfo info;
        ZL_Report r = ZL_DCtx_decompressTyped(dc, &info, dst, dstCap, src, srcSize);
        ret = ZL_isError(r) ? -(int64_t)ZL_errorCode(r) - 1000 : (int64_t)ZL_validResult(r);
        if (ret < 0) break;
    }
    ZL_DCtx_free(dc);
    return ret;
}

/* Writes the frame's decoder list as text (one line per codec: name,
 * transform id, header size, nb inputs/outputs). Returns the number of
 * codecs, or a negative code. */
int64_t ref_describe(const void* src, size_t srcSize, char* out, size_t outCap)
{
    ZL_ReflectionCtx* rc = ZL_ReflectionCtx_create();
    ZL_Report r = ZL_ReflectionCtx_setCompressedFrame(rc, src, srcSize);
    if (ZL_isError(r)) { ZL_ReflectionCtx_free(rc); return -(int64_t)ZL_errorCode(r) - 1000; }
    size_t n = ZL_ReflectionCtx_getNumCodecs_lastChunk(rc);
    size_t pos = 0;
    for (size_t i = 0; i < n && pos + 256 < outCap; i++) {
        const ZL_CodecInfo* ci = ZL_ReflectionCtx_getCodec_lastChunk(rc, i);
        pos += (size_t)snprintf(out + pos, outCap - pos, "%s id=%u hdr=%zu in=%zu out=%zu+%zu\n",
                ZL_CodecInfo_getName(ci), (unsigned)ZL_CodecInfo_getCodecID(ci),
                ZL_CodecInfo_getHeaderSize(ci),
                ZL_CodecInfo_getNumInputs(ci), ZL_CodecInfo_getNumOutputs(ci),
                ZL_CodecInfo_getNumVariableOutputs(ci));
    }
    ZL_ReflectionCtx_free(rc);
    return (int64_t)n;
}

/* XXH3-64 as the reference library computes it (its vendored xxhash). */
#include "openzl/shared/xxhash.h"
uint64_t ref_xxh3_64(const void* src, size_t len) { return XXH3_64bits(src, len); }
