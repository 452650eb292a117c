// Graph building and compression entry points (ZL_Compressor, ZL_CCtx,
// ZL_TypedRef), declared in include/openzl_gb300.h with the reference's
// names, prototypes and identifier values (include/openzl/zl_compressor.h,
// zl_compress.h).
//
// A ZL_Compressor records the graphs a caller registers. At compression the
// starting graph is flattened into its chain of nodes and the terminal graph
// they feed, and that chain is matched against the graphs the GPU encoder
// implements (enc_engine.h). Each of those produces the reference's frame for
// the same graph byte for byte. Any other graph is rejected with
// ZL_ErrorCode_graph_invalid: nothing here compresses on the CPU.
#include <cuda_runtime.h>

#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "../../include/openzl_gb300.h"
#include "device_scope.h"
#include "enc_engine.h"

namespace {

ZL_Report ok(size_t v) { return ZL_Report{ ZL_ErrorCode_no_error, v }; }
ZL_Report fail(int code) { return ZL_Report{ ZL_ErrorCode(code), 0 }; }

// standard identifiers (zl_nodes.h, zl_graphs.h, compress/private_nodes.h)
enum : ZL_IDType {
    N_DELTA = 2, N_TSPLIT = 3, N_ZIGZAG = 4, N_BF16 = 7, N_TOKEN_TO_SERIAL = 10, N_NUM_TO_TOKEN = 11,
    N_NUM_TO_SERIAL = 12, N_BITPACK_INT = 53,
};
enum : ZL_IDType {
    G_ILLEGAL = 0, G_STORE = 2, G_FSE = 3, G_HUFFMAN = 4, G_ENTROPY = 5, G_CONSTANT = 6, G_BITPACK = 8, G_FLATPACK = 9,
};
constexpr ZL_IDType kFirstCustomGraph = 1u << 16; // registered graphs get ids from here

constexpr int kNbParams = 16;

struct DevBuf {
    uint8_t* p = nullptr;
    size_t cap = 0;
    ~DevBuf() { if (p) cudaFree(p); }
    bool reserve(size_t bytes)
    {
        if (bytes <= cap) return true;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return false;
        cap = bytes;
        return true;
    }
};

} // namespace

struct ZL_Compressor_s {
    enum Kind { PIPELINE, TSPLIT, TOKENIZE, MULTI };
    struct Graph {
        Kind kind;
        std::vector<ZL_IDType> nodes; // PIPELINE / MULTI: nodes in order
        std::vector<ZL_IDType> succ;  // successor graphs
        ZL_Type type = ZL_Type_numeric;
        bool sort = false;
    };
    std::map<ZL_IDType, Graph> graphs;
    ZL_IDType next = kFirstCustomGraph;
    ZL_IDType start = G_ILLEGAL;
    int params[kNbParams] = {};
    std::string err; // reason of the last failed call on this compressor

    ZL_GraphID add(Graph g)
    {
        ZL_IDType const id = next++;
        graphs.emplace(id, std::move(g));
        return ZL_GraphID{ id };
    }
    bool known(ZL_IDType gid) const
    {
        return gid == G_STORE || gid == G_FSE || gid == G_HUFFMAN || gid == G_ENTROPY || gid == G_CONSTANT
                || gid == G_BITPACK || gid == G_FLATPACK || graphs.count(gid);
    }
    // The node chain from `gid` to its terminal graph, written as a string of
    // tokens; false for shapes that do not reduce to one chain.
    bool flatten(ZL_IDType gid, std::string& out, int depth = 0) const
    {
        if (depth > 32) return false;
        auto it = graphs.find(gid);
        if (it == graphs.end()) {
            switch (gid) {
                case G_STORE: out += "STORE"; return true;
                case G_FSE: out += "FSE"; return true;
                case G_HUFFMAN: out += "HUFFMAN"; return true;
                case G_ENTROPY: out += "ENTROPY"; return true;
                case G_CONSTANT: out += "CONSTANT"; return true;
                case G_BITPACK: out += "BITPACK"; return true;
                case G_FLATPACK: out += "FLATPACK"; return true;
                default: return false;
            }
        }
        const Graph& g = it->second;
        switch (g.kind) {
            case PIPELINE:
                for (ZL_IDType n : g.nodes) {
                    switch (n) {
                        case N_DELTA: out += "delta>"; break;
                        case N_ZIGZAG: out += "zigzag>"; break;
                        case N_NUM_TO_TOKEN: out += "token>"; break;
                        case N_BITPACK_INT: out += "bitpack>"; break;
                        default: return false;
                    }
                }
                return flatten(g.succ[0], out, depth + 1);
            case TSPLIT:
                out += "tsplit(";
                if (!flatten(g.succ[0], out, depth + 1)) return false;
                out += ")";
                return true;
            case TOKENIZE: {
                if (g.type != ZL_Type_numeric) return false; // numeric tokenize
                out += g.sort ? "tokenize_sorted(" : "tokenize(";
                if (!flatten(g.succ[0], out, depth + 1)) return false;
                out += ",";
                if (!flatten(g.succ[1], out, depth + 1)) return false;
                out += ")";
                return true;
            }
            case MULTI: {
                if (g.nodes[0] != N_BF16 || g.succ.size() != 2) return false;
                out += "bf16(";
                if (!flatten(g.succ[0], out, depth + 1)) return false;
                out += ",";
                if (!flatten(g.succ[1], out, depth + 1)) return false;
                out += ")";
                return true;
            }
            default: return false;
        }
    }
};

struct ZL_TypedRef_s {
    ZL_Type type;
    const void* p;
    size_t width;
    size_t count;
};

struct ZL_CCtx_s {
    int device = ozl::currentDevice(); // the device current at creation: every call encodes there
    const ZL_Compressor_s* comp = nullptr;
    int params[kNbParams] = {};
    ozl::EncodeBatch enc;
    DevBuf in, out;
    cudaStream_t stream = nullptr;
    std::string err;
    ~ZL_CCtx_s()
    {
        if (stream) cudaStreamDestroy(stream);
    }
    int param(ZL_CParam p) const
    {
        int const v = params[p];
        return v ? v : (comp ? comp->params[p] : 0);
    }
    void endOp()
    {
        if (!params[ZL_CParam_stickyParameters]) std::memset(params, 0, sizeof(params));
    }
};

namespace {

// GPU encoder recipe of a flattened chain (enc_engine.h Recipe), or -1.
int recipeOf(const std::string& chain)
{
    static const std::map<std::string, int> table = {
        { "STORE", ozl::RC_STORE },
        { "delta>zigzag>token>tsplit(FSE)", ozl::RC_DZ_TSPLIT_FSE },
        { "delta>zigzag>bitpack>HUFFMAN", ozl::RC_DZ_BITPACK_HUF },
        { "delta>token>tsplit(FSE)", ozl::RC_D_TSPLIT_FSE },
        { "delta>bitpack>HUFFMAN", ozl::RC_D_BITPACK_HUF },
        { "FSE", ozl::RC_FSE },
        { "HUFFMAN", ozl::RC_HUFFMAN },
        { "ENTROPY", ozl::RC_ENTROPY },
        { "delta>STORE", ozl::RC_DELTA_STORE },
        { "zigzag>STORE", ozl::RC_ZIGZAG_STORE },
        { "bitpack>STORE", ozl::RC_BITPACK_STORE },
        { "token>tsplit(STORE)", ozl::RC_TSPLIT_STORE },
        { "CONSTANT", ozl::RC_CONSTANT },
        { "FLATPACK", ozl::RC_FLATPACK },
        { "BITPACK", ozl::RC_BITPACK },
        { "tokenize(STORE,bitpack>HUFFMAN)", ozl::RC_TOKENIZE },
        { "tokenize_sorted(STORE,bitpack>HUFFMAN)", ozl::RC_TOKENIZE_SORTED },
        { "bf16(STORE,FSE)", ozl::RC_BF16 },
    };
    auto it = table.find(chain);
    return it == table.end() ? -1 : it->second;
}

bool numericRecipe(int r)
{
    return r == ozl::RC_DZ_TSPLIT_FSE || r == ozl::RC_DZ_BITPACK_HUF || r == ozl::RC_D_TSPLIT_FSE
            || r == ozl::RC_D_BITPACK_HUF || r == ozl::RC_DELTA_STORE || r == ozl::RC_ZIGZAG_STORE
            || r == ozl::RC_BITPACK_STORE || r == ozl::RC_TSPLIT_STORE || r == ozl::RC_TOKENIZE || r == ozl::RC_TOKENIZE_SORTED
            || r == ozl::RC_BF16;
}

ZL_Report compressOne(ZL_CCtx* c, void* dst, size_t cap, const ZL_TypedRef& in)
{
    c->err.clear();
    int const version = c->param(ZL_CParam_formatVersion);
    if (version == 0) {
        c->err = "formatVersion must be set (ZL_CParam_formatVersion)";
        return fail(ZL_ErrorCode_formatVersion_notSet);
    }
    if (version != 23) {
        c->err = "the GPU encoder writes format version 23 only";
        return fail(ZL_ErrorCode_formatVersion_unsupported);
    }
    if (!c->comp || c->comp->start == G_ILLEGAL) {
        c->err = "no compressor with a starting graph is referenced";
        return fail(ZL_ErrorCode_graph_invalid);
    }
    std::string chain;
    int const recipe = c->comp->flatten(c->comp->start, chain) ? recipeOf(chain) : -1;
    if (recipe < 0) {
        c->err = "graph not implemented by the GPU encoder: " + chain;
        return fail(ZL_ErrorCode_graph_invalid);
    }
    bool const serial = in.type == ZL_Type_serial;
    if (numericRecipe(recipe) && in.type != ZL_Type_numeric) {
        c->err = "the graph's first node takes numeric input";
        return fail(ZL_ErrorCode_node_unexpected_input_type);
    }
    if (!serial && in.type != ZL_Type_numeric) {
        c->err = "struct and string inputs are not on the GPU encoder";
        return fail(ZL_ErrorCode_node_unexpected_input_type);
    }
    size_t const w = serial ? 1 : in.width;
    if (!(w == 1 || w == 2 || w == 4 || w == 8)) return fail(ZL_ErrorCode_parameter_invalid);
    size_t const bytes = in.count * w;
    // checksums: the reference's defaults are on; both toggle together here
    int const ck = c->param(ZL_CParam_contentChecksum), cck = c->param(ZL_CParam_compressedChecksum);
    if ((ck == ZL_TernaryParam_disable) != (cck == ZL_TernaryParam_disable)) {
        c->err = "content and compressed checksums must be enabled or disabled together";
        return fail(ZL_ErrorCode_compressionParameter_invalid);
    }
    bool const checksums = ck != ZL_TernaryParam_disable;
    ozl::DeviceScope const onDevice(c->device);
    if (!c->stream && cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        c->err = "no CUDA device";
        return fail(ZL_ErrorCode_GENERIC);
    }
    size_t const bound = ozl::encodeBound(bytes);
    if (!c->in.reserve(bytes + 64) || !c->out.reserve(bound + 64)) {
        c->err = "device allocation failed";
        return fail(ZL_ErrorCode_allocation);
    }
    if (bytes && cudaMemcpyAsync(c->in.p, in.p, bytes, cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
        return fail(ZL_ErrorCode_GENERIC);
    std::vector<ozl::EncFrameSpec> spec{ ozl::EncFrameSpec{ c->in.p, serial ? bytes : in.count, uint32_t(w), serial,
                                                            recipe } };
    uint8_t* outs[1] = { c->out.p };
    size_t caps[1] = { bound };
    std::vector<size_t> sizes;
    int rc = c->enc.compress(spec, outs, caps, checksums, c->stream, sizes, c->err);
    if (rc) return fail(rc);
    if (sizes[0] > cap) {
        c->err = "destination too small (see ZL_compressBound)";
        return fail(ZL_ErrorCode_dstCapacity_tooSmall);
    }
    if (cudaMemcpyAsync(dst, c->out.p, sizes[0], cudaMemcpyDeviceToHost, c->stream) != cudaSuccess
        || cudaStreamSynchronize(c->stream) != cudaSuccess)
        return fail(ZL_ErrorCode_GENERIC);
    return ok(sizes[0]);
}

} // namespace

extern "C" {

ZL_Compressor* ZL_Compressor_create(void)
{
    try {
        return new ZL_Compressor_s();
    } catch (...) {
        return nullptr;
    }
}

void ZL_Compressor_free(ZL_Compressor* c) { delete c; }

ZL_Report ZL_Compressor_setParameter(ZL_Compressor* c, ZL_CParam p, int value)
{
    if (!c || int(p) <= 0 || int(p) >= kNbParams) return fail(ZL_ErrorCode_parameter_invalid);
    c->params[p] = value;
    return ok(0);
}

int ZL_Compressor_getParameter(const ZL_Compressor* c, ZL_CParam p)
{
    if (!c || int(p) <= 0 || int(p) >= kNbParams) return 0;
    return c->params[p];
}

ZL_GraphID ZL_Compressor_registerStaticGraph_fromPipelineNodes1o(ZL_Compressor* c, const ZL_NodeID* nodes,
                                                                 size_t nbNodes, ZL_GraphID dst)
{
    if (!c || (nbNodes && !nodes) || !c->known(dst.gid)) return ZL_GraphID{ G_ILLEGAL };
    ZL_Compressor_s::Graph g{ ZL_Compressor_s::PIPELINE, {}, { dst.gid } };
    for (size_t i = 0; i < nbNodes; i++) g.nodes.push_back(nodes[i].nid);
    return c->add(std::move(g));
}

ZL_GraphID ZL_Compressor_registerStaticGraph_fromNode1o(ZL_Compressor* c, ZL_NodeID head, ZL_GraphID dst)
{
    return ZL_Compressor_registerStaticGraph_fromPipelineNodes1o(c, &head, 1, dst);
}

ZL_GraphID ZL_Compressor_registerStaticGraph_fromNode(ZL_Compressor* c, ZL_NodeID head, const ZL_GraphID* dsts,
                                                      size_t nbDsts)
{
    if (!c || !dsts || nbDsts == 0) return ZL_GraphID{ G_ILLEGAL };
    if (nbDsts == 1) return ZL_Compressor_registerStaticGraph_fromNode1o(c, head, dsts[0]);
    ZL_Compressor_s::Graph g{ ZL_Compressor_s::MULTI, { head.nid }, {} };
    for (size_t i = 0; i < nbDsts; i++) {
        if (!c->known(dsts[i].gid)) return ZL_GraphID{ G_ILLEGAL };
        g.succ.push_back(dsts[i].gid);
    }
    return c->add(std::move(g));
}

ZL_GraphID ZL_Compressor_registerTransposeSplitGraph(ZL_Compressor* c, ZL_GraphID successor)
{
    if (!c || !c->known(successor.gid)) return ZL_GraphID{ G_ILLEGAL };
    return c->add(ZL_Compressor_s::Graph{ ZL_Compressor_s::TSPLIT, {}, { successor.gid } });
}

ZL_GraphID ZL_Compressor_registerTokenizeGraph(ZL_Compressor* c, ZL_Type inputType, bool sort,
                                               ZL_GraphID alphabetGraph, ZL_GraphID indicesGraph)
{
    if (!c || !c->known(alphabetGraph.gid) || !c->known(indicesGraph.gid)) return ZL_GraphID{ G_ILLEGAL };
    ZL_Compressor_s::Graph g{ ZL_Compressor_s::TOKENIZE, {}, { alphabetGraph.gid, indicesGraph.gid } };
    g.type = inputType;
    g.sort = sort;
    return c->add(std::move(g));
}

ZL_Report ZL_Compressor_selectStartingGraphID(ZL_Compressor* c, ZL_GraphID graph)
{
    if (!c) return fail(ZL_ErrorCode_parameter_invalid);
    if (!c->known(graph.gid)) {
        c->err = "unknown graph ID";
        return fail(ZL_ErrorCode_graph_invalid);
    }
    c->start = graph.gid;
    return ok(0);
}

int ZL_GraphID_isValid(ZL_GraphID g) { return g.gid != G_ILLEGAL; }

/* zl_compressor.h:105 */
const char* ZL_Compressor_getErrorContextString(const ZL_Compressor* c, ZL_Report r)
{
    if (!c || c->err.empty()) return ZL_ErrorCode_toString(r._code);
    return c->err.c_str();
}

size_t ZL_compressBound(size_t totalSrcSize) { return ZL_COMPRESSBOUND(totalSrcSize); }

ZL_CCtx* ZL_CCtx_create(void)
{
    try {
        return new ZL_CCtx_s();
    } catch (...) {
        return nullptr;
    }
}

void ZL_CCtx_free(ZL_CCtx* c) { delete c; }

ZL_Report ZL_CCtx_setParameter(ZL_CCtx* c, ZL_CParam p, int value)
{
    if (!c || int(p) <= 0 || int(p) >= kNbParams) return fail(ZL_ErrorCode_parameter_invalid);
    c->params[p] = value;
    return ok(0);
}

int ZL_CCtx_getParameter(const ZL_CCtx* c, ZL_CParam p)
{
    if (!c || int(p) <= 0 || int(p) >= kNbParams) return 0;
    return c->param(p);
}

ZL_Report ZL_CCtx_resetParameters(ZL_CCtx* c)
{
    if (!c) return fail(ZL_ErrorCode_parameter_invalid);
    std::memset(c->params, 0, sizeof(c->params));
    return ok(0);
}

ZL_Report ZL_CCtx_refCompressor(ZL_CCtx* c, const ZL_Compressor* comp)
{
    if (!c || !comp) return fail(ZL_ErrorCode_parameter_invalid);
    c->comp = comp;
    return ok(0);
}

const char* ZL_CCtx_getErrorContextString(const ZL_CCtx* c, ZL_Report r)
{
    if (!c || c->err.empty()) return ZL_ErrorCode_toString(r._code);
    return c->err.c_str();
}

ZL_Report ZL_CCtx_compress(ZL_CCtx* c, void* dst, size_t cap, const void* src, size_t srcSize)
{
    if (!c || !dst || (srcSize && !src)) return fail(ZL_ErrorCode_parameter_invalid);
    ZL_TypedRef_s in{ ZL_Type_serial, src, 1, srcSize };
    ZL_Report r = compressOne(c, dst, cap, in);
    c->endOp();
    return r;
}

ZL_Report ZL_CCtx_compressTypedRef(ZL_CCtx* c, void* dst, size_t cap, const ZL_TypedRef* input)
{
    if (!c || !dst || !input) return fail(ZL_ErrorCode_parameter_invalid);
    ZL_Report r = compressOne(c, dst, cap, *input);
    c->endOp();
    return r;
}

ZL_Report ZL_CCtx_compressMultiTypedRef(ZL_CCtx* c, void* dst, size_t cap, const ZL_TypedRef* inputs[],
                                        size_t nbInputs)
{
    if (!c || !inputs) return fail(ZL_ErrorCode_parameter_invalid);
    if (nbInputs != 1) {
        c->err = "frames with more than one input are not on the GPU encoder";
        c->endOp();
        return fail(ZL_ErrorCode_temporaryLibraryLimitation);
    }
    return ZL_CCtx_compressTypedRef(c, dst, cap, inputs[0]);
}

ZL_TypedRef* ZL_TypedRef_createSerial(const void* src, size_t srcSize)
{
    return new (std::nothrow) ZL_TypedRef_s{ ZL_Type_serial, src, 1, srcSize };
}

ZL_TypedRef* ZL_TypedRef_createStruct(const void* start, size_t structWidth, size_t structCount)
{
    return new (std::nothrow) ZL_TypedRef_s{ ZL_Type_struct, start, structWidth, structCount };
}

ZL_TypedRef* ZL_TypedRef_createNumeric(const void* start, size_t numWidth, size_t numCount)
{
    if (!(numWidth == 1 || numWidth == 2 || numWidth == 4 || numWidth == 8)) return nullptr;
    if (numCount && (reinterpret_cast<uintptr_t>(start) % numWidth)) return nullptr; // common/stream.c:285
    return new (std::nothrow) ZL_TypedRef_s{ ZL_Type_numeric, start, numWidth, numCount };
}

void ZL_TypedRef_free(ZL_TypedRef* t) { delete t; }

} // extern "C"

void ozl_compressor_set_error(ZL_Compressor* c, const char* msg)
{
    if (c) c->err = msg;
}
