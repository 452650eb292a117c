// C entry points of openzl_gb300 (declared in include/openzl_gb300.h).
//
// The ZL_* functions keep the reference's names and semantics
// (include/openzl/zl_decompress.h, zl_errors.h); the ozl_gpu_* functions are
// the device-resident additions. No exception crosses this boundary.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/openzl_gb300.h"
#include "dec_exec.h"
#include "dec_plan.h"
#include "decode_batch.h"
#include "enc_engine.h"

namespace {

ZL_Report ok(size_t v) { return ZL_Report{ ZL_ErrorCode_no_error, v }; }
ZL_Report fail(int code) { return ZL_Report{ ZL_ErrorCode(code), 0 }; }

} // namespace

namespace ozl {
cudaError_t prepareOnce()
{
    static std::once_flag once;
    static cudaError_t err = cudaSuccess;
    std::call_once(once, [] { err = prepareKernels(); });
    return err;
}
} // namespace ozl

// A planned decode of one or more frames (the C handle).
struct OZL_GpuBatch_s : ozl::DecodeBatch {};

struct ZL_DCtx_s {
    int device = ozl::currentDevice(); // the device current at creation: every call decodes there
    ozl::DecodeBatch batch;
    bool sticky = false;
    int raw[4] = {}; // parameter values as set, for ZL_DCtx_getParameter
    ozl::DevBuf frame, out;
    cudaStream_t stream = nullptr;
    std::string err;
    ~ZL_DCtx_s()
    {
        if (stream) cudaStreamDestroy(stream);
    }
};

// A large batch is encoded in parts of about equal bytes, each by its own
// engine on its own host thread and stream, so that one part's host phases
// (graph discovery, codec decisions, replay) run while another part's
// kernels do. Frames are independent; each part's frames are the bytes a
// whole-batch call would write.
struct OZL_GpuEncoder_s {
    static constexpr int kMaxParts = 16;
    static constexpr uint64_t kSplitBytes = 64ull << 20; // smaller batches: one engine, the caller's stream
    int parts = 8;
    bool shareCores = true; // each part's host phases on its share of the cores
    ozl::EncodeBatch batch[kMaxParts];
    cudaStream_t streams[kMaxParts] = {};
    cudaEvent_t ready = nullptr;
    double phaseMs[ozl::EncodeBatch::kPhases] = {};
    std::string err;
    ~OZL_GpuEncoder_s()
    {
        for (cudaStream_t x : streams)
            if (x) cudaStreamDestroy(x);
        if (ready) cudaEventDestroy(ready);
    }
};

namespace ozl {
// The size of a single-output frame for the library's own decode calls: the
// whole header parsed, frames of several outputs refused (as the
// reference's single-output decompression refuses them).
ZL_Report singleOutputSize(const void* src, size_t size)
{
    if (!src) return fail(ZL_ErrorCode_srcSize_tooSmall);
    FrameHeader h;
    std::string err;
    int const rc = parseFrameHeader(static_cast<const uint8_t*>(src), size, h, err);
    if (rc) return fail(rc);
    if (h.sizes.size() != 1) return fail(ZL_ErrorCode_invalidRequest_singleOutputFrameOnly);
    return ok(size_t(h.outSize));
}
} // namespace ozl

extern "C" {

int ZL_isError(ZL_Report r) { return r._code != ZL_ErrorCode_no_error; }
size_t ZL_validResult(ZL_Report r) { return r._value; }
ZL_ErrorCode ZL_errorCode(ZL_Report r) { return r._code; }

const char* ZL_ErrorCode_toString(ZL_ErrorCode code)
{
    switch (code) {
        case ZL_ErrorCode_no_error: return "No error detected";
        case ZL_ErrorCode_GENERIC: return "Error (generic)";
        case ZL_ErrorCode_srcSize_tooSmall: return "Source size too small";
        case ZL_ErrorCode_srcSize_tooLarge: return "Source size too large";
        case ZL_ErrorCode_dstCapacity_tooSmall: return "Destination capacity too small";
        case ZL_ErrorCode_header_unknown: return "Unknown header";
        case ZL_ErrorCode_frameParameter_unsupported: return "Frame parameter unsupported";
        case ZL_ErrorCode_corruption: return "Corrupted input";
        case ZL_ErrorCode_compressedChecksumWrong: return "Compressed checksum mismatch";
        case ZL_ErrorCode_contentChecksumWrong: return "Content checksum mismatch";
        case ZL_ErrorCode_parameter_invalid: return "Invalid parameter";
        case ZL_ErrorCode_compressionParameter_invalid: return "Invalid compression parameter";
        case ZL_ErrorCode_graph_invalid: return "Graph invalid";
        case ZL_ErrorCode_node_unexpected_input_type: return "Unexpected input type for node";
        case ZL_ErrorCode_node_invalid: return "Node invalid";
        case ZL_ErrorCode_invalidRequest_singleOutputFrameOnly: return "Only single-output frames are supported";
        case ZL_ErrorCode_userBuffers_invalidNum: return "Wrong number of output buffers";
        case ZL_ErrorCode_outputID_invalid: return "Invalid output ID";
        case ZL_ErrorCode_invalidTransform: return "Codec not on the GPU path";
        case ZL_ErrorCode_formatVersion_unsupported: return "Format version unsupported";
        case ZL_ErrorCode_formatVersion_notSet: return "Format version not set";
        case ZL_ErrorCode_allocation: return "Allocation failure";
        case ZL_ErrorCode_temporaryLibraryLimitation: return "Temporary library limitation";
        default: return "Error";
    }
}

OZL_GpuEncoder* ozl_gpu_encoder_create(void)
{
    try {
        return new OZL_GpuEncoder_s();
    } catch (...) {
        return nullptr;
    }
}

void ozl_gpu_encoder_free(OZL_GpuEncoder* e) { delete e; }

size_t ozl_gpu_compress_bound(size_t srcBytes) { return ozl::encodeBound(srcBytes); }

const char* ozl_gpu_encoder_error(const OZL_GpuEncoder* e) { return e ? e->err.c_str() : ""; }

ZL_Report ozl_gpu_encoder_setParts(OZL_GpuEncoder* e, int parts)
{
    int const k = parts < 0 ? -parts : parts;
    if (!e || k < 1 || k > OZL_GpuEncoder_s::kMaxParts) return fail(ZL_ErrorCode_parameter_invalid);
    e->parts = k;
    e->shareCores = parts > 0;
    return ok(0);
}

ZL_Report ozl_gpu_encoder_phases(const OZL_GpuEncoder* e, float* ms, size_t capacity)
{
    if (!e || (capacity && !ms)) return fail(ZL_ErrorCode_parameter_invalid);
    for (size_t i = 0; i < capacity && i < size_t(ozl::EncodeBatch::kPhases); i++) ms[i] = float(e->phaseMs[i]);
    return ok(size_t(ozl::EncodeBatch::kPhases));
}

ZL_Report ozl_gpu_compress_batch(OZL_GpuEncoder* e, size_t n, const void* const* d_srcs, const size_t* nbElts,
                                 const int* eltWidths, const int* recipes, void* const* d_dsts, const size_t* caps,
                                 size_t* frameSizes, int checksums, void* stream)
{
    if (!e || (n && (!d_srcs || !nbElts || !eltWidths || !recipes || !d_dsts || !caps || !frameSizes)))
        return fail(ZL_ErrorCode_parameter_invalid);
    std::vector<ozl::EncFrameSpec> specs(n);
    for (size_t i = 0; i < n; i++) {
        int const w = eltWidths[i];
        if (!(w == 0 || w == 1 || w == 2 || w == 4 || w == 8)) return fail(ZL_ErrorCode_parameter_invalid);
        specs[i] = ozl::EncFrameSpec{ static_cast<const uint8_t*>(d_srcs[i]), nbElts[i], uint32_t(w ? w : 1), w == 0,
                                      recipes[i] };
    }
    std::vector<size_t> sizes;
    e->err.clear();
    uint8_t* const* const outs = reinterpret_cast<uint8_t* const*>(d_dsts);
    cudaStream_t const us = static_cast<cudaStream_t>(stream);
    uint64_t bytes = 0;
    for (const ozl::EncFrameSpec& f : specs) bytes += f.n * f.w;
    int rc = 0;
    if (n < 2 || bytes < OZL_GpuEncoder_s::kSplitBytes) {
        rc = e->batch[0].compress(specs, outs, caps, checksums != 0, us, sizes, e->err);
        if (rc) return fail(rc);
        for (int i = 0; i < ozl::EncodeBatch::kPhases; i++) e->phaseMs[i] = e->batch[0].lastPhaseMs()[i];
    } else {
        // parts of about equal bytes; every part's stream waits for the
        // caller's work on `stream` (the inputs), and every part synchronizes
        // its own
        int const np = int(std::min<size_t>(size_t(e->parts), n));
        std::vector<size_t> cut{ 0 };
        uint64_t acc = 0;
        for (size_t i = 0; i < n && int(cut.size()) < np; i++) {
            acc += specs[i].n * specs[i].w;
            if (acc * uint64_t(np) >= bytes * uint64_t(cut.size()) && i + 1 < n) cut.push_back(i + 1);
        }
        cut.push_back(n);
        int const parts = int(cut.size()) - 1;
        bool okSetup = (e->ready || cudaEventCreateWithFlags(&e->ready, cudaEventDisableTiming) == cudaSuccess);
        for (int p = 0; p < parts; p++)
            okSetup = okSetup && (e->streams[p] || cudaStreamCreateWithFlags(&e->streams[p], cudaStreamNonBlocking) == cudaSuccess);
        okSetup = okSetup && cudaEventRecord(e->ready, us) == cudaSuccess;
        for (int p = 0; p < parts; p++) okSetup = okSetup && cudaStreamWaitEvent(e->streams[p], e->ready, 0) == cudaSuccess;
        if (!okSetup) {
            e->err = "encoder streams could not be set up";
            return fail(ZL_ErrorCode_GENERIC);
        }
        std::vector<std::vector<size_t>> partSizes(parts);
        std::vector<std::string> partErr(parts);
        std::vector<int> partRc(parts, 0);
        unsigned const hw = std::thread::hardware_concurrency();
        unsigned const share = std::max(2u, (hw ? hw : 16u) / unsigned(parts)); // host threads per part
        auto runPart = [&](int p) {
            std::vector<ozl::EncFrameSpec> const sub(specs.begin() + cut[p], specs.begin() + cut[p + 1]);
            e->batch[p].setHostThreads(e->shareCores ? share : 0);
            partRc[p] = e->batch[p].compress(sub, outs + cut[p], caps + cut[p], checksums != 0, e->streams[p],
                                             partSizes[p], partErr[p]);
        };
        std::vector<std::thread> others;
        for (int p = 1; p < parts; p++) others.emplace_back(runPart, p);
        runPart(0);
        for (std::thread& th : others) th.join();
        for (int p = 0; p < parts && !rc; p++)
            if (partRc[p]) {
                rc = partRc[p];
                e->err = partErr[p];
            }
        if (rc) return fail(rc);
        for (int i = 0; i < ozl::EncodeBatch::kPhases; i++) e->phaseMs[i] = 0;
        for (int p = 0; p < parts; p++) {
            sizes.insert(sizes.end(), partSizes[p].begin(), partSizes[p].end());
            for (int i = 0; i < ozl::EncodeBatch::kPhases; i++)
                e->phaseMs[i] = std::max(e->phaseMs[i], e->batch[p].lastPhaseMs()[i]);
        }
    }
    size_t total = 0;
    for (size_t i = 0; i < n; i++) {
        frameSizes[i] = sizes[i];
        total += sizes[i];
    }
    return ok(total);
}

const char* ozl_gpu_version(void) { return "openzl_gb300 0.1 (sm_103a)"; }


ZL_Report ZL_getDecompressedSize(const void* src, size_t size)
{
    // ZL_getFormatVersionFromFrame (common/wire_format.c:10-40): magic
    // numbers outside the known range (padded by 16 versions) are unknown
    // headers, versions outside 8..23 unsupported
    if (!src || size < 4) return fail(ZL_ErrorCode_srcSize_tooSmall);
    const uint8_t* const p = static_cast<const uint8_t*>(src);
    uint32_t const magic = uint32_t(p[0]) | uint32_t(p[1]) << 8 | uint32_t(p[2]) << 16 | uint32_t(p[3]) << 24;
    uint32_t const base = 0xD7B1A5C0u;
    if (magic < base || magic > base + 23 + 16) return fail(ZL_ErrorCode_header_unknown);
    if (magic < base + 8 || magic > base + 23) return fail(ZL_ErrorCode_formatVersion_unsupported);
    unsigned const v = magic - base;
    // getDecompressedSizeV3orMore (decode_frameheader.c:1147-1190), read as
    // the reference reads it: from version 15 a frame whose output token (the
    // byte after the magic, after the flags from version 21) is 64 or more
    // is refused as not single-output; otherwise the size field right after
    // the token (LE32 before version 21, a varint holding size + 1 from 21;
    // 0 means unknown). For frames of several outputs that field is not
    // always output 0's size; the reference returns it all the same.
    size_t const hSize = 4 + (v > 13 ? 1 : 0) + (v >= 21 ? 1 : 0);
    if (size < hSize + 4) return fail(ZL_ErrorCode_srcSize_tooSmall);
    if (v > 14 && p[4 + (v >= 21 ? 1 : 0)] >= 64) return fail(ZL_ErrorCode_invalidRequest_singleOutputFrameOnly);
    if (v < 21) return ok(size_t(uint32_t(p[hSize]) | uint32_t(p[hSize + 1]) << 8 | uint32_t(p[hSize + 2]) << 16
                                 | uint32_t(p[hSize + 3]) << 24));
    uint64_t oSize = 0;
    size_t i = hSize;
    for (unsigned sh = 0;; sh += 7, i++) {
        if (i >= size) return fail(ZL_ErrorCode_srcSize_tooSmall);
        if (sh > 63) return fail(ZL_ErrorCode_corruption);
        oSize |= uint64_t(p[i] & 0x7F) << sh;
        if (!(p[i] & 0x80)) break;
    }
    if (oSize == 0) return fail(ZL_ErrorCode_temporaryLibraryLimitation);
    return ok(size_t(oSize - 1));
}

ZL_Report ozl_frame_info(const void* frame, size_t frameSize, OZL_FrameInfo* info)
{
    if (!info || (!frame && frameSize)) return fail(ZL_ErrorCode_parameter_invalid);
    *info = OZL_FrameInfo{};
    ozl::FrameHeader h;
    std::string err;
    int const rc = ozl::parseFrameHeader(static_cast<const uint8_t*>(frame), frameSize, h, err);
    info->status = rc;
    if (rc) return ok(0);
    std::vector<uint64_t> offs;
    info->formatVersion = h.version;
    info->nbOutputs = uint32_t(h.sizes.size());
    info->flags = (h.hasContentCk ? 1u : 0u) | (h.hasCompressedCk ? 2u : 0u) | (h.hdrCk ? 4u : 0u);
    info->headerBytes = h.end;
    info->output0Bytes = h.outSize;
    info->output0Type = h.outType;
    info->extent = ozl::frameOutputLayout(h, offs);
    return ok(0);
}

ZL_Report ozl_frame_outputs(const void* frame, size_t frameSize, size_t capacity, uint64_t* offsets, uint64_t* sizes,
                            int* types, uint32_t* widths, uint64_t* counts, uint64_t* lensOffsets, uint64_t* extent)
{
    if (!frame) return fail(ZL_ErrorCode_parameter_invalid);
    ozl::DecodePlan plan;
    std::string err;
    const uint8_t* f = static_cast<const uint8_t*>(frame);
    int rc = plan.build(1, &f, &frameSize, nullptr, false, false, err);
    if (rc) return fail(rc);
    const ozl::FramePlan& fp = plan.frames[0];
    size_t const n = fp.outOffs.size();
    for (size_t o = 0; o < n && o < capacity; o++) {
        bool const str = fp.outTypes[o] == ZL_Type_string;
        uint32_t const w = fp.outTypes[o] == ZL_Type_serial || str ? 1 : fp.outWidths[o];
        if (offsets) offsets[o] = fp.outOffs[o];
        if (sizes) sizes[o] = fp.outSizes[o];
        if (types) types[o] = fp.outTypes[o];
        if (widths) widths[o] = w;
        if (counts) counts[o] = str ? fp.nbStrings[o] : fp.outSizes[o] / w;
        if (lensOffsets) lensOffsets[o] = str ? fp.lensOffs[o] : 0;
    }
    if (extent) *extent = fp.decodedSize;
    return ok(n);
}

ZL_Report ZL_getCompressedSize(const void* src, size_t size)
{
    ozl::DecodePlan plan;
    std::string err;
    const uint8_t* f = static_cast<const uint8_t*>(src);
    int rc = plan.build(1, &f, &size, nullptr, false, false, err);
    if (rc) return fail(rc);
    return ok(size_t(plan.frames[0].frameBytes));
}

ZL_DCtx* ZL_DCtx_create(void)
{
    try {
        return new ZL_DCtx_s();
    } catch (...) {
        return nullptr;
    }
}

void ZL_DCtx_free(ZL_DCtx* dctx) { delete dctx; }

ZL_Report ZL_DCtx_setParameter(ZL_DCtx* dctx, ZL_DParam param, int value)
{
    if (!dctx) return fail(ZL_ErrorCode_parameter_invalid);
    switch (param) {
        case ZL_DParam_stickyParameters: dctx->sticky = value != 0; break;
        case ZL_DParam_checkCompressedChecksum: dctx->batch.checkCompressed = value != ZL_TernaryParam_disable; break;
        case ZL_DParam_checkContentChecksum: dctx->batch.checkContent = value != ZL_TernaryParam_disable; break;
        default: return fail(ZL_ErrorCode_parameter_invalid);
    }
    dctx->raw[param] = value;
    return ok(0);
}

/* zl_decompress.h:149: the value set, 0 when unset or unknown */
int ZL_DCtx_getParameter(const ZL_DCtx* dctx, ZL_DParam param)
{
    if (!dctx || int(param) < 1 || int(param) > 3) return 0;
    return dctx->raw[param];
}

/* zl_decompress.h:159: every parameter back to its default, sticky included */
ZL_Report ZL_DCtx_resetParameters(ZL_DCtx* dctx)
{
    if (!dctx) return fail(ZL_ErrorCode_parameter_invalid);
    dctx->sticky = false;
    dctx->batch.checkCompressed = true;
    dctx->batch.checkContent = true;
    for (int& v : dctx->raw) v = 0;
    return ok(0);
}

const char* ZL_DCtx_getErrorContextString(const ZL_DCtx* dctx, ZL_Report report)
{
    if (!dctx) return ZL_ErrorCode_toString(report._code);
    return dctx->err.empty() ? ZL_ErrorCode_toString(report._code) : dctx->err.c_str();
}

static void resetParams(ZL_DCtx* d)
{
    if (!d->sticky) {
        d->batch.checkCompressed = true;
        d->batch.checkContent = true;
        d->raw[ZL_DParam_checkCompressedChecksum] = 0;
        d->raw[ZL_DParam_checkContentChecksum] = 0;
    }
}

ZL_Report ozl_gpu_decompress(ZL_DCtx* dctx, void* d_dst, size_t dstCap, const void* h_frame, const void* d_frame,
                             size_t cSize, void* stream)
{
    if (!dctx || !h_frame || !d_frame) return fail(ZL_ErrorCode_parameter_invalid);
    ozl::DeviceScope const onDevice(dctx->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ZL_Report r = dctx->batch.makePlan(1, &h_frame, &cSize, &d_frame, &d_dst, &dstCap);
    if (!ZL_isError(r)) r = dctx->batch.run(s, false);
    if (!ZL_isError(r)) r = dctx->batch.check(s);
    if (ZL_isError(r)) dctx->err = dctx->batch.err;
    resetParams(dctx);
    return r;
}

// Host buffers in and out: one frame decoded on the DCtx's stream. Fills the
// output's type and element width. Does not reset parameters.
static ZL_Report decodeToHost(ZL_DCtx* dctx, void* dst, size_t dstCap, const void* src, size_t cSize, int* type,
                              uint32_t* width)
{
    if (!dctx || !src || (dstCap && !dst)) return fail(ZL_ErrorCode_parameter_invalid);
    ZL_Report ds = ozl::singleOutputSize(src, cSize);
    if (ZL_isError(ds)) return ds;
    size_t const outSize = ZL_validResult(ds);
    if (outSize > dstCap) return fail(ZL_ErrorCode_dstCapacity_tooSmall);
    ozl::DeviceScope const onDevice(dctx->device);
    if (!dctx->stream && cudaStreamCreateWithFlags(&dctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        dctx->err = "no CUDA device";
        return fail(ZL_ErrorCode_GENERIC);
    }
    if (!dctx->frame.reserve(cSize + 64) || !dctx->out.reserve(outSize + 64)) {
        dctx->err = "device allocation failed";
        return fail(ZL_ErrorCode_allocation);
    }
    cudaStream_t s = dctx->stream;
    if (cudaMemcpyAsync(dctx->frame.data(), src, cSize, cudaMemcpyHostToDevice, s) != cudaSuccess) {
        dctx->err = "copy to device failed";
        return fail(ZL_ErrorCode_GENERIC);
    }
    const void* dF = dctx->frame.data();
    void* dO = dctx->out.data();
    ZL_Report r = dctx->batch.makePlan(1, &src, &cSize, &dF, &dO, &dstCap);
    if (!ZL_isError(r)) r = dctx->batch.run(s, false);
    if (!ZL_isError(r) && outSize
        && cudaMemcpyAsync(dst, dctx->out.data(), outSize, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        r = fail(ZL_ErrorCode_GENERIC);
    if (!ZL_isError(r)) r = dctx->batch.check(s);
    if (ZL_isError(r)) {
        dctx->err = dctx->batch.err;
        return r;
    }
    if (type) *type = dctx->batch.plan.frames[0].outType;
    if (width) *width = dctx->batch.plan.frames[0].outWidth;
    return ok(outSize);
}

ZL_Report ZL_DCtx_decompress(ZL_DCtx* dctx, void* dst, size_t dstCap, const void* src, size_t cSize)
{
    int type = 0;
    ZL_Report r = decodeToHost(dctx, dst, dstCap, src, cSize, &type, nullptr);
    if (!ZL_isError(r) && type != ZL_Type_serial) {
        // decompress2.c:1850-1856: typed outputs go through ZL_DCtx_decompressTyped
        dctx->err = "ZL_DCtx_decompress is only compatible with serialized output";
        r = fail(ZL_ErrorCode_GENERIC);
    }
    if (dctx) resetParams(dctx);
    return r;
}

ZL_Report ZL_DCtx_decompressTyped(ZL_DCtx* dctx, ZL_OutputInfo* info, void* dst, size_t dstCap, const void* src,
                                  size_t cSize)
{
    int type = 0;
    uint32_t width = 1;
    ZL_Report r = decodeToHost(dctx, dst, dstCap, src, cSize, &type, &width);
    if (!ZL_isError(r) && info) {
        info->type = ZL_Type(type);
        info->fixedWidth = type == ZL_Type_serial ? 1 : width;
        info->decompressedByteSize = ZL_validResult(r);
        info->numElts = ZL_validResult(r) / (info->fixedWidth ? info->fixedWidth : 1);
    }
    if (dctx) resetParams(dctx);
    return r;
}

ZL_Report ZL_decompress(void* dst, size_t dstCap, const void* src, size_t cSize)
{
    ZL_DCtx* d = ZL_DCtx_create();
    if (!d) return fail(ZL_ErrorCode_allocation);
    ZL_Report r = ZL_DCtx_decompress(d, dst, dstCap, src, cSize);
    ZL_DCtx_free(d);
    return r;
}

OZL_GpuBatch* ozl_gpu_batch_create(void)
{
    try {
        return new OZL_GpuBatch_s();
    } catch (...) {
        return nullptr;
    }
}

void ozl_gpu_batch_free(OZL_GpuBatch* b) { delete b; }

ZL_Report ozl_gpu_batch_setParameter(OZL_GpuBatch* b, ZL_DParam param, int value)
{
    if (!b) return fail(ZL_ErrorCode_parameter_invalid);
    switch (param) {
        case ZL_DParam_checkCompressedChecksum: b->checkCompressed = value != ZL_TernaryParam_disable; break;
        case ZL_DParam_checkContentChecksum: b->checkContent = value != ZL_TernaryParam_disable; break;
        case ZL_DParam_stickyParameters: break;
        case OZL_DParam_partsPerKind:
            if (value < 1 || value > 8) return fail(ZL_ErrorCode_parameter_invalid);
            b->partsPerKind = value;
            break;
        case OZL_DParam_fseKernel:
            if (value < 0 || value > 2) return fail(ZL_ErrorCode_parameter_invalid);
            b->fseKernel = value;
            break;
        case OZL_DParam_criticalSymbols:
            if (value < 0) return fail(ZL_ErrorCode_parameter_invalid);
            b->criticalSymbols = value;
            break;
        case OZL_DParam_schedule:
            if (value < 0 || value > 1) return fail(ZL_ErrorCode_parameter_invalid);
            b->schedule = value;
            break;
        case OZL_DParam_hostRounds:
            if (value < 1 || value > ozl::DecodeBatch::HostPipe::kRounds) return fail(ZL_ErrorCode_parameter_invalid);
            b->hostRounds = value;
            b->host.reset();
            break;
        case OZL_DParam_hostDepth:
            if (value < 0 || value > ozl::DecodeBatch::HostPipe::kRounds) return fail(ZL_ErrorCode_parameter_invalid);
            b->hostDepth = value;
            b->host.dropGraph();
            break;
        default: return fail(ZL_ErrorCode_parameter_invalid);
    }
    return ok(0);
}

ZL_Report ozl_gpu_batch_plan(OZL_GpuBatch* b, size_t n, const void* const* hF, const size_t* fs,
                             const void* const* dF, void* const* dO, const size_t* caps)
{
    if (!b || !hF || !fs || !dF || !dO) return fail(ZL_ErrorCode_parameter_invalid);
    return b->makePlan(n, hF, fs, dF, dO, caps);
}

ZL_Report ozl_gpu_batch_run(OZL_GpuBatch* b, void* stream, int useGraph)
{
    if (!b) return fail(ZL_ErrorCode_parameter_invalid);
    return b->run(static_cast<cudaStream_t>(stream), useGraph != 0);
}

ZL_Report ozl_gpu_batch_check(OZL_GpuBatch* b, void* stream)
{
    if (!b) return fail(ZL_ErrorCode_parameter_invalid);
    return b->check(static_cast<cudaStream_t>(stream));
}

size_t ozl_gpu_batch_launches(const OZL_GpuBatch* b) { return b ? size_t(b->launches) : 0; }

const char* ozl_gpu_kind_name(int kind)
{
    static const char* names[] = { "copy", "constant", "fse", "huffman", "flatpack", "tokenize",
                                   "float_deconstruct", "transpose", "numeric_pipeline", "xxh3", "huffman16",
                                   "widen" };
    return (kind >= 0 && kind < ozl::KIND_COUNT) ? names[kind] : "?";
}

ZL_Report ozl_gpu_batch_host_timeline(OZL_GpuBatch* b, const void* h_in, size_t inBytes, void* h_out,
                                      size_t outBytes, void* stream, float* rows, size_t capacity)
{
    if (!b || b->dFrames.empty() || (capacity && !rows)) return fail(ZL_ErrorCode_parameter_invalid);
    return b->hostTimeline(h_in, inBytes, h_out, outBytes, static_cast<cudaStream_t>(stream), rows, capacity);
}

ZL_Report ozl_gpu_batch_timeline(OZL_GpuBatch* b, void* stream, float* rows, size_t capacity)
{
    if (!b || (capacity && !rows)) return fail(ZL_ErrorCode_parameter_invalid);
    return b->timeline(static_cast<cudaStream_t>(stream), rows, capacity);
}

ZL_Report ozl_gpu_batch_profile(OZL_GpuBatch* b, void* stream, float* ms, int* kinds, uint64_t* bytes,
                                size_t capacity)
{
    if (!b) return fail(ZL_ErrorCode_parameter_invalid);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ZL_Report const u = b->upload(s);
    if (ZL_isError(u)) return u;
    size_t const n = b->nbLaunches();
    std::vector<cudaEvent_t> ev(n + 1);
    for (auto& e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) return fail(ZL_ErrorCode_GENERIC);
    bool okRun = cudaMemsetAsync(b->status.data(), 0, 4, s) == cudaSuccess;
    cudaEventRecord(ev[0], s);
    for (size_t i = 0; i < n && okRun; i++) {
        size_t p = 0, li = 0;
        b->locate(i, p, li);
        okRun = ozl::runOneLaunch(b->parts[p].layout, li, b->parts[p].pool.data(), b->parts[p].scratch.data(),
                                  reinterpret_cast<uint32_t*>(b->status.data()), s) >= 0;
        cudaEventRecord(ev[i + 1], s);
    }
    okRun = okRun && cudaStreamSynchronize(s) == cudaSuccess;
    for (size_t i = 0; i < n && i < capacity && okRun; i++) {
        float t = 0;
        cudaEventElapsedTime(&t, ev[i], ev[i + 1]);
        size_t p = 0, li = 0;
        b->locate(i, p, li);
        if (ms) ms[i] = t;
        if (kinds) kinds[i] = b->parts[p].layout.launches[li].kind;
        if (bytes) bytes[i] = b->parts[p].layout.launches[li].algoBytes;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    if (!okRun) return fail(ZL_ErrorCode_GENERIC);
    return ok(n);
}

ZL_Report ozl_gpu_batch_autotune(OZL_GpuBatch* b, void* stream, int reps, uint32_t* shapes, size_t capacity)
{
    if (!b || b->dFrames.empty()) return fail(ZL_ErrorCode_parameter_invalid);
    ZL_Report r = b->autotune(static_cast<cudaStream_t>(stream), reps < 1 ? 1 : reps);
    if (ZL_isError(r)) return r;
    for (size_t i = 0; shapes && i < capacity && i < b->nbLaunches(); i++) {
        size_t p = 0, li = 0;
        b->locate(i, p, li);
        shapes[i] = b->parts[p].layout.launches[li].tune;
    }
    return ok(b->nbLaunches());
}

ZL_Report ozl_gpu_batch_run_host(OZL_GpuBatch* b, const void* h_in, size_t inBytes, void* h_out, size_t outBytes,
                                 void* stream, int useGraph)
{
    if (!b || b->dFrames.empty()) return fail(ZL_ErrorCode_parameter_invalid);
    return b->runHost(h_in, inBytes, h_out, outBytes, static_cast<cudaStream_t>(stream), useGraph != 0);
}

const size_t* ozl_gpu_batch_sizes(const OZL_GpuBatch* b) { return b ? b->sizes.data() : nullptr; }

ZL_Report ozl_gpu_xxh3_64(const void* d_data, size_t len, void* stream)
{
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    size_t const scratchBytes = 512 + (len / 1024 + 1) * 72;
    uint8_t* scratch = nullptr;
    if (cudaMalloc(&scratch, scratchBytes + 64) != cudaSuccess) return fail(ZL_ErrorCode_allocation);
    cudaError_t e = ozl::xxh3Device(static_cast<const uint8_t*>(d_data), len,
                                    reinterpret_cast<uint64_t*>(scratch + scratchBytes), scratch, scratchBytes, s);
    uint64_t h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, scratch + scratchBytes, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(scratch);
    if (e != cudaSuccess) return fail(ZL_ErrorCode_GENERIC);
    return ok(size_t(h));
}

const char* ozl_gpu_batch_error(const OZL_GpuBatch* b) { return b ? b->err.c_str() : ""; }


// ---------------------------------------------------------------------------
// Typed buffers (zl_decompress.h:418-599): either wrapping caller memory of a
// stated type and capacity, or filled by the DCtx (host allocation).
struct ZL_TypedBuffer_s {
    bool wrap = false;
    ZL_Type type = ZL_Type_serial;
    size_t width = 1;       // element width (wrap: declared; else from the frame)
    size_t capacity = 0;    // wrap: bytes available
    void* wrapped = nullptr;
    std::vector<uint8_t> own;
    size_t bytes = 0;
    std::vector<uint32_t> lens; // string outputs
};

ZL_TypedBuffer* ZL_TypedBuffer_create(void) { return new (std::nothrow) ZL_TypedBuffer_s(); }
void ZL_TypedBuffer_free(ZL_TypedBuffer* t) { delete t; }

static ZL_TypedBuffer* wrapBuffer(ZL_Type type, void* p, size_t width, size_t bytes)
{
    ZL_TypedBuffer_s* t = new (std::nothrow) ZL_TypedBuffer_s();
    if (!t) return nullptr;
    t->wrap = true;
    t->type = type;
    t->width = width;
    t->capacity = bytes;
    t->wrapped = p;
    return t;
}
ZL_TypedBuffer* ZL_TypedBuffer_createWrapSerial(void* buffer, size_t cap)
{
    return wrapBuffer(ZL_Type_serial, buffer, 1, cap);
}
ZL_TypedBuffer* ZL_TypedBuffer_createWrapStruct(void* buffer, size_t width, size_t n)
{
    return width ? wrapBuffer(ZL_Type_struct, buffer, width, width * n) : nullptr;
}
ZL_TypedBuffer* ZL_TypedBuffer_createWrapNumeric(void* buffer, size_t width, size_t n)
{
    if (!(width == 1 || width == 2 || width == 4 || width == 8)) return nullptr;
    return wrapBuffer(ZL_Type_numeric, buffer, width, width * n);
}
ZL_Type ZL_TypedBuffer_type(const ZL_TypedBuffer* t) { return t ? t->type : ZL_Type_serial; }
size_t ZL_TypedBuffer_byteSize(const ZL_TypedBuffer* t) { return t ? t->bytes : 0; }
const void* ZL_TypedBuffer_rPtr(const ZL_TypedBuffer* t)
{
    if (!t) return nullptr;
    return t->wrap ? t->wrapped : static_cast<const void*>(t->own.data());
}
size_t ZL_TypedBuffer_numElts(const ZL_TypedBuffer* t)
{
    if (t && t->type == ZL_Type_string) return t->lens.size();
    return t && t->width ? t->bytes / t->width : 0;
}
const uint32_t* ZL_TypedBuffer_rStringLens(const ZL_TypedBuffer* t)
{
    return t && t->type == ZL_Type_string ? t->lens.data() : nullptr;
}
size_t ZL_TypedBuffer_eltWidth(const ZL_TypedBuffer* t) { return t ? t->width : 0; }

ZL_Report ZL_DCtx_decompressMultiTBuffer(ZL_DCtx* dctx, ZL_TypedBuffer* outputs[], size_t nbOutputs,
                                         const void* src, size_t cSize);

ZL_Report ZL_DCtx_decompressTBuffer(ZL_DCtx* dctx, ZL_TypedBuffer* out, const void* src, size_t cSize)
{
    if (!dctx || !out || !src) return fail(ZL_ErrorCode_parameter_invalid);
    {
        // a string output carries its lengths: the multi-output path fills both
        ozl::FrameHeader h;
        std::string e;
        if (!ozl::parseFrameHeader(static_cast<const uint8_t*>(src), cSize, h, e) && h.types.size() == 1
            && h.types[0] == ZL_Type_string) {
            ZL_TypedBuffer* one[1] = { out };
            ZL_Report r = ZL_DCtx_decompressMultiTBuffer(dctx, one, 1, src, cSize);
            return ZL_isError(r) ? r : ok(out->bytes);
        }
    }
    ZL_Report ds = ozl::singleOutputSize(src, cSize);
    if (ZL_isError(ds)) { resetParams(dctx); return ds; }
    size_t const outSize = ZL_validResult(ds);
    void* dst;
    size_t cap;
    if (out->wrap) {
        dst = out->wrapped;
        cap = out->capacity;
    } else {
        try {
            out->own.resize(outSize + 1);
        } catch (...) {
            resetParams(dctx);
            return fail(ZL_ErrorCode_allocation);
        }
        dst = out->own.data();
        cap = outSize;
    }
    int type = 0;
    uint32_t width = 1;
    ZL_Report r = decodeToHost(dctx, dst, cap, src, cSize, &type, &width);
    if (!ZL_isError(r)) {
        size_t const w = type == ZL_Type_serial ? 1 : width;
        if (out->wrap && (ZL_Type(type) != out->type || (type != ZL_Type_serial && w != out->width))) {
            dctx->err = "the wrapped buffer's type or width differs from the frame's output";
            r = fail(ZL_ErrorCode_GENERIC);
        } else {
            out->type = ZL_Type(type);
            out->width = w;
            out->bytes = ZL_validResult(r);
        }
    }
    resetParams(dctx);
    return r;
}

// All outputs of a frame, decoded on the device into one destination (each
// output at its 16-byte-aligned offset), then copied to the typed buffers
// (decompress2.c:1580-1775).
ZL_Report ZL_DCtx_decompressMultiTBuffer(ZL_DCtx* dctx, ZL_TypedBuffer* outputs[], size_t nbOutputs,
                                         const void* src, size_t cSize)
{
    if (!dctx || !outputs || !src) return fail(ZL_ErrorCode_parameter_invalid);
    for (size_t o = 0; o < nbOutputs; o++)
        if (!outputs[o]) return fail(ZL_ErrorCode_parameter_invalid);
    dctx->err.clear();
    ozl::FrameHeader h;
    int rc = ozl::parseFrameHeader(static_cast<const uint8_t*>(src), cSize, h, dctx->err);
    if (rc) { resetParams(dctx); return fail(rc); }
    if (h.sizes.size() != nbOutputs) { // decompress2.c:845
        dctx->err = "the frame holds " + std::to_string(h.sizes.size()) + " outputs";
        resetParams(dctx);
        return fail(ZL_ErrorCode_userBuffers_invalidNum);
    }
    std::vector<uint64_t> offs, lensOffs;
    uint64_t const extent = ozl::frameOutputLayout(h, offs, &lensOffs);
    auto done = [&](ZL_Report r) {
        resetParams(dctx);
        return r;
    };
    ozl::DeviceScope const onDevice(dctx->device);
    if (!dctx->stream && cudaStreamCreateWithFlags(&dctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        dctx->err = "no CUDA device";
        return done(fail(ZL_ErrorCode_GENERIC));
    }
    if (!dctx->frame.reserve(cSize + 64) || !dctx->out.reserve(extent + 64)) {
        dctx->err = "device allocation failed";
        return done(fail(ZL_ErrorCode_allocation));
    }
    cudaStream_t s = dctx->stream;
    if (cudaMemcpyAsync(dctx->frame.data(), src, cSize, cudaMemcpyHostToDevice, s) != cudaSuccess) {
        dctx->err = "copy to device failed";
        return done(fail(ZL_ErrorCode_GENERIC));
    }
    const void* dF = dctx->frame.data();
    void* dO = dctx->out.data();
    size_t cap = size_t(extent);
    ZL_Report r = dctx->batch.makePlan(1, &src, &cSize, &dF, &dO, &cap);
    if (!ZL_isError(r)) r = dctx->batch.run(s, false);
    if (!ZL_isError(r)) r = dctx->batch.check(s);
    if (ZL_isError(r)) {
        dctx->err = dctx->batch.err;
        return done(r);
    }
    const ozl::FramePlan& fp = dctx->batch.plan.frames[0];
    for (size_t o = 0; o < nbOutputs; o++) {
        ZL_TypedBuffer_s* out = outputs[o];
        size_t const bytes = size_t(fp.outSizes[o]);
        ZL_Type const type = ZL_Type(fp.outTypes[o]);
        size_t const w = type == ZL_Type_serial || type == ZL_Type_string ? 1 : fp.outWidths[o];
        void* dst;
        if (type == ZL_Type_string) {
            if (out->wrap) { dctx->err = "string outputs need a DCtx-allocated buffer"; return done(fail(ZL_ErrorCode_GENERIC)); }
            try {
                out->lens.resize(size_t(fp.nbStrings[o]));
            } catch (...) {
                return done(fail(ZL_ErrorCode_allocation));
            }
            if (!out->lens.empty()
                && cudaMemcpyAsync(out->lens.data(), static_cast<uint8_t*>(dO) + lensOffs[o], 4 * out->lens.size(),
                                   cudaMemcpyDeviceToHost, s) != cudaSuccess)
                return done(fail(ZL_ErrorCode_GENERIC));
        }
        if (out->wrap) {
            if (bytes > out->capacity) { dctx->err = "output buffer too small"; return done(fail(ZL_ErrorCode_dstCapacity_tooSmall)); }
            if (type != out->type || (type != ZL_Type_serial && w != out->width)) {
                dctx->err = "a wrapped buffer's type or width differs from the frame's output";
                return done(fail(ZL_ErrorCode_GENERIC));
            }
            dst = out->wrapped;
        } else {
            try {
                out->own.resize(bytes + 1);
            } catch (...) {
                return done(fail(ZL_ErrorCode_allocation));
            }
            dst = out->own.data();
        }
        if (bytes && cudaMemcpyAsync(dst, static_cast<uint8_t*>(dO) + offs[o], bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return done(fail(ZL_ErrorCode_GENERIC));
        out->type = type;
        out->width = w;
        out->bytes = bytes;
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) return done(fail(ZL_ErrorCode_GENERIC));
    return done(ok(nbOutputs));
}

// ---------------------------------------------------------------------------
// Frame information from the frame header (decode_frameheader.c:290-470).
struct ZL_FrameInfo_s {
    unsigned version;
    std::vector<int> types;
    std::vector<uint64_t> sizes, nbStrings;
};

ZL_FrameInfo* ZL_FrameInfo_create(const void* src, size_t cSize)
{
    if (!src) return nullptr;
    ozl::FrameHeader h;
    std::string err;
    if (ozl::parseFrameHeader(static_cast<const uint8_t*>(src), cSize, h, err)) return nullptr;
    ZL_FrameInfo_s* fi = new (std::nothrow) ZL_FrameInfo_s();
    if (!fi) return nullptr;
    fi->version = h.version;
    fi->types = h.types; // the planner's type codes are ZL_Type's values
    fi->sizes = h.sizes;
    fi->nbStrings = h.nbStrings;
    return fi;
}
void ZL_FrameInfo_free(ZL_FrameInfo* fi) { delete fi; }
ZL_Report ZL_FrameInfo_getFormatVersion(const ZL_FrameInfo* fi)
{
    return fi ? ok(fi->version) : fail(ZL_ErrorCode_parameter_invalid);
}
ZL_Report ZL_FrameInfo_getNumOutputs(const ZL_FrameInfo* fi)
{
    return fi ? ok(fi->sizes.size()) : fail(ZL_ErrorCode_parameter_invalid);
}
// decode_frameheader.c:421-437: an ID past the outputs is outputID_invalid
static bool badOutput(const ZL_FrameInfo* fi, int id) { return id < 0 || size_t(id) >= fi->sizes.size(); }
ZL_Report ZL_FrameInfo_getOutputType(const ZL_FrameInfo* fi, int id)
{
    if (!fi) return fail(ZL_ErrorCode_parameter_invalid);
    if (badOutput(fi, id)) return fail(ZL_ErrorCode_outputID_invalid);
    return ok(size_t(fi->types[size_t(id)]));
}
ZL_Report ZL_FrameInfo_getDecompressedSize(const ZL_FrameInfo* fi, int id)
{
    if (!fi) return fail(ZL_ErrorCode_parameter_invalid);
    if (badOutput(fi, id)) return fail(ZL_ErrorCode_outputID_invalid);
    return ok(size_t(fi->sizes[size_t(id)]));
}
ZL_Report ZL_FrameInfo_getNumElts(const ZL_FrameInfo* fi, int id)
{
    if (!fi) return fail(ZL_ErrorCode_parameter_invalid);
    if (badOutput(fi, id)) return fail(ZL_ErrorCode_outputID_invalid);
    // decode_frameheader.c:448-453: frames before v21 carry no element counts
    if (fi->version < 21) return fail(ZL_ErrorCode_GENERIC);
    // decode_frameheader.c:455-467: counts known for serial outputs only
    int const t = fi->types[size_t(id)];
    if (t == ZL_Type_struct || t == ZL_Type_numeric) return fail(ZL_ErrorCode_temporaryLibraryLimitation);
    if (t == ZL_Type_string) return ok(size_t(fi->nbStrings[size_t(id)]));
    return ok(size_t(fi->sizes[size_t(id)]));
}

} // extern "C"
