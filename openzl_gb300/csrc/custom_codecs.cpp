// Custom-codec registration entry points (include/openzl/zl_ctransform.h:170,
// :287, :359; include/openzl/zl_dtransform.h:97, :177, :217).
//
// A custom codec runs the caller's own host functions and writes a custom
// transform ID into the frame (common/wire_format.h:91-94, :199). Neither fits
// this library: there is no device form of a host callback, and a custom
// transform cannot give the standard codecs' frame bytes. The entry points are
// exported so that programs built against the reference's headers link; each
// refuses the registration. Encoders return ZL_NODE_ILLEGAL (the reference's
// failure value, zl_ctransform.h:369) and record the reason on the
// compressor; decoders return ZL_ErrorCode_temporaryLibraryLimitation.
//
// The reference takes ownership of a descriptor's opaque pointer even when
// registration fails (zl_ctransform.h:141-146, zl_dtransform.h:82-87), so a
// refusal still calls its free function once. The descriptors are read
// through layout mirrors of the reference's structs, kept private here: the
// public header declares the descriptor types opaque, since nothing else in
// this library reads them.
#include <cstddef>

#include "../../include/openzl_gb300.h"

// compress_api.cpp: records the reason a registration failed on the compressor
void ozl_compressor_set_error(ZL_Compressor* c, const char* msg);

namespace {

// zl_common_types.h:24-48
struct OpaquePtr {
    void* ptr;
    void* freeOpaquePtr;
    void (*freeFn)(void* freeOpaquePtr, void* ptr);
};
// zl_localParams.h:56-126: three {pointer, count} pairs
struct LocalParams {
    const void* p0; size_t n0;
    const void* p1; size_t n1;
    const void* p2; size_t n2;
};
// zl_ctransform.h:65-70
struct StateMgr {
    void* (*stateAlloc)(void);
    void (*stateFree)(void*);
    size_t optionalStateID;
};
// zl_ctransform.h:116-128 (typed), :223-231 (variable outputs), :316-323 (multiple inputs)
struct TypedGraphDesc { ZL_IDType CTid; int inStreamType; const int* outTypes; size_t nbOut; };
struct VOGraphDesc { ZL_IDType CTid; int inStreamType; const int* soTypes; size_t nbSO; const int* voTypes; size_t nbVO; };
struct MIGraphDesc {
    ZL_IDType CTid; const int* inTypes; size_t nbIn; int lastVariable;
    const int* soTypes; size_t nbSO; const int* voTypes; size_t nbVO;
};
// encoder descriptors: graph, function, local params, name, state manager, opaque
template <class G> struct EncoderDesc {
    G gd;
    void* fn;
    LocalParams localParams;
    const char* name;
    StateMgr mgr;
    OpaquePtr opaque;
};
// decoder descriptors: graph, function, name, state manager, opaque
template <class G> struct DecoderDesc {
    G gd;
    void* fn;
    const char* name;
    StateMgr mgr;
    OpaquePtr opaque;
};

// offsets of `opaque` in the reference's structs on LP64 targets
static_assert(offsetof(EncoderDesc<TypedGraphDesc>, opaque) == 112, "ZL_TypedEncoderDesc layout");
static_assert(offsetof(EncoderDesc<VOGraphDesc>, opaque) == 128, "ZL_VOEncoderDesc layout");
static_assert(offsetof(EncoderDesc<MIGraphDesc>, opaque) == 152, "ZL_MIEncoderDesc layout");
static_assert(offsetof(DecoderDesc<TypedGraphDesc>, opaque) == 64, "ZL_TypedDecoderDesc layout");
static_assert(offsetof(DecoderDesc<VOGraphDesc>, opaque) == 80, "ZL_VODecoderDesc layout");
static_assert(offsetof(DecoderDesc<MIGraphDesc>, opaque) == 104, "ZL_MIDecoderDesc layout");

void release(const OpaquePtr& o)
{
    if (o.freeFn) o.freeFn(o.freeOpaquePtr, o.ptr);
}

template <class D> ZL_NodeID refuseEncoder(ZL_Compressor* c, const void* desc)
{
    if (desc) release(static_cast<const D*>(desc)->opaque);
    ozl_compressor_set_error(c, "custom encoders are not supported: the GPU path implements the standard codecs only");
    return ZL_NodeID{ 0 };
}

template <class D> ZL_Report refuseDecoder(ZL_DCtx* d, const void* desc)
{
    if (desc) release(static_cast<const D*>(desc)->opaque);
    (void)d;
    return ZL_Report{ ZL_ErrorCode_temporaryLibraryLimitation, 0 };
}

} // namespace

extern "C" {

ZL_NodeID ZL_Compressor_registerTypedEncoder(ZL_Compressor* c, const ZL_TypedEncoderDesc* d)
{
    return refuseEncoder<EncoderDesc<TypedGraphDesc>>(c, d);
}

ZL_NodeID ZL_Compressor_registerVOEncoder(ZL_Compressor* c, const ZL_VOEncoderDesc* d)
{
    return refuseEncoder<EncoderDesc<VOGraphDesc>>(c, d);
}

ZL_NodeID ZL_Compressor_registerMIEncoder(ZL_Compressor* c, const ZL_MIEncoderDesc* d)
{
    return refuseEncoder<EncoderDesc<MIGraphDesc>>(c, d);
}

ZL_Report ZL_DCtx_registerTypedDecoder(ZL_DCtx* dctx, const ZL_TypedDecoderDesc* d)
{
    return refuseDecoder<DecoderDesc<TypedGraphDesc>>(dctx, d);
}

ZL_Report ZL_DCtx_registerVODecoder(ZL_DCtx* dctx, const ZL_VODecoderDesc* d)
{
    return refuseDecoder<DecoderDesc<VOGraphDesc>>(dctx, d);
}

ZL_Report ZL_DCtx_registerMIDecoder(ZL_DCtx* dctx, const ZL_MIDecoderDesc* d)
{
    return refuseDecoder<DecoderDesc<MIGraphDesc>>(dctx, d);
}

} // extern "C"
