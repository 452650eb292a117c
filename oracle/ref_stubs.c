/* Stubs for the zstd and lz4 codec bindings of the reference library.
 *
 * The reference links its zstd/lz4 codecs against third-party libraries
 * (zstd 1.5.7, lz4 1.10.0) that are not vendored with its sources. Neither
 * codec is on the numeric codec-graph path, so the oracle build replaces the
 * four binding files (src/openzl/codecs/{zstd,lz4}/*_binding.c) with these
 * error-returning stand-ins. Test infrastructure only.
 */
#include "openzl/zl_compressor.h"
#include "openzl/zl_ctransform.h"
#include "openzl/zl_dtransform.h"
#include "openzl/zl_errors.h"
#include "openzl/codecs/zl_lz4.h"

#include <string.h>

ZL_Report DI_zstd(ZL_Decoder* d, const ZL_Input* ins[]);
ZL_Report EI_zstd(ZL_Encoder* e, const ZL_Input* ins[], size_t n);
void* DIZSTD_createDCtx(void);
void DIZSTD_freeDCtx(void* s);
void* EIZSTD_createCCtx(void);
void EIZSTD_freeCCtx(void* s);
ZL_Report DI_lz4(ZL_Decoder* d, const ZL_Input* ins[]);
ZL_Report EI_lz4(ZL_Encoder* e, const ZL_Input* ins[], size_t n);
ZL_GraphID ZL_Compressor_registerZstdGraph_withLevel(ZL_Compressor* c, int l);

ZL_Report DI_zstd(ZL_Decoder* d, const ZL_Input* ins[])
{
    (void)d; (void)ins;
    return ZL_returnError(ZL_ErrorCode_GENERIC);
}
ZL_Report EI_zstd(ZL_Encoder* e, const ZL_Input* ins[], size_t n)
{
    (void)e; (void)ins; (void)n;
    return ZL_returnError(ZL_ErrorCode_GENERIC);
}
void* DIZSTD_createDCtx(void) { return (void*)1; }
void DIZSTD_freeDCtx(void* s) { (void)s; }
void* EIZSTD_createCCtx(void) { return (void*)1; }
void EIZSTD_freeCCtx(void* s) { (void)s; }
ZL_Report DI_lz4(ZL_Decoder* d, const ZL_Input* ins[])
{
    (void)d; (void)ins;
    return ZL_returnError(ZL_ErrorCode_GENERIC);
}
ZL_Report EI_lz4(ZL_Encoder* e, const ZL_Input* ins[], size_t n)
{
    (void)e; (void)ins; (void)n;
    return ZL_returnError(ZL_ErrorCode_GENERIC);
}
ZL_GraphID ZL_Compressor_registerZstdGraph_withLevel(ZL_Compressor* c, int l)
{
    (void)c; (void)l;
    return ZL_GRAPH_ILLEGAL;
}
ZL_RESULT_OF(ZL_GraphID) ZL_Compressor_buildLZ4Graph(ZL_Compressor* c, int l)
{
    (void)c; (void)l;
    ZL_RESULT_OF(ZL_GraphID) r;
    memset(&r, 0, sizeof(r));
    r._code = ZL_ErrorCode_GENERIC;
    return r;
}
