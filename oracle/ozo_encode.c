/* CPU restatement of the OpenZL encoder for the numeric graph recipes
 * (test infrastructure only). */
#include "ozo_internal.h"

size_t ozo_compress_bound(size_t srcSize) { return srcSize * 2 + 4096; }

int64_t ozo_compress(int recipe, const void* src, size_t nbElts, int eltWidth,
                     void* dst, size_t dstCap, int checksums)
{
    (void)recipe; (void)src; (void)nbElts; (void)eltWidth; (void)dst; (void)dstCap; (void)checksums;
    return -OZO_ERR_UNSUPPORTED;
}
