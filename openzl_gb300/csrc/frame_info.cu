// Frame-header summaries parsed on the device (ozl_gpu_frame_info), one
// thread per frame, for frames that live in device memory. The parse
// restates the host planner's parseFrameHeader and frameOutputLayout
// (dec_plan.cpp) without containers, with the same checks in the same order
// and the same error codes, after src/openzl/decompress/decode_frameheader.c:
// 58-190 (format versions 8-20: output count and types from byte 4 onwards,
// LE32 sizes) and 94-107, 148-250, 270-370 (versions 21-23: flags byte,
// packed types, varint sizes, string counts, comment, header checksum byte).
// The GPU tests compare every record with the host's on the reference's
// frames and on truncated and corrupted copies.
#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/openzl_gb300.h"

namespace ozl {
namespace {

constexpr uint32_t kMagicBase = 0xD7B1A5C0u;
enum : int { FI_SERIAL = 1, FI_STRUCT = 2, FI_NUMERIC = 4, FI_STRING = 8 };
enum : int { FI_SRC_SMALL = 3, FI_CORRUPT = 12, FI_VERSION = 60, FI_LIMIT = 81 };

__device__ __forceinline__ int fiType(uint32_t code)
{
    return code == 0 ? FI_SERIAL : code == 1 ? FI_STRUCT : code == 2 ? FI_NUMERIC : FI_STRING;
}

// LEB128 varint of at most ten bytes from [p, end); advances p
__device__ bool fiVarint(const uint8_t*& p, const uint8_t* end, uint64_t& v)
{
    v = 0;
    for (int sh = 0; sh < 70; sh += 7) {
        if (p >= end) return false;
        uint8_t const b = *p++;
        v |= uint64_t(b & 0x7f) << sh;
        if (!(b & 0x80)) return true;
    }
    return false;
}

__device__ int fiParse(const uint8_t* src, uint64_t size, OZL_FrameInfo& o)
{
    if (size < 8) return FI_SRC_SMALL;
    uint32_t const magic = uint32_t(src[0]) | (uint32_t(src[1]) << 8) | (uint32_t(src[2]) << 16) | (uint32_t(src[3]) << 24);
    if (magic < kMagicBase + 8 || magic > kMagicBase + 23) return FI_VERSION;
    uint32_t const version = magic - kMagicBase;
    uint64_t nbOut = 1, pos = 4, extent = 0;
    int type0 = FI_SERIAL;
    uint64_t size0 = 0, end = 0;
    uint32_t flags = 0;
    if (version < 21) {
        if (version >= 15) {
            if (size < pos + 1 + 4) return FI_SRC_SMALL;
            uint8_t t = src[pos++];
            nbOut = uint64_t(t >> 6) + 1;
            if (nbOut == 4) {
                if (pos >= size) return FI_SRC_SMALL;
                t = src[pos++];
                nbOut = uint64_t(t >> 4) + 4;
            }
            if (nbOut == 19) {
                if (pos >= size) return FI_SRC_SMALL;
                t = src[pos++];
                nbOut = uint64_t(t) + 19;
            }
            if (nbOut == 274) {
                if (pos + 2 > size) return FI_SRC_SMALL;
                nbOut = uint64_t(src[pos] | (src[pos + 1] << 8)) + 274;
                pos += 2;
            }
        } else if (version == 14) {
            pos++; // the type byte
        }
        if (nbOut > 2048) return FI_LIMIT;
        // types: outputs 0-2 in byte 4, 3-4 in byte 5, then four per byte
        uint64_t typePos = pos;
        if (version >= 14 && nbOut > 5) {
            uint64_t const nb = (nbOut - 5 + 3) / 4;
            if (pos + nb > size) return FI_SRC_SMALL;
            pos += nb;
        }
        auto typeOf = [&](uint64_t n) -> int {
            if (version < 14) return FI_SERIAL;
            if (n < 3) return fiType((src[4] >> (2 * n)) & 3);
            if (n < 5) return fiType((src[5] >> (2 * (n - 3))) & 3);
            return fiType((src[typePos + (n - 5) / 4] >> (((n - 5) % 4) * 2)) & 3);
        };
        if (pos + 4 * nbOut > size) return FI_SRC_SMALL;
        for (uint64_t n = 0; n < nbOut; n++)
            if (typeOf(n) == FI_STRING) return FI_LIMIT;
        for (uint64_t n = 0; n < nbOut; n++) {
            const uint8_t* q = src + pos + 4 * n;
            uint64_t const sz = uint64_t(q[0]) | (uint64_t(q[1]) << 8) | (uint64_t(q[2]) << 16) | (uint64_t(q[3]) << 24);
            extent = ((extent + 15) & ~uint64_t(15)) + sz;
            if (n == 0) size0 = sz;
        }
        type0 = typeOf(0);
        end = pos + 4 * nbOut;
    } else {
        if (size < 9) return FI_SRC_SMALL;
        uint8_t const fl = src[4];
        bool const hasContent = fl & 1, hasCompressed = (fl >> 1) & 1, hasComment = (fl >> 2) & 1;
        uint8_t const t1 = src[5];
        pos = 6;
        nbOut = t1 & 15;
        uint64_t done = 0;
        if (nbOut == 15) {
            if (pos >= size) return FI_SRC_SMALL;
            uint8_t const t2 = src[pos++];
            nbOut = (uint64_t(t2) << 4) + (t1 >> 4) + 15;
        }
        if (nbOut == 0) return FI_CORRUPT;
        if (nbOut > 2048) return FI_LIMIT;
        if ((t1 & 15) != 15) done = 2;
        uint64_t const typePos = pos;
        if (nbOut > done) {
            uint64_t const nb = (nbOut - done + 3) / 4;
            if (pos + nb > size) return FI_SRC_SMALL;
            pos += nb;
        }
        auto typeOf = [&](uint64_t n) -> int {
            if (n < done) return fiType((t1 >> (4 + 2 * n)) & 3);
            return fiType((src[typePos + (n - done) / 4] >> (((n - done) % 4) * 2)) & 3);
        };
        // sizes (all, as the host parses them), then the string counts in
        // output order beside a second pass over the sizes
        const uint8_t* const lim = src + size;
        const uint8_t* p = src + pos;
        for (uint64_t n = 0; n < nbOut; n++) {
            uint64_t v;
            if (!fiVarint(p, lim, v)) return FI_SRC_SMALL;
            if (v == 0) return FI_LIMIT;
        }
        const uint8_t* ps = src + pos; // sizes again
        const uint8_t* pc = p;         // string counts
        for (uint64_t n = 0; n < nbOut; n++) {
            uint64_t v, ns = 0;
            fiVarint(ps, lim, v);
            int const ty = typeOf(n);
            if (ty == FI_STRING && !fiVarint(pc, lim, ns)) return FI_SRC_SMALL;
            extent = ((extent + 15) & ~uint64_t(15)) + (v - 1);
            if (ty == FI_STRING) extent = ((extent + 15) & ~uint64_t(15)) + 4 * ns;
            if (n == 0) {
                size0 = v - 1;
                type0 = ty;
            }
        }
        p = pc;
        if (version >= 22 && hasComment) {
            uint64_t c;
            if (!fiVarint(p, lim, c) || c == 0 || c > uint64_t(lim - p)) return FI_CORRUPT;
            p += c;
        }
        end = uint64_t(p - src);
        flags = (hasContent ? 1u : 0u) | (hasCompressed ? 2u : 0u);
        if (hasCompressed) {
            if (end + 1 > size) return FI_SRC_SMALL;
            flags |= 4u;
            end++;
        }
    }
    o.formatVersion = version;
    o.nbOutputs = uint32_t(nbOut);
    o.flags = flags;
    o.headerBytes = end;
    o.output0Bytes = size0;
    o.output0Type = type0;
    o.extent = extent;
    return 0;
}

__global__ void __launch_bounds__(128) kFrameInfo(const uint8_t* const* __restrict__ frames,
                                                  const uint64_t* __restrict__ sizes, uint64_t n,
                                                  OZL_FrameInfo* __restrict__ out)
{
    uint64_t const i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    OZL_FrameInfo o{};
    int const rc = fiParse(frames[i], sizes[i], o);
    if (rc) {
        o = OZL_FrameInfo{};
        o.status = rc;
    }
    out[i] = o;
}

} // namespace
} // namespace ozl

extern "C" ZL_Report ozl_gpu_frame_info(const void* const* d_frames, const uint64_t* d_frameSizes, size_t n,
                                        OZL_FrameInfo* d_info, void* stream)
{
    if (n && (!d_frames || !d_frameSizes || !d_info)) return ZL_Report{ ZL_ErrorCode_parameter_invalid, 0 };
    if (!n) return ZL_Report{ ZL_ErrorCode_no_error, 0 };
    uint64_t const grid = (uint64_t(n) + 127) / 128;
    if (grid > 0x7fffffffu) return ZL_Report{ ZL_ErrorCode_parameter_invalid, 0 };
    ozl::kFrameInfo<<<unsigned(grid), 128, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const uint8_t* const*>(d_frames), d_frameSizes, n, d_info);
    if (cudaGetLastError() != cudaSuccess) return ZL_Report{ ZL_ErrorCode_GENERIC, 0 };
    return ZL_Report{ ZL_ErrorCode_no_error, n };
}
