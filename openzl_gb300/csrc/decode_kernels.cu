// sm_103a decode kernels for OpenZL's numeric codec graph.
//
// All work here is integer and HBM/latency bound: no tensor cores. Each
// kernel takes a task array plus, for data-parallel kinds, a tile list; the
// host planner (dec_plan.cpp) builds both. Kernels never trap: malformed
// input sets the batch status word (first error wins) and the kernel moves
// on. Every spin-wait is bounded.
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "dec_tasks.h"
#include "dec_exec.h"
#include "stream_ring.cuh"

namespace ozl {

// ---------------------------------------------------------------------------
// helpers

__device__ __forceinline__ void reportError(uint32_t* status, uint32_t code)
{
    atomicCAS(status, 0u, code);
}

// 8 bytes from any address inside a buffer that this library allocated with
// at least 16 bytes of slack on both sides of every stream it reads this way.
__device__ __forceinline__ uint64_t ld64Any(const uint8_t* p)
{
    uintptr_t const a = reinterpret_cast<uintptr_t>(p) & ~uintptr_t(7);
    unsigned const s = unsigned(reinterpret_cast<uintptr_t>(p) - a) * 8u;
    uint64_t const lo = *reinterpret_cast<const uint64_t*>(a);
    if (s == 0) return lo;
    uint64_t const hi = *reinterpret_cast<const uint64_t*>(a + 8);
    return (lo >> s) | (hi << (64u - s));
}

__device__ __forceinline__ uint64_t ldElem(const uint8_t* p, uint32_t w)
{
    switch (w) {
        case 1: return *p;
        case 2: return (reinterpret_cast<uintptr_t>(p) & 1) ? (uint64_t(p[0]) | (uint64_t(p[1]) << 8))
                                                           : *reinterpret_cast<const uint16_t*>(p);
        case 4:
            if (!(reinterpret_cast<uintptr_t>(p) & 3)) return *reinterpret_cast<const uint32_t*>(p);
            return uint64_t(p[0]) | (uint64_t(p[1]) << 8) | (uint64_t(p[2]) << 16) | (uint64_t(p[3]) << 24);
        default:
            if (!(reinterpret_cast<uintptr_t>(p) & 7)) return *reinterpret_cast<const uint64_t*>(p);
            {
                uint64_t v = 0;
                for (int b = 0; b < 8; b++) v |= uint64_t(p[b]) << (8 * b);
                return v;
            }
    }
}

__device__ __forceinline__ void stElem(uint8_t* p, uint64_t v, uint32_t w)
{
    switch (w) {
        case 1: *p = uint8_t(v); break;
        case 2:
            if (!(reinterpret_cast<uintptr_t>(p) & 1)) *reinterpret_cast<uint16_t*>(p) = uint16_t(v);
            else { p[0] = uint8_t(v); p[1] = uint8_t(v >> 8); }
            break;
        case 4:
            if (!(reinterpret_cast<uintptr_t>(p) & 3)) *reinterpret_cast<uint32_t*>(p) = uint32_t(v);
            else for (int b = 0; b < 4; b++) p[b] = uint8_t(v >> (8 * b));
            break;
        default:
            if (!(reinterpret_cast<uintptr_t>(p) & 7)) *reinterpret_cast<uint64_t*>(p) = v;
            else for (int b = 0; b < 8; b++) p[b] = uint8_t(v >> (8 * b));
    }
}

__device__ __forceinline__ uint64_t umin64(uint64_t a, uint64_t b) { return a < b ? a : b; }

__device__ __forceinline__ uint64_t widthMask(uint32_t w)
{
    return w >= 8 ? ~0ull : ((1ull << (8 * w)) - 1);
}

// ---------------------------------------------------------------------------
// copy / constant: tiles of kTileBytes output bytes

// 16 bytes starting `off` bytes (1..15) into the 32 bytes (u0, u1); q and r
// are off / 4 and (off % 4) * 8, uniform across the block
__device__ __forceinline__ uint4 shiftCombine(uint4 u0, uint4 u1, uint32_t q, uint32_t r)
{
    uint32_t y0, y1, y2, y3, y4;
    switch (q) {
        case 0: y0 = u0.x; y1 = u0.y; y2 = u0.z; y3 = u0.w; y4 = u1.x; break;
        case 1: y0 = u0.y; y1 = u0.z; y2 = u0.w; y3 = u1.x; y4 = u1.y; break;
        case 2: y0 = u0.z; y1 = u0.w; y2 = u1.x; y3 = u1.y; y4 = u1.z; break;
        default: y0 = u0.w; y1 = u1.x; y2 = u1.y; y3 = u1.z; y4 = u1.w; break;
    }
    return make_uint4(__funnelshift_r(y0, y1, r), __funnelshift_r(y1, y2, r), __funnelshift_r(y2, y3, r),
                      __funnelshift_r(y3, y4, r));
}

// Copies one tile: bytes up to the destination's 16-byte boundary, then
// 16-byte stores, each from the two aligned 16-byte source blocks that hold
// its bytes (both blocks hold bytes of the source, so nothing outside the
// source's blocks is read), then the tail bytes.
__global__ void __launch_bounds__(256) kCopy(const CopyTask* __restrict__ tasks, const TileRef* __restrict__ tiles)
{
    TileRef const tr = tiles[blockIdx.x];
    CopyTask const t = tasks[tr.task];
    uint64_t const b0 = uint64_t(tr.tile) * kTileBytes;
    uint64_t const b1 = min(t.bytes, b0 + kTileBytes);
    uint64_t const head = min(b1 - b0, uint64_t((16 - (reinterpret_cast<uintptr_t>(t.dst + b0) & 15)) & 15));
    for (uint64_t i = b0 + threadIdx.x; i < b0 + head; i += blockDim.x) t.dst[i] = t.src[i];
    uint64_t const a0 = b0 + head;
    uint64_t const nv = (b1 - a0) / 16;
    uint4* const d = reinterpret_cast<uint4*>(t.dst + a0);
    uintptr_t const sa = reinterpret_cast<uintptr_t>(t.src + a0);
    uint32_t const off = uint32_t(sa & 15);
    const uint4* const s = reinterpret_cast<const uint4*>(sa - off);
    if (off == 0) {
#pragma unroll 4
        for (uint64_t i = threadIdx.x; i < nv; i += blockDim.x) d[i] = __ldg(s + i);
    } else {
        uint32_t const q = off >> 2, r = (off & 3) * 8;
#pragma unroll 4
        for (uint64_t i = threadIdx.x; i < nv; i += blockDim.x) d[i] = shiftCombine(__ldg(s + i), __ldg(s + i + 1), q, r);
    }
    for (uint64_t i = a0 + nv * 16 + threadIdx.x; i < b1; i += blockDim.x) t.dst[i] = t.src[i];
}

__global__ void kConst(const ConstTask* __restrict__ tasks, const TileRef* __restrict__ tiles)
{
    TileRef const tr = tiles[blockIdx.x];
    ConstTask const t = tasks[tr.task];
    uint64_t const total = t.n * t.w;
    uint64_t const b0 = uint64_t(tr.tile) * kTileBytes;
    uint64_t const b1 = min(total, b0 + kTileBytes);
    if (t.w == 1) {
        uint8_t const v = t.value[0];
        uint32_t const v4 = v * 0x01010101u;
        // head bytes up to 16-byte alignment, then 16-byte stores
        uint64_t a = b0;
        uintptr_t const base = reinterpret_cast<uintptr_t>(t.out);
        uint64_t const alignStart = min(b1, (((base + b0 + 15) & ~uintptr_t(15)) - base));
        for (uint64_t i = a + threadIdx.x; i < alignStart; i += blockDim.x) t.out[i] = v;
        a = alignStart;
        uint64_t const nv = (b1 - a) / 16;
        uint4 const q = make_uint4(v4, v4, v4, v4);
        uint4* d = reinterpret_cast<uint4*>(t.out + a);
        for (uint64_t i = threadIdx.x; i < nv; i += blockDim.x) d[i] = q;
        for (uint64_t i = a + nv * 16 + threadIdx.x; i < b1; i += blockDim.x) t.out[i] = v;
    } else {
        for (uint64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) t.out[i] = t.value[i % t.w];
    }
}

// XXH3's published secret and primes (the checksum kernels below and the
// content-checksum block sums fused into the numeric pipeline).
__constant__ uint8_t kXxhSecret[192] = {
    0xb8, 0xfe, 0x6c, 0x39, 0x23, 0xa4, 0x4b, 0xbe, 0x7c, 0x01, 0x81, 0x2c, 0xf7, 0x21, 0xad, 0x1c,
    0xde, 0xd4, 0x6d, 0xe9, 0x83, 0x90, 0x97, 0xdb, 0x72, 0x40, 0xa4, 0xa4, 0xb7, 0xb3, 0x67, 0x1f,
    0xcb, 0x79, 0xe6, 0x4e, 0xcc, 0xc0, 0xe5, 0x78, 0x82, 0x5a, 0xd0, 0x7d, 0xcc, 0xff, 0x72, 0x21,
    0xb8, 0x08, 0x46, 0x74, 0xf7, 0x43, 0x24, 0x8e, 0xe0, 0x35, 0x90, 0xe6, 0x81, 0x3a, 0x26, 0x4c,
    0x3c, 0x28, 0x52, 0xbb, 0x91, 0xc3, 0x00, 0xcb, 0x88, 0xd0, 0x65, 0x8b, 0x1b, 0x53, 0x2e, 0xa3,
    0x71, 0x64, 0x48, 0x97, 0xa2, 0x0d, 0xf9, 0x4e, 0x38, 0x19, 0xef, 0x46, 0xa9, 0xde, 0xac, 0xd8,
    0xa8, 0xfa, 0x76, 0x3f, 0xe3, 0x9c, 0x34, 0x3f, 0xf9, 0xdc, 0xbb, 0xc7, 0xc7, 0x0b, 0x4f, 0x1d,
    0x8a, 0x51, 0xe0, 0x4b, 0xcd, 0xb4, 0x59, 0x31, 0xc8, 0x9f, 0x7e, 0xc9, 0xd9, 0x78, 0x73, 0x64,
    0xea, 0xc5, 0xac, 0x83, 0x34, 0xd3, 0xeb, 0xc3, 0xc5, 0x81, 0xa0, 0xff, 0xfa, 0x13, 0x63, 0xeb,
    0x17, 0x0d, 0xdd, 0x51, 0xb7, 0xf0, 0xda, 0x49, 0xd3, 0x16, 0x55, 0x26, 0x29, 0xd4, 0x68, 0x9e,
    0x2b, 0x16, 0xbe, 0x58, 0x7d, 0x47, 0xa1, 0xfc, 0x8f, 0xf8, 0xb8, 0xd1, 0x7a, 0xd0, 0x31, 0xce,
    0x45, 0xcb, 0x3a, 0x8f, 0x95, 0x16, 0x04, 0x28, 0xaf, 0xd7, 0xfb, 0xca, 0xbb, 0x4b, 0x40, 0x7e,
};

#define XP32_1 0x9E3779B1u
#define XP32_2 0x85EBCA77u
#define XP32_3 0xC2B2AE3Du
#define XP64_1 0x9E3779B185EBCA87ull
#define XP64_2 0xC2B2AE3D27D4EB4Full
#define XP64_3 0x165667B19E3779F9ull
#define XP64_4 0x85EBCA77C2B2AE63ull
#define XP64_5 0x27D4EB2F165667C5ull
#define XPMX1 0x165667919E3779F9ull
#define XPMX2 0x9FB21C651E98DF25ull

__device__ __forceinline__ uint64_t secret64(int off)
{
    uint64_t v = 0;
    for (int b = 0; b < 8; b++) v |= uint64_t(kXxhSecret[off + b]) << (8 * b);
    return v;
}
__device__ __forceinline__ uint32_t secret32(int off)
{
    return uint32_t(kXxhSecret[off]) | (uint32_t(kXxhSecret[off + 1]) << 8) | (uint32_t(kXxhSecret[off + 2]) << 16)
            | (uint32_t(kXxhSecret[off + 3]) << 24);
}
// ---------------------------------------------------------------------------
// Fused numeric pipeline: source (plain elements, byte planes or LSB-first
// bit-packed fields) -> optional zigzag -> optional delta -> output elements.
//
// Delta decoding is an exclusive prefix sum: out[i] = first + sum(src[0..i))
// modulo 2^(8w), src holding n-1 elements (decode_delta_kernel.c:232). A tile
// is kNumTileBytes of output (kNumTileBytes / w elements); thread t owns the
// 64 output bytes 64t..64t+63 of its tile and holds them as 16 words of
// little-endian elements, so every width keeps 64 bytes of loads in flight
// per thread. Byte and 16-bit elements are zigzagged and scanned four or two
// to a word with SIMD byte/halfword adds. Plain sources and planes are read
// with 16- or 8-byte loads (shifted into place when misaligned); bit-packed
// sources are staged through shared memory with coalesced loads, one pad
// word after every 32 so that the threads' field reads spread over the
// banks. Delta tasks take three launches, none of which waits on another
// CTA: the sum of every tile's sources, an exclusive scan of those sums per
// task (one warp per task), then the final pass that scans inside the tile
// and adds the tile's prefix.
constexpr int kNPThreads = 256;
constexpr int kNW = 16;                                   // words per thread
constexpr uint32_t kNPBytes = 4 * kNW;                    // 64 output bytes per thread
static_assert(kNPBytes * kNPThreads == kNumTileBytes, "tile = threads x bytes per thread");
constexpr uint32_t kNPStageWords = kNumTileBytes / 4 + 8; // the fields of a tile plus partial blocks at both ends
constexpr uint32_t kNPStagePadded = kNPStageWords + kNPStageWords / 32 + 1;

__device__ __forceinline__ uint32_t npPad(uint32_t q) { return q + (q >> 5); }

// NQ 16-byte blocks from p (any alignment; every block read holds bytes of
// the range) into w[0 .. 4 NQ)
template <int NQ>
__device__ __forceinline__ void npLdq(const uint8_t* p, uint32_t* w)
{
    uintptr_t const a = reinterpret_cast<uintptr_t>(p) & ~uintptr_t(15);
    uint32_t const off = uint32_t(reinterpret_cast<uintptr_t>(p) - a);
    const uint4* const s = reinterpret_cast<const uint4*>(a);
    if (off == 0) {
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            uint4 const u = __ldg(s + q);
            w[4 * q] = u.x; w[4 * q + 1] = u.y; w[4 * q + 2] = u.z; w[4 * q + 3] = u.w;
        }
    } else {
        uint32_t const qq = off >> 2, r = (off & 3) * 8;
        uint4 prev = __ldg(s);
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            uint4 const nxt = __ldg(s + q + 1);
            uint4 const u = shiftCombine(prev, nxt, qq, r);
            w[4 * q] = u.x; w[4 * q + 1] = u.y; w[4 * q + 2] = u.z; w[4 * q + 3] = u.w;
            prev = nxt;
        }
    }
}

// 8 bytes from p (any alignment) into w[0], w[1], from the aligned 8-byte
// words that hold them
__device__ __forceinline__ void npLd8(const uint8_t* p, uint32_t* w)
{
    uintptr_t const a = reinterpret_cast<uintptr_t>(p) & ~uintptr_t(7);
    uint32_t const off = uint32_t(reinterpret_cast<uintptr_t>(p) - a);
    const uint2* const s = reinterpret_cast<const uint2*>(a);
    uint2 const u0 = __ldg(s);
    if (off == 0) {
        w[0] = u0.x;
        w[1] = u0.y;
    } else {
        uint2 const u1 = __ldg(s + 1);
        uint32_t const r = (off & 3) * 8;
        uint32_t const x0 = off < 4 ? u0.x : u0.y, x1 = off < 4 ? u0.y : u1.x, x2 = off < 4 ? u1.x : u1.y;
        w[0] = __funnelshift_r(x0, x1, r);
        w[1] = __funnelshift_r(x1, x2, r);
    }
}

// Loads the thread's source elements j0 .. j0 + 64/W (those below nSrc; the
// rest read as 0) as 16 words of little-endian elements. `stage` holds the
// tile's bit-packed words (padded) for SRC_BITPACK, bit `sbit` being the
// first field of the tile.
template <int W, int MODE>
__device__ __forceinline__ void npLoad(const NumPipeTask& t, uint64_t j0, uint64_t nSrc, const uint32_t* stage,
                                       uint32_t sbit, uint32_t tileRel, uint32_t (&w)[kNW])
{
    constexpr uint32_t E = kNPBytes / W;
    uint32_t const cs = j0 < nSrc ? uint32_t(umin64(E, nSrc - j0)) : 0u;
    if constexpr (MODE == SRC_PLAIN) {
        if (cs == E) {
            npLdq<kNW / 4>(t.src + j0 * W, w);
        } else {
            const uint8_t* const p = t.src + j0 * W;
#pragma unroll
            for (int m = 0; m < kNW; m++) {
                uint32_t x = 0;
#pragma unroll
                for (int y = 0; y < 4; y++)
                    if (uint32_t(4 * m + y) < cs * W) x |= uint32_t(p[4 * m + y]) << (8 * y);
                w[m] = x;
            }
        }
    } else if constexpr (MODE == SRC_PLANES) {
        constexpr int PW = int(E / 4); // words per plane
        uint32_t raw[kNW];
        if (cs == E) {
#pragma unroll
            for (int b = 0; b < W; b++) {
                if constexpr (PW >= 4) npLdq<PW / 4>(t.planes[b] + j0, raw + PW * b);
                else npLd8(t.planes[b] + j0, raw + PW * b);
            }
        } else {
#pragma unroll
            for (int b = 0; b < W; b++) {
                const uint8_t* const pl = t.planes[b] + j0;
#pragma unroll
                for (int m = 0; m < PW; m++) {
                    uint32_t x = 0;
#pragma unroll
                    for (int y = 0; y < 4; y++)
                        if (uint32_t(4 * m + y) < cs) x |= uint32_t(pl[4 * m + y]) << (8 * y);
                    raw[PW * b + m] = x;
                }
            }
        }
        if constexpr (W == 1) {
#pragma unroll
            for (int m = 0; m < kNW; m++) w[m] = raw[m];
        } else if constexpr (W == 2) {
#pragma unroll
            for (int m = 0; m < kNW; m++) w[m] = __byte_perm(raw[m >> 1], raw[PW + (m >> 1)], (m & 1) ? 0x7362 : 0x5140);
        } else {
            // 4x4 byte transposes of planes 0-3 (and 4-7 for the high words)
#pragma unroll
            for (int h = 0; h < W / 4; h++) {
#pragma unroll
                for (int g = 0; g < PW; g++) {
                    uint32_t const* const pl = raw + PW * (4 * h);
                    uint32_t const p0 = pl[g], p1 = pl[PW + g], p2 = pl[2 * PW + g], p3 = pl[3 * PW + g];
                    uint32_t const t0 = __byte_perm(p0, p1, 0x5140), t1 = __byte_perm(p0, p1, 0x7362);
                    uint32_t const t2 = __byte_perm(p2, p3, 0x5140), t3 = __byte_perm(p2, p3, 0x7362);
                    uint32_t const e[4] = { __byte_perm(t0, t2, 0x5410), __byte_perm(t0, t2, 0x7632),
                                            __byte_perm(t1, t3, 0x5410), __byte_perm(t1, t3, 0x7632) };
#pragma unroll
                    for (int j = 0; j < 4; j++) w[(W / 4) * (4 * g + j) + h] = e[j];
                }
            }
        }
    } else {
        // LSB-first fields of nbBits (1..8W) from the staged words
        uint32_t const nb = t.nbBits;
#pragma unroll
        for (int m = 0; m < kNW; m++) w[m] = 0;
#pragma unroll
        for (uint32_t k = 0; k < E; k++) {
            uint64_t x = 0;
            if (k < cs) {
                uint32_t const bit = sbit + (tileRel + k) * nb;
                uint32_t const q = bit >> 5, r = bit & 31;
                uint32_t const w0 = stage[npPad(q)];
                uint32_t const w1 = (r + nb > 32) ? stage[npPad(q + 1)] : 0u;
                x = __funnelshift_r(w0, w1, r);
                if (r + nb > 64) x |= uint64_t(__funnelshift_r(w1, stage[npPad(q + 2)], r)) << 32;
                else if (nb > 32) x |= uint64_t(w1 >> r) << 32;
                if (nb < 64) x &= (1ull << nb) - 1;
            }
            if constexpr (W == 1) w[k >> 2] |= uint32_t(x) << (8 * (k & 3));
            else if constexpr (W == 2) w[k >> 1] |= uint32_t(x) << (16 * (k & 1));
            else if constexpr (W == 4) w[k] = uint32_t(x);
            else {
                w[2 * k] = uint32_t(x);
                w[2 * k + 1] = uint32_t(x >> 32);
            }
        }
    }
}

template <int W>
__device__ __forceinline__ void npZigzag(uint32_t (&w)[kNW])
{
#pragma unroll
    for (int m = 0; m < kNW; m++) {
        uint32_t const x = w[m];
        if constexpr (W == 1) w[m] = ((x >> 1) & 0x7f7f7f7fu) ^ ((x & 0x01010101u) * 0xffu);
        else if constexpr (W == 2) w[m] = ((x >> 1) & 0x7fff7fffu) ^ ((x & 0x00010001u) * 0xffffu);
        else if constexpr (W == 4) w[m] = (x >> 1) ^ (0u - (x & 1u));
    }
    if constexpr (W == 8) {
#pragma unroll
        for (int m = 0; m < kNW; m += 2) {
            uint64_t const v = uint64_t(w[m]) | (uint64_t(w[m + 1]) << 32);
            uint64_t const z = (v >> 1) ^ (0ull - (v & 1ull));
            w[m] = uint32_t(z);
            w[m + 1] = uint32_t(z >> 32);
        }
    }
}

// sum of the thread's elements (modulo 2^(8W) after masking)
template <int W>
__device__ __forceinline__ uint64_t npSum(const uint32_t (&w)[kNW])
{
    if constexpr (W == 1) {
        uint32_t acc = 0;
#pragma unroll
        for (int m = 0; m < kNW; m++) acc = __vadd4(acc, w[m]);
        return (acc & 0xff) + ((acc >> 8) & 0xff) + ((acc >> 16) & 0xff) + (acc >> 24);
    } else if constexpr (W == 2) {
        uint32_t acc = 0;
#pragma unroll
        for (int m = 0; m < kNW; m++) acc = __vadd2(acc, w[m]);
        return (acc & 0xffff) + (acc >> 16);
    } else if constexpr (W == 4) {
        uint32_t acc = 0;
#pragma unroll
        for (int m = 0; m < kNW; m++) acc += w[m];
        return acc;
    } else {
        uint64_t acc = 0;
#pragma unroll
        for (int m = 0; m < kNW; m += 2) acc += uint64_t(w[m]) | (uint64_t(w[m + 1]) << 32);
        return acc;
    }
}

// exclusive scan of the thread's elements in place
template <int W>
__device__ __forceinline__ void npScan(uint32_t (&w)[kNW])
{
    if constexpr (W == 1) {
        uint32_t c = 0;
#pragma unroll
        for (int m = 0; m < kNW; m++) {
            uint32_t p = __vadd4(w[m], w[m] << 8);
            p = __vadd4(p, p << 16);
            w[m] = __vadd4(p << 8, c * 0x01010101u);
            c = (c + (p >> 24)) & 0xffu;
        }
    } else if constexpr (W == 2) {
        uint32_t c = 0;
#pragma unroll
        for (int m = 0; m < kNW; m++) {
            uint32_t const p = __vadd2(w[m], w[m] << 16);
            w[m] = __vadd2(p << 16, c * 0x00010001u);
            c = (c + (p >> 16)) & 0xffffu;
        }
    } else if constexpr (W == 4) {
        uint32_t c = 0;
#pragma unroll
        for (int m = 0; m < kNW; m++) {
            uint32_t const x = w[m];
            w[m] = c;
            c += x;
        }
    } else {
        uint64_t c = 0;
#pragma unroll
        for (int m = 0; m < kNW; m += 2) {
            uint64_t const x = uint64_t(w[m]) | (uint64_t(w[m + 1]) << 32);
            w[m] = uint32_t(c);
            w[m + 1] = uint32_t(c >> 32);
            c += x;
        }
    }
}

// adds `add` (modulo 2^(8W)) to every element
template <int W>
__device__ __forceinline__ void npAdd(uint32_t (&w)[kNW], uint64_t add)
{
    if constexpr (W == 1) {
        uint32_t const a = uint32_t(add & 0xff) * 0x01010101u;
#pragma unroll
        for (int m = 0; m < kNW; m++) w[m] = __vadd4(w[m], a);
    } else if constexpr (W == 2) {
        uint32_t const a = uint32_t(add & 0xffff) * 0x00010001u;
#pragma unroll
        for (int m = 0; m < kNW; m++) w[m] = __vadd2(w[m], a);
    } else if constexpr (W == 4) {
#pragma unroll
        for (int m = 0; m < kNW; m++) w[m] += uint32_t(add);
    } else {
#pragma unroll
        for (int m = 0; m < kNW; m += 2) {
            uint64_t const v = (uint64_t(w[m]) | (uint64_t(w[m + 1]) << 32)) + add;
            w[m] = uint32_t(v);
            w[m + 1] = uint32_t(v >> 32);
        }
    }
}

// Stages the tile's bit-packed source in shared memory (padded words): the
// 16-byte blocks from the one holding the tile's first field to the one
// holding its last source bit. Returns the bit offset of the first field.
__device__ __forceinline__ uint32_t npStage(const NumPipeTask& t, uint64_t e0, uint64_t nSrc, uint32_t te,
                                            uint32_t* stage)
{
    uint64_t const firstBit = uint64_t(reinterpret_cast<uintptr_t>(t.src) & 15) * 8 + e0 * t.nbBits;
    uintptr_t const a = (reinterpret_cast<uintptr_t>(t.src) & ~uintptr_t(15)) + (firstBit >> 7) * 16;
    uint32_t const sbit = uint32_t(firstBit & 127);
    uint64_t const nFields = e0 < nSrc ? umin64(te, nSrc - e0) : 0;
    uint32_t const nq = nFields ? uint32_t((sbit + nFields * t.nbBits + 127) >> 7) : 0u;
    const uint4* const src = reinterpret_cast<const uint4*>(a);
    for (uint32_t q = threadIdx.x; q < nq; q += kNPThreads) {
        uint4 const u = __ldg(src + q);
        uint32_t const d = npPad(4 * q); // a block never straddles a pad word
        stage[d] = u.x;
        stage[d + 1] = u.y;
        stage[d + 2] = u.z;
        stage[d + 3] = u.w;
    }
    __syncthreads();
    return sbit;
}

template <int W>
__device__ __forceinline__ void npStore(uint8_t* out, uint32_t cnt, const uint32_t (&w)[kNW])
{
    constexpr uint32_t E = kNPBytes / W;
    if (cnt == E && !(reinterpret_cast<uintptr_t>(out) & 15)) {
#pragma unroll
        for (int q = 0; q < kNW / 4; q++)
            reinterpret_cast<uint4*>(out)[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
    } else {
#pragma unroll
        for (int k = 0; k < int(kNPBytes); k++)
            if (uint32_t(k) < cnt * W) out[k] = uint8_t(w[k >> 2] >> (8 * (k & 3)));
    }
}

// shared scratch of one tile
struct NPShared {
    uint32_t stage[kNPStagePadded];
    uint64_t warpVal[kNPThreads / 32];
    uint64_t key[24]; // XXH3 secret words at byte offsets 0, 8, ..., 184 (fused block sums)
};

// XXH3 block sums of the output, fused into the output pass. The thread's 64
// bytes (w, little-endian) are stripe tid % 16 of 1 KiB block `blk` of the
// checksummed output; the 16 threads of a block are one half-warp. Each
// thread adds its stripe's increments to 8 accumulators (acc[i ^ 1] +=
// d[i]; acc[i] += lo32(d[i] ^ k[i]) * hi32(d[i] ^ k[i]), k[i] the secret word
// at byte 8 (stripe + i)), then the half-warp reduce-scatters them: after
// four exchanges (4 + 2 + 1 + 1 shuffles) every lane holds the block total of
// accumulator 4 bit3 + 2 bit2 + bit1 of its lane index, and the even lane
// writes it where phase 1 would have. Every lane of the warp takes part; only
// blocks below hashBlocks are written.
__device__ __forceinline__ void npHashStripe(const NumPipeTask& t, const uint32_t* w, uint64_t blk,
                                             const uint64_t* key)
{
    uint32_t const lane = threadIdx.x & 31, s = lane & 15;
    uint64_t acc[8];
#pragma unroll
    for (int i = 0; i < 8; i++) acc[i] = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        uint64_t const d = uint64_t(w[2 * i]) | (uint64_t(w[2 * i + 1]) << 32);
        uint64_t const x = d ^ key[s + i];
        acc[i ^ 1] += d;
        acc[i] += uint64_t(uint32_t(x)) * (x >> 32);
    }
    bool const b3 = s & 8, b2 = s & 4, b1 = s & 2;
    uint64_t v4[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        uint64_t const send = b3 ? acc[k] : acc[k + 4];
        uint64_t const keep = b3 ? acc[k + 4] : acc[k];
        v4[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    uint64_t v2[2];
#pragma unroll
    for (int k = 0; k < 2; k++) {
        uint64_t const send = b2 ? v4[k] : v4[k + 2];
        uint64_t const keep = b2 ? v4[k + 2] : v4[k];
        v2[k] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    uint64_t v = (b1 ? v2[1] : v2[0]) + __shfl_xor_sync(0xffffffffu, b1 ? v2[0] : v2[1], 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    if (!(s & 1) && blk < t.hashBlocks) t.blockSums[8 * blk + 4 * b3 + 2 * b2 + b1] = v;
}

template <int W, int MODE>
__device__ __forceinline__ void npReduceTile(const NumPipeTask& t, const TileRef& tr, uint64_t* sums, uint32_t g,
                                             NPShared& sh)
{
    constexpr uint32_t TE = kNumTileBytes / W, E = kNPBytes / W;
    uint32_t const tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    uint64_t const e0 = uint64_t(tr.tile) * TE;
    uint64_t const nSrc = t.n ? t.n - 1 : 0;
    uint32_t sbit = 0;
    if constexpr (MODE == SRC_BITPACK) sbit = npStage(t, e0, nSrc, TE, sh.stage);
    uint32_t w[kNW];
    npLoad<W, MODE>(t, e0 + uint64_t(tid) * E, nSrc, sh.stage, sbit, tid * E, w);
    if (t.zigzag) npZigzag<W>(w);
    uint64_t acc = npSum<W>(w);
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, m);
    if (lane == 0) sh.warpVal[wid] = acc;
    __syncthreads();
    if (tid == 0) {
        uint64_t tot = 0;
#pragma unroll
        for (int w2 = 0; w2 < kNPThreads / 32; w2++) tot += sh.warpVal[w2];
        sums[g] = tot;
    }
}

template <int W, int MODE>
__device__ __forceinline__ void npTile(const NumPipeTask& t, const TileRef& tr, uint32_t g, const uint64_t* prefix,
                                       NPShared& sh)
{
    constexpr uint32_t TE = kNumTileBytes / W, E = kNPBytes / W;
    uint32_t const tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    uint64_t const e0 = uint64_t(tr.tile) * TE;
    uint64_t const j0 = e0 + uint64_t(tid) * E;
    uint32_t const cnt = j0 < t.n ? uint32_t(umin64(E, t.n - j0)) : 0;
    uint64_t const nSrc = t.delta ? (t.n ? t.n - 1 : 0) : t.n;
    uint32_t sbit = 0;
    if constexpr (MODE == SRC_BITPACK) sbit = npStage(t, e0, nSrc, TE, sh.stage);
    uint32_t w[kNW];
    npLoad<W, MODE>(t, j0, nSrc, sh.stage, sbit, tid * E, w);
    if (t.zigzag) npZigzag<W>(w);
    if (t.delta) {
        uint64_t const tot = npSum<W>(w);
        npScan<W>(w);
        // exclusive scan of thread totals within the warp, then across warps
        uint64_t incl = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint64_t const y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= uint32_t(o)) incl += y;
        }
        if (lane == 31) sh.warpVal[wid] = incl;
        __syncthreads();
        uint64_t warpPre = 0;
#pragma unroll
        for (int w2 = 0; w2 < kNPThreads / 32; w2++) warpPre += uint32_t(w2) < wid ? sh.warpVal[w2] : 0;
        npAdd<W>(w, t.first + prefix[g] + warpPre + (incl - tot));
    }
    if (cnt) npStore<W>(t.out + j0 * W, cnt, w);
    if (t.blockSums) npHashStripe(t, w, (uint64_t(tr.tile) * kNumTileBytes + uint64_t(tid) * kNPBytes) >> 10, sh.key);
}

template <int W>
__device__ __forceinline__ void npTileW(const NumPipeTask& t, const TileRef& tr, uint32_t g, const uint64_t* prefix,
                                        NPShared& sh)
{
    switch (t.srcMode) {
        case SRC_PLAIN: npTile<W, SRC_PLAIN>(t, tr, g, prefix, sh); break;
        case SRC_PLANES: npTile<W, SRC_PLANES>(t, tr, g, prefix, sh); break;
        default: npTile<W, SRC_BITPACK>(t, tr, g, prefix, sh); break;
    }
}

template <int W>
__device__ __forceinline__ void npReduceW(const NumPipeTask& t, const TileRef& tr, uint64_t* sums, uint32_t g,
                                          NPShared& sh)
{
    switch (t.srcMode) {
        case SRC_PLAIN: npReduceTile<W, SRC_PLAIN>(t, tr, sums, g, sh); break;
        case SRC_PLANES: npReduceTile<W, SRC_PLANES>(t, tr, sums, g, sh); break;
        default: npReduceTile<W, SRC_BITPACK>(t, tr, sums, g, sh); break;
    }
}

// pass 1 (delta tasks): sum of each tile's sources
__global__ void __launch_bounds__(kNPThreads) kNumReduce(const NumPipeTask* __restrict__ tasks,
                                                         const TileRef* __restrict__ tiles,
                                                         uint64_t* __restrict__ sums)
{
    __shared__ NPShared sh;
    uint32_t const g = blockIdx.x;
    TileRef const tr = tiles[g];
    NumPipeTask const t = tasks[tr.task];
    if (!t.delta) return;
    switch (t.w) {
        case 1: npReduceW<1>(t, tr, sums, g, sh); break;
        case 2: npReduceW<2>(t, tr, sums, g, sh); break;
        case 4: npReduceW<4>(t, tr, sums, g, sh); break;
        default: npReduceW<8>(t, tr, sums, g, sh); break;
    }
}

// pass 2: exclusive scan of tile sums per task, one warp per task
__global__ void __launch_bounds__(256) kNumPrefix(const NumPipeTask* __restrict__ tasks, uint32_t nbTasks,
                                                  const uint64_t* __restrict__ sums, uint64_t* __restrict__ prefix)
{
    uint32_t const ti = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t const lane = threadIdx.x & 31;
    if (ti >= nbTasks) return;
    NumPipeTask const t = tasks[ti];
    if (!t.delta) return;
    uint32_t const te = kNumTileBytes / t.w;
    uint32_t const nT = uint32_t((t.n + te - 1) / te);
    // 256 tiles per round: lane L scans tiles 8L .. 8L + 7 of the round in
    // registers, the warp scans the lanes' totals
    const uint64_t* const in = sums + t.tileBase;
    uint64_t* const out = prefix + t.tileBase;
    uint64_t running = 0;
    for (uint32_t k0 = 0; k0 < nT; k0 += 256) {
        uint32_t const k = k0 + 8 * lane;
        uint64_t x[8];
        uint64_t tot = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            x[j] = k + j < nT ? in[k + j] : 0;
            tot += x[j];
        }
        uint64_t incl = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint64_t const y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= uint32_t(o)) incl += y;
        }
        uint64_t run = running + incl - tot;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            if (k + j < nT) out[k + j] = run;
            run += x[j];
        }
        running += __shfl_sync(0xffffffffu, incl, 31);
    }
}

// pass 3: the output
__global__ void __launch_bounds__(kNPThreads) kNumPipe(const NumPipeTask* __restrict__ tasks,
                                                       const TileRef* __restrict__ tiles,
                                                       const uint64_t* __restrict__ prefix)
{
    __shared__ NPShared sh;
    uint32_t const g = blockIdx.x;
    TileRef const tr = tiles[g];
    NumPipeTask const t = tasks[tr.task];
    if (t.blockSums) { // the same task for the whole CTA
        if (threadIdx.x < 24) sh.key[threadIdx.x] = secret64(int(8 * threadIdx.x));
        __syncthreads();
    }
    switch (t.w) {
        case 1: npTileW<1>(t, tr, g, prefix, sh); break;
        case 2: npTileW<2>(t, tr, g, prefix, sh); break;
        case 4: npTileW<4>(t, tr, g, prefix, sh); break;
        default: npTileW<8>(t, tr, g, prefix, sh); break;
    }
}

// ---------------------------------------------------------------------------
// generic transpose (any width)
__global__ void kTranspose(const TransposeTask* __restrict__ tasks, const TileRef* __restrict__ tiles)
{
    TileRef const tr = tiles[blockIdx.x];
    TransposeTask const t = tasks[tr.task];
    uint64_t const e0 = uint64_t(tr.tile) * kTileElems;
    uint64_t const e1 = umin64(t.n, e0 + kTileElems);
    for (uint64_t i = e0 + threadIdx.x; i < e1; i += blockDim.x)
        for (uint32_t b = 0; b < t.W; b++) t.out[i * t.W + b] = t.planes[b][i];
}

// ---------------------------------------------------------------------------
// tokenize: dictionary gather out[i] = alphabet[idx[i]]
__global__ void kTokenize(const TokenizeTask* __restrict__ tasks, const TileRef* __restrict__ tiles,
                          uint32_t* __restrict__ status)
{
    TileRef const tr = tiles[blockIdx.x];
    TokenizeTask const t = tasks[tr.task];
    uint64_t const e0 = uint64_t(tr.tile) * kTileElems;
    uint64_t const e1 = umin64(t.n, e0 + kTileElems);
    bool bad = false;
    for (uint64_t i = e0 + threadIdx.x; i < e1; i += blockDim.x) {
        uint64_t const k = ldElem(t.idx + i * t.iw, t.iw);
        if (k >= t.alphabetSize) { bad = true; continue; }
        if (t.w == 4 || t.w == 2 || t.w == 1 || t.w == 8) stElem(t.out + i * t.w, ldElem(t.alphabet + k * t.w, t.w), t.w);
        else for (uint32_t b = 0; b < t.w; b++) t.out[i * t.w + b] = t.alphabet[k * t.w + b];
    }
    if (bad) reportError(status, DERR_CORRUPTION);
}

// ---------------------------------------------------------------------------
// string lengths to 4 bytes (NUMOP_write32_fromNumerics in
// DI_revert_VSF_separation, decode_conversion_binding.c:245-250)
__global__ void kWiden(const WidenTask* __restrict__ tasks, const TileRef* __restrict__ tiles,
                       uint32_t* __restrict__ status)
{
    TileRef const tr = tiles[blockIdx.x];
    WidenTask const t = tasks[tr.task];
    uint64_t const e0 = uint64_t(tr.tile) * kTileElems;
    uint64_t const e1 = umin64(t.n, e0 + kTileElems);
    bool bad = false;
    for (uint64_t i = e0 + threadIdx.x; i < e1; i += blockDim.x) {
        uint64_t const v = ldElem(t.src + i * t.w, t.w);
        bad |= v > 0xffffffffull;
        t.dst[i] = uint32_t(v);
    }
    if (bad) reportError(status, DERR_CORRUPTION);
}

// ---------------------------------------------------------------------------
// float deconstruct (decode_float_deconstruct_kernel.c semantics)
__global__ void kFloatDec(const FloatDecTask* __restrict__ tasks, const TileRef* __restrict__ tiles)
{
    TileRef const tr = tiles[blockIdx.x];
    FloatDecTask const t = tasks[tr.task];
    uint64_t const e0 = uint64_t(tr.tile) * kTileElems;
    uint64_t const e1 = umin64(t.n, e0 + kTileElems);
    for (uint64_t i = e0 + threadIdx.x; i < e1; i += blockDim.x) {
        uint32_t const ex = t.exponent[i];
        if (t.eltType == 1) {
            uint32_t const s = t.signFrac[i];
            stElem(t.out + 2 * i, uint16_t((s >> 1) | (s << 15) | (ex << 7)), 2);
        } else if (t.eltType == 2) {
            uint32_t const s = uint32_t(t.signFrac[2 * i]) | (uint32_t(t.signFrac[2 * i + 1]) << 8);
            stElem(t.out + 2 * i, uint16_t((s >> 1) | (s << 15) | (ex << 10)), 2);
        } else {
            uint32_t const s = uint32_t(t.signFrac[3 * i]) | (uint32_t(t.signFrac[3 * i + 1]) << 8)
                    | (uint32_t(t.signFrac[3 * i + 2]) << 16);
            stElem(t.out + 4 * i, (ex << 23) | (s << 31) | (s >> 1), 4);
        }
    }
}

// ---------------------------------------------------------------------------
// flatpack: alphabet + LSB-first indices terminated by a 1 bit
// Flatpack: out[i] = alphabet[field i], fields of nbBits (1..8) LSB-first.
// The alphabet sits in shared memory; each thread decodes 8 consecutive
// fields from a 64-bit window (three aligned words of the packed stream,
// funnel-shifted) and stores them with one 8-byte store. Only words that hold
// bytes of the packed stream are read (its last word holds the terminator).
__global__ void __launch_bounds__(256) kFlatpack(const FlatpackTask* __restrict__ tasks,
                                                 const TileRef* __restrict__ tiles, uint32_t* __restrict__ status)
{
    __shared__ uint8_t sAlpha[256];
    TileRef const tr = tiles[blockIdx.x];
    FlatpackTask const t = tasks[tr.task];
    uint32_t const as = min(t.alphabetSize, 256u);
    for (uint32_t i = threadIdx.x; i < as; i += blockDim.x) sAlpha[i] = t.alphabet[i];
    __syncthreads();
    uint32_t const nb = t.nbBits, mask = (1u << nb) - 1u;
    const uint32_t* const pw = reinterpret_cast<const uint32_t*>(reinterpret_cast<uintptr_t>(t.packed) & ~uintptr_t(3));
    uint64_t const sb = (reinterpret_cast<uintptr_t>(t.packed) & 3) * 8;
    uint64_t const qLast = (sb + t.n * nb) >> 5;
    uint64_t const e0 = uint64_t(tr.tile) * kTileBytes;
    uint64_t const e1 = umin64(t.n, e0 + kTileBytes);
    bool bad = false;
    for (uint64_t k0 = e0 + 8ull * threadIdx.x; k0 < e1; k0 += 8ull * blockDim.x) {
        uint32_t const cnt = uint32_t(umin64(8, e1 - k0));
        uint64_t const bit = sb + k0 * nb;
        uint64_t const q = bit >> 5;
        uint32_t const r = uint32_t(bit & 31);
        uint32_t const w0 = __ldg(pw + q);
        uint32_t const w1 = q + 1 <= qLast ? __ldg(pw + q + 1) : 0u;
        uint32_t const w2 = q + 2 <= qLast ? __ldg(pw + q + 2) : 0u;
        uint32_t const lo = __funnelshift_r(w0, w1, r), hi = __funnelshift_r(w1, w2, r);
        uint32_t o[2] = { 0u, 0u };
#pragma unroll
        for (uint32_t j = 0; j < 8; j++) {
            uint32_t const sh = j * nb;
            uint32_t const f = (sh < 32 ? __funnelshift_r(lo, hi, sh) : hi >> (sh - 32)) & mask;
            uint32_t v = 0;
            if (j < cnt) {
                if (f < as) v = sAlpha[f];
                else bad = true;
            }
            o[j >> 2] |= v << (8 * (j & 3));
        }
        uint8_t* const dst = t.out + k0;
        if (cnt == 8 && !(reinterpret_cast<uintptr_t>(dst) & 7)) {
            *reinterpret_cast<uint2*>(dst) = make_uint2(o[0], o[1]);
        } else {
#pragma unroll
            for (uint32_t j = 0; j < 8; j++)
                if (j < cnt) dst[j] = uint8_t(o[j >> 2] >> (8 * (j & 3)));
        }
    }
    if (tr.tile == 0 && threadIdx.x == 0) {
        // terminator: the bit after the last index is set and is the last set bit
        uint64_t const endBit = t.n * t.nbBits;
        uint8_t const last = t.packed[endBit >> 3];
        if (!((last >> (endBit & 7)) & 1) || (last >> (endBit & 7)) != 1) bad = true;
    }
    if (bad) reportError(status, DERR_CORRUPTION);
}

// ---------------------------------------------------------------------------
// Backward bit readers (FSE / Huffman bitstreams): fields are read most
// significant bit first from the end of the stream towards its start.
//
// Each lane stages its stream through a small ring of 16-byte chunks in
// shared memory, filled by asynchronous copies (cp.async) issued AHEAD chunks
// before they are needed; the bit window in registers refills from the ring.
__device__ __forceinline__ bool streamStart(const uint8_t* p, uint32_t size, const uint8_t*& g16, int32_t& pos,
                                            int32_t& end)
{
    if (size == 0) return false;
    uint8_t const last = p[size - 1];
    if (last == 0) return false;
    uintptr_t const a = reinterpret_cast<uintptr_t>(p) & ~uintptr_t(15);
    g16 = reinterpret_cast<const uint8_t*>(a);
    end = int32_t(reinterpret_cast<uintptr_t>(p) - a) * 8;
    pos = end + int32_t(size - 1) * 8 + (31 - __clz(uint32_t(last)));
    return true;
}

// Backward bit reader (FSE and Huffman decoders): three stream words in
// registers, a (bits [cb + 64, cb + 96)) above b and c (bits [cb, cb + 32)),
// cb = 32 * kb, and g = cb + 96 - pos, the bits of the window already read.
// Invariant: g <= 32 at the start of every step. The four-symbol loops take
// the 64 bits just below pos as one left-aligned register pair (hi, lo) =
// two funnel shifts of (a, b, c), peel each field off the top of the pair,
// and then call advance() once with the step's total. A step reads at most
// four fields of at most 12 bits (FSE tableLog <= 12, Huffman codes <= 12
// bits), i.e. n <= 48, so g + n <= 80 < 96 stays inside the three words, and
// advance() drops one or two words without a branch, leaving g <= 32 again.
// read(nb) is the one-field path (stream heads, tails and initial states):
// it takes window(g), the 32 bits starting g bits below the top of the
// window. prepare(), once per step, makes the next two words of the ring
// readable. Words below the stream are never consumed by a valid stream
// (finished() checks that the stream ends exactly at its first bit), so the
// ring's stale contents may stand in for them.
template <int RING, int AHEAD>
struct BitWin3 {
    StreamRing<RING, AHEAD> r;
    uint32_t a, b, c;
    int32_t kb, g, end;

    __device__ __forceinline__ bool init(const uint8_t* p, uint32_t size, uint32_t* ring)
    {
        int32_t pos;
        if (!streamStart(p, size, r.g16, pos, end)) return false;
        r.ring = ring;
        r.start(pos);
        int32_t const jt = (pos - 1) >> 5; // word of the top unread bit
        a = r.word(jt);
        b = r.word(jt - 1);
        c = r.word(jt - 2);
        kb = jt - 2;
        g = (kb + 3) * 32 - pos; // in [0, 32)
        return true;
    }
    __device__ __forceinline__ void prepare()
    {
        int32_t const m = (kb - 2) >> 2;
        if (m < r.low) {
            r.low = m;
            r.issue(m - AHEAD);
            asm volatile("cp.async.wait_group %0;" ::"n"(AHEAD) : "memory");
        }
    }
    // the 32 bits starting o bits below the top of the window (o <= 56)
    __device__ __forceinline__ uint32_t window(int32_t o) const
    {
        uint32_t const hiPair = __funnelshift_l(b, a, uint32_t(o));      // o < 32
        uint32_t const loPair = __funnelshift_l(c, b, uint32_t(o - 32)); // 32 <= o <= 56
        return o < 32 ? hiPair : loPair;
    }
    // drops the n bits read since the start of the step (g + n <= 96)
    __device__ __forceinline__ void advance(int32_t n)
    {
        uint32_t const w1 = r.ring[(kb - 1) & (4 * RING - 1)];
        uint32_t const w2 = r.ring[(kb - 2) & (4 * RING - 1)];
        g += n;
        bool const one = g > 32, two = g > 64;
        uint32_t const na = two ? c : (one ? b : a);
        uint32_t const nb = two ? w1 : (one ? c : b);
        uint32_t const nc = two ? w2 : (one ? w1 : c);
        a = na;
        b = nb;
        c = nc;
        int32_t const k = int32_t(one) + int32_t(two);
        kb -= k;
        g -= 32 * k;
    }
    // one field of nb bits (nb <= 12) just below pos
    __device__ __forceinline__ uint32_t read(uint32_t nb)
    {
        prepare();
        uint32_t const f = __funnelshift_l(window(g), 0u, nb);
        advance(int32_t(nb));
        return f;
    }
    __device__ __forceinline__ bool finished() const { return (kb + 3) * 32 - g == end; }
};

// ---------------------------------------------------------------------------
// FSE: one lane per chunk. Each lane keeps its decoding table in shared
// memory as two arrays over the cells: a 16-bit entry holding the cell's
// newStateBase (bits 4-15) and nbBits (bits 0-3), and the cell's symbol byte.
// Three bytes a cell (6 KiB at tableLog 11) let about 32 chunks reside per
// SM. A decoder state is a cell index: a transition is one 16-bit load, the
// symbol one byte load, and the fields of a pair of transitions come out of
// one 32-bit window by funnel shifts.
//
// Table construction restates src/openzl/fse/decompress/fse_decompress.c:
// 73-171; decode order restates fse_decompress.c:255-337 (state i % nbStates
// emits symbol i; the last symbol of each state has no transition).
constexpr uint32_t kFseCtaSmem = 224 * 1024; // up to 32 tableLog-11 lanes per CTA (one warp)
constexpr uint32_t kFseDefaultLanes = 6;       // streams per CTA when the autotuner has not run

constexpr int kFseRing = 16, kFseAhead = 12; // stream ring: 256 bytes per lane, 192 bytes ahead

// per lane: 16-bit entries (2 << tableLog), symbols (1 << tableLog), stream
// ring (16-byte aligned for tableLog >= 4)
__host__ __device__ __forceinline__ uint32_t fseSlotBytes(uint32_t tlMax) { return (3u << tlMax) + 16u * kFseRing; }
__host__ __device__ __forceinline__ uint32_t fseSmemBytes(uint32_t lanes, uint32_t tlMax)
{
    return lanes * fseSlotBytes(tlMax);
}

// Builds the decoding table of task t in the slot at byte `slot` of the CTA's
// shared memory with all 32 lanes of the warp (every lane calls it); `cum`
// and `next` are the CTA's build scratch (257 and 256 entries).
//  - Counts: the normalized counts go to the counters; a warp scan of
//    the positive counts gives each symbol's first occurrence (cum), and the
//    count -1 symbols take the top cells in symbol order.
//  - Spread: occurrence k (symbols in order, each repeated count times) goes
//    to the k-th cell of the sequence 0, step, 2 step, ... (mod size) that is
//    not a top cell; 32 sequence positions per round, ranked by a ballot.
//  - Cells, 32 per round in increasing order: a cell's state x is its
//    symbol's counter plus the number of lower lanes of the round holding
//    the same symbol (__match_any_sync); the highest such lane advances the
//    counter.
// The result equals the serial construction of fse_decompress.c:73-171.
__device__ __forceinline__ void fseBuildWarp(const FseTask& t, uint8_t* smem, uint32_t slot, uint32_t tlMax,
                                             uint16_t* cum, uint16_t* next)
{
    uint32_t const lane = threadIdx.x;
    uint32_t const lt = (1u << lane) - 1u;
    uint16_t* const tab = reinterpret_cast<uint16_t*>(smem + slot);
    uint8_t* const symOf = smem + slot + (2u << tlMax);
    uint32_t const tl = t.tableLog;
    uint32_t const size = 1u << tl, mask = size - 1;
    uint32_t const step = (size >> 1) + (size >> 3) + 3;
    uint32_t const nbSym = t.nbSym;
    // normalized counts (16-byte aligned in the parameter block, which has
    // slack after its end) into the counters: at most 32 16-byte blocks
    uint32_t const nv = (nbSym * 2 + 15) >> 4;
    if (lane < nv) reinterpret_cast<uint4*>(next)[lane] = __ldg(reinterpret_cast<const uint4*>(t.norm) + lane);
    __syncwarp();
    // lane j: symbols 8j .. 8j + 7
    int v[8];
    uint32_t sumC = 0, sumNeg = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        uint32_t const sy = 8 * lane + k;
        v[k] = sy < nbSym ? int(int16_t(next[sy])) : 0;
        sumC += v[k] > 0 ? uint32_t(v[k]) : 0u;
        sumNeg += v[k] == -1 ? 1u : 0u;
    }
    uint32_t inC = sumC, inNeg = sumNeg;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t const yc = __shfl_up_sync(0xffffffffu, inC, o), yn = __shfl_up_sync(0xffffffffu, inNeg, o);
        if (lane >= uint32_t(o)) {
            inC += yc;
            inNeg += yn;
        }
    }
    uint32_t const totalNeg = __shfl_sync(0xffffffffu, inNeg, 31);
    uint32_t const high = size - 1 - totalNeg;
    uint32_t c0 = inC - sumC, n0 = inNeg - sumNeg;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        uint32_t const sy = 8 * lane + k;
        cum[sy] = uint16_t(c0);
        c0 += v[k] > 0 ? uint32_t(v[k]) : 0u;
        if (v[k] == -1) {
            symOf[size - 1 - n0] = uint8_t(sy);
            next[sy] = 1;
            n0++;
        }
    }
    if (lane == 31) cum[256] = uint16_t(c0);
    __syncwarp();
    // spread
    uint32_t sCur = 0, cumNext = cum[1], occBase = 0;
    for (uint32_t b0 = 0; b0 < size; b0 += 32) {
        uint32_t const pos = ((b0 + lane) * step) & mask;
        bool const valid = totalNeg < size && pos <= high; // all cells are top cells when every count is -1
        uint32_t const bal = __ballot_sync(0xffffffffu, valid);
        if (valid) {
            uint32_t const occ = occBase + __popc(bal & lt);
            while (occ >= cumNext && sCur < 255) cumNext = cum[++sCur + 1];
            symOf[pos] = uint8_t(sCur);
        }
        occBase += __popc(bal);
    }
    __syncwarp();
    // cells
    for (uint32_t b0 = 0; b0 < size; b0 += 32) {
        uint32_t const u = b0 + lane;
        uint32_t const sy = symOf[u];
        uint32_t const m = __match_any_sync(0xffffffffu, sy);
        uint32_t const base = next[sy];
        __syncwarp();
        if (lane == 31u - __clz(m)) next[sy] = uint16_t(base + __popc(m));
        uint32_t const x = base + __popc(m & lt);
        uint32_t const nb = tl - (31 - __clz(x));
        uint32_t const ns = (x << nb) - size;
        tab[u] = uint16_t((ns << 4) | nb);
        __syncwarp();
    }
}

__global__ void __launch_bounds__(32) kFse(const FseTask* __restrict__ tasks, uint32_t nbTasks, uint32_t lanes,
                                           uint32_t tableLogMax, uint32_t* __restrict__ status)
{
    extern __shared__ __align__(16) uint8_t smemFse[];
    __shared__ uint16_t sCum[260];
    __shared__ __align__(16) uint16_t sNext[256];
    uint32_t const lane = threadIdx.x;
    // every lane of the warp builds every table of the CTA, one at a time
    for (uint32_t k = 0; k < lanes; k++) {
        uint32_t const tk = blockIdx.x * lanes + k;
        if (tk >= nbTasks) break;
        FseTask const tt = tasks[tk];
        fseBuildWarp(tt, smemFse, k * fseSlotBytes(tableLogMax), tableLogMax, sCum, sNext);
    }
    if (lane >= lanes) return;
    uint32_t const ti = blockIdx.x * lanes + lane;
    if (ti >= nbTasks) return;
    FseTask const t = tasks[ti];
    uint32_t const slot = lane * fseSlotBytes(tableLogMax);
    uint32_t* const ring = reinterpret_cast<uint32_t*>(smemFse + slot + (3u << tableLogMax));
    const uint16_t* const tab = reinterpret_cast<const uint16_t*>(smemFse + slot);
    const uint8_t* const symOf = smemFse + slot + (2u << tableLogMax);
    uint32_t const tl = t.tableLog;

    BitWin3<kFseRing, kFseAhead> br;
    if (!br.init(t.bits, t.bitsSize, ring)) { reportError(status, DERR_CORRUPTION); return; }
    uint32_t const nst = t.nbStates;
    uint32_t st0 = br.read(tl), st1 = br.read(tl), st2 = 0, st3 = 0;
    if (nst == 4) {
        st2 = br.read(tl);
        st3 = br.read(tl);
    }
    uint32_t const n = t.dstSize;
    uint32_t const lastTr = n > nst ? n - nst : 0; // symbols [0, lastTr) have a transition
    uint8_t* const out = t.out;
    auto ent = [&](uint32_t st) -> uint32_t { return tab[st]; };
    auto sym = [&](uint32_t st) -> uint32_t { return symOf[st]; };
    auto nbOf = [](uint32_t e) -> uint32_t { return e & 15u; };
    auto nextOf = [](uint32_t e, uint32_t f) -> uint32_t { return (e >> 4) + f; };
    // one transition: its field is the top bits of the 64-bit register window
    // (hi, lo), which then shifts them out; four fields take at most 48 bits
    auto take = [](uint32_t e, uint32_t& hi, uint32_t& lo) -> uint32_t {
        uint32_t const nb = e & 15u;
        uint32_t const f = __funnelshift_l(hi, 0u, nb);
        hi = __funnelshift_l(lo, hi, nb);
        lo <<= nb;
        return (e >> 4) + f;
    };
    // one symbol from st0, then the states rotate
    auto single = [&](uint32_t i) {
        uint32_t const e = ent(st0);
        out[i] = uint8_t(sym(st0));
        uint32_t ns = st0;
        if (i < lastTr) ns = nextOf(e, br.read(nbOf(e)));
        if (nst == 4) {
            st0 = st1; st1 = st2; st2 = st3; st3 = ns;
        } else {
            st0 = st1; st1 = ns;
        }
    };
    uint32_t i = 0;
    uint32_t const head = min(n, uint32_t((4 - (reinterpret_cast<uintptr_t>(out) & 3)) & 3));
    for (; i < head; i++) single(i);
    if (nst == 4) {
        for (; i + 4 <= lastTr; i += 4) {
            br.prepare();
            // the 64 bits below pos, left-aligned (g is in [0, 32])
            uint32_t hi = __funnelshift_lc(br.b, br.a, uint32_t(br.g));
            uint32_t lo = __funnelshift_lc(br.c, br.b, uint32_t(br.g));
            uint32_t const ea = ent(st0), eb = ent(st1), ec = ent(st2), ed = ent(st3);
            uint32_t const ya = sym(st0), yb = sym(st1), yc = sym(st2), yd = sym(st3);
            st0 = take(ea, hi, lo);
            st1 = take(eb, hi, lo);
            st2 = take(ec, hi, lo);
            st3 = take(ed, hi, lo);
            br.advance(int32_t(nbOf(ea) + nbOf(eb) + nbOf(ec) + nbOf(ed)));
            *reinterpret_cast<uint32_t*>(out + i) =
                __byte_perm(__byte_perm(ya, yb, 0x0040), __byte_perm(yc, yd, 0x0040), 0x5410);
        }
    } else {
        for (; i + 4 <= lastTr; i += 4) {
            br.prepare();
            uint32_t hi = __funnelshift_lc(br.b, br.a, uint32_t(br.g));
            uint32_t lo = __funnelshift_lc(br.c, br.b, uint32_t(br.g));
            uint32_t const ea = ent(st0), eb = ent(st1);
            uint32_t const ya = sym(st0), yb = sym(st1);
            st0 = take(ea, hi, lo);
            st1 = take(eb, hi, lo);
            uint32_t const ec = ent(st0), ed = ent(st1);
            uint32_t const yc = sym(st0), yd = sym(st1);
            st0 = take(ec, hi, lo);
            st1 = take(ed, hi, lo);
            br.advance(int32_t(nbOf(ea) + nbOf(eb) + nbOf(ec) + nbOf(ed)));
            *reinterpret_cast<uint32_t*>(out + i) =
                __byte_perm(__byte_perm(ya, yb, 0x0040), __byte_perm(yc, yd, 0x0040), 0x5410);
        }
    }
    for (; i < n; i++) single(i);
    asm volatile("cp.async.wait_all;" ::: "memory"); // no copy outlives the lane
    if (!br.finished()) reportError(status, DERR_CORRUPTION);
}

// FSE with one lane per state: a warp decodes up to eight streams, four lanes
// each (lane k of a group runs state k of its stream, k < nbStates). Symbol
// i uses state i % nbStates, so one step decodes nbStates consecutive
// symbols, one per lane. The lanes of a group keep identical copies of the
// stream's bit window (the same arithmetic on the same words); each looks up
// its own state's cell, a scan over the group's field widths (two shuffles)
// gives its field's offset below the top of the window, and the group's
// total (a third shuffle) advances every copy. The stream's ring is filled by
// the group's first lane; a full-warp __syncwarp() per step makes its
// completed copies visible to the other lanes, so the step loop is
// warp-uniform (streams of a CTA are of similar length: tasks are sorted
// longest first) and ends when no lane of the warp has a symbol left. Tables
// as kFse (one per stream, built by the whole warp).
constexpr uint32_t kFse4Variant = kTuneFseLanePerState; // Launch::tune flag (dec_exec.h)

__global__ void __launch_bounds__(32) kFse4(const FseTask* __restrict__ tasks, uint32_t nbTasks, uint32_t streams,
                                            uint32_t tableLogMax, uint32_t* __restrict__ status)
{
    extern __shared__ __align__(16) uint8_t smemFse[];
    __shared__ uint16_t sCum[260];
    __shared__ __align__(16) uint16_t sNext[256];
    uint32_t const lane = threadIdx.x;
    for (uint32_t q = 0; q < streams; q++) {
        uint32_t const tk = blockIdx.x * streams + q;
        if (tk >= nbTasks) break;
        FseTask const tt = tasks[tk];
        fseBuildWarp(tt, smemFse, q * fseSlotBytes(tableLogMax), tableLogMax, sCum, sNext);
    }
    uint32_t const grp = lane >> 2, k = lane & 3;
    uint32_t const ti = blockIdx.x * streams + grp;
    FseTask t{};
    bool ok = grp < streams && ti < nbTasks;
    if (ok) t = tasks[ti];
    uint32_t const slot = grp * fseSlotBytes(tableLogMax);
    uint32_t* const ring = reinterpret_cast<uint32_t*>(smemFse + slot + (3u << tableLogMax));
    const uint16_t* const tab = reinterpret_cast<const uint16_t*>(smemFse + slot);
    const uint8_t* const symOf = smemFse + slot + (2u << tableLogMax);
    uint32_t const tl = t.tableLog, ns = t.nbStates;
    if (ok && ((ns != 2 && ns != 4) || tl > tableLogMax)) { // the planner admits neither
        if (k == 0) reportError(status, DERR_CORRUPTION);
        ok = false;
    }
    // stream start and ring fill (first lane of the group issues the copies)
    StreamRing<kFseRing, kFseAhead> r;
    int32_t pos = 0, end = 0;
    if (ok && !streamStart(t.bits, t.bitsSize, r.g16, pos, end)) {
        if (k == 0) reportError(status, DERR_CORRUPTION);
        ok = false;
    }
    r.ring = ring;
    r.low = 0;
    if (ok) {
        int32_t const mt = (pos - 1) >> 7;
        if (k == 0) {
            for (int32_t m = mt; m >= mt - kFseAhead; m--) r.issue(m);
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        r.low = mt;
    }
    __syncwarp();
    // window: a (bits [cb + 64, cb + 96)), b, c; g = bits of the window read
    uint32_t a = 0, b = 0, c = 0;
    int32_t kb = 0, g = 0;
    if (ok) {
        int32_t const jt = (pos - 1) >> 5;
        a = jt >= 0 ? ring[jt & (4 * kFseRing - 1)] : 0u;
        b = jt - 1 >= 0 ? ring[(jt - 1) & (4 * kFseRing - 1)] : 0u;
        c = jt - 2 >= 0 ? ring[(jt - 2) & (4 * kFseRing - 1)] : 0u;
        kb = jt - 2;
        g = (kb + 3) * 32 - pos;
    }
    // the group's fields of one step: lane k reads nb bits below the k-th
    // lower lanes' fields; returns the field, sets the group's total
    auto fields = [&](uint32_t nb, uint32_t& total) -> uint32_t {
        uint32_t x = nb;
        uint32_t const y1 = __shfl_up_sync(0xffffffffu, x, 1, 4);
        if (k >= 1) x += y1;
        uint32_t const y2 = __shfl_up_sync(0xffffffffu, x, 2, 4);
        if (k >= 2) x += y2;
        total = __shfl_sync(0xffffffffu, x, 3, 4);
        uint32_t const off = x - nb; // <= 36
        uint32_t const hi = __funnelshift_lc(b, a, uint32_t(g));
        uint32_t const lo = __funnelshift_lc(c, b, uint32_t(g));
        uint32_t const w = off < 32 ? __funnelshift_l(lo, hi, off) : (lo << (off - 32));
        return __funnelshift_rc(w, 0u, 32u - nb);
    };
    // drop n bits (n <= 48, g <= 32): one or two words from the ring
    auto advance = [&](uint32_t n) {
        // the next two words below the window must be in the ring
        int32_t const m = (kb - 2) >> 2;
        if (ok && m < r.low) {
            r.low = m;
            if (k == 0) {
                r.issue(m - kFseAhead);
                asm volatile("cp.async.wait_group %0;" ::"n"(kFseAhead) : "memory");
            }
        }
        __syncwarp();
        // a lane without a stream has no ring (its slot may lie past the CTA's memory)
        uint32_t const w1 = ok ? ring[(kb - 1) & (4 * kFseRing - 1)] : 0u;
        uint32_t const w2 = ok ? ring[(kb - 2) & (4 * kFseRing - 1)] : 0u;
        g += int32_t(n);
        bool const one = g > 32, two = g > 64;
        uint32_t const na = two ? c : (one ? b : a);
        uint32_t const nb2 = two ? w1 : (one ? c : b);
        uint32_t const nc = two ? w2 : (one ? w1 : c);
        a = na;
        b = nb2;
        c = nc;
        int32_t const kk = int32_t(one) + int32_t(two);
        kb -= kk;
        g -= 32 * kk;
    };
    // initial states: state k is the k-th field of tableLog bits from the top
    uint32_t st = 0, total = 0;
    {
        bool const mine = ok && k < ns;
        uint32_t const f = fields(mine ? tl : 0u, total);
        st = f;
        advance(total);
    }
    uint32_t const n = ok ? t.dstSize : 0;
    uint32_t const lastTr = n > ns ? n - ns : 0; // symbols [0, lastTr) have a transition
    uint8_t* const out = t.out;
    for (uint32_t i = 0;; i += ns) {
        bool const act = ok && k < ns && i + k < n;
        if (!__any_sync(0xffffffffu, act)) break;
        bool const tr = act && i + k < lastTr;
        uint32_t const e = act ? uint32_t(tab[st]) : 0u;
        uint32_t const y = act ? uint32_t(symOf[st]) : 0u;
        uint32_t const f = fields(tr ? (e & 15u) : 0u, total);
        if (tr) st = (e >> 4) + f;
        if (act) out[i + k] = uint8_t(y);
        advance(total);
    }
    if (k == 0) asm volatile("cp.async.wait_all;" ::: "memory"); // no copy outlives the lane
    if (ok && k == 0 && (kb + 3) * 32 - g != end) reportError(status, DERR_CORRUPTION);
}

// ---------------------------------------------------------------------------
// Huffman: weights -> canonical table (symbols ranked by weight then value;
// weight w spans 2^(w-1) cells, nbBits = tableLog + 1 - w), after
// src/openzl/fse/decompress/huf_decompress.c:342-454. One warp per CTA
// decodes eight chunks, four lanes per chunk (one per stream of a 4X chunk;
// lane 0 alone for 1X) sharing the chunk's table (entry: symbol |
// nbBits << 8). Table slots hold tableLog 11, the largest the reference's
// encoder emits (encode_entropy_binding.c:222, HUF_TABLELOG_DEFAULT); chunks
// with tableLog 12 take two adjacent slots and are decoded in a second round
// when their neighbour's slot is busy.
constexpr uint32_t kHufTableLog = 12;
constexpr uint32_t kHufChunks = 8;
constexpr uint32_t kHufSlotCells = 1u << 11;
constexpr uint32_t kHufSlotBytes = kHufSlotCells * 2 + 512 + 4;

__device__ bool hufRank(const uint8_t* weights, uint32_t nbW, uint16_t* first, uint32_t& tlOut)
{
    uint32_t counts[13];
#pragma unroll
    for (int k = 0; k < 13; k++) counts[k] = 0;
    uint32_t sum = 0;
    if (nbW > 256) return false;
    for (uint32_t s = 0; s < nbW; s++) {
        uint32_t const w = weights[s];
        if (w > 12) return false;
#pragma unroll
        for (int k = 1; k < 13; k++) counts[k] += (w == uint32_t(k));
        sum += (1u << w) >> 1;
    }
    if (sum == 0 || (sum & (sum - 1))) return false;
    uint32_t const tl = 31 - __clz(sum);
    if (tl > kHufTableLog) return false;
    uint32_t nz = 0;
#pragma unroll
    for (int k = 1; k < 13; k++) nz += counts[k];
    if (nz < 2) return false;
    uint32_t start[13];
    uint32_t p = 0;
#pragma unroll
    for (int k = 1; k < 13; k++) {
        start[k] = p;
        if (uint32_t(k) <= tl) p += counts[k] << (k - 1);
    }
    for (uint32_t s = 0; s < nbW; s++) {
        uint32_t const w = weights[s];
        uint32_t f = 0;
#pragma unroll
        for (int k = 1; k < 13; k++)
            if (w == uint32_t(k)) { f = start[k]; start[k] += 1u << (k - 1); }
        first[s] = uint16_t(f);
    }
    tlOut = tl;
    return true;
}

constexpr int kHufRing = 8, kHufAhead = 5; // stream ring: 128 bytes per lane, 80 bytes ahead
// rings after the slots and the spare ranks
__host__ __device__ __forceinline__ uint32_t hufRingOff(uint32_t chunks) { return (chunks * kHufSlotBytes + 512 + 15) & ~15u; }

__device__ __forceinline__ void hufDecodeStream(const HufTask& t, const uint16_t* dt, uint32_t tl, uint32_t sIdx,
                                                uint32_t* ring, uint32_t* status)
{
    const uint8_t* sp;
    uint32_t ssize, n, o0;
    if (t.x4) {
        if (t.bitsSize < 10) { if (sIdx == 0) reportError(status, DERR_CORRUPTION); return; }
        uint32_t const l1 = t.bits[0] | (t.bits[1] << 8);
        uint32_t const l2 = t.bits[2] | (t.bits[3] << 8);
        uint32_t const l3 = t.bits[4] | (t.bits[5] << 8);
        if (6ull + l1 + l2 + l3 > t.bitsSize) { if (sIdx == 0) reportError(status, DERR_CORRUPTION); return; }
        uint32_t const l4 = t.bitsSize - 6 - l1 - l2 - l3;
        uint32_t const seg = (t.dstSize + 3) / 4;
        if (3ull * seg > t.dstSize) { if (sIdx == 0) reportError(status, DERR_CORRUPTION); return; }
        uint32_t off = 6;
        off += sIdx > 0 ? l1 : 0;
        off += sIdx > 1 ? l2 : 0;
        off += sIdx > 2 ? l3 : 0;
        sp = t.bits + off;
        ssize = sIdx == 0 ? l1 : (sIdx == 1 ? l2 : (sIdx == 2 ? l3 : l4));
        o0 = seg * sIdx;
        n = sIdx == 3 ? t.dstSize - 3 * seg : seg;
    } else {
        if (sIdx != 0) return;
        sp = t.bits;
        ssize = t.bitsSize;
        o0 = 0;
        n = t.dstSize;
    }
    BitWin3<kHufRing, kHufAhead> br;
    if (!br.init(sp, ssize, ring)) { reportError(status, DERR_CORRUPTION); return; }
    uint8_t* const out = t.out + o0;
    uint32_t const sh = 32u - tl;
    uint32_t i = 0;
    // one symbol; its code is at most tl <= 12 bits
    auto single = [&]() -> uint32_t {
        br.prepare();
        uint32_t const e = dt[__funnelshift_lc(br.b, br.a, uint32_t(br.g)) >> sh];
        br.advance(int32_t(e >> 8));
        return e;
    };
    // unaligned head, then four symbols per refill and per 32-bit store: the
    // 64 bits below pos, left-aligned in (hi, lo), hold the four codes
    uint32_t const head = min(n, uint32_t((4 - (reinterpret_cast<uintptr_t>(out) & 3)) & 3));
    for (; i < head; i++) out[i] = uint8_t(single());
    for (; i + 4 <= n; i += 4) {
        br.prepare();
        uint32_t hi = __funnelshift_lc(br.b, br.a, uint32_t(br.g));
        uint32_t lo = __funnelshift_lc(br.c, br.b, uint32_t(br.g));
        uint32_t const e0 = dt[hi >> sh];
        uint32_t const n0 = e0 >> 8;
        hi = __funnelshift_l(lo, hi, n0);
        lo <<= n0;
        uint32_t const e1 = dt[hi >> sh];
        uint32_t const n1 = e1 >> 8;
        hi = __funnelshift_l(lo, hi, n1);
        lo <<= n1;
        uint32_t const e2 = dt[hi >> sh];
        uint32_t const n2 = e2 >> 8;
        hi = __funnelshift_l(lo, hi, n2);
        uint32_t const e3 = dt[hi >> sh];
        br.advance(int32_t(n0 + n1 + n2 + (e3 >> 8)));
        *reinterpret_cast<uint32_t*>(out + i) = __byte_perm(__byte_perm(e0, e1, 0x0040), __byte_perm(e2, e3, 0x0040), 0x5410);
    }
    for (; i < n; i++) out[i] = uint8_t(single());
    asm volatile("cp.async.wait_all;" ::: "memory"); // no copy outlives the lane
    if (!br.finished()) reportError(status, DERR_CORRUPTION);
}

__global__ void __launch_bounds__(32) kHuf(const HufTask* __restrict__ tasks, uint32_t nbTasks, uint32_t chunks,
                                           uint32_t* __restrict__ status)
{
    extern __shared__ __align__(16) uint8_t smemHuf[];
    __shared__ uint32_t sTl[kHufChunks];
    __shared__ uint8_t sOk[kHufChunks];
    uint32_t const c = threadIdx.x >> 2;       // chunk slot in this CTA
    uint32_t const sIdx = threadIdx.x & 3;     // stream within the chunk
    uint32_t const ti = blockIdx.x * chunks + c;
    bool const active = ti < nbTasks;
    uint8_t* const slot = smemHuf + size_t(c) * kHufSlotBytes;
    uint16_t* const first = reinterpret_cast<uint16_t*>(slot + kHufSlotCells * 2); // first cell per symbol
    HufTask t{};
    if (active) t = tasks[ti];
    if (sIdx == 0) {
        uint32_t tl = 0;
        bool const ok = active && hufRank(t.weights, t.nbWeights, first, tl);
        sOk[c] = ok ? 1 : 0;
        sTl[c] = tl;
        if (active && !ok) reportError(status, DERR_CORRUPTION);
    }
    __syncwarp();
    // tableLog <= 11: each chunk in its own slot
    uint32_t const tl = sTl[c];
    bool const narrow = active && sOk[c] && tl <= 11;
    uint16_t* const dt = reinterpret_cast<uint16_t*>(slot);
    if (narrow) {
        for (uint32_t s = sIdx; s < t.nbWeights; s += 4) {
            uint32_t const w = t.weights[s];
            if (!w) continue;
            uint32_t const len = 1u << (w - 1);
            uint16_t const e = uint16_t(s | ((tl + 1 - w) << 8));
            uint32_t const f = first[s];
            for (uint32_t u = 0; u < len; u++) dt[f + u] = e;
        }
    }
    __syncwarp();
    uint32_t* const ring = reinterpret_cast<uint32_t*>(smemHuf + hufRingOff(chunks)) + threadIdx.x * 4 * kHufRing;
    if (narrow) hufDecodeStream(t, dt, tl, sIdx, ring, status);
    __syncwarp();
    // tableLog 12 (valid, but never emitted by the reference's encoder): one
    // chunk at a time, its table across the first slots, ranks recomputed
    // into the spare area after the slots
    uint16_t* const wideFirst = reinterpret_cast<uint16_t*>(smemHuf + size_t(chunks) * kHufSlotBytes);
    uint16_t* const wide = reinterpret_cast<uint16_t*>(smemHuf);
    for (uint32_t k = 0; k < chunks; k++) {
        if (!(sOk[k] && sTl[k] > 11)) continue; // warp-uniform
        HufTask const tk = tasks[blockIdx.x * chunks + k];
        if (threadIdx.x == 0) {
            uint32_t tlk = 0;
            hufRank(tk.weights, tk.nbWeights, wideFirst, tlk);
        }
        __syncwarp();
        uint32_t const tlk = sTl[k];
        for (uint32_t s = threadIdx.x; s < tk.nbWeights; s += blockDim.x) { // 4 x chunks threads
            uint32_t const w = tk.weights[s];
            if (!w) continue;
            uint32_t const len = 1u << (w - 1);
            uint16_t const e = uint16_t(s | ((tlk + 1 - w) << 8));
            uint32_t const f = wideFirst[s];
            for (uint32_t u = 0; u < len; u++) wide[f + u] = e;
        }
        __syncwarp();
        if (threadIdx.x < 4) hufDecodeStream(tk, wide, tlk, threadIdx.x, ring, status);
        __syncwarp();
    }
}

// Backward bit reader of the 16-bit Huffman decoder. The window is the three
// stream words kb + 2 (top), kb + 1 and kb, loaded through the read-only data
// cache at each step (a lane walks down one 128-byte line every few dozen
// steps, so nearly all loads hit L1), and g = 32 * (kb + 3) - pos in
// [0, 32): the 64 bits just below pos, most significant first, are two
// funnel shifts of them. A step reads at most 48 bits; advance() drops them
// with three integer operations. Word indices are clamped at 0, the 16-byte
// block that holds the stream's first byte: words below the stream are never
// consumed by a valid stream (finished() checks that the stream ends exactly
// at its first bit), so any word may stand in for them, and nothing outside
// the stream's blocks is read.
struct BitLdg {
    const uint32_t* base; // the 16-byte block holding the stream's first byte
    int32_t kb, g, end;

    __device__ __forceinline__ bool init(const uint8_t* p, uint32_t size)
    {
        int32_t pos;
        const uint8_t* g16;
        if (!streamStart(p, size, g16, pos, end)) return false;
        base = reinterpret_cast<const uint32_t*>(g16);
        int32_t const jt = (pos - 1) >> 5;
        kb = jt - 2;
        g = (kb + 3) * 32 - pos;
        return true;
    }
    // the 64 bits below pos, most significant first
    __device__ __forceinline__ void window(uint32_t& hi, uint32_t& lo) const
    {
        uint32_t const c = __ldg(base + max(kb, 0)), b = __ldg(base + max(kb + 1, 0)), a = __ldg(base + max(kb + 2, 0));
        hi = __funnelshift_l(b, a, uint32_t(g));
        lo = __funnelshift_l(c, b, uint32_t(g));
    }
    __device__ __forceinline__ void advance(uint32_t n)
    {
        g += int32_t(n);
        kb -= g >> 5;
        g &= 31;
    }
    // one field of nb bits (nb <= 12) just below pos
    __device__ __forceinline__ uint32_t read(uint32_t nb)
    {
        uint32_t hi, lo;
        window(hi, lo);
        advance(nb);
        return __funnelshift_l(hi, 0u, nb);
    }
    __device__ __forceinline__ bool finished() const { return (kb + 3) * 32 - g == end; }
};

// ---------------------------------------------------------------------------
// 16-bit-symbol Huffman (huffman_struct_v2), one CTA per chunk. Tables reach
// 2^20 cells (tableLog <= 20), so instead of a cell table the CTA keeps, per
// weight, the first cell and the first index into the symbols sorted by
// (weight, value): the cell range of weight w spans count[w] << (w - 1)
// cells, weight 1 (the longest code) first, and a symbol of weight w spans
// 2^(w-1) consecutive cells and codes on tableLog + 1 - w bits
// (decode_huffman_kernel.c:35-71). Decoding a symbol peeks tableLog bits,
// finds the weight whose cell range holds them (binary search over at most
// 20 ranks) and indexes the sorted symbols. The validity rules of
// decode_entropy_binding.c:349-412 apply: weights at most 20, at least two
// of them non-zero, the sum of 2^(w-1) a power of two. One lane decodes each
// of the one or four streams; like the reference, a stream is not required
// to end exactly at its first bit (the planner checked that the stream table
// fills the input exactly).
__global__ void __launch_bounds__(128) kHuf16(const Huf16Task* __restrict__ tasks, uint32_t* __restrict__ status)
{
    __shared__ uint32_t sCount[32], sStart[32], sBase[32], sNext[32];
    __shared__ uint32_t sTl, sOk;
    __shared__ unsigned long long sSum;
    Huf16Task const t = tasks[blockIdx.x];
    uint32_t const tid = threadIdx.x, lane = tid & 31;
    if (tid < 32) sCount[tid] = 0;
    if (tid == 0) {
        sSum = 0;
        sOk = 1;
    }
    __syncthreads();
    unsigned long long part = 0;
    bool bad = false;
    for (uint32_t s = tid; s < t.nbWeights; s += blockDim.x) {
        uint32_t const w = t.weights[s];
        if (w > 20) {
            bad = true;
        } else if (w) {
            atomicAdd(&sCount[w], 1u);
            part += 1ull << (w - 1);
        }
    }
    if (bad) sOk = 0;
    if (part) atomicAdd(&sSum, part);
    __syncthreads();
    if (tid == 0) {
        uint64_t const sum = sSum;
        uint32_t nz = 0;
        for (int w = 1; w <= 20; w++) nz += sCount[w];
        uint32_t tl = 0;
        while (tl < 63 && (2ull << tl) <= sum) tl++;
        bool const ok = sOk && nz >= 2 && sum != 0 && !(sum & (sum - 1)) && tl <= 20;
        if (ok) {
            uint32_t pos = 0, base = 0;
            for (uint32_t w = 1; w <= tl; w++) {
                sStart[w] = pos;
                sBase[w] = base;
                sNext[w] = base;
                pos += sCount[w] << (w - 1);
                base += sCount[w];
            }
            sStart[tl + 1] = 1u << tl;
        }
        sTl = tl;
        sOk = ok ? 1u : 0u;
    }
    __syncthreads();
    if (!sOk) {
        if (tid == 0) reportError(status, DERR_CORRUPTION);
        return;
    }
    uint32_t const tl = sTl;
    // symbols sorted by (weight, value): 32 at a time, ranked among the lanes
    // holding the same weight
    if (tid < 32) {
        for (uint32_t b0 = 0; b0 < t.nbWeights; b0 += 32) {
            uint32_t const s = b0 + lane;
            uint32_t const w = s < t.nbWeights ? t.weights[s] : 0u;
            uint32_t const m = __match_any_sync(0xffffffffu, w);
            uint32_t const base = w ? sNext[w] : 0u;
            __syncwarp();
            if (w) {
                if (lane == 31u - __clz(m)) sNext[w] = base + __popc(m);
                t.sorted[base + __popc(m & ((1u << lane) - 1u))] = uint16_t(s);
            }
            __syncwarp();
        }
    }
    __syncthreads();
    if (tid >= t.nbStreams) return;
    BitLdg br;
    if (!br.init(t.stream[tid], t.streamSize[tid])) {
        reportError(status, DERR_CORRUPTION);
        return;
    }
    uint8_t* const out = t.out + 2ull * t.dstOff[tid];
    bool const al = !(reinterpret_cast<uintptr_t>(out) & 1);
    uint32_t const n = t.count[tid];
    for (uint32_t i = 0; i < n; i++) {
        uint32_t hi, lo;
        br.window(hi, lo);
        uint32_t const v = hi >> (32 - tl);
        uint32_t a = 1, b = tl;
        while (a < b) {
            uint32_t const mid = (a + b + 1) >> 1;
            if (sStart[mid] <= v) a = mid;
            else b = mid - 1;
        }
        uint32_t const sym = t.sorted[sBase[a] + ((v - sStart[a]) >> (a - 1))];
        if (al) {
            reinterpret_cast<uint16_t*>(out)[i] = uint16_t(sym);
        } else {
            out[2 * i] = uint8_t(sym);
            out[2 * i + 1] = uint8_t(sym >> 8);
        }
        br.advance(tl + 1 - a);
    }
}

// ---------------------------------------------------------------------------
// XXH3-64 checksums. Phase 1: per 1 KiB block, the 16-stripe sum of every
// accumulator lane's increments (they commute within a block). Phase 2: per
// task, the block chain acc = scramble(acc + blockSum) on 8 lanes, then the
// tail stripes and the final merge on one lane (the secret and primes are
// defined above the numeric pipeline). Where the numeric pipeline writes a
// content-checksummed output, it computes that output's block sums itself
// and phase 1 skips those blocks.
__device__ __forceinline__ uint64_t fold128(uint64_t a, uint64_t b)
{
    return (a * b) ^ __umul64hi(a, b);
}
__device__ __forceinline__ uint64_t xAvalanche(uint64_t h)
{
    h ^= h >> 37;
    h *= XPMX1;
    return h ^ (h >> 32);
}
__device__ __forceinline__ uint64_t x64Avalanche(uint64_t h)
{
    h ^= h >> 33;
    h *= XP64_2;
    h ^= h >> 29;
    h *= XP64_3;
    return h ^ (h >> 32);
}
__device__ __forceinline__ uint64_t ldData(const uint8_t* p, bool aligned)
{
    if (aligned && !(reinterpret_cast<uintptr_t>(p) & 7)) return *reinterpret_cast<const uint64_t*>(p);
    uint64_t v = 0;
    for (int b = 0; b < 8; b++) v |= uint64_t(p[b]) << (8 * b);
    return v;
}
__device__ __forceinline__ uint64_t mix16(const uint8_t* in, int soff, bool al)
{
    return fold128(ldData(in, al) ^ secret64(soff), ldData(in + 8, al) ^ secret64(soff + 8));
}

__device__ uint64_t xxh3Short(const uint8_t* in, uint64_t len, bool al)
{
    if (len <= 16) {
        if (len > 8) {
            uint64_t lo = ldData(in, al) ^ (secret64(24) ^ secret64(32));
            uint64_t hi = ldData(in + len - 8, al) ^ (secret64(40) ^ secret64(48));
            uint64_t const swapped = (uint64_t(__byte_perm(uint32_t(lo), 0, 0x0123)) << 32)
                    | __byte_perm(uint32_t(lo >> 32), 0, 0x0123);
            uint64_t acc = len + swapped + hi + fold128(lo, hi);
            return xAvalanche(acc);
        }
        if (len >= 4) {
            uint64_t i1 = 0, i2 = 0;
            for (int b = 0; b < 4; b++) {
                i1 |= uint64_t(in[b]) << (8 * b);
                i2 |= uint64_t(in[len - 4 + b]) << (8 * b);
            }
            uint64_t k = (i2 + (i1 << 32)) ^ (secret64(8) ^ secret64(16));
            k ^= ((k << 49) | (k >> 15)) ^ ((k << 24) | (k >> 40));
            k *= XPMX2;
            k ^= (k >> 35) + len;
            k *= XPMX2;
            return k ^ (k >> 28);
        }
        if (len > 0) {
            uint32_t c = (uint32_t(in[0]) << 16) | (uint32_t(in[len >> 1]) << 24) | in[len - 1] | (uint32_t(len) << 8);
            return x64Avalanche(uint64_t(c) ^ uint64_t(secret32(0) ^ secret32(4)));
        }
        return x64Avalanche(secret64(56) ^ secret64(64));
    }
    if (len <= 128) {
        uint64_t acc = len * XP64_1;
        if (len > 32) {
            if (len > 64) {
                if (len > 96) {
                    acc += mix16(in + 48, 96, al);
                    acc += mix16(in + len - 64, 112, al);
                }
                acc += mix16(in + 32, 64, al);
                acc += mix16(in + len - 48, 80, al);
            }
            acc += mix16(in + 16, 32, al);
            acc += mix16(in + len - 32, 48, al);
        }
        acc += mix16(in, 0, al);
        acc += mix16(in + len - 16, 16, al);
        return xAvalanche(acc);
    }
    uint64_t acc = len * XP64_1;
    uint64_t const rounds = len / 16;
    for (uint64_t i = 0; i < 8; i++) acc += mix16(in + 16 * i, int(16 * i), al);
    acc = xAvalanche(acc);
    for (uint64_t i = 8; i < rounds; i++) acc += mix16(in + 16 * i, int(16 * (i - 8) + 3), al);
    acc += mix16(in + len - 16, 136 - 17, al);
    return xAvalanche(acc);
}

// Phase 1: one warp per 1 KiB block. Lane L holds 16 bytes of each half
// block (stripe L/4 (+8), words 2(L%4) and 2(L%4)+1), read as one aligned
// 16-byte load; for data that is not 16-byte aligned the lane funnels its
// aligned chunk with the next lane's (the last lane loads one more chunk,
// which holds at least one byte of the task's data). Each lane adds both
// words' increments (acc[i] += data[i^1] + lo32(data[i]^key[i]) * hi32(...))
// and the warp reduces over stripes.
__device__ __forceinline__ uint4 funnel16(uint4 c, uint4 n, uint32_t off)
{
    uint32_t const q = off >> 2, r = (off & 3) * 8;
    uint32_t w[4];
    switch (q) {
        case 0:
            w[0] = __funnelshift_r(c.x, c.y, r); w[1] = __funnelshift_r(c.y, c.z, r);
            w[2] = __funnelshift_r(c.z, c.w, r); w[3] = __funnelshift_r(c.w, n.x, r);
            break;
        case 1:
            w[0] = __funnelshift_r(c.y, c.z, r); w[1] = __funnelshift_r(c.z, c.w, r);
            w[2] = __funnelshift_r(c.w, n.x, r); w[3] = __funnelshift_r(n.x, n.y, r);
            break;
        case 2:
            w[0] = __funnelshift_r(c.z, c.w, r); w[1] = __funnelshift_r(c.w, n.x, r);
            w[2] = __funnelshift_r(n.x, n.y, r); w[3] = __funnelshift_r(n.y, n.z, r);
            break;
        default:
            w[0] = __funnelshift_r(c.w, n.x, r); w[1] = __funnelshift_r(n.x, n.y, r);
            w[2] = __funnelshift_r(n.y, n.z, r); w[3] = __funnelshift_r(n.z, n.w, r);
            break;
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

__device__ __forceinline__ void hashBlock(const HashTask* __restrict__ tasks, TileRef const br, const uint64_t* sKey,
                                          uint32_t lane)
{
    HashTask const t = tasks[br.task];
    const uint8_t* const blk = t.data + uint64_t(br.tile) * kHashBlock;
    uintptr_t const base = reinterpret_cast<uintptr_t>(blk) & ~uintptr_t(15);
    uint32_t const off = uint32_t(reinterpret_cast<uintptr_t>(blk) - base);
    const uint4* const A = reinterpret_cast<const uint4*>(base);
    uint32_t const j = lane & 3, sl = lane >> 2;
    uint4 c[2];
    c[0] = __ldg(A + lane);
    c[1] = __ldg(A + 32 + lane);
    if (off) {
        uint4 const ext = lane == 31 ? __ldg(A + 64) : make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int r = 0; r < 2; r++) {
            uint4 n;
            n.x = __shfl_down_sync(0xffffffffu, c[r].x, 1);
            n.y = __shfl_down_sync(0xffffffffu, c[r].y, 1);
            n.z = __shfl_down_sync(0xffffffffu, c[r].z, 1);
            n.w = __shfl_down_sync(0xffffffffu, c[r].w, 1);
            // lane 31's next chunk: round 0 -> lane 0 of round 1; round 1 -> ext
            uint32_t const x = __shfl_sync(0xffffffffu, c[1].x, 0), y = __shfl_sync(0xffffffffu, c[1].y, 0);
            uint32_t const z = __shfl_sync(0xffffffffu, c[1].z, 0), w = __shfl_sync(0xffffffffu, c[1].w, 0);
            if (lane == 31) n = r == 0 ? make_uint4(x, y, z, w) : ext;
            c[r] = funnel16(c[r], n, off);
        }
    }
    uint64_t a0 = 0, a1 = 0;
#pragma unroll
    for (int r = 0; r < 2; r++) {
        uint32_t const st = sl + 8 * r;
        uint64_t const w0 = uint64_t(c[r].x) | (uint64_t(c[r].y) << 32);
        uint64_t const w1 = uint64_t(c[r].z) | (uint64_t(c[r].w) << 32);
        uint64_t const k0 = w0 ^ sKey[st + 2 * j], k1 = w1 ^ sKey[st + 2 * j + 1];
        a0 += w1 + uint64_t(uint32_t(k0)) * (k0 >> 32);
        a1 += w0 + uint64_t(uint32_t(k1)) * (k1 >> 32);
    }
#pragma unroll
    for (int m = 4; m < 32; m <<= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, m);
        a1 += __shfl_xor_sync(0xffffffffu, a1, m);
    }
    if (lane < 4) {
        t.blockSums[8ull * br.tile + 2 * lane] = a0;
        t.blockSums[8ull * br.tile + 2 * lane + 1] = a1;
    }
}

__global__ void __launch_bounds__(256) kHashBlocks(const HashTask* __restrict__ tasks,
                                                   const TileRef* __restrict__ blocks, uint32_t nbBlocks)
{
    __shared__ uint64_t sKey[24]; // secret words at byte offsets 0, 8, ..., 184
    if (threadIdx.x < 24) sKey[threadIdx.x] = secret64(int(8 * threadIdx.x));
    __syncthreads();
    uint32_t const lane = threadIdx.x & 31;
    // grid-stride over the blocks, one warp per block at a time: the secret
    // is staged once per CTA
    uint32_t const nw = gridDim.x * (blockDim.x >> 5);
    for (uint32_t warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); warp < nbBlocks; warp += nw)
        hashBlock(tasks, blocks[warp], sKey, lane);
}


// The block chain of accumulator lane & 7 over nb blocks (all 32 lanes of the
// warp call it; see kHashFinish), starting from init, with key words
// (klo, khi); sb: the warp's 264 words of shared memory. Returns the
// accumulator after the last block. Kept out of line: compiled inside
// kHashFinish the same loop ran slower (the chain of a 256 MiB input took
// 5.13 ms there, 4.78 ms here).
__device__ __noinline__ uint64_t xxhBlockChain(const uint64_t* __restrict__ bs, uint32_t nb, uint64_t init,
                                           uint32_t klo, uint32_t khi, uint64_t* sb)
{
    uint32_t const lane = threadIdx.x & 31, i = lane & 7;
    uint64_t const total = 8ull * nb;
    // batches of 32 blocks: the current one, the next, and the one after
    // it in flight (two batches of chain steps cover an L2 round trip)
    uint64_t cur[8], nxt[8];
#pragma unroll
    for (int m = 0; m < 8; m++) {
        uint64_t const idx = uint64_t(lane) + 32u * m;
        cur[m] = idx < total ? __ldg(bs + idx) : 0;
        nxt[m] = idx + 256 < total ? __ldg(bs + idx + 256) : 0;
    }
    uint64_t const y0 = init + __shfl_sync(0xffffffffu, cur[0], int(i)); // init + sum of block 0
    uint32_t ylo = uint32_t(y0), yhi = uint32_t(y0 >> 32);
    for (uint32_t b0 = 0; b0 < nb; b0 += 32) {
        uint64_t nx2[8];
#pragma unroll
        for (int m = 0; m < 8; m++) {
            uint64_t const idx = 8ull * (b0 + 64) + lane + 32u * m;
            nx2[m] = idx < total ? __ldg(bs + idx) : 0;
        }
        uint32_t const cnt = min(32u, nb - b0);
#pragma unroll
        for (int m = 0; m < 8; m++) sb[lane + 32 * m] = cur[m];
        if (lane < 8) sb[256 + lane] = nxt[0];
        __syncwarp();
        // one chain step with the sum of block b0 + k + 1 (0 past the last block)
        auto step = [&](int k) {
            uint64_t const nv = sb[8 * (k + 1) + i];
            uint32_t const tt = ylo ^ (yhi >> 15) ^ klo;
            uint32_t const u = yhi ^ khi;
            uint64_t const r = uint64_t(tt) * XP32_1 + nv;
            ylo = uint32_t(r);
            yhi = uint32_t(r >> 32) + u * XP32_1;
        };
        if (cnt == 32) { // full batches without a per-block predicate
#pragma unroll
            for (int k = 0; k < 32; k++) step(k);
        } else {
#pragma unroll
            for (int k = 0; k < 32; k++)
                if (uint32_t(k) < cnt) step(k);
        }
        __syncwarp(); // the batch's sums are read before the next batch overwrites them
#pragma unroll
        for (int m = 0; m < 8; m++) {
            cur[m] = nxt[m];
            nxt[m] = nx2[m];
        }
    }
    // after the last block y = acc (its next sum is 0); with no block,
    // y = init + 0
    return (uint64_t(yhi) << 32) | ylo;
}

// Phase 2: one warp per task. Lane i (and its copies i + 8, i + 16, i + 24)
// runs the block chain of accumulator i, then the trailing partial stripes
// and the final stripe, and lane 0 merges.
__global__ void kHashFinish(const HashTask* __restrict__ tasks, uint32_t nbTasks, uint32_t* __restrict__ status)
{
    uint32_t const ti = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t const lane = threadIdx.x & 31;
    if (ti >= nbTasks) return;
    HashTask const t = tasks[ti];
    bool const al = t.aligned8 != 0;
    uint64_t h;
    if (t.len <= 240) {
        if (lane != 0) return;
        h = xxh3Short(t.data, t.len, al);
    } else {
        uint32_t const i = lane & 7;
        uint64_t const init = i == 0 ? XP32_3 : i == 1 ? XP64_1 : i == 2 ? XP64_2 : i == 3 ? XP64_3
                            : i == 4 ? XP64_4 : i == 5 ? XP32_2 : i == 6 ? XP64_5 : XP32_1;
        uint64_t const key = secret64(int(192 - 64 + 8 * i));
        uint32_t const klo = uint32_t(key), khi = uint32_t(key >> 32);
        // The block chain acc = scramble(acc + sum), scramble(x) = ((x ^
        // (x >> 47)) ^ key) * PRIME32_1, is serial; its inputs are not. The
        // warp loads the sums of 32 blocks at a time (coalesced, the next
        // batch while the current one runs), and lane i takes the value of
        // block k for accumulator i from lane 8 * (k % 4) + i.
        //
        // The chain runs on y = acc + sum of the block about to be scrambled,
        // in 32-bit halves: x >> 47 only reaches the low half (y.hi >> 15), so
        // with t = y.lo ^ (y.hi >> 15) ^ key.lo and u = y.hi ^ key.hi the next
        // y is t * P + next sum (one 32x32+64-bit multiply-add) with u * P
        // added to its high half. Per block the dependent path is a shift, a
        // xor and two multiply-adds; the sums' additions leave it. Each batch
        // of sums is staged in the warp's shared memory and read per block:
        // in a micro-benchmark of the loop alone, 27 cycles a block on GB300
        // against 38 when taken by warp shuffles.
        // per warp: the sums of a batch of 32 blocks, then the next batch's first
        __shared__ uint64_t sBatch[8][256 + 8];
        uint32_t const nb = t.nbBlocks;
        uint64_t acc = xxhBlockChain(t.blockSums, nb, init, klo, khi, sBatch[threadIdx.x >> 5]);
        uint64_t const len = t.len;
        uint64_t const nbStripes = ((len - 1) - uint64_t(kHashBlock) * nb) / 64;
        const uint8_t* const last = t.data + uint64_t(kHashBlock) * nb;
        for (uint64_t st = 0; st < nbStripes; st++) {
            uint64_t const v = ldData(last + 64 * st + 8 * i, al);
            uint64_t const vx = __shfl_xor_sync(0xffffffffu, v, 1);
            uint64_t const x = v ^ secret64(int(8 * st + 8 * i));
            acc += vx + uint64_t(uint32_t(x)) * (x >> 32);
        }
        {
            uint64_t const v = ldData(t.data + len - 64 + 8 * i, al);
            uint64_t const vx = __shfl_xor_sync(0xffffffffu, v, 1);
            uint64_t const x = v ^ secret64(192 - 64 - 7 + 8 * int(i));
            acc += vx + uint64_t(uint32_t(x)) * (x >> 32);
        }
        // merge: pairs (2k, 2k+1) folded with secret words at 11 + 16k
        uint64_t const odd = __shfl_xor_sync(0xffffffffu, acc, 1);
        uint64_t part = 0;
        if (!(i & 1)) {
            int const k = int(i >> 1);
            part = fold128(acc ^ secret64(11 + 16 * k), odd ^ secret64(11 + 16 * k + 8));
        }
        part += __shfl_xor_sync(0xffffffffu, part, 2);
        part += __shfl_xor_sync(0xffffffffu, part, 4);
        if (lane != 0) return;
        h = xAvalanche(len * XP64_1 + part);
    }
    if (t.hashOut) *t.hashOut = h;
    bool const ok = t.low8 ? ((h & 255) == t.expected) : (uint32_t(h) == t.expected);
    if (!ok && t.errCode) reportError(status, t.errCode);
}

} // namespace ozl

// ---------------------------------------------------------------------------
// dispatch
namespace ozl {

namespace {
uint32_t fseLanes(uint32_t tlMax)
{
    uint32_t lanes = 32;
    while (lanes > 1 && fseSmemBytes(lanes, tlMax) > kFseCtaSmem) lanes--;
    return lanes;
}
uint32_t hufSmem(uint32_t chunks) { return hufRingOff(chunks) + 4 * chunks * 16 * kHufRing; }
// kHashBlocks grid: one warp per block up to eight full CTAs per SM, then
// grid-stride (any grid size is correct)
uint32_t hashGrid(uint32_t nbBlocks)
{
    static int sms = 0;
    if (!sms) {
        int dev = 0, n = 0;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess)
            sms = n;
        if (sms <= 0) sms = 152;
    }
    uint32_t const want = (nbBlocks + 7) / 8;
    uint32_t const cap = uint32_t(sms) * 8;
    return want < cap ? (want ? want : 1) : cap;
}
static_assert(2 * kHufSlotBytes >= (2u << kHufTableLog), "a tableLog-12 table fits two slots");
} // namespace

cudaError_t prepareKernels()
{
    cudaError_t e = cudaFuncSetAttribute(kFse, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kFseCtaSmem));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(kFse4, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kFseCtaSmem));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(kHuf, cudaFuncAttributeMaxDynamicSharedMemorySize, int(hufSmem(kHufChunks)));
}

uint32_t tuneCandidates(const Launch& l, uint32_t* out, uint32_t cap)
{
    uint32_t n = 0;
    if (l.kind == KIND_FSE) {
        uint32_t const mx = fseLanes(l.param0);
        for (uint32_t c : { 32u, 16u, 8u, 6u, 5u, 4u, 3u, 2u })
            if (c <= mx && n < cap) out[n++] = c;
        for (uint32_t c : { 8u, 6u, 4u }) // kFse4: streams per warp
            if (c <= mx && n < cap) out[n++] = kFse4Variant | c;
    } else if (l.kind == KIND_HUF) {
        for (uint32_t c : { 8u, 6u, 4u, 2u })
            if (n < cap) out[n++] = c;
    }
    return n;
}

long runLaunches(const DeviceLayout& L, uint8_t* dPool, uint8_t* dScratch, uint32_t* dStatus, cudaStream_t s)
{
    long count = 0;
    for (size_t i = 0; i < L.launches.size(); i++) {
        long const n = runOneLaunch(L, i, dPool, dScratch, dStatus, s);
        if (n < 0) return -1;
        count += n;
    }
    return count;
}

long runOneLaunch(const DeviceLayout& L, size_t li, uint8_t* dPool, uint8_t* dScratch, uint32_t* dStatus,
                  cudaStream_t s)
{
    long count = 0;
    {
        const Launch& l = L.launches[li];
        const void* tasks = dPool + l.taskOff;
        const TileRef* tiles = reinterpret_cast<const TileRef*>(dPool + l.tileOff);
        switch (l.kind) {
            case KIND_COPY:
                kCopy<<<l.nbTiles, 256, 0, s>>>(static_cast<const CopyTask*>(tasks), tiles);
                break;
            case KIND_CONST:
                kConst<<<l.nbTiles, 256, 0, s>>>(static_cast<const ConstTask*>(tasks), tiles);
                break;
            case KIND_FSE: {
                uint32_t const maxLanes = fseLanes(l.param0);
                // untuned: large tables six streams per warp, the autotuner's
                // choice on the mixed-frame workload (wider CTAs wait on their
                // serial table builds and leave too few warps per SM to hide
                // latency); small tables as many as fit
                if (l.tune & kFse4Variant) { // one lane per state, up to eight streams per warp
                    uint32_t streams = l.tune & 0xFFu;
                    if (streams > 8) streams = 8;
                    if (streams > maxLanes) streams = maxLanes;
                    if (streams == 0) streams = 1;
                    uint32_t const grid = (l.nbTasks + streams - 1) / streams;
                    kFse4<<<grid, 32, fseSmemBytes(streams, l.param0), s>>>(static_cast<const FseTask*>(tasks), l.nbTasks,
                                                                            streams, l.param0, dStatus);
                    break;
                }
                uint32_t const dflt = l.param0 <= 8 || maxLanes < kFseDefaultLanes ? maxLanes : kFseDefaultLanes;
                uint32_t const lanes = l.tune && l.tune <= maxLanes ? l.tune : dflt;
                uint32_t const grid = (l.nbTasks + lanes - 1) / lanes;
                kFse<<<grid, 32, fseSmemBytes(lanes, l.param0), s>>>(static_cast<const FseTask*>(tasks), l.nbTasks,
                                                                     lanes, l.param0, dStatus);
                break;
            }
            case KIND_HUF: {
                uint32_t const chunks = l.tune && l.tune <= kHufChunks ? l.tune : kHufChunks;
                uint32_t const grid = (l.nbTasks + chunks - 1) / chunks;
                kHuf<<<grid, 4 * chunks, hufSmem(chunks), s>>>(static_cast<const HufTask*>(tasks), l.nbTasks, chunks,
                                                               dStatus);
                break;
            }
            case KIND_FLATPACK:
                kFlatpack<<<l.nbTiles, 256, 0, s>>>(static_cast<const FlatpackTask*>(tasks), tiles, dStatus);
                break;
            case KIND_HUF16:
                if (l.nbTasks) kHuf16<<<l.nbTasks, 128, 0, s>>>(static_cast<const Huf16Task*>(tasks), dStatus);
                break;
            case KIND_WIDEN:
                kWiden<<<l.nbTiles, 256, 0, s>>>(static_cast<const WidenTask*>(tasks), tiles, dStatus);
                break;
            case KIND_TOKENIZE:
                kTokenize<<<l.nbTiles, 256, 0, s>>>(static_cast<const TokenizeTask*>(tasks), tiles, dStatus);
                break;
            case KIND_FLOATDEC:
                kFloatDec<<<l.nbTiles, 256, 0, s>>>(static_cast<const FloatDecTask*>(tasks), tiles);
                break;
            case KIND_TRANSPOSE:
                kTranspose<<<l.nbTiles, 256, 0, s>>>(static_cast<const TransposeTask*>(tasks), tiles);
                break;
            case KIND_NUMPIPE: {
                const NumPipeTask* const np = static_cast<const NumPipeTask*>(tasks);
                uint64_t* prefix = nullptr;
                if (l.needsScan) {
                    uint64_t* const sums = reinterpret_cast<uint64_t*>(dScratch + l.statusOff);
                    prefix = sums + l.nbTiles;
                    kNumReduce<<<l.nbTiles, kNPThreads, 0, s>>>(np, tiles, sums);
                    kNumPrefix<<<(l.nbTasks * 32 + 255) / 256, 256, 0, s>>>(np, l.nbTasks, sums, prefix);
                    count += 2;
                }
                kNumPipe<<<l.nbTiles, kNPThreads, 0, s>>>(np, tiles, prefix);
                break;
            }
            case KIND_HASH: {
                if (l.nbTiles) {
                    kHashBlocks<<<hashGrid(l.nbTiles), 256, 0, s>>>(static_cast<const HashTask*>(tasks), tiles,
                                                                   l.nbTiles);
                    count++;
                }
                uint32_t const grid = (l.nbTasks * 32 + 255) / 256;
                kHashFinish<<<grid, 256, 0, s>>>(static_cast<const HashTask*>(tasks), l.nbTasks, dStatus);
                break;
            }
            default:
                return -1;
        }
        count++;
        if (cudaPeekAtLastError() != cudaSuccess) return -1;
    }
    return count;
}

} // namespace ozl

// ---------------------------------------------------------------------------
// standalone XXH3-64 of a device buffer, and launch helpers for the encoder
namespace ozl {
void launchCopy(const CopyTask* tasks, const TileRef* tiles, uint32_t nbTiles, cudaStream_t s)
{
    if (nbTiles) kCopy<<<nbTiles, 256, 0, s>>>(tasks, tiles);
}

void launchHash(const HashTask* tasks, uint32_t nbTasks, const TileRef* blocks, uint32_t nbBlocks, uint32_t* status,
                cudaStream_t s)
{
    if (nbBlocks) kHashBlocks<<<hashGrid(nbBlocks), 256, 0, s>>>(tasks, blocks, nbBlocks);
    if (nbTasks) kHashFinish<<<(nbTasks * 32 + 255) / 256, 256, 0, s>>>(tasks, nbTasks, status);
}

cudaError_t xxh3Device(const uint8_t* data, uint64_t len, uint64_t* dHashOut, uint8_t* dScratch,
                       uint64_t scratchBytes, cudaStream_t s)
{
    uint32_t const nbBlocks = len > 240 ? uint32_t((len - 1) / kHashBlock) : 0;
    size_t const need = 256 + size_t(nbBlocks) * (64 + sizeof(TileRef));
    if (need > scratchBytes) return cudaErrorInvalidValue;
    HashTask t{};
    t.data = data;
    t.len = len;
    t.blockSums = reinterpret_cast<uint64_t*>(dScratch + 256);
    t.nbBlocks = nbBlocks;
    t.aligned8 = (reinterpret_cast<uintptr_t>(data) & 7) == 0;
    t.hashOut = dHashOut;
    HashTask* dTask = reinterpret_cast<HashTask*>(dScratch);
    TileRef* dTiles = reinterpret_cast<TileRef*>(dScratch + 256 + size_t(nbBlocks) * 64);
    cudaError_t e = cudaMemcpyAsync(dTask, &t, sizeof(t), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    if (nbBlocks) {
        std::vector<TileRef> tiles(nbBlocks);
        for (uint32_t k = 0; k < nbBlocks; k++) tiles[k] = TileRef{ 0, k };
        e = cudaMemcpyAsync(dTiles, tiles.data(), nbBlocks * sizeof(TileRef), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return e;
        kHashBlocks<<<hashGrid(nbBlocks), 256, 0, s>>>(dTask, dTiles, nbBlocks);
    }
    kHashFinish<<<1, 32, 0, s>>>(dTask, 1, nullptr);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s);
}
} // namespace ozl

// ---------------------------------------------------------------------------
// Allocation-free XXH3 (ozl_gpu_xxh3_64_static): the hash kernels above, fed
// from one file-scope device array instead of allocated scratch.
//
// Array layout: [0, 128) the task, [128, 136) the result, [256, ...) the
// per-block sums (64 bytes per 1 KiB block), then the block list (8 bytes per
// block). Nothing in it has to start at zero: each call writes the task, the
// block list and every block sum it reads, and clears the result word first.
// Calls that overlap on the GPU share the array and race.
#include "../../include/openzl_gb300.h"

namespace {

constexpr uint64_t kStaticMaxLen = OZL_XXH3_STATIC_MAX_LEN;
constexpr uint32_t kStaticMaxBlocks = uint32_t(kStaticMaxLen / ozl::kHashBlock);
constexpr size_t kStaticScratch = OZL_XXH3_STATIC_SCRATCH;
static_assert(kStaticScratch >= 256 + size_t(kStaticMaxBlocks) * (64 + sizeof(ozl::TileRef)), "scratch layout");
static_assert(sizeof(ozl::HashTask) <= 128, "task slot");

static __device__ __align__(256) uint8_t gXxh3Scratch[kStaticScratch];

// Writes the task and the block list into the array (one launch, no host copy).
__global__ void kStageHashStatic(ozl::HashTask t, ozl::HashTask* dTask, ozl::TileRef* dBlocks, uint32_t nbBlocks,
                                 uint64_t* dResult)
{
    uint32_t const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        *dTask = t;
        *dResult = 0;
    }
    if (i < nbBlocks) dBlocks[i] = ozl::TileRef{ 0, i };
}

// Device address of the array in the current device's context, looked up on
// every call (no allocation): a cached address would go stale if the host
// application reset the device and the module reloaded elsewhere.
cudaError_t staticScratch(uint8_t** out)
{
    void* p = nullptr;
    cudaError_t const e = cudaGetSymbolAddress(&p, gXxh3Scratch);
    if (e != cudaSuccess) return e;
    *out = static_cast<uint8_t*>(p);
    return cudaSuccess;
}

} // namespace

extern "C" ZL_Report ozl_gpu_xxh3_64_static(const void* d_data, size_t len, void* stream)
{
    if (len > kStaticMaxLen) return ZL_Report{ ZL_ErrorCode_srcSize_tooLarge, 0 };
    if (!d_data && len) return ZL_Report{ ZL_ErrorCode_parameter_invalid, 0 };
    uint8_t* base = nullptr;
    if (staticScratch(&base) != cudaSuccess) return ZL_Report{ ZL_ErrorCode_GENERIC, 0 };
    cudaStream_t const s = static_cast<cudaStream_t>(stream);
    uint32_t const nbBlocks = len > 240 ? uint32_t((len - 1) / ozl::kHashBlock) : 0;
    auto* dTask = reinterpret_cast<ozl::HashTask*>(base);
    auto* dResult = reinterpret_cast<uint64_t*>(base + 128);
    auto* dSums = reinterpret_cast<uint64_t*>(base + 256);
    auto* dBlocks = reinterpret_cast<ozl::TileRef*>(base + 256 + size_t(kStaticMaxBlocks) * 64);
    ozl::HashTask t{};
    t.data = static_cast<const uint8_t*>(d_data);
    t.len = len;
    t.blockSums = dSums;
    t.nbBlocks = nbBlocks;
    t.aligned8 = (reinterpret_cast<uintptr_t>(d_data) & 7) == 0;
    t.hashOut = dResult;
    uint32_t const stageThreads = nbBlocks > 0 ? nbBlocks : 1;
    kStageHashStatic<<<(stageThreads + 255) / 256, 256, 0, s>>>(t, dTask, dBlocks, nbBlocks, dResult);
    if (nbBlocks) ozl::kHashBlocks<<<ozl::hashGrid(nbBlocks), 256, 0, s>>>(dTask, dBlocks, nbBlocks);
    ozl::kHashFinish<<<1, 32, 0, s>>>(dTask, 1, nullptr);
    if (cudaGetLastError() != cudaSuccess) return ZL_Report{ ZL_ErrorCode_GENERIC, 0 };
    uint64_t h = 0;
    if (cudaMemcpyAsync(&h, dResult, 8, cudaMemcpyDeviceToHost, s) != cudaSuccess
        || cudaStreamSynchronize(s) != cudaSuccess)
        return ZL_Report{ ZL_ErrorCode_GENERIC, 0 };
    return ZL_Report{ ZL_ErrorCode_no_error, size_t(h) };
}

