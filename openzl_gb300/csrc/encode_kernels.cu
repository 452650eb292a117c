// sm_103a encode kernels for OpenZL's numeric codec graph.
//
// Data-parallel front ends (delta/zigzag with byte-split or bit packing),
// per-chunk histograms, and the entropy bitstreams (FSE with 2/4 interleaved
// states, Huffman 1X/4X). Bitstream kernels run one lane per chunk (FSE) or
// per stream (Huffman) with that chunk's coding table in shared memory; the
// bit order restates src/openzl/fse/bitstream.h (fields appended LSB-first,
// a final 1 marker bit).
#include <cstdint>
#include <type_traits>

#include <cuda_runtime.h>

#include "enc_exec.h"
#include "enc_tables.h"
#include "fse_norm.h"
#include "huf_tree.h"
#include "enc_tasks.h"
#include "stream_ring.cuh"

namespace ozl {

namespace {

__device__ __forceinline__ uint64_t ldW(const uint8_t* p, uint32_t w)
{
    uint64_t v = 0;
    if (w == 1) return *p;
    if (w == 2 && !(reinterpret_cast<uintptr_t>(p) & 1)) return *reinterpret_cast<const uint16_t*>(p);
    if (w == 4 && !(reinterpret_cast<uintptr_t>(p) & 3)) return *reinterpret_cast<const uint32_t*>(p);
    if (w == 8 && !(reinterpret_cast<uintptr_t>(p) & 7)) return *reinterpret_cast<const uint64_t*>(p);
    for (uint32_t b = 0; b < w; b++) v |= uint64_t(p[b]) << (8 * b);
    return v;
}

__device__ __forceinline__ void stW(uint8_t* p, uint64_t v, uint32_t w)
{
    if (w == 1) { *p = uint8_t(v); return; }
    if (w == 2 && !(reinterpret_cast<uintptr_t>(p) & 1)) { *reinterpret_cast<uint16_t*>(p) = uint16_t(v); return; }
    if (w == 4 && !(reinterpret_cast<uintptr_t>(p) & 3)) { *reinterpret_cast<uint32_t*>(p) = uint32_t(v); return; }
    if (w == 8 && !(reinterpret_cast<uintptr_t>(p) & 7)) { *reinterpret_cast<uint64_t*>(p) = v; return; }
    for (uint32_t b = 0; b < w; b++) p[b] = uint8_t(v >> (8 * b));
}

__device__ __forceinline__ uint64_t transformed(const EncNumTask& t, uint64_t i)
{
    uint64_t const m = t.w >= 8 ? ~0ull : ((1ull << (8 * t.w)) - 1);
    uint64_t v;
    if (t.delta) v = (ldW(t.src + (i + 1) * t.w, t.w) - ldW(t.src + i * t.w, t.w)) & m;
    else v = ldW(t.src + i * t.w, t.w);
    if (t.zigzag) {
        uint64_t const sign = (v >> (8 * t.w - 1)) & 1;
        v = ((v << 1) ^ (0 - sign)) & m;
    }
    return v;
}

// Packs `cnt` fields of nbBits (LSB-first) that start at a 32-bit boundary of
// `out`; complete words are stored whole, the final partial word bytewise.
struct WordPacker {
    uint8_t* out;
    uint64_t acc = 0;
    uint32_t nb = 0;
    uint32_t pos = 0; // bytes written
    __device__ explicit WordPacker(uint8_t* o) : out(o) {}
    // invariant: nb < 32 between calls
    __device__ __forceinline__ void put(uint64_t v, uint32_t bits)
    {
        if (bits > 32) {
            put(v & 0xffffffffu, 32);
            put(v >> 32, bits - 32);
            return;
        }
        uint64_t const m = bits == 32 ? 0xffffffffull : ((1ull << bits) - 1);
        acc |= (v & m) << nb;
        nb += bits;
        if (nb >= 32) {
            *reinterpret_cast<uint32_t*>(out + pos) = uint32_t(acc);
            pos += 4;
            acc >>= 32;
            nb -= 32;
        }
    }
    __device__ __forceinline__ void finish(uint32_t totalBytes)
    {
        while (pos < totalBytes) {
            out[pos++] = uint8_t(acc);
            acc >>= 8;
        }
    }
};

} // namespace

// ---------------------------------------------------------------------------
// per-task maximum of the transformed values (bit width of bitpack_int)
__global__ void kEncMax(const EncNumTask* __restrict__ tasks, const TileRef* __restrict__ tiles,
                        unsigned long long* __restrict__ maxima)
{
    TileRef const tr = tiles[blockIdx.x];
    EncNumTask const t = tasks[tr.task];
    uint64_t const e0 = uint64_t(tr.tile) * kEncTile;
    uint64_t const e1 = min(t.n, e0 + kEncTile);
    uint64_t mx = 0;
    for (uint64_t i = e0 + threadIdx.x; i < e1; i += blockDim.x) {
        uint64_t const v = transformed(t, i);
        mx = v > mx ? v : mx;
    }
    for (int o = 16; o > 0; o >>= 1) {
        uint64_t const x = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = x > mx ? x : mx;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(&maxima[t.maxSlot], (unsigned long long)mx);
}

// Element e of consecutive W-byte elements held as little-endian words.
template <int W>
__device__ __forceinline__ uint64_t elemOf(const uint32_t* u, int e)
{
    if constexpr (W == 8) return uint64_t(u[2 * e]) | (uint64_t(u[2 * e + 1]) << 32);
    else if constexpr (W == 4) return u[e];
    else if constexpr (W == 2) return (u[e >> 1] >> (16 * (e & 1))) & 0xffffu;
    else return (u[e >> 2] >> (8 * (e & 3))) & 0xffu;
}

// The thread's 32 elements [i0, i0 + 32) of a full tile when the source is
// 16-byte aligned, in rounds of R elements (64 bytes for 8-byte elements,
// else 16 elements) loaded as 16-byte vectors; the element after a round,
// which delta needs, is the next round's first (loaded one round ahead) or
// one more load after the last. Values are transformed in registers and
// written as vectors (plain, byte planes) or packed fields. Returns false
// (the caller takes the element loop) when an output is not 16-byte aligned.
template <int W>
__device__ __forceinline__ bool encNumVec(const EncNumTask& t, uint64_t i0)
{
    constexpr int R = W == 8 ? 8 : 16, NV = R * W / 16, ROUNDS = 32 / R;
    if (t.mode == EOUT_PLAIN && (reinterpret_cast<uintptr_t>(t.out) & 15)) return false;
    if (t.mode == EOUT_PLANES && ((reinterpret_cast<uintptr_t>(t.out) | t.planeStride) & 15)) return false;
    using V = typename std::conditional<W == 8, uint64_t, uint32_t>::type;
    uint64_t const m = W >= 8 ? ~0ull : ((1ull << (8 * W)) - 1);
    const uint4* const src = reinterpret_cast<const uint4*>(t.src + i0 * W);
    WordPacker wp(t.out + (i0 / 32) * 4 * t.nbBits);
    uint32_t u[4 * NV], nx[4 * NV];
#pragma unroll
    for (int q = 0; q < NV; q++) reinterpret_cast<uint4*>(u)[q] = __ldg(src + q);
#pragma unroll
    for (int h = 0; h < ROUNDS; h++) {
        uint64_t after = 0; // the first element after this round
        if (h + 1 < ROUNDS) {
#pragma unroll
            for (int q = 0; q < NV; q++) reinterpret_cast<uint4*>(nx)[q] = __ldg(src + NV * (h + 1) + q);
            after = elemOf<W>(nx, 0);
        } else if (t.delta) {
            after = ldW(t.src + (i0 + 32) * W, W);
        }
        V v[R];
#pragma unroll
        for (int e = 0; e < R; e++) {
            uint64_t x = elemOf<W>(u, e);
            if (t.delta) x = ((e + 1 < R ? elemOf<W>(u, e + 1) : after) - x) & m;
            if (t.zigzag) x = ((x << 1) ^ (0 - ((x >> (8 * W - 1)) & 1))) & m;
            v[e] = V(x);
        }
        uint64_t const j = i0 + uint64_t(R) * h;
        if (t.mode == EOUT_PLAIN) {
            uint32_t o[4 * NV];
#pragma unroll
            for (int q = 0; q < 4 * NV; q++) o[q] = 0;
#pragma unroll
            for (int e = 0; e < R; e++) {
                if constexpr (W == 8) {
                    o[2 * e] = uint32_t(v[e]);
                    o[2 * e + 1] = uint32_t(uint64_t(v[e]) >> 32);
                } else {
                    o[(e * W) >> 2] |= uint32_t(v[e]) << (8 * ((e * W) & 3));
                }
            }
            uint4* const dst = reinterpret_cast<uint4*>(t.out + j * W);
#pragma unroll
            for (int q = 0; q < NV; q++) dst[q] = reinterpret_cast<const uint4*>(o)[q];
        } else if (t.mode == EOUT_PLANES) {
#pragma unroll
            for (int b = 0; b < W; b++) {
                uint32_t wd[R / 4];
#pragma unroll
                for (int q = 0; q < R / 4; q++) {
                    uint32_t x = 0;
#pragma unroll
                    for (int c = 0; c < 4; c++) x |= uint32_t((uint64_t(v[4 * q + c]) >> (8 * b)) & 0xffu) << (8 * c);
                    wd[q] = x;
                }
                uint8_t* const p = t.out + b * t.planeStride + j;
                if constexpr (R == 16) *reinterpret_cast<uint4*>(p) = make_uint4(wd[0], wd[1], wd[2], wd[3]);
                else *reinterpret_cast<uint2*>(p) = make_uint2(wd[0], wd[1]);
            }
        } else {
#pragma unroll
            for (int e = 0; e < R; e++) wp.put(uint64_t(v[e]), t.nbBits);
        }
        if (h + 1 < ROUNDS) {
#pragma unroll
            for (int q = 0; q < 4 * NV; q++) u[q] = nx[q];
        }
    }
    if (t.mode == EOUT_BITPACK) wp.finish(4 * t.nbBits);
    return true;
}

// front end: delta/zigzag then plain, byte planes or bit packing.
// 128 threads x 32 consecutive elements per tile.
__global__ void __launch_bounds__(128) kEncNum(const EncNumTask* __restrict__ tasks, const TileRef* __restrict__ tiles)
{
    TileRef const tr = tiles[blockIdx.x];
    EncNumTask const t = tasks[tr.task];
    uint64_t const i0 = uint64_t(tr.tile) * kEncTile + uint64_t(threadIdx.x) * 32;
    if (i0 >= t.n) return;
    uint32_t const cnt = uint32_t(min(uint64_t(32), t.n - i0));
    // full rounds from a 16-byte aligned source (the source holds element
    // i0 + 32 when delta reads it: n output elements come from n + 1)
    if (cnt == 32 && !(reinterpret_cast<uintptr_t>(t.src) & 15) && (!t.delta || i0 + 32 <= t.n)) {
        bool done = false;
        switch (t.w) {
            case 1: done = encNumVec<1>(t, i0); break;
            case 2: done = encNumVec<2>(t, i0); break;
            case 4: done = encNumVec<4>(t, i0); break;
            case 8: done = encNumVec<8>(t, i0); break;
            default: break;
        }
        if (done) return;
    }
    if (t.mode == EOUT_PLAIN) {
        for (uint32_t k = 0; k < cnt; k++) stW(t.out + (i0 + k) * t.w, transformed(t, i0 + k), t.w);
    } else if (t.mode == EOUT_PLANES) {
        uint64_t v[32];
        for (uint32_t k = 0; k < cnt; k++) v[k] = transformed(t, i0 + k);
        for (uint32_t b = 0; b < t.w; b++) {
            uint8_t* const p = t.out + b * t.planeStride + i0;
            if (cnt == 32 && !(reinterpret_cast<uintptr_t>(p) & 15)) {
                uint32_t wds[8];
                for (int q = 0; q < 8; q++) {
                    uint32_t x = 0;
                    for (int c = 0; c < 4; c++) x |= uint32_t((v[4 * q + c] >> (8 * b)) & 0xff) << (8 * c);
                    wds[q] = x;
                }
                reinterpret_cast<uint4*>(p)[0] = make_uint4(wds[0], wds[1], wds[2], wds[3]);
                reinterpret_cast<uint4*>(p)[1] = make_uint4(wds[4], wds[5], wds[6], wds[7]);
            } else {
                for (uint32_t k = 0; k < cnt; k++) p[k] = uint8_t(v[k] >> (8 * b));
            }
        }
    } else {
        // 32 fields start at bit 32*nbBits*(i0/32): a 4-byte boundary
        WordPacker wp(t.out + (i0 / 32) * 4 * t.nbBits);
        for (uint32_t k = 0; k < cnt; k++) wp.put(transformed(t, i0 + k), t.nbBits);
        wp.finish(uint32_t((uint64_t(cnt) * t.nbBits + 7) / 8));
    }
}

// serial bit packing / flatpack indices
__global__ void __launch_bounds__(128) kPack(const PackTask* __restrict__ tasks, const TileRef* __restrict__ tiles)
{
    TileRef const tr = tiles[blockIdx.x];
    PackTask const t = tasks[tr.task];
    uint64_t const i0 = uint64_t(tr.tile) * kEncTile + uint64_t(threadIdx.x) * 32;
    if (i0 >= t.n) return;
    uint32_t const cnt = uint32_t(min(uint64_t(32), t.n - i0));
    WordPacker wp(t.out + (i0 / 32) * 4 * t.nbBits);
    for (uint32_t k = 0; k < cnt; k++) {
        uint32_t const s = t.src[i0 + k];
        wp.put(t.map ? t.map[s] : s, t.nbBits);
    }
    uint32_t bits = cnt * t.nbBits;
    if (t.map && i0 + cnt == t.n) {
        wp.put(1, 1); // flatpack terminator
        bits += 1;
    }
    wp.finish((bits + 7) / 8);
}

// 256-bin histogram of one chunk per CTA
__global__ void __launch_bounds__(256) kHist(const HistTask* __restrict__ tasks, uint32_t* __restrict__ hists)
{
    __shared__ uint32_t h[8][256];
    HistTask const t = tasks[blockIdx.x];
    for (int k = threadIdx.x; k < 8 * 256; k += 256) (&h[0][0])[k] = 0;
    __syncthreads();
    uint32_t* const mine = h[threadIdx.x & 7];
    uint32_t const n = t.n;
    uint32_t i = threadIdx.x * 4;
    bool const al = !(reinterpret_cast<uintptr_t>(t.src) & 3);
    if (al) {
        for (; i + 4 <= n; i += 1024) {
            uint32_t const x = *reinterpret_cast<const uint32_t*>(t.src + i);
            atomicAdd(&mine[x & 0xff], 1u);
            atomicAdd(&mine[(x >> 8) & 0xff], 1u);
            atomicAdd(&mine[(x >> 16) & 0xff], 1u);
            atomicAdd(&mine[x >> 24], 1u);
        }
        for (uint32_t k = i; k < n && k < i + 4; k++) atomicAdd(&mine[t.src[k]], 1u);
    } else {
        for (uint32_t k = threadIdx.x; k < n; k += 256) atomicAdd(&mine[t.src[k]], 1u);
    }
    __syncthreads();
    uint32_t s = 0;
    for (int r = 0; r < 8; r++) s += h[r][threadIdx.x];
    hists[uint64_t(t.outIndex) * 256 + threadIdx.x] = s;
}

// ---------------------------------------------------------------------------
// forward bit writer into a 4-byte aligned buffer of `cap` bytes; writes past
// the capacity are dropped and reported through the returned size (> cap).
struct BitOut {
    uint8_t* out;
    uint32_t cap;
    uint64_t acc = 0;
    uint32_t nb = 0;
    uint32_t pos = 0;
    __device__ BitOut(uint8_t* o, uint32_t c) : out(o), cap(c) {}
    __device__ __forceinline__ void add(uint32_t v, uint32_t bits)
    {
        acc |= uint64_t(v & ((1u << bits) - 1u)) << nb;
        nb += bits;
        if (nb >= 32) {
            if (pos + 4 <= cap) *reinterpret_cast<uint32_t*>(out + pos) = uint32_t(acc);
            pos += 4;
            acc >>= 32;
            nb -= 32;
        }
    }
    // appends `bits` <= 32 bits of v (bits above them zero) with one flush
    // check: used for two fields combined, so that the fields of a step are
    // computed before any branch
    __device__ __forceinline__ void add2(uint32_t v, uint32_t bits)
    {
        acc |= uint64_t(v) << nb;
        nb += bits;
        if (nb >= 32) {
            if (pos + 4 <= cap) *reinterpret_cast<uint32_t*>(out + pos) = uint32_t(acc);
            pos += 4;
            acc >>= 32;
            nb -= 32;
        }
    }
    __device__ __forceinline__ uint32_t close()
    {
        add(1, 1);
        while (nb > 0) {
            if (pos < cap) out[pos] = uint8_t(acc);
            pos++;
            acc >>= 8;
            nb = nb > 8 ? nb - 8 : 0;
        }
        return pos;
    }
};

// FSE coding tables on the device, one warp per chunk: lane 0 normalizes the
// histogram and writes the normalized-count header (fse_norm.h, serial as in
// the reference); the warp builds the encoding table (FSE_buildCTable_wksp,
// fse_compress.c:69-207). Cells: the count -1 symbols take the top cells in
// symbol order; occurrence k of the other symbols (in symbol order, each
// repeated count times) goes to the k-th cell of the sequence 0, step,
// 2 step, ... (mod size) below the top cells, 32 positions per round ranked
// by a ballot. States: a symbol's state slots, from its cumulative count,
// take its cells in increasing order, ranked within the round by
// __match_any_sync. The result equals the serial construction.
constexpr int kFseTabWarps = 4;
struct FseBuildSmem {
    uint32_t count[256];
    int16_t norm[256];
    uint16_t posCum[260];  // occurrences before each symbol (positive counts)
    uint16_t cumul[260];   // state slots before each symbol (count -1 takes one)
    uint16_t next[256];
    uint8_t symbolAt[2048];
};

__global__ void __launch_bounds__(32 * kFseTabWarps) kFseTables(const FseTableTask* __restrict__ tasks, uint32_t nbTasks,
                                                                uint32_t* __restrict__ sizes,
                                                                uint32_t* __restrict__ errors)
{
    __shared__ FseBuildSmem sm[kFseTabWarps];
    uint32_t const wid = threadIdx.x >> 5, lane = threadIdx.x & 31, lt = (1u << lane) - 1;
    uint32_t const ti = blockIdx.x * kFseTabWarps + wid;
    if (ti >= nbTasks) return; // the whole warp
    FseTableTask const t = tasks[ti];
    FseBuildSmem& S = sm[wid];
    uint32_t const tl = t.tableLog, maxSym = t.maxSym;
    uint32_t const size = 1u << tl, mask = size - 1, step = (size >> 1) + (size >> 3) + 3;
    if (tl < 5 || tl > 11 || maxSym > 255) { // outside what the encoder emits
        if (lane == 0) atomicOr(errors, 1u);
        return;
    }
    for (uint32_t k = lane; k < 256; k += 32) {
        S.count[k] = t.hist[k];
        S.norm[k] = 0;
    }
    __syncwarp();
    if (lane == 0 && !ent::fseNormalizeCounts(S.norm, tl, S.count, t.n, maxSym)) atomicOr(errors, 1u);
    __syncwarp();
    // lane j: symbols 8j .. 8j + 7; scans of occurrences, state slots and
    // top cells
    int v[8];
    uint32_t sp = 0, sc = 0, sn = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        uint32_t const sy = 8 * lane + k;
        v[k] = sy <= maxSym ? int(S.norm[sy]) : 0;
        sp += v[k] > 0 ? uint32_t(v[k]) : 0u;
        sc += v[k] == -1 ? 1u : (v[k] > 0 ? uint32_t(v[k]) : 0u);
        sn += v[k] == -1 ? 1u : 0u;
    }
    uint32_t ip = sp, ic = sc, in = sn;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t const yp = __shfl_up_sync(0xffffffffu, ip, o), yc = __shfl_up_sync(0xffffffffu, ic, o),
                       yn = __shfl_up_sync(0xffffffffu, in, o);
        if (lane >= uint32_t(o)) {
            ip += yp;
            ic += yc;
            in += yn;
        }
    }
    uint32_t const totalNeg = __shfl_sync(0xffffffffu, in, 31);
    uint32_t const high = size - 1 - totalNeg;
    uint32_t p0 = ip - sp, c0 = ic - sc, n0 = in - sn;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        uint32_t const sy = 8 * lane + k;
        S.posCum[sy] = uint16_t(p0);
        S.cumul[sy] = uint16_t(c0);
        S.next[sy] = uint16_t(c0);
        p0 += v[k] > 0 ? uint32_t(v[k]) : 0u;
        c0 += v[k] == -1 ? 1u : (v[k] > 0 ? uint32_t(v[k]) : 0u);
        if (v[k] == -1) {
            S.symbolAt[size - 1 - n0] = uint8_t(sy);
            n0++;
        }
    }
    if (lane == 31) {
        S.posCum[256] = uint16_t(p0);
        S.cumul[256] = uint16_t(c0);
    }
    __syncwarp();
    // spread
    uint32_t sCur = 0, cumNext = S.posCum[1], occBase = 0;
    for (uint32_t b0 = 0; b0 < size; b0 += 32) {
        uint32_t const pos = ((b0 + lane) * step) & mask;
        bool const valid = totalNeg < size && pos <= high;
        uint32_t const bal = __ballot_sync(0xffffffffu, valid);
        if (valid) {
            uint32_t const occ = occBase + __popc(bal & lt);
            while (occ >= cumNext && sCur < 255) cumNext = S.posCum[++sCur + 1];
            S.symbolAt[pos] = uint8_t(sCur);
        }
        occBase += __popc(bal);
    }
    __syncwarp();
    // state table
    ent::FseCTable* const ct = reinterpret_cast<ent::FseCTable*>(t.ctable);
    for (uint32_t b0 = 0; b0 < size; b0 += 32) {
        uint32_t const u = b0 + lane;
        uint32_t const sy = S.symbolAt[u];
        uint32_t const m = __match_any_sync(0xffffffffu, sy);
        uint32_t const base = S.next[sy];
        __syncwarp();
        if (lane == 31u - __clz(m)) S.next[sy] = uint16_t(base + __popc(m));
        ct->state[base + __popc(m & lt)] = uint16_t(size + u);
        __syncwarp();
    }
    for (uint32_t sy = lane; sy < 256; sy += 32) {
        int const c = sy <= maxSym ? int(S.norm[sy]) : 0;
        ent::fseSymbolDeltas(c, tl, S.cumul[sy], ct->deltaNbBits[sy], ct->deltaFindState[sy]);
    }
    for (uint32_t sy = lane; sy <= maxSym; sy += 32) t.norm[sy] = S.norm[sy];
    if (lane == 0) {
        ct->tableLog = uint16_t(tl);
        ct->maxSym = uint16_t(maxSym);
        sizes[t.sizeSlot] = uint32_t(ent::fseWriteNCountTo(t.ncount, S.norm, maxSym, tl));
    }
}

// Huffman code lengths and codes on the device, one warp per chunk: the
// build (huf_tree.h, as the reference's HUF_buildCTable) is serial, so lane 0
// runs it on the warp's shared nodes; the warp loads the histogram and writes
// the weights.
constexpr int kHufTabWarps = 4;
struct HufBuildSmem {
    ent::HufNode nodes[ent::kHufNodes];
    uint32_t count[256];
    uint8_t nbBits[256];
};

__global__ void __launch_bounds__(32 * kHufTabWarps) kHufTables(const HufTableTask* __restrict__ tasks, uint32_t nbTasks)
{
    __shared__ HufBuildSmem sm[kHufTabWarps];
    __shared__ uint32_t sTl[kHufTabWarps];
    uint32_t const wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t const ti = blockIdx.x * kHufTabWarps + wid;
    if (ti >= nbTasks) return; // the whole warp
    HufTableTask const t = tasks[ti];
    HufBuildSmem& S = sm[wid];
    for (uint32_t k = lane; k < 256; k += 32) S.count[k] = t.hist[k];
    __syncwarp();
    ent::HufCTable* const ct = reinterpret_cast<ent::HufCTable*>(t.ctable);
    if (lane == 0) {
        unsigned const tl = ent::hufBuildCodes(S.nodes, ct->value, S.nbBits, S.count, t.maxSym, t.maxNbBits);
        ct->tableLog = tl;
        sTl[wid] = tl;
    }
    __syncwarp();
    uint32_t const tl = sTl[wid];
    for (uint32_t k = lane; k < 256; k += 32) {
        uint32_t const nb = S.nbBits[k];
        ct->nbBits[k] = uint8_t(nb);
        if (k <= t.maxSym) t.weights[k] = uint8_t(nb ? tl + 1 - nb : 0);
    }
}

// Sources are read from their end, four symbols per 32-bit word, through a
// per-lane ring of 16-byte blocks in shared memory filled by cp.async ahead
// of use (the lanes of a warp read unrelated chunks, so direct byte loads
// stall the warp on every lane's cache misses).
constexpr int kEncRing = 8, kEncAhead = 5; // 128 bytes per lane, 80 bytes ahead
using EncRing = StreamRing<kEncRing, kEncAhead>;

// Reader of the words that hold a source's bytes [q - 4, q), q falling by 4
// per call; q is a byte position above the 16-byte block of the source's
// first byte.
struct BackWords {
    EncRing r;
    int32_t k;   // word holding byte q - 4
    uint32_t sh; // (q - 4) % 4, in bits
    uint32_t hi; // word k + 1
    // `src`, `n` > 0 bytes; `ip` the count of bytes not yet read from the top
    __device__ __forceinline__ void start(const uint8_t* src, uint32_t n, uint32_t ip, uint32_t* ring)
    {
        uintptr_t const a = reinterpret_cast<uintptr_t>(src) & ~uintptr_t(15);
        uint32_t const off = uint32_t(reinterpret_cast<uintptr_t>(src) - a);
        r.g16 = reinterpret_cast<const uint8_t*>(a);
        r.ring = ring;
        r.start(int32_t(off + n) * 8);
        int32_t const q = int32_t(off + ip);
        k = (q - 4) >> 2;
        sh = uint32_t((q - 4) & 3) * 8;
        hi = sh ? r.word(k + 1) : 0u;
    }
    // bytes [q - 4, q) of the source, the lowest in bits 0-7
    __device__ __forceinline__ uint32_t next()
    {
        uint32_t const lo = r.word(k);
        uint32_t const w = sh ? __funnelshift_r(lo, hi, sh) : lo;
        hi = lo;
        k--;
        return w;
    }
};

// FSE: one lane per chunk; the lane's table (2^tableLog next states and the
// per-symbol transform) lives in shared memory, then its source ring.
constexpr uint32_t kFseEncLanes = 16;
constexpr uint32_t kFseLaneTables = 2048 * 2 + 256 * 8;
constexpr uint32_t kFseLaneBytes = kFseLaneTables + 16 * kEncRing;
static_assert(kFseLaneTables % 16 == 0 && kFseLaneBytes % 16 == 0, "16-byte aligned rings");

__global__ void __launch_bounds__(32) kFseEnc(const FseEncTask* __restrict__ tasks, uint32_t nbTasks,
                                              uint32_t* __restrict__ sizes)
{
    extern __shared__ uint8_t smemFseEnc[];
    uint32_t const lane = threadIdx.x;
    uint32_t const ti = blockIdx.x * kFseEncLanes + lane;
    if (lane >= kFseEncLanes || ti >= nbTasks) return;
    FseEncTask const t = tasks[ti];
    uint8_t* const base = smemFseEnc + size_t(lane) * kFseLaneBytes;
    uint32_t* const dnb = reinterpret_cast<uint32_t*>(base);
    int32_t* const dfs = reinterpret_cast<int32_t*>(base + 1024);
    uint16_t* const st = reinterpret_cast<uint16_t*>(base + 2048);
    const ent::FseCTable* ct = reinterpret_cast<const ent::FseCTable*>(t.ctable);
    for (int s = 0; s < 256; s++) {
        dnb[s] = ct->deltaNbBits[s];
        dfs[s] = ct->deltaFindState[s];
    }
    uint32_t const size = 1u << t.tableLog;
    for (uint32_t u = 0; u < size; u++) st[u] = ct->state[u];

    uint32_t const n = t.n, ns = t.nbStates;
    BitOut bo(t.out, t.n + t.n / 128 + 512);
    uint32_t v[4];
    auto initState = [&](uint32_t sym) -> uint32_t {
        uint32_t const nbOut = (dnb[sym] + (1u << 15)) >> 16;
        uint32_t const x = (nbOut << 16) - dnb[sym];
        return st[(x >> nbOut) + dfs[sym]];
    };
    auto encode = [&](uint32_t& state, uint32_t sym) {
        uint32_t const nbOut = (state + dnb[sym]) >> 16;
        bo.add(state, nbOut);
        state = st[(state >> nbOut) + dfs[sym]];
    };
    // The start-up loops reach the states by a run-time index. Each access
    // is a switch over the four constant indexes: indexing the array itself
    // would put it, and with it every state of the main loop, in local memory.
    auto initAt = [&](uint32_t k, uint32_t sym) {
        uint32_t const x = initState(sym);
        switch (k) {
            case 0: v[0] = x; break;
            case 1: v[1] = x; break;
            case 2: v[2] = x; break;
            default: v[3] = x; break;
        }
    };
    auto encodeAt = [&](uint32_t k, uint32_t sym) {
        switch (k) {
            case 0: encode(v[0], sym); break;
            case 1: encode(v[1], sym); break;
            case 2: encode(v[2], sym); break;
            default: encode(v[3], sym); break;
        }
    };
    int64_t ip = n;
    uint32_t s = ns - (n % ns);
    for (uint32_t k = 0; k < ns; k++) initAt((s++) % ns, t.src[--ip]);
    for (uint32_t k = 0; k < n % ns; k++) encodeAt((s++) % ns, t.src[--ip]);
    // ip is a multiple of nbStates now: four symbols per word, states in
    // turn. One transition of state x for symbol y: nbOut = (x + dnb[y]) >>
    // 16, its field is the low nbOut bits of x, its next state st[(x >>
    // nbOut) + dfs[y]]. The fields of two transitions are joined (at most
    // 2 x 12 bits) and appended with one flush check, after the states of
    // the step have been computed, so the states' chains overlap.
    auto step = [&](uint32_t& xa, uint32_t ya, uint32_t& xb, uint32_t yb) {
        uint32_t const na = (xa + dnb[ya]) >> 16, nb = (xb + dnb[yb]) >> 16;
        uint32_t const fa = xa & ((1u << na) - 1u), fb = xb & ((1u << nb) - 1u);
        xa = st[(xa >> na) + dfs[ya]];
        xb = st[(xb >> nb) + dfs[yb]];
        bo.add2(fa | (fb << na), na + nb);
    };
    if (ip >= 4) {
        BackWords bw;
        bw.start(t.src, n, uint32_t(ip), reinterpret_cast<uint32_t*>(base + kFseLaneTables));
        if (ns == 4) {
            for (; ip >= 4; ip -= 4) {
                uint32_t const w = bw.next();
                uint32_t const y0 = w >> 24, y1 = (w >> 16) & 0xffu, y2 = (w >> 8) & 0xffu, y3 = w & 0xffu;
                uint32_t const n0 = (v[0] + dnb[y0]) >> 16, n1 = (v[1] + dnb[y1]) >> 16;
                uint32_t const n2 = (v[2] + dnb[y2]) >> 16, n3 = (v[3] + dnb[y3]) >> 16;
                uint32_t const f01 = (v[0] & ((1u << n0) - 1u)) | ((v[1] & ((1u << n1) - 1u)) << n0);
                uint32_t const f23 = (v[2] & ((1u << n2) - 1u)) | ((v[3] & ((1u << n3) - 1u)) << n2);
                v[0] = st[(v[0] >> n0) + dfs[y0]];
                v[1] = st[(v[1] >> n1) + dfs[y1]];
                v[2] = st[(v[2] >> n2) + dfs[y2]];
                v[3] = st[(v[3] >> n3) + dfs[y3]];
                bo.add2(f01, n0 + n1);
                bo.add2(f23, n2 + n3);
            }
        } else {
            for (; ip >= 4; ip -= 4) {
                uint32_t const w = bw.next();
                step(v[0], w >> 24, v[1], (w >> 16) & 0xffu);
                step(v[0], (w >> 8) & 0xffu, v[1], w & 0xffu);
            }
        }
        asm volatile("cp.async.wait_all;" ::: "memory"); // no copy outlives the lane
    }
    for (; ip > 0; ip -= 2) { // two states: the last pair
        encode(v[0], t.src[ip - 1]);
        encode(v[1], t.src[ip - 2]);
    }
    bo.add(v[0], t.tableLog);
    bo.add(v[1], t.tableLog);
    if (ns == 4) {
        bo.add(v[2], t.tableLog);
        bo.add(v[3], t.tableLog);
    }
    sizes[t.sizeSlot] = bo.close();
}

// FSE, long chunks (four states, kFseLongMin symbols or more), in two
// launches. The four states' chains are independent: only the order in which
// their fields are appended couples them.
//  - kFseEncStates: four lanes per chunk, lane k running state k's chain. It
//    writes one 16-bit entry per transition (the field in bits 0-11, its
//    width in bits 12-15) at the field's index in append order, and after its
//    last transition its state's flush (tableLog bits) at index n - 4 + k. A
//    chunk's n entries are then its bitstream's fields in order.
//  - kFseEncPack: one warp per chunk appends the entries, 128 per round (four
//    per lane): a warp scan of the lanes' widths places them, they are ORed
//    into a window of words in shared memory, and the complete words go out
//    (a word only when it fits the capacity, as in the one-lane encoder);
//    then the end mark and the last bytes.
// The bytes equal kFseEnc's for the same chunk.
constexpr uint32_t kFseStChunks = 8; // chunks per CTA (one warp, four lanes each)
constexpr uint32_t kFseStSlot = kFseLaneTables + 4 * 16 * kEncRing;
static_assert(kFseStSlot % 16 == 0, "16-byte aligned rings");

__global__ void __launch_bounds__(32) kFseEncStates(const FseEncTask* __restrict__ tasks, uint32_t nbTasks)
{
    extern __shared__ __align__(16) uint8_t smemFseSt[];
    uint32_t const lane = threadIdx.x, g = lane >> 2, k = lane & 3u;
    uint32_t const ti = blockIdx.x * kFseStChunks + g;
    if (ti >= nbTasks) return; // the four lanes of a group leave together
    unsigned const gm = 0xFu << (4 * g);
    FseEncTask const t = tasks[ti];
    uint8_t* const base = smemFseSt + size_t(g) * kFseStSlot;
    uint32_t* const dnb = reinterpret_cast<uint32_t*>(base);
    int32_t* const dfs = reinterpret_cast<int32_t*>(base + 1024);
    uint16_t* const st = reinterpret_cast<uint16_t*>(base + 2048);
    const ent::FseCTable* ct = reinterpret_cast<const ent::FseCTable*>(t.ctable);
    for (uint32_t y = k; y < 256; y += 4) {
        dnb[y] = ct->deltaNbBits[y];
        dfs[y] = ct->deltaFindState[y];
    }
    uint32_t const size = 1u << t.tableLog;
    for (uint32_t u = k; u < size; u += 4) st[u] = ct->state[u];
    __syncwarp(gm);

    uint32_t const n = t.n, r = n & 3u, s0 = 4u - r;
    // the c-th symbol from the end belongs to state (s0 + c) % 4; the last
    // four symbols start the states and emit nothing
    uint32_t const cInit = (k + 4u - (s0 & 3u)) & 3u;
    uint32_t v;
    {
        uint32_t const y = t.src[n - 1 - cInit];
        uint32_t const nbOut = (dnb[y] + (1u << 15)) >> 16;
        uint32_t const x = (nbOut << 16) - dnb[y];
        v = st[(x >> nbOut) + dfs[y]];
    }
    auto trans = [&](uint32_t y) -> uint32_t {
        uint32_t const nb = (v + dnb[y]) >> 16;
        uint32_t const e = (v & ((1u << nb) - 1u)) | (nb << 12);
        v = st[(v >> nb) + dfs[y]];
        return e;
    };
    uint16_t* const fo = t.fields;
    for (uint32_t c = 4; c < 4 + r; c++) // the n % 4 single symbols, fields 0 .. r - 1
        if (((s0 + c) & 3u) == k) fo[c - 4] = uint16_t(trans(t.src[n - 1 - c]));
    // then four symbols per word (its top byte for state 0), fields
    // r + 4 t + k of step t. The next step's symbol and its two per-symbol
    // entries do not depend on the state: they load while the state's
    // next-state load is in flight, so a transition's chain is one shared
    // load and a few integer operations.
    uint32_t ip = n - 4 - r;
    if (ip) {
        BackWords bw;
        bw.start(t.src, n, ip, reinterpret_cast<uint32_t*>(base + kFseLaneTables) + k * 4 * kEncRing);
        uint32_t const shift = 24 - 8 * k;
        uint32_t y = (bw.next() >> shift) & 0xffu;
        uint32_t a = dnb[y];
        int32_t b = dfs[y];
        for (uint32_t f = r + k;; f += 4) {
            uint32_t const nb = (v + a) >> 16;
            uint32_t const e = (v & ((1u << nb) - 1u)) | (nb << 12);
            uint32_t const next = (v >> nb) + b;
            ip -= 4;
            if (ip) {
                y = (bw.next() >> shift) & 0xffu;
                a = dnb[y];
                b = dfs[y];
            }
            v = st[next];
            fo[f] = uint16_t(e);
            if (!ip) break;
        }
        asm volatile("cp.async.wait_all;" ::: "memory"); // no copy outlives the lane
    }
    fo[n - 4 + k] = uint16_t((v & (size - 1u)) | (t.tableLog << 12));
}

constexpr uint32_t kFsePackWarps = 4;

__global__ void __launch_bounds__(32 * kFsePackWarps) kFseEncPack(const FseEncTask* __restrict__ tasks,
                                                                   uint32_t nbTasks, uint32_t* __restrict__ sizes)
{
    // 64-word windows: a round places at most 128 x 12 bits (48 words) above
    // the partial word carried from the round before
    __shared__ uint32_t win[kFsePackWarps][64];
    uint32_t const lane = threadIdx.x & 31u, wi = threadIdx.x >> 5;
    uint32_t const ti = blockIdx.x * kFsePackWarps + wi;
    if (ti >= nbTasks) return; // the whole warp
    FseEncTask const t = tasks[ti];
    uint32_t* const w = win[wi];
    w[lane] = 0;
    w[lane + 32] = 0;
    __syncwarp();
    uint32_t const n = t.n, cap = t.n + t.n / 128 + 512; // the one-lane encoder's capacity
    uint8_t* const out = t.out;
    uint32_t B = 0, wb = 0; // bits placed; first word not written yet
    auto flushWords = [&](uint32_t upTo) { // words [wb, upTo) are complete
        for (uint32_t q = wb + lane; q < upTo; q += 32) {
            uint32_t const x = w[q & 63u];
            w[q & 63u] = 0;
            if (4 * q + 4 <= cap) *reinterpret_cast<uint32_t*>(out + 4 * q) = x;
        }
        __syncwarp();
        wb = upTo;
    };
    const uint2* const src = reinterpret_cast<const uint2*>(t.fields);
    uint32_t const nw = (n + 3) >> 2; // entries in groups of four
    uint2 d = lane < nw ? src[lane] : make_uint2(0u, 0u);
    for (uint32_t i0 = 0; i0 < nw; i0 += 32) {
        uint2 const cur = d;
        uint32_t const inext = i0 + 32 + lane;
        d = inext < nw ? src[inext] : make_uint2(0u, 0u); // the next round's entries, in flight
        uint32_t const j = 4 * (i0 + lane);
        uint32_t e0 = cur.x & 0xffffu, e1 = cur.x >> 16, e2 = cur.y & 0xffffu, e3 = cur.y >> 16;
        if (j + 0 >= n) e0 = 0;
        if (j + 1 >= n) e1 = 0;
        if (j + 2 >= n) e2 = 0;
        if (j + 3 >= n) e3 = 0;
        uint32_t const sum = (e0 >> 12) + (e1 >> 12) + (e2 >> 12) + (e3 >> 12);
        uint32_t inc = sum;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            uint32_t const y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        uint32_t p = B + inc - sum;
        auto place = [&](uint32_t e) {
            uint32_t const nb = e >> 12, f = e & 0xfffu;
            if (nb) {
                uint32_t const q = p >> 5, sh = p & 31u;
                atomicOr(&w[q & 63u], f << sh);
                if (sh + nb > 32) atomicOr(&w[(q + 1) & 63u], f >> (32 - sh));
            }
            p += nb;
        };
        place(e0);
        place(e1);
        place(e2);
        place(e3);
        B += __shfl_sync(0xffffffffu, inc, 31);
        __syncwarp();
        flushWords(B >> 5);
    }
    // the end mark; a word it completes goes out as a word, then the bytes
    if (lane == 0) w[(B >> 5) & 63u] |= 1u << (B & 31u);
    B += 1;
    __syncwarp();
    flushWords(B >> 5);
    uint32_t const bytes = (B + 7) >> 3;
    for (uint32_t b = 4 * wb + lane; b < bytes; b += 32)
        if (b < cap) out[b] = uint8_t(w[(b >> 2) & 63u] >> (8 * (b & 3u)));
    if (lane == 0) sizes[t.sizeSlot] = bytes;
}

// Huffman: one lane per stream (4 per chunk for 4X); symbols are appended
// from the end of the stream to its start. Each stream writes at its own
// offset of the chunk buffer; the frame assembly joins them.
constexpr uint32_t kHufEncChunks = 8;

__device__ __forceinline__ uint32_t hufStreamCap(uint32_t seg) { return ((seg + (seg >> 3) + 64) + 15) & ~15u; }

__global__ void __launch_bounds__(32) kHufEnc(const HufEncTask* __restrict__ tasks, uint32_t nbTasks,
                                              uint32_t* __restrict__ sizes)
{
    __shared__ uint16_t val[kHufEncChunks][256];
    __shared__ uint8_t nbb[kHufEncChunks][256];
    __shared__ __align__(16) uint32_t rings[4 * kHufEncChunks][4 * kEncRing];
    uint32_t const c = threadIdx.x >> 2, k = threadIdx.x & 3;
    uint32_t const ti = blockIdx.x * kHufEncChunks + c;
    bool const active = ti < nbTasks;
    HufEncTask t{};
    if (active) {
        t = tasks[ti];
        const ent::HufCTable* ct = reinterpret_cast<const ent::HufCTable*>(t.ctable);
        for (int s = k; s < 256; s += 4) {
            val[c][s] = ct->value[s];
            nbb[c][s] = ct->nbBits[s];
        }
    }
    __syncwarp();
    if (!active) return;
    uint32_t start, len;
    uint8_t* out;
    if (t.x4) {
        uint32_t const seg = (t.n + 3) / 4;
        start = seg * k;
        len = k < 3 ? seg : t.n - 3 * seg;
        out = t.out + 16 + k * hufStreamCap(seg);
    } else {
        if (k) return;
        start = 0;
        len = t.n;
        out = t.out;
    }
    BitOut bo(out, t.x4 ? hufStreamCap((t.n + 3) / 4) : t.n + t.n / 8 + 64);
    const uint8_t* const src = t.src + start;
    uint32_t i = len;
    if (i >= 4) {
        BackWords bw;
        bw.start(src, len, len, rings[threadIdx.x]);
        for (; i >= 4; i -= 4) {
            // codes of at most 11 bits (the table's values hold no bits above
            // their length): two joined per append
            uint32_t const w = bw.next();
            uint32_t const s3 = w >> 24, s2 = (w >> 16) & 0xffu, s1 = (w >> 8) & 0xffu, s0 = w & 0xffu;
            uint32_t const b3 = nbb[c][s3], b2 = nbb[c][s2], b1 = nbb[c][s1], b0 = nbb[c][s0];
            uint32_t const c3 = val[c][s3], c2 = val[c][s2], c1 = val[c][s1], c0 = val[c][s0];
            bo.add2(c3 | (c2 << b3), b3 + b2);
            bo.add2(c1 | (c0 << b1), b1 + b0);
        }
        asm volatile("cp.async.wait_all;" ::: "memory"); // no copy outlives the lane
    }
    for (; i > 0; i--) {
        uint32_t const s = src[i - 1];
        bo.add(val[c][s], nbb[c][s]);
    }
    sizes[t.sizeSlot + k] = bo.close();
}

// 16-bit chunk statistics (the counts ZS_Histogram_count16 takes,
// src/openzl/shared/histogram.c:37-80, plus first occurrences for tokenize):
// one tile of kEncTile values per CTA, global atomics per value; the maximum
// is reduced per warp first.
__global__ void __launch_bounds__(256) kHist16(const Hist16Task* __restrict__ tasks,
                                               const TileRef* __restrict__ tiles)
{
    TileRef const tr = tiles[blockIdx.x];
    Hist16Task const t = tasks[tr.task];
    uint32_t const i0 = tr.tile * kEncTile;
    uint32_t mx = 0;
    for (uint32_t k = threadIdx.x; k < kEncTile; k += 256) {
        uint32_t const i = i0 + k;
        if (i >= t.n) break;
        uint32_t const v = uint32_t(t.src[2 * i]) | (uint32_t(t.src[2 * i + 1]) << 8);
        atomicAdd(&t.count[v], 1u);
        atomicMin(&t.first[v], i);
        mx = max(mx, v);
    }
    mx = __reduce_max_sync(0xffffffffu, mx);
    if ((threadIdx.x & 31) == 0) atomicMax(t.maxOut, mx);
}

// tokenize indices: binary search of each value among the chunk's sorted
// distinct values (fewer than 256, staged in shared memory)
__global__ void __launch_bounds__(256) kTok16(const Tok16Task* __restrict__ tasks, const TileRef* __restrict__ tiles)
{
    __shared__ uint16_t keys[256];
    __shared__ uint8_t ids[256];
    TileRef const tr = tiles[blockIdx.x];
    Tok16Task const t = tasks[tr.task];
    for (uint32_t k = threadIdx.x; k < t.na; k += 256) {
        keys[k] = t.keys[k];
        ids[k] = t.ids[k];
    }
    __syncthreads();
    uint32_t const i0 = tr.tile * kEncTile;
    for (uint32_t k = threadIdx.x; k < kEncTile; k += 256) {
        uint32_t const i = i0 + k;
        if (i >= t.n) break;
        uint32_t const v = uint32_t(t.src[2 * i]) | (uint32_t(t.src[2 * i + 1]) << 8);
        uint32_t lo = 0, hi = t.na; // first key >= v
        while (lo < hi) {
            uint32_t const mid = (lo + hi) >> 1;
            if (keys[mid] < v) lo = mid + 1;
            else hi = mid;
        }
        t.idx[i] = ids[lo < t.na ? lo : 0];
    }
}

// 16-bit-symbol Huffman streams (ZS_largeHuffmanEncodeUsingCTable and its 4X
// split, src/openzl/codecs/entropy/encode_huffman_kernel.c:413-508): stream k
// of a 4X chunk holds size/4 + 1 symbols, the last one the rest; symbols are
// appended from the end of the stream to its start, then a 1 bit closes it.
// sizes[sizeSlot + k] gets the bitstream's size, sizes[sizeSlot + 4 + k] its
// whole bytes (the reference's writer fails once these reach its capacity
// less 8 bytes).
__global__ void __launch_bounds__(128) kHuf16Enc(const Huf16EncTask* __restrict__ tasks, uint32_t nbTasks,
                                                 uint32_t* __restrict__ sizes)
{
    uint32_t const g = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t const ti = g >> 2, k = g & 3;
    if (ti >= nbTasks) return;
    Huf16EncTask const t = tasks[ti];
    if (!t.x4 && k) return;
    uint32_t const chunk = t.x4 ? t.n / 4 + 1 : t.n;
    uint32_t const start = min(t.n, k * chunk);
    uint32_t const len = min(chunk, t.n - start);
    uint8_t* const out = t.out + uint64_t(k) * t.streamCap;
    BitOut bo(out + 8, t.streamCap - 8);
    const uint8_t* const src = t.src + 2ull * start;
    uint64_t bits = 1;
    for (uint32_t i = len; i > 0; i--) {
        uint32_t const v = uint32_t(src[2 * (i - 1)]) | (uint32_t(src[2 * (i - 1) + 1]) << 8);
        uint32_t const nb = __ldg(t.nbBits + v);
        bo.add(__ldg(t.code + v), nb);
        bits += nb;
    }
    uint32_t const size = bo.close();
    *reinterpret_cast<uint32_t*>(out) = len;
    *reinterpret_cast<uint32_t*>(out + 4) = size;
    sizes[t.sizeSlot + k] = size;
    sizes[t.sizeSlot + 4 + k] = uint32_t(bits / 8);
}

__global__ void __launch_bounds__(256) kRemap(const RemapTask* __restrict__ tasks, const TileRef* __restrict__ tiles)
{
    TileRef const tr = tiles[blockIdx.x];
    RemapTask const t = tasks[tr.task];
    uint64_t const e0 = uint64_t(tr.tile) * kEncTile;
    uint64_t const e1 = min(t.n, e0 + kEncTile);
    for (uint64_t i = e0 + threadIdx.x; i < e1; i += blockDim.x)
        stW(t.idx + i * t.iw, t.rankOf[ldW(t.idx + i * t.iw, t.iw)], t.iw);
}

__global__ void kPut(const PutTask* __restrict__ tasks, uint32_t n)
{
    uint32_t const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    PutTask const t = tasks[i];
    uint64_t const h = *t.hash;
    for (uint32_t b = 0; b < t.bytes; b++) t.dst[b] = uint8_t(h >> (8 * b));
}

// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// bf16 deconstruct: 4096 elements per tile
__global__ void __launch_bounds__(256) kBf16(const Bf16Task* __restrict__ tasks, const TileRef* __restrict__ tiles)
{
    TileRef const tr = tiles[blockIdx.x];
    Bf16Task const t = tasks[tr.task];
    uint64_t const e0 = uint64_t(tr.tile) * kEncTile;
    uint64_t const e1 = e0 + kEncTile < t.n ? e0 + kEncTile : t.n;
    for (uint64_t i = e0 + threadIdx.x; i < e1; i += blockDim.x) {
        uint32_t const x = uint32_t(t.src[2 * i]) | (uint32_t(t.src[2 * i + 1]) << 8);
        t.signFrac[i] = uint8_t(((x >> 15) & 1) | ((x & 0x7f) << 1));
        t.exponent[i] = uint8_t(x >> 7);
    }
}

// ---------------------------------------------------------------------------
// tokenize: open-addressing table of distinct values with their first index
__device__ __forceinline__ uint64_t tokHash(uint64_t k)
{
    // splitmix64 finalizer
    k ^= k >> 30;
    k *= 0xbf58476d1ce4e5b9ull;
    k ^= k >> 27;
    k *= 0x94d049bb133111ebull;
    return k ^ (k >> 31);
}

__global__ void __launch_bounds__(256) kTokInsert(const TokTask* __restrict__ tasks, const TileRef* __restrict__ tiles,
                                                  uint32_t* __restrict__ errors)
{
    TileRef const tr = tiles[blockIdx.x];
    TokTask const t = tasks[tr.task];
    uint64_t const e0 = uint64_t(tr.tile) * kEncTile;
    uint64_t const e1 = e0 + kEncTile < t.n ? e0 + kEncTile : t.n;
    for (uint64_t i = e0 + threadIdx.x; i < e1; i += blockDim.x) {
        uint64_t const k = ldW(t.src + i * t.w, t.w);
        uint64_t h = tokHash(k) & t.capMask;
        bool placed = false;
        for (uint64_t probe = 0; probe <= t.capMask && !placed; probe++) {
            volatile uint32_t* const st = t.state + h;
            uint32_t s = *st;
            if (s == 0) {
                if (atomicCAS(t.state + h, 0u, 1u) == 0u) {
                    t.key[h] = k;
                    __threadfence();
                    atomicExch(t.state + h, 2u);
                    atomicMin(t.first + h, uint32_t(i));
                    placed = true;
                    break;
                }
                s = *st;
            }
            // another element is writing this slot: wait (bounded) for its key
            uint32_t spins = 0;
            while (s == 1 && spins < (1u << 22)) {
                s = *st;
                spins++;
            }
            if (s != 2) break;
            __threadfence();
            if (*reinterpret_cast<volatile uint64_t*>(t.key + h) == k) {
                atomicMin(t.first + h, uint32_t(i));
                placed = true;
                break;
            }
            h = (h + 1) & t.capMask;
        }
        if (!placed) atomicAdd(errors, 1u);
    }
}

// Marks first occurrences (rank[i] = 1) and records each element's slot;
// per-tile mark counts go to tileSums.
__global__ void __launch_bounds__(256) kTokMark(const TokTask* __restrict__ tasks, const TileRef* __restrict__ tiles,
                                                uint64_t* __restrict__ tileSums, uint32_t* __restrict__ errors)
{
    __shared__ uint32_t warpCnt[8];
    TileRef const tr = tiles[blockIdx.x];
    TokTask const t = tasks[tr.task];
    uint64_t const e0 = uint64_t(tr.tile) * kEncTile;
    uint64_t const e1 = e0 + kEncTile < t.n ? e0 + kEncTile : t.n;
    uint32_t cnt = 0;
    for (uint64_t i = e0 + threadIdx.x; i < e1; i += blockDim.x) {
        uint64_t const k = ldW(t.src + i * t.w, t.w);
        uint64_t h = tokHash(k) & t.capMask;
        uint64_t probe = 0;
        while (probe <= t.capMask && !(t.state[h] == 2 && t.key[h] == k)) {
            h = (h + 1) & t.capMask;
            probe++;
        }
        if (probe > t.capMask) {
            atomicAdd(errors, 1u);
            t.slotOf[i] = 0;
            t.rank[i] = 0;
            continue;
        }
        t.slotOf[i] = uint32_t(h);
        uint32_t const m = t.first[h] == uint32_t(i) ? 1u : 0u;
        t.rank[i] = m;
        cnt += m;
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) warpCnt[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t tot = 0;
        for (int w = 0; w < 8; w++) tot += warpCnt[w];
        tileSums[blockIdx.x] = tot;
    }
}

// one warp per task: exclusive scan of its tiles' mark counts; the total is
// the alphabet size
__global__ void __launch_bounds__(256) kTokPrefix(const TokTask* __restrict__ tasks, uint32_t nbTasks,
                                                  const uint64_t* __restrict__ tileSums,
                                                  uint64_t* __restrict__ tilePrefix, uint32_t* __restrict__ counts)
{
    uint32_t const ti = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t const lane = threadIdx.x & 31;
    if (ti >= nbTasks) return;
    TokTask const t = tasks[ti];
    uint32_t const nT = uint32_t((t.n + kEncTile - 1) / kEncTile);
    uint64_t running = 0;
    for (uint32_t k0 = 0; k0 < nT; k0 += 32) {
        uint32_t const k = k0 + lane;
        uint64_t const x = k < nT ? tileSums[t.tileBase + k] : 0;
        uint64_t incl = x;
        for (int o = 1; o < 32; o <<= 1) {
            uint64_t const y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= uint32_t(o)) incl += y;
        }
        if (k < nT) tilePrefix[t.tileBase + k] = running + incl - x;
        running += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) counts[ti] = uint32_t(running);
}

// marks -> exclusive ranks, 16 consecutive elements per thread
__global__ void __launch_bounds__(256) kTokRank(const TokTask* __restrict__ tasks, const TileRef* __restrict__ tiles,
                                                const uint64_t* __restrict__ tilePrefix)
{
    __shared__ uint32_t warpTot[8];
    TileRef const tr = tiles[blockIdx.x];
    TokTask const t = tasks[tr.task];
    uint32_t const tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    uint64_t const base = uint64_t(tr.tile) * kEncTile + uint64_t(tid) * 16;
    uint32_t v[16];
    uint32_t acc = 0;
#pragma unroll
    for (int k = 0; k < 16; k++) {
        uint32_t const m = base + k < t.n ? t.rank[base + k] : 0u;
        v[k] = acc;
        acc += m;
    }
    uint32_t incl = acc;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t const y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= uint32_t(o)) incl += y;
    }
    if (lane == 31) warpTot[wid] = incl;
    __syncthreads();
    uint32_t pre = 0;
    for (uint32_t w = 0; w < wid; w++) pre += warpTot[w];
    uint32_t const add = uint32_t(tilePrefix[blockIdx.x]) + pre + (incl - acc);
#pragma unroll
    for (int k = 0; k < 16; k++)
        if (base + k < t.n) t.rank[base + k] = v[k] + add;
}

// indices and alphabet
__global__ void __launch_bounds__(256) kTokEmit(const TokTask* __restrict__ tasks, const TileRef* __restrict__ tiles)
{
    TileRef const tr = tiles[blockIdx.x];
    TokTask const t = tasks[tr.task];
    uint64_t const e0 = uint64_t(tr.tile) * kEncTile;
    uint64_t const e1 = e0 + kEncTile < t.n ? e0 + kEncTile : t.n;
    for (uint64_t i = e0 + threadIdx.x; i < e1; i += blockDim.x) {
        uint32_t const f = t.first[t.slotOf[i]];
        uint32_t const r = t.rank[f];
        stW(t.idx + i * t.iw, r, t.iw);
        if (f == uint32_t(i)) stW(t.alphabet + uint64_t(r) * t.w, ldW(t.src + i * t.w, t.w), t.w);
    }
}

cudaError_t prepareEncodeKernels()
{
    cudaError_t const e = cudaFuncSetAttribute(kFseEnc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               int(kFseEncLanes * kFseLaneBytes));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(kFseEncStates, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(kFseStChunks * kFseStSlot));
}

uint32_t hufEncStreamCap(uint32_t seg) { return ((seg + (seg >> 3) + 64) + 15) & ~15u; }

void launchEncMax(const EncNumTask* t, const TileRef* tiles, uint32_t nbTiles, unsigned long long* maxima,
                  cudaStream_t s)
{
    if (nbTiles) kEncMax<<<nbTiles, 256, 0, s>>>(t, tiles, maxima);
}
void launchEncNum(const EncNumTask* t, const TileRef* tiles, uint32_t nbTiles, cudaStream_t s)
{
    if (nbTiles) kEncNum<<<nbTiles, 128, 0, s>>>(t, tiles);
}
void launchPack(const PackTask* t, const TileRef* tiles, uint32_t nbTiles, cudaStream_t s)
{
    if (nbTiles) kPack<<<nbTiles, 128, 0, s>>>(t, tiles);
}
void launchHist(const HistTask* t, uint32_t n, uint32_t* hists, cudaStream_t s)
{
    if (n) kHist<<<n, 256, 0, s>>>(t, hists);
}
void launchFseTables(const FseTableTask* t, uint32_t n, uint32_t* sizes, uint32_t* errors, cudaStream_t s)
{
    if (n) kFseTables<<<(n + kFseTabWarps - 1) / kFseTabWarps, 32 * kFseTabWarps, 0, s>>>(t, n, sizes, errors);
}

void launchHufTables(const HufTableTask* t, uint32_t n, cudaStream_t s)
{
    if (n) kHufTables<<<(n + kHufTabWarps - 1) / kHufTabWarps, 32 * kHufTabWarps, 0, s>>>(t, n);
}

void launchFseEnc(const FseEncTask* t, uint32_t n, uint32_t* sizes, cudaStream_t s)
{
    if (n) kFseEnc<<<(n + kFseEncLanes - 1) / kFseEncLanes, 32, kFseEncLanes * kFseLaneBytes, s>>>(t, n, sizes);
}
void launchFseEncLong(const FseEncTask* t, uint32_t n, uint32_t* sizes, cudaStream_t s)
{
    if (!n) return;
    kFseEncStates<<<(n + kFseStChunks - 1) / kFseStChunks, 32, kFseStChunks * kFseStSlot, s>>>(t, n);
    kFseEncPack<<<(n + kFsePackWarps - 1) / kFsePackWarps, 32 * kFsePackWarps, 0, s>>>(t, n, sizes);
}
void launchHufEnc(const HufEncTask* t, uint32_t n, uint32_t* sizes, cudaStream_t s)
{
    if (n) kHufEnc<<<(n + kHufEncChunks - 1) / kHufEncChunks, 32, 0, s>>>(t, n, sizes);
}
void launchPut(const PutTask* t, uint32_t n, cudaStream_t s)
{
    if (n) kPut<<<(n + 127) / 128, 128, 0, s>>>(t, n);
}


void launchBf16(const Bf16Task* t, const TileRef* tiles, uint32_t nbTiles, cudaStream_t s)
{
    if (nbTiles) kBf16<<<nbTiles, 256, 0, s>>>(t, tiles);
}

void launchTokCount(const TokTask* t, uint32_t nbTasks, const TileRef* tiles, uint32_t nbTiles, uint64_t* tileSums,
                    uint64_t* tilePrefix, uint32_t* counts, uint32_t* errors, cudaStream_t s)
{
    if (!nbTiles) return;
    kTokInsert<<<nbTiles, 256, 0, s>>>(t, tiles, errors);
    kTokMark<<<nbTiles, 256, 0, s>>>(t, tiles, tileSums, errors);
    kTokPrefix<<<(nbTasks * 32 + 255) / 256, 256, 0, s>>>(t, nbTasks, tileSums, tilePrefix, counts);
    kTokRank<<<nbTiles, 256, 0, s>>>(t, tiles, tilePrefix);
}

void launchHist16(const Hist16Task* t, const TileRef* tiles, uint32_t nbTiles, cudaStream_t s)
{
    if (nbTiles) kHist16<<<nbTiles, 256, 0, s>>>(t, tiles);
}
void launchTok16(const Tok16Task* t, const TileRef* tiles, uint32_t nbTiles, cudaStream_t s)
{
    if (nbTiles) kTok16<<<nbTiles, 256, 0, s>>>(t, tiles);
}
void launchHuf16Enc(const Huf16EncTask* t, uint32_t n, uint32_t* sizes, cudaStream_t s)
{
    if (n) kHuf16Enc<<<(4 * n + 127) / 128, 128, 0, s>>>(t, n, sizes);
}

void launchRemap(const RemapTask* t, const TileRef* tiles, uint32_t nbTiles, cudaStream_t s)
{
    if (nbTiles) kRemap<<<nbTiles, 256, 0, s>>>(t, tiles);
}

void launchTokEmit(const TokTask* t, const TileRef* tiles, uint32_t nbTiles, cudaStream_t s)
{
    if (nbTiles) kTokEmit<<<nbTiles, 256, 0, s>>>(t, tiles);
}

} // namespace ozl
