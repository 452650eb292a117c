// Device task descriptors of the GPU decoder. The host planner
// (dec_plan.cpp) fills these from frame headers; the kernels (decode.cu)
// consume them. All pointers are device pointers resolved at plan time.
#pragma once
#include <cstddef>
#include <cstdint>

namespace ozl {

// Error codes a kernel records in the batch status word (first error wins).
enum DevError : uint32_t {
    DERR_NONE = 0,
    DERR_CORRUPTION = 12,
    DERR_COMPRESSED_CK = 13,
    DERR_CONTENT_CK = 14,
    DERR_TIMEOUT = 80,
};

// Fused numeric pipeline: source -> [zigzag] -> [delta prefix sum] -> out.
// Covers delta/zigzag/transpose-split/bitpack decoders and the chains of them
// that OpenZL numeric graphs produce.
enum NumSrc : uint8_t {
    SRC_PLAIN = 0,   // numeric elements of width w at `src`
    SRC_PLANES = 1,  // w byte planes; element i byte b = planes[b][i]
    SRC_BITPACK = 2, // LSB-first fields of nbBits at `src`
};

struct NumPipeTask {
    uint8_t* out;
    const uint8_t* src;
    const uint8_t* const* planes; // SRC_PLANES: device array of w pointers
    uint64_t n;                   // output elements
    uint64_t first;               // delta: first value (from the codec header)
    uint32_t w;                   // element width: 1, 2, 4 or 8
    uint8_t srcMode;
    uint8_t nbBits;
    uint8_t zigzag;
    uint8_t delta;                // source holds n-1 elements when set
    uint32_t tileBase;            // first tile index of this task in its launch
    uint32_t nbTiles;
    // Content checksum fused into the output pass: when set, the XXH3 block
    // sums (8 lanes per 1 KiB block, as kHashBlocks writes them) of the first
    // hashBlocks blocks of `out` are written here.
    uint64_t* blockSums;
    uint32_t hashBlocks;
};

// Generic transpose-split for arbitrary widths: out[i*W + b] = planes[b][i].
struct TransposeTask {
    uint8_t* out;
    const uint8_t* const* planes;
    uint64_t n;
    uint32_t W;
    uint32_t tileBase;
};

struct CopyTask {
    uint8_t* dst;
    const uint8_t* src;
    uint64_t bytes;
    uint32_t tileBase;
};

struct ConstTask {
    uint8_t* out;
    const uint8_t* value; // one element of width w
    uint64_t n;
    uint32_t w;
    uint32_t tileBase;
};

struct FseTask {
    uint8_t* out;
    const uint8_t* bits;
    const int16_t* norm;  // normalized counts (nbSym entries)
    uint32_t bitsSize;
    uint32_t dstSize;
    uint16_t nbSym;
    uint8_t nbStates;
    uint8_t tableLog;
};

// 16-bit-symbol Huffman (huffman_struct_v2): one or four backward streams
// whose byte ranges and symbol counts the planner read from the stored
// bitstream; `sorted` is scratch for the symbols ranked by (weight, value).
struct Huf16Task {
    uint8_t* out;              // dstSize 16-bit symbols
    const uint8_t* weights;    // nbWeights bytes
    uint16_t* sorted;          // nbWeights entries of scratch
    const uint8_t* stream[4];
    uint32_t streamSize[4];
    uint32_t count[4];         // symbols per stream
    uint32_t dstOff[4];        // first symbol of each stream
    uint32_t nbWeights;
    uint32_t nbStreams;
};

struct HufTask {
    uint8_t* out;
    const uint8_t* bits;
    const uint8_t* weights;
    uint32_t bitsSize;
    uint32_t dstSize;
    uint16_t nbWeights;
    uint8_t x4;
};

// String lengths of width w (1, 2 or 8 bytes) to 4-byte lengths; a value
// above 2^32 - 1 is corruption.
struct WidenTask {
    const uint8_t* src;
    uint32_t* dst;
    uint64_t n;
    uint32_t w;
    uint32_t tileBase;
};

struct TokenizeTask {
    uint8_t* out;
    const uint8_t* alphabet;
    const uint8_t* idx;
    uint64_t n;
    uint32_t alphabetSize;
    uint32_t w;   // alphabet element width
    uint32_t iw;  // index width
    uint32_t tileBase;
};

struct FloatDecTask {
    uint8_t* out;
    const uint8_t* signFrac;
    const uint8_t* exponent;
    uint64_t n;
    uint32_t eltType; // 0 float32, 1 bfloat16, 2 float16
    uint32_t tileBase;
};

struct FlatpackTask {
    uint8_t* out;
    const uint8_t* alphabet;
    const uint8_t* packed;
    uint64_t n;
    uint32_t alphabetSize;
    uint32_t nbBits;
    uint32_t tileBase;
};

// XXH3-64 low-32 check of a contiguous region.
struct HashTask {
    const uint8_t* data;
    uint64_t len;
    uint64_t* blockSums;   // scratch: 8 lanes per 1 KiB block
    uint32_t expected;
    uint32_t errCode;      // DERR_CONTENT_CK or DERR_COMPRESSED_CK
    uint32_t blockBase;    // first block index in the launch's block list
    uint32_t nbBlocks;     // full 1 KiB blocks accumulated in phase 1
    uint32_t low8;         // compare the low 8 bits only (frame-header checksum)
    uint32_t aligned8;     // data pointer is 8-byte aligned
    uint64_t* hashOut;     // optional: receives the full 64-bit hash
};

// One tile of a tiled launch: task index and tile index within the task.
struct TileRef {
    uint32_t task;
    uint32_t tile;
};

constexpr uint32_t kTileElems = 4096;     // element tile of the element-wise kernels
constexpr uint32_t kNumTileBytes = 16384; // numeric-pipeline tile: kNumTileBytes / w output elements
constexpr uint32_t kTileBytes = 65536;    // byte-oriented tile
constexpr uint32_t kHashBlock = 1024;     // XXH3 block length

} // namespace ozl
