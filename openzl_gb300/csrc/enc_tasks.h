// Device task descriptors of the GPU encoder (built by enc_engine.cpp,
// consumed by encode_kernels.cu).
#pragma once
#include <cstdint>

#include "dec_tasks.h"

namespace ozl {

// Numeric front end of a frame: values v[i] of width w, optionally delta
// (v[i] - v[i-1], the first value goes to the codec header) and zigzag, then
// one of: planes (byte-split), LSB-first bit packing, or plain numeric.
enum EncOut : uint8_t {
    EOUT_PLAIN = 0,
    EOUT_PLANES = 1,
    EOUT_BITPACK = 2,
};

struct EncNumTask {
    const uint8_t* src;  // input elements (width w)
    uint8_t* out;        // PLAIN / BITPACK output, or plane 0 for PLANES
    uint64_t n;          // output elements (input elements - 1 with delta)
    uint64_t planeStride;// PLANES: byte distance between consecutive planes
    uint32_t w;
    uint8_t delta, zigzag, mode, nbBits;
    uint32_t maxSlot;    // index of this task's max accumulator
    uint32_t tileBase;
};

// 256-bin histogram of a byte chunk.
struct HistTask {
    const uint8_t* src;
    uint32_t n;
    uint32_t outIndex;   // histogram slot
};

// FSE coding tables of one chunk built on the device from its histogram:
// normalized counts (the chunk's numeric stream), their header (fse_ncount)
// and the encoding table that kFseEnc reads.
struct FseTableTask {
    const uint32_t* hist;    // 256 counts
    uint64_t n;              // symbols in the chunk
    uint8_t* ctable;         // ent::FseCTable
    int16_t* norm;           // maxSym + 1 normalized counts
    uint8_t* ncount;         // header, at most 520 bytes
    uint32_t maxSym;
    uint32_t tableLog;
    uint32_t sizeSlot;       // where the header's size is written
    uint32_t pad;
};

// Huffman code lengths and codes of one chunk built on the device from its
// histogram, and the chunk's weights stream (tableLog + 1 - length, 0 for
// absent symbols).
struct HufTableTask {
    const uint32_t* hist;    // 256 counts
    uint8_t* ctable;         // ent::HufCTable
    uint8_t* weights;        // maxSym + 1 weights
    uint32_t maxSym;
    uint32_t maxNbBits;      // the chunk's table log bound
};

struct FseEncTask {
    const uint8_t* src;
    uint8_t* out;            // capacity: n + n/128 + 512 bytes
    const uint8_t* ctable;   // ent::FseCTable on the device
    uint32_t n;
    uint32_t sizeSlot;       // where the bitstream size is written
    uint32_t nbStates;
    uint32_t tableLog;
    uint16_t* fields;        // chunks of kFseLongMin symbols or more: fseFieldBytes(n) of scratch
};
// Chunks of four states and at least this many symbols encode with one lane
// per state (kFseEncStates, then kFseEncPack); shorter ones one lane each.
constexpr uint32_t kFseLongMin = 4096;
// scratch of a long chunk: one 16-bit entry per field, padded to 8 bytes
inline size_t fseFieldBytes(uint32_t n) { return 2 * ((size_t(n) + 3) & ~size_t(3)) + 16; }

struct HufEncTask {
    const uint8_t* src;
    uint8_t* out;            // capacity: n + n/256 + 1024 bytes
    const uint8_t* ctable;   // ent::HufCTable on the device
    uint32_t n;
    uint32_t sizeSlot;
    uint32_t x4;
};

// Serial bit packing (flatpack indices when `map` is set): element i takes
// nbBits at bit i*nbBits; flatpack appends a terminating 1 bit.
struct PackTask {
    const uint8_t* src;
    uint8_t* out;
    const uint8_t* map;      // flatpack: symbol -> index (256 bytes), or null
    uint64_t n;
    uint32_t nbBits;
    uint32_t tileBase;
};

struct PutTask {
    uint8_t* dst;            // frame byte where a checksum lands
    const uint64_t* hash;    // computed hash
    uint32_t bytes;          // 4 (low 32 bits) or 1 (low 8 bits)
};

// bf16 deconstruct (encode_float_deconstruct_kernel.c): per element, the
// sign|fraction byte (sign in bit 0, the 7 fraction bits above it) and the
// exponent byte.
struct Bf16Task {
    const uint8_t* src;
    uint8_t* signFrac;
    uint8_t* exponent;
    uint64_t n;
};

// Tokenize with the alphabet in first-occurrence order: a per-frame
// open-addressing table keeps each distinct value's first index; marking the
// elements that are first occurrences and prefix-summing the marks gives each
// value its alphabet rank.
struct TokTask {
    const uint8_t* src;   // n elements of width w
    uint64_t n;
    uint32_t w;
    uint32_t iw;          // index width (1, 2 or 4), known after counting
    uint64_t capMask;     // table capacity - 1 (a power of two)
    uint32_t* state;      // 0 empty, 1 being written, 2 ready
    uint64_t* key;
    uint32_t* first;      // first element index of the slot's value
    uint32_t* slotOf;     // per element: the slot of its value
    uint32_t* rank;       // per element: marks, then exclusive rank of the marks
    uint8_t* alphabet;    // distinct values, width w
    uint8_t* idx;         // per element: alphabet index, width iw
    uint32_t tileBase;    // first tile of this task in its launch
};

// 16-bit chunk statistics: per 2-byte value its count and the index of its
// first occurrence (initialised to 0xffffffff), and the largest value.
struct Hist16Task {
    const uint8_t* src;   // n little-endian 2-byte values
    uint32_t n;
    uint32_t* count;      // 65536 slots
    uint32_t* first;      // 65536 slots
    uint32_t* maxOut;     // one word, initialised to 0
};

// Tokenize indices of a 16-bit chunk with fewer than 256 distinct values:
// `keys` holds the values in increasing order and `ids` their alphabet index.
struct Tok16Task {
    const uint8_t* src;
    uint8_t* idx;
    const uint16_t* keys;
    const uint8_t* ids;
    uint32_t n, na;
};

// 16-bit-symbol Huffman (huffman_struct_v2) streams of one chunk: stream k
// (k < 4 when x4, else 0) is written at out + k * streamCap as LE32 symbol
// count, LE32 bitstream size, bitstream; its bitstream size goes to
// sizes[sizeSlot + k].
struct Huf16EncTask {
    const uint8_t* src;
    uint8_t* out;
    const uint16_t* code;   // per value 0..maxSym
    const uint8_t* nbBits;
    uint32_t n, streamCap, sizeSlot, x4;
};

// Sorted tokenize: indices in first-occurrence order renumbered to the
// sorted alphabet's order, idx[i] = rankOf[idx[i]].
struct RemapTask {
    uint8_t* idx;
    const uint32_t* rankOf;
    uint64_t n;
    uint32_t iw;
};

constexpr uint32_t kEncTile = 4096; // elements per numeric/pack tile (32 per thread)

} // namespace ozl
