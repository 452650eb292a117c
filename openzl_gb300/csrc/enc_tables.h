// Host-side entropy decisions and coding tables for the GPU encoder.
//
// These are the small, per-chunk computations between the GPU histogram pass
// and the GPU bitstream pass: OpenZL's chunk codec choice
// (src/openzl/codecs/entropy/encode_entropy_binding.c:602-762) from 256-bin
// histograms, FSE normalization and encoding tables
// (src/openzl/fse/compress/fse_compress.c), and Huffman code lengths
// (src/openzl/fse/compress/huf_compress.c). Their results must equal the
// reference's bit for bit, so the arithmetic is restated exactly, including
// the one double-precision entropy estimate (computed without FMA).
#pragma once
#include <cstddef>
#include <cstdint>

namespace ozl {
namespace ent {

enum ChunkCodec : int {
    CC_STORE = 0,
    CC_CONSTANT,
    CC_FLATPACK,
    CC_BITPACK,
    CC_FSE,
    CC_HUF,
    CC_TOK16, // 16-bit chunk: tokenize (alphabet + 8-bit indices)
    CC_HUF16, // 16-bit chunk: huffman_struct_v2
};

struct Histo {
    uint32_t count[256];
    uint64_t n;
    unsigned maxSym;
    unsigned card;
    void finish(); // fills maxSym and card from count
};

// Entropy backend modes: the FSE graph, the Huffman graph, the entropy graph.
enum : int { EM_FSE = 0, EM_HUF = 1, EM_ANY = 2 };

// Chunk codec choice for a serial chunk under a backend mode
// (entropyCompressChunk, encode_entropy_binding.c:602-762).
ChunkCodec chooseCodec(const Histo& h, int mode);
// The estimates it compares (DataStatsU8, src/openzl/shared/data_stats.c):
// the entropy in bits per symbol (ZL_calculateEntropyU8), the fast Huffman
// size from it (DataStatsU8_estimateHuffmanSizeFast), and the flat-packed
// and bit-packed sizes.
double entropyEstimate(const uint32_t* count, uint64_t total);
uint64_t hufSizeFast(double entropy, uint64_t n);
uint64_t flatpackedSize(const Histo& h);
uint64_t bitpackedSize(const Histo& h);

// FSE: table log, normalized counts, encoding tables.
unsigned fseTableLog(unsigned maxTableLog, uint64_t srcSize, unsigned maxSym, unsigned minus);
bool fseNormalize(int16_t* norm, unsigned tableLog, const uint32_t* count, uint64_t total, unsigned maxSym);
size_t fseWriteNCount(uint8_t* out, const int16_t* norm, unsigned maxSym, unsigned tableLog);

// Device-ready FSE encoding table: next-state table sorted by symbol, and
// per-symbol (deltaNbBits, deltaFindState).
struct FseCTable {
    uint16_t tableLog;
    uint16_t maxSym;
    uint32_t deltaNbBits[256];
    int32_t deltaFindState[256];
    uint16_t state[2048];
};
void fseBuildCTable(FseCTable& ct, const int16_t* norm, unsigned maxSym, unsigned tableLog);

// Huffman: code lengths and canonical codes for a histogram.
struct HufCTable {
    uint16_t value[256];
    uint8_t nbBits[256];
    uint32_t tableLog;
};
unsigned hufBuild(HufCTable& ct, const uint32_t* count, unsigned maxSym, unsigned maxNbBits);

// Chunk codec choice for a 16-bit struct chunk (the 2-byte branch of
// entropyCompressChunk, encode_entropy_binding.c:612-681), whatever the
// backend mode: CC_CONSTANT, CC_BITPACK (read as little-endian numbers),
// CC_STORE, CC_TOK16 or CC_HUF16. `count` holds values 0..maxSym.
ChunkCodec chooseCodec16(const uint32_t* count, unsigned maxSym, uint64_t n, unsigned card);

// 16-bit-symbol Huffman code (ZS_largeHuffmanBuildCTable with maxNbBits 0,
// src/openzl/codecs/entropy/encode_huffman_kernel.c:34-374): code and length
// of each value 0..maxSym. Returns the table log, or -1.
int huf16Build(uint16_t* code, uint8_t* nbBits, const uint32_t* count, unsigned maxSym);

int nextPow2Bits(uint64_t v);

} // namespace ent
} // namespace ozl
