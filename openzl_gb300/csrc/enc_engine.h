// Batched GPU compressor for OpenZL numeric graphs.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace ozl {

// Graph shapes of the numeric path (numbering shared with the tests' graph
// recipes): which nodes precede which entropy graph.
enum Recipe : int {
    RC_STORE = 0,
    RC_DZ_TSPLIT_FSE = 1,   // delta -> zigzag -> to-struct -> transpose split -> FSE per plane
    RC_DZ_BITPACK_HUF = 2,  // delta -> zigzag -> bitpack_int -> Huffman
    RC_D_TSPLIT_FSE = 3,    // delta -> to-struct -> transpose split -> FSE per plane
    RC_D_BITPACK_HUF = 4,   // delta -> bitpack_int -> Huffman
    RC_TOKENIZE = 5,        // tokenize (numeric, first-occurrence order): alphabet -> store, indices -> bitpack_int -> Huffman
    RC_BF16 = 6,            // bf16 deconstruct: sign|fraction -> store, exponent -> FSE
    RC_FSE = 7,
    RC_HUFFMAN = 8,
    RC_DELTA_STORE = 9,
    RC_ZIGZAG_STORE = 10,
    RC_BITPACK_STORE = 11,
    RC_TSPLIT_STORE = 12,
    RC_CONSTANT = 13,
    RC_FLATPACK = 14,
    RC_BITPACK = 15,
    RC_TOKENIZE_SORTED = 16, // tokenize with the alphabet in increasing order
    RC_ENTROPY = 17,        // ZL_GRAPH_ENTROPY: FSE or Huffman per chunk (EBM_any)
};

struct EncFrameSpec {
    const uint8_t* dIn; // device input
    uint64_t n;         // elements
    uint32_t w;         // element width (serial inputs: 1)
    bool serial;        // serial input (else numeric)
    int recipe;
};

class EncodeBatch {
  public:
    EncodeBatch();
    ~EncodeBatch();
    // Compresses every frame into dOut[i] (capacity caps[i]); frame sizes go
    // to `sizes`. Runs on `stream` and synchronizes it. Returns 0 or a ZL code.
    int compress(const std::vector<EncFrameSpec>& frames, uint8_t* const* dOut, const size_t* caps,
                 bool checksums, cudaStream_t stream, std::vector<size_t>& sizes, std::string& err);
    size_t lastLaunches() const { return launches_; }
    // Wall-clock milliseconds of the last compress() call's phases A-G (a
    // phase that ends in a stream synchronize includes its device work).
    static constexpr int kPhases = 7;
    const double* lastPhaseMs() const { return phaseMs_; }
    // host threads of the parallel host phases (0: the machine's, at most 16)
    void setHostThreads(unsigned n) { hostThreads_ = n; }

    struct Impl;

  private:
    Impl* impl_;
    size_t launches_ = 0;
    double phaseMs_[kPhases] = {};
    unsigned hostThreads_ = 0;
};

// Worst-case frame size for `srcBytes` of input (ZL_compressBound-style).
size_t encodeBound(size_t srcBytes);

} // namespace ozl
