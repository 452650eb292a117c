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

struct FseEncTask {
    const uint8_t* src;
    uint8_t* out;            // capacity: n + n/128 + 512 bytes
    const uint8_t* ctable;   // ent::FseCTable on the device
    uint32_t n;
    uint32_t sizeSlot;       // where the bitstream size is written
    uint32_t nbStates;
    uint32_t tableLog;
};

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

constexpr uint32_t kEncTile = 4096; // elements per numeric/pack tile (32 per thread)

} // namespace ozl
