// Per-lane stream ring in shared memory, shared by the decoders (backward
// bitstreams) and the encoders (sources read from their end).
#pragma once
#include <cstdint>

namespace ozl {

// Chunks are the 16-byte-aligned blocks of global memory that hold at least
// one byte of the stream (such a block never crosses a page), counted from
// the block holding the stream's first byte. Positions are bit indices above
// bit 0 of that block.
template <int RING, int AHEAD>
struct StreamRing {
    static_assert((RING & (RING - 1)) == 0 && AHEAD + 1 <= RING, "ring shape");
    const uint8_t* g16;  // 16-byte aligned block holding the stream's first byte
    uint32_t* ring;      // RING * 4 words of shared memory, 16-byte aligned
    int32_t low;         // lowest chunk whose words have been read

    __device__ __forceinline__ void issue(int32_t m)
    {
        if (m >= 0) {
            uint32_t const dst = uint32_t(__cvta_generic_to_shared(ring + 4 * (m & (RING - 1))));
            asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(g16 + 16 * size_t(m)) : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    // Starts the ring for a stream whose top bit is at position pos (> 0).
    __device__ __forceinline__ void start(int32_t pos)
    {
        int32_t const mt = (pos - 1) >> 7;
        for (int32_t m = mt; m >= mt - AHEAD; m--) issue(m);
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        low = mt;
    }
    // Word k (descending order after start(); k may be negative: 0).
    __device__ __forceinline__ uint32_t word(int32_t k)
    {
        if (k < 0) return 0u;
        int32_t const m = k >> 2;
        if (m < low) {
            low = m;
            issue(m - AHEAD);
            asm volatile("cp.async.wait_group %0;" ::"n"(AHEAD) : "memory");
        }
        return ring[k & (4 * RING - 1)];
    }
};

} // namespace ozl
