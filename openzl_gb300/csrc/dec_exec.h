// Kernel dispatch for a laid-out decode plan.
#pragma once
#include <cuda_runtime.h>

#include "dec_plan.h"

namespace ozl {

// Enqueues every launch of `layout` on `stream`. `dPool` holds the uploaded
// descriptor pool, `dScratch` the look-back status and hash block sums,
// `dStatus` the batch error word. Returns the number of kernels launched, or
// a negative value if a launch could not be issued.
long runLaunches(const DeviceLayout& layout, uint8_t* dPool, uint8_t* dScratch, uint32_t* dStatus,
                 cudaStream_t stream);

// Applies the shared-memory carve-out attributes the entropy kernels need.
// Call once per device before the first launch (and before graph capture).
cudaError_t prepareKernels();
// Launch::tune of an FSE launch: streams per CTA in the low byte; this flag
// selects the kernel with one lane per decoder state (kFse4) instead of one
// lane per stream (kFse).
constexpr uint32_t kTuneFseLanePerState = 0x100;

// Launch shapes the autotuner may try for a launch (chunks per CTA); 0 if none.
uint32_t tuneCandidates(const Launch& l, uint32_t* out, uint32_t cap);

// Enqueues launch `i` of `layout` alone (the building block of runLaunches).
// Returns the number of kernels it issued, or a negative value on failure.
long runOneLaunch(const DeviceLayout& layout, size_t i, uint8_t* dPool, uint8_t* dScratch, uint32_t* dStatus,
                  cudaStream_t stream);

// Launch helpers shared with the encoder.
void launchCopy(const CopyTask* tasks, const TileRef* tiles, uint32_t nbTiles, cudaStream_t s);
void launchHash(const HashTask* tasks, uint32_t nbTasks, const TileRef* blocks, uint32_t nbBlocks,
                uint32_t* status, cudaStream_t s);

// XXH3-64 of `len` device bytes at `data`; the hash lands in *dHashOut.
// Needs 256 + 72 * ceil(len / 1 KiB) bytes of device scratch. Synchronizes `s`.
cudaError_t xxh3Device(const uint8_t* data, uint64_t len, uint64_t* dHashOut, uint8_t* dScratch,
                       uint64_t scratchBytes, cudaStream_t s);

} // namespace ozl
