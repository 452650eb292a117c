// Host-side decode planner: turns OpenZL frames into device task lists.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "dec_tasks.h"

namespace ozl {

// Kernel families, in the order they launch within one dependency level.
enum Kind : int {
    KIND_COPY = 0,
    KIND_CONST,
    KIND_FSE,
    KIND_HUF,
    KIND_FLATPACK,
    KIND_TOKENIZE,
    KIND_FLOATDEC,
    KIND_TRANSPOSE,
    KIND_NUMPIPE,
    KIND_HASH,
    KIND_HUF16, // launched after KIND_HUF within a level
    KIND_WIDEN, // string lengths to 4 bytes
    KIND_COUNT
};

struct Launch {
    int kind;
    int level;
    size_t taskOff;   // byte offset of the task array in the descriptor pool
    uint32_t nbTasks;
    size_t tileOff;   // byte offset of the TileRef array (tiled kinds)
    uint32_t nbTiles;
    size_t statusOff; // scratch offset of look-back status (NUMPIPE with delta)
    size_t statusBytes;
    bool needsScan;
    uint32_t param0;  // kind-specific launch shape (FSE: max table log)
    uint32_t tune;    // chunks per CTA chosen by the autotuner (FSE, Huffman); 0 = default
    uint64_t algoBytes; // bytes the launch must read plus write (roofline numerator)
};

// Where a stream's bytes live.
enum LocKind : int { L_NONE = 0, L_FRAME, L_ARENA, L_OUT, L_PARAM, L_SUB, L_ALIAS };

struct PlanStream {
    int type = 0;
    uint32_t w = 1;
    uint64_t n = 0;
    int producer = -1; // node index, -1 = stored
    int loc = L_NONE;
    int frame = -1;    // for L_FRAME / L_OUT
    int parent = -1;   // for L_SUB / L_ALIAS
    uint64_t off = 0;  // offset within the location
    const uint8_t* host = nullptr; // host copy of the content, when known at plan time
    int lens = -1;     // string streams: the stream of 4-byte string lengths
    uint64_t bytes() const { return n * w; }
};

struct PlanNode {
    uint32_t id = 0;          // standard transform ID
    int frame = -1;
    const uint8_t* hdr = nullptr;
    size_t hsz = 0;
    std::vector<int> ins;     // streams, in the decoder's own input order
    int out = -1;
    bool dead = false;        // absorbed by a fused consumer, or a no-op view
    int level = 0;
    // fused numeric pipeline parameters
    uint8_t srcMode = SRC_PLAIN, nbBits = 0, zigzag = 0, delta = 0;
    uint64_t paramOff = 0;    // FSE: normalized counts in the parameter block
};

enum HashWhere : uint8_t { HW_FRAME = 0, HW_OUTPUT = 1, HW_ARENA = 2 };

struct PlanHash {
    int frame;
    uint8_t where;      // HW_*: the frame (compressed), its output (content), the arena (gathered outputs)
    uint64_t off, len;
    uint32_t expected;
    uint32_t err;
    bool low8;          // frame-header checksum: compare the low 8 bits only
};

// Output bytes that a frame stores verbatim (no decoder regenerates them).
struct PlanCopy {
    int frame;
    uint64_t frameOff, outOff, bytes;
};

// String lengths narrower than 4 bytes, widened into an output's lengths.
struct PlanWiden {
    int stream;
    int frame;
    uint64_t outOff;
};

// One output's block gathered into the arena, so that the content checksum
// of a multi-output block hashes contiguous bytes.
struct PlanGather {
    int frame;
    uint64_t outOff, arenaOff, bytes;
};

struct FramePlan {
    uint64_t decodedSize = 0;  // destination bytes: every output, each at a 16-byte-aligned offset
    uint64_t frameBytes = 0;   // compressed size, with the end-of-frame byte (v21+)
    int outType = 0;           // output 0
    uint32_t outWidth = 1;
    std::vector<uint64_t> outOffs, outSizes; // per output: offset in the destination, bytes
    std::vector<int> outTypes;
    std::vector<uint32_t> outWidths;
    std::vector<uint64_t> lensOffs;          // string outputs: offset of their 4-byte lengths
    std::vector<uint64_t> nbStrings;         // string outputs: strings in the frame header
    std::vector<uint64_t> stringsDone;       // string outputs: strings placed so far
};

// Frame-header fields shared by the planner and the frame-information calls.
struct FrameHeader {
    unsigned version = 0;
    bool hasContentCk = false;    // v21+; older frames carry the flags per block
    bool hasCompressedCk = false;
    std::vector<int> types;       // TY_* per output
    std::vector<uint64_t> sizes;  // decompressed bytes per output (strings: content bytes)
    std::vector<uint64_t> nbStrings; // string outputs: number of strings (0 for other types)
    int outType = 0;              // output 0
    uint64_t outSize = 0;
    size_t end = 0;               // first byte after the header
    bool hdrCk = false;           // v21+: header checksum byte at end - 1
};

// Parses the frame header (src/openzl/decompress/decode_frameheader.c:58-190,
// 270-370). Format versions 8..23, up to 2048 outputs; string outputs from
// format version 21 (older headers carry no string counts). Returns 0 or a
// ZL error code: formatVersion_unsupported (60), srcSize_tooSmall (3),
// temporaryLibraryLimitation (81) for unknown sizes or string outputs before
// v21, corruption (12).
int parseFrameHeader(const uint8_t* src, size_t size, FrameHeader& h, std::string& err);

// Where the batch API writes a frame's outputs in its destination: one after
// another, each at a 16-byte-aligned offset; a string output's 4-byte lengths
// follow its content at the next 16-byte-aligned offset (`lensOffsets`, 0 for
// other types). Returns the bytes needed.
uint64_t frameOutputLayout(const FrameHeader& h, std::vector<uint64_t>& offsets, std::vector<uint64_t>* lensOffsets = nullptr);

class DecodePlan {
  public:
    // Parses and plans. Returns 0 or a ZL error code; `err` gets a message.
    int build(size_t nbFrames, const uint8_t* const* hFrames, const size_t* frameSizes,
              const size_t* dstCapacities, bool checkContent, bool checkCompressed,
              std::string& err);
    // The same plan built on up to `threads` host threads: runs of frames
    // planned apart, then joined with their stream, node, frame, arena and
    // parameter references moved to the joined positions. Arena blocks are
    // 64-byte multiples and parameter blocks start 16-byte aligned, so the
    // joined plan equals the serial one. Small batches, or any error (for its
    // exact message), take the serial build.
    int buildParallel(size_t nbFrames, const uint8_t* const* hFrames, const size_t* frameSizes,
                      const size_t* dstCapacities, bool checkContent, bool checkCompressed, std::string& err,
                      unsigned threads);

    std::vector<FramePlan> frames;
    std::vector<PlanStream> streams;
    std::vector<PlanNode> nodes;
    std::vector<PlanHash> hashes;
    std::vector<PlanCopy> directCopies;
    std::vector<PlanGather> gathers;
    std::vector<PlanWiden> widens;
    std::vector<uint8_t> params;  // host-decoded small streams (FSE normalized counts)
    uint64_t arenaBytes = 0;
    uint64_t totalOut = 0;

  private:
    int planFrame(int f, const uint8_t* src, size_t size, size_t dstCap, bool ckContent,
                  bool ckCompressed, std::string& err);
    // `produced` holds each output's bytes so far; the block adds its own
    int planBlock(int f, unsigned version, const uint8_t* src, size_t size, size_t start, size_t* consumed,
                  bool hasContentCk, bool hasCompressedCk, bool ckContent, bool ckCompressed,
                  std::vector<uint64_t>& produced, std::string& err);
};

// Resolved, device-ready plan: task pools and launch list.
struct DeviceLayout {
    std::vector<uint8_t> pool;     // task descriptors, tile lists, pointer arrays
    std::vector<Launch> launches;
    uint64_t arenaBytes = 0;       // intermediate streams
    uint64_t scratchBytes = 0;     // look-back status + hash block sums
    uint64_t paramBytes = 0;
};

// Produces task descriptors with absolute device addresses.
// With `frameMask`, only the work of the frames it marks is laid out (the
// plan's arena and parameter placements are shared by all such parts).
int layoutPlan(const DecodePlan& plan, const uint8_t* const* dFrames, uint8_t* const* dOuts,
               uint8_t* dArena, uint8_t* dParams, uint8_t* dScratch, uint8_t* dPool,
               DeviceLayout& out, std::string& err, const std::vector<char>* frameMask = nullptr);

} // namespace ozl
