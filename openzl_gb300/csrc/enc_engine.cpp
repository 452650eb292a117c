// Batched GPU compressor: host orchestration.
//
// One compress() call encodes many frames in a fixed sequence of phases, each
// one batched across all frames:
//   A. front end on the GPU: per-frame maximum (for bit packing), then
//      delta/zigzag with byte planes, bit packing or plain output; content
//      checksums of the inputs;
//   B. graph discovery on the host: which streams enter an entropy graph and
//      how they are chunked (sizes only);
//   C. 256-bin histograms of every chunk on the GPU;
//   D. per-chunk codec choice and coding tables on the host (the small,
//      exactly-specified arithmetic of the reference);
//   E. entropy bitstreams (FSE, Huffman, bit packing, flatpack) on the GPU;
//   F. graph replay on the host, in the reference's node-creation order
//      (src/openzl/compress/cctx.c:700-1230), giving each frame's decoder map,
//      codec headers and stored streams (encode_frameheader.c:441-834);
//   G. frame assembly and block/header checksums on the GPU.
#include "enc_engine.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstddef>
#include <cstring>
#include <memory>
#include <mutex>
#include <thread>

#include "dec_exec.h"
#include "enc_exec.h"
#include "enc_tables.h"
#include "enc_tasks.h"

namespace ozl {

namespace {

enum : int { T_SERIAL = 1, T_STRUCT = 2, T_NUMERIC = 4 };
enum : uint32_t {
    TR_DELTA = 1, TR_ZIGZAG = 3, TR_TSPLIT = 4, TR_CONV_STRUCT_TO_SERIAL = 6, TR_CONV_NUM_TO_STRUCT = 8,
    TR_CONV_NUM_TO_SERIAL = 10, TR_BITPACK_SERIAL = 27, TR_BITPACK_INT = 28, TR_FLATPACK = 29, TR_SPLITN = 40,
    TR_CONST_SERIAL = 44, TR_FSE = 49, TR_HUF = 50, TR_NCOUNT = 52, TR_FLOAT_DECONSTRUCT = 33,
    TR_TOKENIZE_NUMERIC = 37, TR_CONV_STRUCT_TO_NUM = 7, TR_TOKENIZE_FIXED = 36, TR_CONST_FIXED = 45,
    TR_SPLITN_STRUCT = 47, TR_HUF16 = 51,
};
constexpr uint64_t kMinStream = 10;   // ZL_MINSTREAMSIZE_DEFAULT
constexpr uint64_t kChunk = 1 << 15;  // entropy chunk size
constexpr uint64_t kMinChunking = 100000;

struct DevBuf {
    uint8_t* p = nullptr;
    size_t cap = 0;
    ~DevBuf()
    {
        if (p) cudaFree(p);
    }
    bool reserve(size_t bytes)
    {
        bytes += 256;
        if (bytes <= cap) return true;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return false;
        cap = bytes;
        return true;
    }
    uint8_t* data() const { return p + 64; }
};

// bump allocator over a size pass / real pass
struct Bump {
    uint8_t* base = nullptr;
    size_t used = 0;
    uint8_t* take(size_t bytes, size_t align = 64)
    {
        used = (used + align - 1) & ~(align - 1);
        uint8_t* r = base ? base + used : nullptr;
        used += bytes;
        return r;
    }
};

struct Piece {
    const uint8_t* dev = nullptr;
    const uint8_t* host = nullptr;
    uint64_t bytes = 0;
};

enum : int { M_FSE = 0, M_HUF, M_CONSTANT, M_FLATPACK, M_BITPACK, M_ANY };

// Discovery's record of one entropy job.
struct JobSeed {
    const uint8_t* dsrc;
    uint64_t n;
    int mode;
    bool wide;
    unsigned width; // element width in bytes
};

struct Job {
    // arrays without initializers are written before they are read, so
    // sizing the job list does not zero them
    Job() {}
    Job(Job&&) = default;
    Job& operator=(Job&&) = default;
    const uint8_t* dsrc = nullptr;    // device content
    std::vector<uint8_t> hsrc;        // host content (Huffman weights)
    const uint8_t* dstaged = nullptr; // device copy of hsrc
    uint64_t n = 0;
    int mode = M_FSE;
    ent::Histo hist{};
    int codec = ent::CC_STORE;
    // FSE: tables built on the device (kFseTables) from the histogram
    unsigned tl = 0, nbStates = 2;
    uint8_t* dNorm = nullptr;   // normalized counts (numeric i16)
    uint8_t* dNcount = nullptr; // their header
    uint32_t ncountSlot = 0;
    size_t ncountSize = 0;
    // Huffman: code lengths and codes built on the device (kHufTables), the
    // weights brought back for the nested FSE graph and the frame
    std::vector<uint8_t> weights;
    int weightsJob = -1;
    bool x4 = false;
    uint8_t jump[6];
    // bit packing / flatpack
    unsigned packBits = 0;
    uint64_t packBytes = 0;
    uint8_t map[256];
    std::vector<uint8_t> alphabet;
    uint8_t constVal = 0;
    // device outputs and sizes
    uint8_t* out = nullptr;
    uint32_t sizeSlot = 0;
    uint32_t sizes[4] = { 0, 0, 0, 0 };
    const uint8_t* dTable = nullptr;
    uint16_t* dFields = nullptr; // long FSE chunks: the per-state encoders' fields
    // 16-bit chunks (struct of 2-byte values)
    bool wide = false;
    unsigned width = 1; // element width in bytes
    unsigned maxSym16 = 0, card16 = 0;
    std::vector<uint32_t> count16, first16; // values 0..maxSym16
    uint8_t const16[2] = { 0, 0 };
    // huffman_struct_v2
    int tl16 = 0;
    std::vector<uint16_t> code16;
    std::vector<uint8_t> nbBits16;
    uint32_t streamCap = 0;
    uint32_t full[4] = { 0, 0, 0, 0 };      // whole bytes of each bitstream
    const uint8_t* dNbBits = nullptr;
    // tokenize: alphabet in first-occurrence order, sorted lookup, indices
    std::vector<uint8_t> alphabet16;        // little-endian 2-byte values
    std::vector<uint16_t> tokKeys;
    std::vector<uint8_t> tokIds;
    int idxJob = -1;                        // Huffman-graph job of the indices
    uint8_t* idxOut = nullptr;
    const uint8_t* dKeys = nullptr;
    const uint8_t* dIds = nullptr;
    unsigned alphaBits = 0;                 // bit packing of the alphabet
    uint64_t alphaBytes = 0;
    const uint8_t* alphaStaged = nullptr;
    uint8_t* alphaOut = nullptr;
};

struct RStream {
    int type;
    uint32_t w;
    uint64_t n;
    std::vector<Piece> pieces; // content (contiguous device pointer is pieces[0] when single)
    bool store = false;
    uint64_t bytes() const { return n * w; }
};

struct RNode {
    uint32_t trid;
    uint8_t hdr[16];
    size_t hsz = 0;
    int in;
    int outStart, nbOut, nbSO;
};

// Per-frame front-end plan (phase A).
struct Front {
    int mode = -1;            // -1 none, else EncOut
    bool delta = false, zigzag = false;
    uint8_t* out = nullptr;
    uint64_t n = 0;           // output elements
    uint64_t planeStride = 0;
    unsigned nbBits = 0;
    uint64_t outBytes = 0;
    uint32_t maxSlot = 0;
    bool needMax = false;
    bool needFirst = false;   // delta: the first element goes to the codec header
    uint64_t first = 0;
    int special = 0;          // 1: bf16 deconstruct, 2: tokenize
    uint8_t* signFrac = nullptr, *exponent = nullptr;  // bf16 outputs
    uint8_t* alphabet = nullptr, *idx = nullptr;       // tokenize outputs
    uint32_t iw = 0;          // tokenize index width
    uint64_t na = 0;          // tokenize alphabet size
    uint32_t tokSlot = 0;
};

} // namespace

// Pinned host staging of the blobs the host computes for the device (coding
// tables, Huffman weights, tokenize keys), uploaded in one copy.
struct PinnedBuf {
    uint8_t* p = nullptr;
    size_t cap = 0;
    ~PinnedBuf()
    {
        if (p) cudaFreeHost(p);
    }
    bool reserve(size_t bytes)
    {
        if (bytes <= cap) return true;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        if (cudaHostAlloc(reinterpret_cast<void**>(&p), bytes, cudaHostAllocDefault) != cudaSuccess) return false;
        cap = bytes;
        return true;
    }
};

// host threads of the calling compress() (0: the machine's, at most 16)
thread_local unsigned tlHostThreads = 0;

// fn(i) for i < n on up to 16 host threads (chunks of 64 indices)
template <class F>
void parallelFor(size_t n, F fn)
{
    unsigned const hw = std::thread::hardware_concurrency();
    unsigned const nt = std::min(tlHostThreads ? tlHostThreads : 16u, hw ? hw : 1u);
    if (n < 256 || nt < 2) {
        for (size_t i = 0; i < n; i++) fn(i);
        return;
    }
    std::atomic<size_t> next{ 0 };
    auto work = [&] {
        for (size_t i; (i = next.fetch_add(64)) < n;)
            for (size_t k = i; k < std::min(n, i + 64); k++) fn(k);
    };
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt; t++) th.emplace_back(work);
    work();
    for (auto& x : th) x.join();
}

struct EncodeBatch::Impl {
    DevBuf bufA, bufE, bufF, bufSmall, bufT, bufW, bufR, bufH;
    // the inputs' content checksums run on their own stream (a long input's
    // block chain is serial), from the front end until the assembly writes
    // them into the frames
    cudaStream_t hashStream = nullptr;
    cudaEvent_t hashStart = nullptr, hashDone = nullptr;
    bool hashPending = false;
    ~Impl()
    {
        if (hashStream) cudaStreamDestroy(hashStream);
        if (hashStart) cudaEventDestroy(hashStart);
        if (hashDone) cudaEventDestroy(hashDone);
    }
    PinnedBuf stage, stageH;
    std::vector<Job> jobs;           // data chunks (discovery order), then nested weights jobs
    size_t nbDataJobs = 0;
    bool checksums = true;
};

EncodeBatch::EncodeBatch() : impl_(new Impl) {}
EncodeBatch::~EncodeBatch() { delete impl_; }

size_t encodeBound(size_t srcBytes) { return srcBytes + srcBytes / 16 + 4096; }

namespace {

// ---------------------------------------------------------------------------
// Graph engine (one frame). In discovery mode entropy chunks are registered
// as jobs; in replay mode their decisions and encoded outputs are used.
struct Engine {
    bool discover;
    std::vector<Job>* jobs;
    std::vector<JobSeed>* seeds; // discovery: the frame's jobs in order
    size_t* jobCursor;          // next data-job index (same order in both modes)
    std::vector<RStream> s;
    std::vector<RNode> nd;
    const Front* front;
    int err = 0;

    int newStream(int type, uint32_t w, uint64_t n)
    {
        s.push_back(RStream{ type, w, n, {}, false });
        return int(s.size() - 1);
    }
    RNode& newNode(uint32_t trid, int in, int nbSO)
    {
        RNode x{};
        x.trid = trid;
        x.in = in;
        x.outStart = int(s.size());
        x.nbSO = nbSO;
        nd.push_back(x);
        return nd.back();
    }
    static std::vector<Piece> slice(const std::vector<Piece>& p, uint64_t off, uint64_t len)
    {
        // contiguous single-piece sources only
        std::vector<Piece> r;
        if (p.empty()) return r;
        Piece x = p[0];
        if (x.dev) x.dev += off;
        if (x.host) x.host += off;
        x.bytes = len;
        r.push_back(x);
        return r;
    }

    int convNumToSerial(int in)
    {
        RNode& x = newNode(TR_CONV_NUM_TO_SERIAL, in, 1);
        x.hdr[0] = uint8_t(ent::nextPow2Bits(s[in].w));
        x.hsz = 1;
        int o = newStream(T_SERIAL, 1, s[in].bytes());
        s[o].pieces = s[in].pieces;
        nd.back().nbOut = 1;
        return o;
    }
    int convStructToSerial(int in)
    {
        RNode& x = newNode(TR_CONV_STRUCT_TO_SERIAL, in, 1);
        uint64_t v = s[in].w;
        size_t k = 0;
        while (v >= 0x80) { x.hdr[k++] = uint8_t(v | 0x80); v >>= 7; }
        x.hdr[k++] = uint8_t(v);
        x.hsz = k;
        int o = newStream(T_SERIAL, 1, s[in].bytes());
        s[o].pieces = s[in].pieces;
        nd.back().nbOut = 1;
        return o;
    }
    // ZL_NODE_INTERPRET_TOKEN_AS_LE (encode_conversion_binding.c:179-189)
    int convStructToNum(int in)
    {
        newNode(TR_CONV_STRUCT_TO_NUM, in, 1);
        int o = newStream(T_NUMERIC, s[in].w, s[in].n);
        s[o].pieces = s[in].pieces;
        nd.back().nbOut = 1;
        return o;
    }
    int convNumToStruct(int in)
    {
        newNode(TR_CONV_NUM_TO_STRUCT, in, 1);
        int o = newStream(T_STRUCT, s[in].w, s[in].n);
        s[o].pieces = s[in].pieces;
        nd.back().nbOut = 1;
        return o;
    }
    // implicit conversion (src/openzl/compress/implicit_conversion.c:18-34)
    int convertFor(int sid, int mask)
    {
        int const t = s[sid].type;
        if (t & mask) return sid;
        if ((t & T_NUMERIC) && (mask & T_STRUCT)) return convNumToStruct(sid);
        if ((t & T_STRUCT) && (mask & T_SERIAL)) return convStructToSerial(sid);
        if ((t & T_NUMERIC) && (mask & T_SERIAL)) return convNumToSerial(sid);
        err = 43;
        return sid;
    }

    // ---- graphs ----------------------------------------------------------
    enum G {
        G_STORE, G_SERIAL_STORE, G_FSE, G_HUF, G_ENTROPY, G_CONSTANT, G_BITPACK, G_FLATPACK, G_NCOUNT, G_TSPLIT_FSE,
        G_TSPLIT_STORE, G_BITPACK_HUF, G_JOB, G_TOKENIZE, G_BF16, G_BITPACK16, G_ALPHAPACK
    };
    struct Succ {
        int g, sid, job;
    };

    void runSuccs(std::vector<Succ>& l)
    {
        // successors run in edge-creation (stream id) order (cctx.c:660-690)
        std::stable_sort(l.begin(), l.end(), [](const Succ& a, const Succ& b) { return a.sid < b.sid; });
        for (const Succ& x : l) {
            if (err) return;
            runSuccessor(x.g, x.sid, x.job);
        }
    }

    // small single inputs are stored (cctx.c:1125-1140)
    void runSuccessor(int g, int sid, int job = -1)
    {
        if (err) return;
        if (g != G_SERIAL_STORE && s[sid].bytes() < kMinStream) g = G_STORE;
        if (g == G_STORE && s[sid].bytes() < kMinStream) {
            graph(G_SERIAL_STORE, sid, -1);
            return;
        }
        graph(g, sid, job);
    }

    Job* jobFor(int sid, int mode, int explicitJob)
    {
        if (explicitJob >= 0) return &(*jobs)[size_t(explicitJob)];
        size_t const j = (*jobCursor)++;
        if (discover) {
            seeds->push_back(JobSeed{ s[sid].pieces.empty() ? nullptr : s[sid].pieces[0].dev, s[sid].n, mode,
                                      s[sid].w == 2, unsigned(s[sid].w) });
            return nullptr;
        }
        return &(*jobs)[j];
    }

    // entropyCompressChunk (encode_entropy_binding.c:602-762)
    void entropyChunk(int sid, int mode, std::vector<Succ>& succ, int explicitJob)
    {
        if (s[sid].n <= 1) {
            succ.push_back({ G_STORE, sid, -1 });
            return;
        }
        Job* j = jobFor(sid, mode, explicitJob);
        if (!j) return; // discovery
        if (j->wide) {
            wideChunk(sid, *j, succ);
            return;
        }
        switch (j->codec) {
            case ent::CC_STORE: succ.push_back({ G_STORE, sid, -1 }); return;
            case ent::CC_CONSTANT: succ.push_back({ G_JOB, sid, int(j - jobs->data()) | (G_CONSTANT << 24) }); return;
            case ent::CC_FLATPACK: succ.push_back({ G_JOB, sid, int(j - jobs->data()) | (G_FLATPACK << 24) }); return;
            case ent::CC_BITPACK: succ.push_back({ G_JOB, sid, int(j - jobs->data()) | (G_BITPACK << 24) }); return;
            case ent::CC_FSE: {
                RNode& x = newNode(TR_FSE, sid, 2);
                x.hdr[0] = uint8_t(j->nbStates);
                size_t const nbBytes = size_t(ent::nextPow2Bits(j->n + 1) + 7) / 8;
                for (size_t b = 0; b < nbBytes; b++) x.hdr[1 + b] = uint8_t(j->n >> (8 * b));
                x.hsz = nbBytes + 1;
                int ns = newStream(T_NUMERIC, 2, j->hist.maxSym + 1);
                s[ns].pieces.push_back(Piece{ j->dNorm, nullptr, 2ull * (j->hist.maxSym + 1) });
                int bs = newStream(T_SERIAL, 1, j->sizes[0]);
                s[bs].pieces.push_back(Piece{ j->out, nullptr, j->sizes[0] });
                nd.back().nbOut = 2;
                succ.push_back({ G_NCOUNT, ns, int(j - jobs->data()) });
                succ.push_back({ G_STORE, bs, -1 });
                return;
            }
            case ent::CC_HUF: {
                RNode& x = newNode(TR_HUF, sid, 2);
                x.hdr[0] = uint8_t(j->x4 ? 1 : 0);
                size_t const nbBytes = size_t(ent::nextPow2Bits(j->n + 1) + 7) / 8;
                for (size_t b = 0; b < nbBytes; b++) x.hdr[1 + b] = uint8_t(j->n >> (8 * b));
                x.hsz = nbBytes + 1;
                int ws = newStream(T_NUMERIC, 1, j->weights.size());
                s[ws].pieces.push_back(Piece{ nullptr, j->weights.data(), j->weights.size() });
                uint64_t total = 0;
                for (int k = 0; k < (j->x4 ? 4 : 1); k++) total += j->sizes[k];
                int bs = newStream(T_SERIAL, 1, total + (j->x4 ? 6 : 0));
                if (j->x4) {
                    s[bs].pieces.push_back(Piece{ nullptr, j->jump, 6 });
                    uint32_t const cap = hufEncStreamCap(uint32_t((j->n + 3) / 4));
                    for (int k = 0; k < 4; k++) s[bs].pieces.push_back(Piece{ j->out + 16 + uint64_t(k) * cap, nullptr, j->sizes[k] });
                } else {
                    s[bs].pieces.push_back(Piece{ j->out, nullptr, j->sizes[0] });
                }
                nd.back().nbOut = 2;
                succ.push_back({ G_FSE, ws, j->weightsJob });
                succ.push_back({ G_STORE, bs, -1 });
                return;
            }
        }
    }

    // the 2-byte branch of entropyCompressChunk (encode_entropy_binding.c:
    // 612-681), from the decision taken on the chunk's statistics
    void wideChunk(int sid, Job& j, std::vector<Succ>& succ)
    {
        int const ji = int(&j - jobs->data());
        switch (j.codec) {
            case ent::CC_STORE: succ.push_back({ G_STORE, sid, -1 }); return;
            case ent::CC_CONSTANT: succ.push_back({ G_JOB, sid, ji | (G_CONSTANT << 24) }); return;
            case ent::CC_BITPACK: {
                int const o = convStructToNum(sid);
                succ.push_back({ G_JOB, o, ji | (G_BITPACK16 << 24) });
                return;
            }
            case ent::CC_TOK16: { // tokenize_struct (first-occurrence order)
                newNode(TR_TOKENIZE_FIXED, sid, 2);
                size_t const na = j.alphabet16.size() / 2;
                int const a = newStream(T_STRUCT, 2, na);
                s[a].pieces.push_back(Piece{ nullptr, j.alphabet16.data(), j.alphabet16.size() });
                int const o = newStream(T_NUMERIC, 1, j.n);
                s[o].pieces.push_back(Piece{ j.idxOut, nullptr, j.n });
                nd.back().nbOut = 2;
                if (ent::nextPow2Bits(uint64_t(j.maxSym16) + 1) < 16) {
                    int const c = convStructToNum(a);
                    succ.push_back({ G_JOB, c, ji | (G_ALPHAPACK << 24) });
                } else {
                    succ.push_back({ G_STORE, a, -1 });
                }
                succ.push_back({ G_HUF, o, j.idxJob });
                return;
            }
            case ent::CC_HUF16: { // EI_huffman_struct_v2 (encode_entropy_binding.c:287-367)
                RNode& x = newNode(TR_HUF16, sid, 2);
                x.hdr[0] = uint8_t(j.x4 ? 1 : 0);
                size_t const nbBytes = size_t(ent::nextPow2Bits(j.n + 1) + 7) / 8;
                for (size_t b = 0; b < nbBytes; b++) x.hdr[1 + b] = uint8_t(j.n >> (8 * b));
                x.hsz = nbBytes + 1;
                int const ws = newStream(T_NUMERIC, 1, j.weights.size());
                s[ws].pieces.push_back(Piece{ nullptr, j.weights.data(), j.weights.size() });
                uint64_t total = 0;
                int const ns = j.x4 ? 4 : 1;
                for (int k = 0; k < ns; k++) total += 8 + j.sizes[k];
                int const bs = newStream(T_SERIAL, 1, total);
                for (int k = 0; k < ns; k++)
                    s[bs].pieces.push_back(Piece{ j.out + uint64_t(k) * j.streamCap, nullptr, 8ull + j.sizes[k] });
                nd.back().nbOut = 2;
                succ.push_back({ G_FSE, ws, j.weightsJob });
                succ.push_back({ G_STORE, bs, -1 });
                return;
            }
            default: err = 32; return;
        }
    }

    void entropyGraph(int sid, int mode, int explicitJob)
    {
        std::vector<Succ> succ;
        // doEntropyConversion (encode_entropy_binding.c:764-810): width 1 to
        // serial, numeric width 2 to struct
        if (s[sid].w == 1 && s[sid].type != T_SERIAL)
            sid = s[sid].type == T_NUMERIC ? convNumToSerial(sid) : convStructToSerial(sid);
        else if (s[sid].w == 2 && s[sid].type == T_NUMERIC)
            sid = convNumToStruct(sid);
        if (s[sid].w != 1 && s[sid].w != 2) { err = 81; return; }
        uint64_t const n = s[sid].n;
        if (n < kMinChunking) {
            entropyChunk(sid, mode, succ, explicitJob);
        } else {
            uint64_t const nb = (n + kChunk - 1) / kChunk;
            uint32_t const w = s[sid].w;
            int const type = s[sid].type;
            newNode(type == T_STRUCT ? TR_SPLITN_STRUCT : TR_SPLITN, sid, 0);
            int const first = int(s.size());
            uint64_t pos = 0;
            std::vector<Piece> src = s[sid].pieces;
            for (uint64_t k = 0; k < nb; k++) {
                uint64_t const len = k + 1 < nb ? kChunk : n - pos;
                int o = newStream(type, w, len);
                s[o].pieces = slice(src, pos * w, len * w);
                pos += len;
            }
            nd.back().nbOut = int(nb);
            for (uint64_t k = 0; k < nb; k++) entropyChunk(first + int(k), mode, succ, -1);
        }
        runSuccs(succ);
    }

    void graph(int g, int sid, int job)
    {
        std::vector<Succ> succ;
        if (g == G_JOB) {
            g = job >> 24;
            job &= 0xffffff;
        }
        switch (g) {
            case G_SERIAL_STORE:
                sid = convertFor(sid, T_SERIAL);
                s[sid].store = true;
                return;
            case G_STORE: runSuccessor(G_SERIAL_STORE, sid); return;
            case G_FSE: sid = convertFor(sid, T_SERIAL); entropyGraph(sid, M_FSE, job); return;
            case G_HUF: entropyGraph(sid, M_HUF, job); return;
            case G_ENTROPY: entropyGraph(sid, M_ANY, job); return;
            case G_CONSTANT: {
                Job& j = (*jobs)[size_t(job)];
                bool const fixed = s[sid].type != T_SERIAL; // 2-byte struct chunks
                RNode& x = newNode(fixed ? TR_CONST_FIXED : TR_CONST_SERIAL, sid, 1);
                uint64_t v = s[sid].n;
                size_t k = 0;
                while (v >= 0x80) { x.hdr[k++] = uint8_t(v | 0x80); v >>= 7; }
                x.hdr[k++] = uint8_t(v);
                x.hsz = k;
                int o = newStream(s[sid].type, s[sid].w, 1);
                if (j.mode == M_CONSTANT && j.dsrc) // the constant graph: the input's first element
                    s[o].pieces.push_back(Piece{ j.dsrc, nullptr, s[sid].w });
                else
                    s[o].pieces.push_back(Piece{ nullptr, fixed ? j.const16 : &j.constVal, s[sid].w });
                nd.back().nbOut = 1;
                runSuccessor(G_SERIAL_STORE, o);
                return;
            }
            case G_BITPACK: {
                Job& j = (*jobs)[size_t(job)];
                RNode& x = newNode(TR_BITPACK_SERIAL, sid, 1);
                uint64_t const maxN = j.packBytes * 8 / j.packBits;
                x.hdr[0] = uint8_t(j.packBits - 1);
                x.hsz = 1;
                if (maxN > j.n) { x.hdr[1] = uint8_t(maxN - j.n); x.hsz = 2; }
                int o = newStream(T_SERIAL, 1, j.packBytes);
                s[o].pieces.push_back(Piece{ j.out, nullptr, j.packBytes });
                nd.back().nbOut = 1;
                runSuccessor(G_SERIAL_STORE, o);
                return;
            }
            case G_BITPACK16:
            case G_ALPHAPACK: { // ZL_GRAPH_BITPACK on 2-byte numbers (TR_BITPACK_INT)
                Job& j = (*jobs)[size_t(job)];
                bool const alpha = g == G_ALPHAPACK;
                unsigned const bits = alpha ? j.alphaBits : j.packBits;
                uint64_t const bytes = alpha ? j.alphaBytes : j.packBytes;
                uint64_t const n = s[sid].n;
                RNode& x = newNode(TR_BITPACK_INT, sid, 1);
                uint64_t const maxN = bytes * 8 / bits;
                x.hdr[0] = uint8_t((1u << 6) | (bits - 1));
                x.hsz = 1;
                if (maxN > n) { x.hdr[1] = uint8_t(maxN - n); x.hsz = 2; }
                int o = newStream(T_SERIAL, 1, bytes);
                s[o].pieces.push_back(Piece{ alpha ? j.alphaOut : j.out, nullptr, bytes });
                nd.back().nbOut = 1;
                runSuccessor(G_SERIAL_STORE, o);
                return;
            }
            case G_FLATPACK: {
                Job& j = (*jobs)[size_t(job)];
                sid = convertFor(sid, T_SERIAL);
                newNode(TR_FLATPACK, sid, 2);
                int a = newStream(T_SERIAL, 1, j.alphabet.size());
                s[a].pieces.push_back(Piece{ nullptr, j.alphabet.data(), j.alphabet.size() });
                int p = newStream(T_SERIAL, 1, j.packBytes);
                s[p].pieces.push_back(Piece{ j.out, nullptr, j.packBytes });
                nd.back().nbOut = 2;
                succ.push_back({ G_SERIAL_STORE, a, -1 });
                succ.push_back({ G_SERIAL_STORE, p, -1 });
                runSuccs(succ);
                return;
            }
            case G_NCOUNT: {
                Job& j = (*jobs)[size_t(job)];
                newNode(TR_NCOUNT, sid, 1);
                int o = newStream(T_SERIAL, 1, j.ncountSize);
                s[o].pieces.push_back(Piece{ j.dNcount, nullptr, j.ncountSize });
                nd.back().nbOut = 1;
                runSuccessor(G_SERIAL_STORE, o);
                return;
            }
            case G_TSPLIT_FSE:
            case G_TSPLIT_STORE: {
                sid = convertFor(sid, T_STRUCT);
                uint32_t const W = s[sid].w;
                uint64_t const m = s[sid].n;
                newNode(TR_TSPLIT, sid, 0);
                int const first = int(s.size());
                for (uint32_t b = 0; b < W; b++) {
                    int o = newStream(T_SERIAL, 1, m);
                    if (front->mode == EOUT_PLANES) s[o].pieces.push_back(Piece{ front->out + b * front->planeStride, nullptr, m });
                }
                nd.back().nbOut = int(W);
                for (uint32_t b = 0; b < W; b++) succ.push_back({ g == G_TSPLIT_FSE ? G_FSE : G_STORE, first + int(b), -1 });
                runSuccs(succ);
                return;
            }
            case G_TOKENIZE: { // encode_tokenize_binding.c:423 (numeric, first-occurrence order)
                sid = convertFor(sid, T_NUMERIC);
                newNode(TR_TOKENIZE_NUMERIC, sid, 2);
                int const a = newStream(s[sid].type, s[sid].w, front->na);
                s[a].pieces.push_back(Piece{ front->alphabet, nullptr, front->na * s[sid].w });
                int const o = newStream(T_NUMERIC, front->iw, s[sid].n);
                s[o].pieces.push_back(Piece{ front->idx, nullptr, s[sid].n * front->iw });
                nd.back().nbOut = 2;
                succ.push_back({ G_STORE, a, -1 });
                succ.push_back({ G_BITPACK_HUF, o, -1 });
                runSuccs(succ);
                return;
            }
            case G_BF16: { // encode_float_deconstruct_binding.c:14-80
                sid = convertFor(sid, T_NUMERIC);
                RNode& x = newNode(TR_FLOAT_DECONSTRUCT, sid, 2);
                x.hdr[0] = 1; // bfloat16
                x.hsz = 1;
                uint64_t const n = s[sid].n;
                int const sf = newStream(T_STRUCT, 1, n);
                s[sf].pieces.push_back(Piece{ front->signFrac, nullptr, n });
                int const ex = newStream(T_SERIAL, 1, n);
                s[ex].pieces.push_back(Piece{ front->exponent, nullptr, n });
                nd.back().nbOut = 2;
                succ.push_back({ G_STORE, sf, -1 });
                succ.push_back({ G_FSE, ex, -1 });
                runSuccs(succ);
                return;
            }
            case G_BITPACK_HUF: {
                sid = convertFor(sid, T_NUMERIC);
                RNode& x = newNode(TR_BITPACK_INT, sid, 1);
                static const uint8_t lg[9] = { 0, 0, 1, 0, 2, 0, 0, 0, 3 };
                uint64_t const n = s[sid].n;
                uint64_t const bytes = (n * front->nbBits + 7) / 8;
                uint64_t const maxN = bytes * 8 / front->nbBits;
                x.hdr[0] = uint8_t((lg[s[sid].w] << 6) | (front->nbBits - 1));
                x.hsz = 1;
                if (maxN > n) { x.hdr[1] = uint8_t(maxN - n); x.hsz = 2; }
                int o = newStream(T_SERIAL, 1, bytes);
                s[o].pieces.push_back(Piece{ front->out, nullptr, bytes });
                nd.back().nbOut = 1;
                runSuccessor(job == 1 ? G_STORE : G_HUF, o);
                return;
            }
            default: err = 32; return;
        }
    }

    // Pipeline steps of the numeric recipes, each hop a successor.
    void pipeline(int recipe, int in)
    {
        int cur = in;
        auto hop = [&](bool first) -> bool {
            if (!first && s[cur].bytes() < kMinStream) {
                runSuccessor(G_STORE, cur);
                return false;
            }
            return true;
        };
        bool const delta = recipe == RC_DZ_TSPLIT_FSE || recipe == RC_DZ_BITPACK_HUF || recipe == RC_D_TSPLIT_FSE
                || recipe == RC_D_BITPACK_HUF || recipe == RC_DELTA_STORE;
        bool const zz = recipe == RC_DZ_TSPLIT_FSE || recipe == RC_DZ_BITPACK_HUF || recipe == RC_ZIGZAG_STORE;
        bool first = true;
        if (delta) {
            RNode& x = newNode(TR_DELTA, cur, 1);
            uint32_t const w = s[cur].w;
            for (uint32_t b = 0; b < w; b++) x.hdr[b] = uint8_t(front->first >> (8 * b));
            x.hsz = w;
            uint64_t const n = s[cur].n;
            int o = newStream(T_NUMERIC, s[cur].w, n ? n - 1 : 0);
            nd.back().nbOut = 1;
            // delta output content: the front end writes it when it is the
            // last step (plain) or when it is stored because it is small
            if (front->mode == EOUT_PLAIN && !front->zigzag) s[o].pieces.push_back(Piece{ front->out, nullptr, front->outBytes });
            cur = o;
            first = false;
            if (!hop(false)) return;
        }
        if (zz) {
            if (!first && !hop(false)) return;
            newNode(TR_ZIGZAG, cur, 1);
            int o = newStream(T_NUMERIC, s[cur].w, s[cur].n);
            nd.back().nbOut = 1;
            if (front->mode == EOUT_PLAIN) s[o].pieces.push_back(Piece{ front->out, nullptr, front->outBytes });
            cur = o;
            first = false;
        }
        switch (recipe) {
            case RC_DZ_TSPLIT_FSE:
            case RC_D_TSPLIT_FSE: {
                if (!hop(first)) return;
                cur = convNumToStruct(cur);
                runSuccessor(G_TSPLIT_FSE, cur);
                return;
            }
            case RC_TSPLIT_STORE: {
                if (!hop(first)) return;
                cur = convNumToStruct(cur);
                runSuccessor(G_TSPLIT_STORE, cur);
                return;
            }
            case RC_DZ_BITPACK_HUF:
            case RC_D_BITPACK_HUF: runSuccessor(G_BITPACK_HUF, cur, 0); return;
            case RC_BITPACK_STORE: runSuccessor(G_BITPACK_HUF, cur, 1); return;
            case RC_DELTA_STORE:
            case RC_ZIGZAG_STORE: runSuccessor(G_STORE, cur); return;
            default: err = 32; return;
        }
    }
};

uint8_t typeCode(int t) { return t == T_SERIAL ? 0 : (t == T_STRUCT ? 1 : 2); }

void pushVarint(std::vector<uint8_t>& o, uint64_t v)
{
    while (v >= 0x80) {
        o.push_back(uint8_t(v | 0x80));
        v >>= 7;
    }
    o.push_back(uint8_t(v));
}

void pushBits(std::vector<uint8_t>& o, const std::vector<uint32_t>& v, int nbBits)
{
    size_t const base = o.size();
    o.resize(base + (v.size() * size_t(nbBits) + 7) / 8, 0);
    for (size_t i = 0; i < v.size(); i++) {
        size_t bit = i * size_t(nbBits);
        for (int b = 0; b < nbBits; b++, bit++)
            if ((v[i] >> b) & 1) o[base + (bit >> 3)] |= uint8_t(1u << (bit & 7));
    }
}

} // namespace

// ---------------------------------------------------------------------------
int EncodeBatch::compress(const std::vector<EncFrameSpec>& frames, uint8_t* const* dOut, const size_t* caps,
                          bool checksums, cudaStream_t st, std::vector<size_t>& sizes, std::string& err)
{
    Impl& I = *impl_;
    launches_ = 0;
    static std::once_flag prepOnce;
    static cudaError_t prepErr = cudaSuccess;
    std::call_once(prepOnce, [] { prepErr = prepareEncodeKernels(); });
    if (prepErr != cudaSuccess) { err = "kernel attributes"; return 1; }
    size_t const nf = frames.size();
    sizes.assign(nf, 0);
    std::vector<Front> fronts(nf);
    tlHostThreads = hostThreads_;
    for (double& m : phaseMs_) m = 0;
    auto clock0 = std::chrono::steady_clock::now();
    int phase = 0;
    auto endPhase = [&]() { // closes phase `phase` and opens the next
        auto const now = std::chrono::steady_clock::now();
        if (phase < kPhases) phaseMs_[phase] = std::chrono::duration<double, std::milli>(now - clock0).count();
        clock0 = now;
        phase++;
    };

    // ---- phase A: front-end plan -------------------------------------------------
    for (size_t f = 0; f < nf; f++) {
        const EncFrameSpec& F = frames[f];
        Front& fr = fronts[f];
        uint64_t const inBytes = F.n * F.w;
        int const r = F.recipe;
        bool const hasDelta = r == RC_DZ_TSPLIT_FSE || r == RC_DZ_BITPACK_HUF || r == RC_D_TSPLIT_FSE
                || r == RC_D_BITPACK_HUF || r == RC_DELTA_STORE;
        bool const hasZz = r == RC_DZ_TSPLIT_FSE || r == RC_DZ_BITPACK_HUF || r == RC_ZIGZAG_STORE;
        if (F.serial || inBytes < kMinStream) continue; // no numeric front end
        if (r == RC_FSE || r == RC_HUFFMAN || r == RC_ENTROPY) continue; // the graphs read the input itself
        if (r == RC_BF16) {
            if (F.w != 2) { err = "bf16 deconstruct takes 2-byte elements"; return 54; }
            fr.special = 1;
            fr.n = F.n;
            continue;
        }
        if (r == RC_TOKENIZE || r == RC_TOKENIZE_SORTED) {
            if (F.n >= (1ull << 32)) { err = "tokenize input too large"; return 4; }
            fr.special = 2;
            fr.n = F.n;
            fr.mode = EOUT_BITPACK; // the indices, bit-packed
            continue;
        }
        fr.needFirst = hasDelta;
        uint64_t const m = hasDelta ? F.n - 1 : F.n;
        if (hasDelta && m * F.w < kMinStream) {
            fr.mode = EOUT_PLAIN; // small delta output: stored as is
            fr.delta = true;
            fr.n = m;
            continue;
        }
        fr.delta = hasDelta;
        fr.zigzag = hasZz;
        fr.n = m;
        if (r == RC_DZ_TSPLIT_FSE || r == RC_D_TSPLIT_FSE || r == RC_TSPLIT_STORE) fr.mode = EOUT_PLANES;
        else if (r == RC_DZ_BITPACK_HUF || r == RC_D_BITPACK_HUF || r == RC_BITPACK_STORE) { fr.mode = EOUT_BITPACK; fr.needMax = true; }
        else fr.mode = EOUT_PLAIN;
    }
    // maxima for bit packing
    std::vector<EncNumTask> maxTasks;
    std::vector<TileRef> maxTiles;
    uint32_t nbMax = 0;
    for (size_t f = 0; f < nf; f++) {
        Front& fr = fronts[f];
        if (!fr.needMax) continue;
        fr.maxSlot = nbMax++;
        EncNumTask t{};
        t.src = frames[f].dIn;
        t.n = fr.n;
        t.w = frames[f].w;
        t.delta = fr.delta;
        t.zigzag = fr.zigzag;
        t.maxSlot = fr.maxSlot;
        for (uint32_t k = 0; k < (fr.n + kEncTile - 1) / kEncTile; k++) maxTiles.push_back(TileRef{ uint32_t(maxTasks.size()), k });
        maxTasks.push_back(t);
    }
    // content checksums of the inputs, computed on the device now and
    // written into the frames during assembly
    std::vector<HashTask> contentHash;
    std::vector<TileRef> contentBlocks;
    {
        size_t smallBytes = 4096 + maxTasks.size() * sizeof(EncNumTask) + maxTiles.size() * sizeof(TileRef)
                + nbMax * 8 + nf * (sizeof(HashTask) + 8) + 64 + nf * (8 + sizeof(CopyTask) + sizeof(TileRef)) + 256;
        uint64_t blocks = 0;
        for (size_t f = 0; f < nf; f++) {
            uint64_t const len = frames[f].n * frames[f].w;
            if (len > 240) blocks += (len - 1) / kHashBlock;
        }
        smallBytes += blocks * (64 + sizeof(TileRef)) + 1024;
        // a previous call that failed may have left its checksums running on
        // the side stream, which reads this buffer
        if (I.hashPending) {
            cudaEventSynchronize(I.hashDone);
            I.hashPending = false;
        }
        if (!I.bufSmall.reserve(smallBytes)) { err = "device allocation failed"; return 70; }
        Bump b{ I.bufSmall.data(), 0 };
        auto* dMaxTasks = reinterpret_cast<EncNumTask*>(b.take(maxTasks.size() * sizeof(EncNumTask) + 1));
        auto* dMaxTiles = reinterpret_cast<TileRef*>(b.take(maxTiles.size() * sizeof(TileRef) + 1));
        auto* dMax = reinterpret_cast<unsigned long long*>(b.take(nbMax * 8 + 8));
        auto* dHashOut = reinterpret_cast<uint64_t*>(b.take(nf * 8 + 8));
        auto* dHashTasks = reinterpret_cast<HashTask*>(b.take(nf * sizeof(HashTask) + 1));
        auto* dSums = reinterpret_cast<uint64_t*>(b.take(blocks * 64 + 64));
        auto* dBlocks = reinterpret_cast<TileRef*>(b.take(blocks * sizeof(TileRef) + 8));
        auto* dFirst = reinterpret_cast<uint64_t*>(b.take(nf * 8 + 8));
        auto* dFirstCopies = reinterpret_cast<CopyTask*>(b.take(nf * sizeof(CopyTask) + 8));
        auto* dFirstTiles = reinterpret_cast<TileRef*>(b.take(nf * sizeof(TileRef) + 8));
        // first elements of the delta inputs, gathered into one array
        std::vector<CopyTask> firstCopies;
        std::vector<TileRef> firstTiles;
        for (size_t f = 0; f < nf; f++)
            if (fronts[f].needFirst) {
                firstTiles.push_back(TileRef{ uint32_t(firstCopies.size()), 0 });
                firstCopies.push_back(CopyTask{ reinterpret_cast<uint8_t*>(dFirst + f), frames[f].dIn, frames[f].w, 0 });
            }
        if (!firstCopies.empty()) {
            cudaMemsetAsync(dFirst, 0, nf * 8, st);
            cudaMemcpyAsync(dFirstCopies, firstCopies.data(), firstCopies.size() * sizeof(CopyTask), cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(dFirstTiles, firstTiles.data(), firstTiles.size() * sizeof(TileRef), cudaMemcpyHostToDevice, st);
            launchCopy(dFirstCopies, dFirstTiles, uint32_t(firstTiles.size()), st);
            launches_++;
        }
        if (checksums) {
            uint64_t bb = 0;
            for (size_t f = 0; f < nf; f++) {
                HashTask h{};
                h.data = frames[f].dIn;
                h.len = frames[f].n * frames[f].w;
                h.aligned8 = (reinterpret_cast<uintptr_t>(h.data) & 7) == 0;
                h.nbBlocks = h.len > 240 ? uint32_t((h.len - 1) / kHashBlock) : 0;
                h.blockSums = dSums + 8 * bb;
                h.hashOut = dHashOut + f;
                for (uint32_t k = 0; k < h.nbBlocks; k++) contentBlocks.push_back(TileRef{ uint32_t(f), k });
                bb += h.nbBlocks;
                contentHash.push_back(h);
            }
        }
        if (!maxTasks.empty()) {
            cudaMemcpyAsync(dMaxTasks, maxTasks.data(), maxTasks.size() * sizeof(EncNumTask), cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(dMaxTiles, maxTiles.data(), maxTiles.size() * sizeof(TileRef), cudaMemcpyHostToDevice, st);
            cudaMemsetAsync(dMax, 0, nbMax * 8, st);
            launchEncMax(dMaxTasks, dMaxTiles, uint32_t(maxTiles.size()), dMax, st);
            launches_++;
        }
        if (!contentHash.empty()) {
            bool const ok = (I.hashStream || cudaStreamCreateWithFlags(&I.hashStream, cudaStreamNonBlocking) == cudaSuccess)
                            && (I.hashStart || cudaEventCreateWithFlags(&I.hashStart, cudaEventDisableTiming) == cudaSuccess)
                            && (I.hashDone || cudaEventCreateWithFlags(&I.hashDone, cudaEventDisableTiming) == cudaSuccess);
            if (!ok) { err = "checksum stream could not be set up"; return 1; }
            cudaStream_t const hs = I.hashStream;
            cudaEventRecord(I.hashStart, st); // the inputs are ready on `st`
            cudaStreamWaitEvent(hs, I.hashStart, 0);
            cudaMemcpyAsync(dHashTasks, contentHash.data(), contentHash.size() * sizeof(HashTask), cudaMemcpyHostToDevice, hs);
            if (!contentBlocks.empty())
                cudaMemcpyAsync(dBlocks, contentBlocks.data(), contentBlocks.size() * sizeof(TileRef), cudaMemcpyHostToDevice, hs);
            launchHash(dHashTasks, uint32_t(contentHash.size()), dBlocks, uint32_t(contentBlocks.size()), nullptr, hs);
            cudaEventRecord(I.hashDone, hs);
            I.hashPending = true;
            launches_ += contentBlocks.empty() ? 1 : 2;
        }
        std::vector<unsigned long long> maxima(nbMax);
        if (nbMax) cudaMemcpyAsync(maxima.data(), dMax, nbMax * 8, cudaMemcpyDeviceToHost, st);
        std::vector<uint64_t> firsts(firstCopies.empty() ? 0 : nf);
        if (!firstCopies.empty()) cudaMemcpyAsync(firsts.data(), dFirst, nf * 8, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) { err = "device error in phase A"; return 1; }
        for (size_t f = 0; f < nf; f++)
            if (fronts[f].needFirst) fronts[f].first = firsts[f];
        for (size_t f = 0; f < nf; f++)
            if (fronts[f].needMax) {
                uint64_t const mx = maxima[fronts[f].maxSlot];
                fronts[f].nbBits = 1 + (mx ? unsigned(63 - __builtin_clzll(mx)) : 0);
            }
        // keep the content hash outputs' addresses
        for (size_t f = 0; f < contentHash.size(); f++) contentHash[f].hashOut = dHashOut + f;
    }

    // tokenize: distinct values in first-occurrence order, counted then emitted
    {
        std::vector<size_t> tokFrames;
        for (size_t f = 0; f < nf; f++)
            if (fronts[f].special == 2) tokFrames.push_back(f);
        if (!tokFrames.empty()) {
            std::vector<TokTask> tt(tokFrames.size());
            std::vector<TileRef> tiles;
            uint8_t *dTasks = nullptr, *dTiles = nullptr, *dSums = nullptr, *dPre = nullptr, *dCnt = nullptr;
            auto layoutT = [&](Bump& b) {
                tiles.clear();
                for (size_t k = 0; k < tokFrames.size(); k++) {
                    size_t const f = tokFrames[k];
                    uint64_t const n = frames[f].n;
                    uint32_t const w = frames[f].w;
                    uint64_t cap = 1024;
                    while (cap < 2 * n) cap <<= 1;
                    TokTask& t = tt[k];
                    t = TokTask{};
                    t.src = frames[f].dIn;
                    t.n = n;
                    t.w = w;
                    t.capMask = cap - 1;
                    t.state = reinterpret_cast<uint32_t*>(b.take(4 * cap));
                    t.key = reinterpret_cast<uint64_t*>(b.take(8 * cap));
                    t.first = reinterpret_cast<uint32_t*>(b.take(4 * cap));
                    t.slotOf = reinterpret_cast<uint32_t*>(b.take(4 * n + 64));
                    t.rank = reinterpret_cast<uint32_t*>(b.take(4 * n + 64));
                    t.alphabet = b.take(uint64_t(w) * n + 64);
                    t.idx = b.take(4 * n + 64);
                    t.tileBase = uint32_t(tiles.size());
                    for (uint32_t j = 0; j < (n + kEncTile - 1) / kEncTile; j++) tiles.push_back(TileRef{ uint32_t(k), j });
                    fronts[f].tokSlot = uint32_t(k);
                }
                dTasks = b.take(tt.size() * sizeof(TokTask));
                dTiles = b.take(tiles.size() * sizeof(TileRef));
                dSums = b.take(tiles.size() * 8 + 8);
                dPre = b.take(tiles.size() * 8 + 8);
                dCnt = b.take(tt.size() * 4 + 8); // counts, then the error count
            };
            Bump sizeT;
            layoutT(sizeT);
            if (!I.bufT.reserve(sizeT.used)) { err = "device allocation failed"; return 70; }
            Bump realT{ I.bufT.data(), 0 };
            layoutT(realT);
            for (const TokTask& t : tt) {
                cudaMemsetAsync(t.state, 0, 4 * (t.capMask + 1), st);
                cudaMemsetAsync(t.first, 0xff, 4 * (t.capMask + 1), st);
            }
            uint32_t* const counts = reinterpret_cast<uint32_t*>(dCnt);
            uint32_t* const errors = counts + tt.size();
            cudaMemsetAsync(dCnt, 0, tt.size() * 4 + 8, st);
            cudaMemcpyAsync(dTasks, tt.data(), tt.size() * sizeof(TokTask), cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(dTiles, tiles.data(), tiles.size() * sizeof(TileRef), cudaMemcpyHostToDevice, st);
            launchTokCount(reinterpret_cast<const TokTask*>(dTasks), uint32_t(tt.size()),
                           reinterpret_cast<const TileRef*>(dTiles), uint32_t(tiles.size()),
                           reinterpret_cast<uint64_t*>(dSums), reinterpret_cast<uint64_t*>(dPre), counts, errors, st);
            launches_ += 4;
            std::vector<uint32_t> hc(tt.size() + 1);
            cudaMemcpyAsync(hc.data(), dCnt, (tt.size() + 1) * 4, cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) { err = "device error in tokenize"; return 1; }
            if (hc[tt.size()]) { err = "tokenize table overflow"; return 1; }
            for (size_t k = 0; k < tt.size(); k++) {
                Front& fr = fronts[tokFrames[k]];
                uint64_t const na = hc[k];
                fr.na = na;
                fr.iw = na <= 256 ? 1 : (na <= 65536 ? 2 : 4); // encode_tokenize_binding.c:195-205
                uint64_t const mx = na ? na - 1 : 0;
                fr.nbBits = 1 + (mx ? unsigned(63 - __builtin_clzll(mx)) : 0);
                fr.alphabet = tt[k].alphabet;
                fr.idx = tt[k].idx;
                tt[k].iw = fr.iw;
            }
            cudaMemcpyAsync(dTasks, tt.data(), tt.size() * sizeof(TokTask), cudaMemcpyHostToDevice, st);
            launchTokEmit(reinterpret_cast<const TokTask*>(dTasks), reinterpret_cast<const TileRef*>(dTiles),
                          uint32_t(tiles.size()), st);
            launches_++;
            // sorted alphabets (encode_tokenize_binding.c:185-193): the
            // first-occurrence alphabet comes back, is sorted here by increasing
            // unsigned value, goes back, and the indices are renumbered on the
            // device through each first-occurrence rank's sorted position
            std::vector<size_t> sk;
            for (size_t k = 0; k < tt.size(); k++)
                if (frames[tokFrames[k]].recipe == RC_TOKENIZE_SORTED && fronts[tokFrames[k]].na) sk.push_back(k);
            if (!sk.empty()) {
                std::vector<std::vector<uint8_t>> alpha(sk.size());
                for (size_t i = 0; i < sk.size(); i++) {
                    const TokTask& t = tt[sk[i]];
                    alpha[i].resize(fronts[tokFrames[sk[i]]].na * t.w);
                    cudaMemcpyAsync(alpha[i].data(), t.alphabet, alpha[i].size(), cudaMemcpyDeviceToHost, st);
                }
                if (cudaStreamSynchronize(st) != cudaSuccess) { err = "device error in tokenize"; return 1; }
                std::vector<std::vector<uint32_t>> rankOf(sk.size());
                uint64_t rankBytes = 0;
                std::vector<TileRef> rtiles;
                for (size_t i = 0; i < sk.size(); i++) {
                    const TokTask& t = tt[sk[i]];
                    size_t const na = fronts[tokFrames[sk[i]]].na;
                    std::vector<uint64_t> val(na);
                    for (size_t j = 0; j < na; j++) {
                        uint64_t v = 0;
                        for (uint32_t b = 0; b < t.w; b++) v |= uint64_t(alpha[i][j * t.w + b]) << (8 * b);
                        val[j] = v;
                    }
                    std::vector<uint32_t> order(na);
                    for (size_t j = 0; j < na; j++) order[j] = uint32_t(j);
                    std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return val[a] < val[b]; });
                    rankOf[i].resize(na);
                    std::vector<uint8_t> sorted(na * t.w);
                    for (size_t j = 0; j < na; j++) {
                        rankOf[i][order[j]] = uint32_t(j);
                        std::memcpy(&sorted[j * t.w], &alpha[i][size_t(order[j]) * t.w], t.w);
                    }
                    alpha[i].swap(sorted);
                    rankBytes += (4 * na + 255) & ~uint64_t(255);
                    for (uint32_t k = 0; k < (t.n + kEncTile - 1) / kEncTile; k++) rtiles.push_back(TileRef{ uint32_t(i), k });
                }
                size_t const need = rankBytes + sk.size() * sizeof(RemapTask) + rtiles.size() * sizeof(TileRef) + 1024;
                if (!I.bufR.reserve(need)) { err = "device allocation failed"; return 70; }
                Bump rb{ I.bufR.data(), 0 };
                std::vector<RemapTask> rt(sk.size());
                for (size_t i = 0; i < sk.size(); i++) {
                    const TokTask& t = tt[sk[i]];
                    auto* dRank = reinterpret_cast<uint32_t*>(rb.take(4 * rankOf[i].size(), 256));
                    cudaMemcpyAsync(dRank, rankOf[i].data(), 4 * rankOf[i].size(), cudaMemcpyHostToDevice, st);
                    cudaMemcpyAsync(t.alphabet, alpha[i].data(), alpha[i].size(), cudaMemcpyHostToDevice, st);
                    rt[i] = RemapTask{ t.idx, dRank, t.n, t.iw };
                }
                auto* dRt = reinterpret_cast<RemapTask*>(rb.take(rt.size() * sizeof(RemapTask)));
                auto* dRtiles = reinterpret_cast<TileRef*>(rb.take(rtiles.size() * sizeof(TileRef)));
                cudaMemcpyAsync(dRt, rt.data(), rt.size() * sizeof(RemapTask), cudaMemcpyHostToDevice, st);
                cudaMemcpyAsync(dRtiles, rtiles.data(), rtiles.size() * sizeof(TileRef), cudaMemcpyHostToDevice, st);
                launchRemap(dRt, dRtiles, uint32_t(rtiles.size()), st);
                launches_++;
                // the host copies above are pageable: they complete before the
                // calls return, so the vectors may go out of scope
                if (cudaStreamSynchronize(st) != cudaSuccess) { err = "device error in tokenize"; return 1; }
            }
        }
    }

    // front-end outputs
    {
        Bump sizeB;
        auto layoutA = [&](Bump& b) {
            for (size_t f = 0; f < nf; f++) {
                Front& fr = fronts[f];
                if (fr.special == 1) {
                    fr.signFrac = b.take(fr.n + 64, 64);
                    fr.exponent = b.take(fr.n + 64, 64);
                    continue;
                }
                if (fr.mode < 0) continue;
                uint32_t const w = fr.special == 2 ? fr.iw : frames[f].w;
                if (fr.mode == EOUT_PLANES) {
                    fr.planeStride = (fr.n + 63) & ~uint64_t(63);
                    fr.outBytes = fr.n; // per plane
                    fr.out = b.take(fr.planeStride * w + 64, 64);
                } else if (fr.mode == EOUT_BITPACK) {
                    fr.outBytes = (fr.n * fr.nbBits + 7) / 8;
                    fr.out = b.take(fr.outBytes + 64, 64);
                } else {
                    fr.outBytes = fr.n * w;
                    fr.out = b.take(fr.outBytes + 64, 64);
                }
            }
        };
        layoutA(sizeB);
        if (!I.bufA.reserve(sizeB.used)) { err = "device allocation failed"; return 70; }
        Bump real{ I.bufA.data(), 0 };
        layoutA(real);
    }
    {
        std::vector<EncNumTask> tasks;
        std::vector<TileRef> tiles;
        for (size_t f = 0; f < nf; f++) {
            Front& fr = fronts[f];
            if (fr.mode < 0 || fr.n == 0) continue;
            EncNumTask t{};
            t.src = fr.special == 2 ? fr.idx : frames[f].dIn;
            t.out = fr.out;
            t.n = fr.n;
            t.planeStride = fr.planeStride;
            t.w = fr.special == 2 ? fr.iw : frames[f].w;
            t.delta = fr.delta;
            t.zigzag = fr.zigzag;
            t.mode = uint8_t(fr.mode);
            t.nbBits = uint8_t(fr.nbBits);
            for (uint32_t k = 0; k < (fr.n + kEncTile - 1) / kEncTile; k++) tiles.push_back(TileRef{ uint32_t(tasks.size()), k });
            tasks.push_back(t);
        }
        std::vector<Bf16Task> bt;
        std::vector<TileRef> btiles;
        for (size_t f = 0; f < nf; f++) {
            Front& fr = fronts[f];
            if (fr.special != 1 || fr.n == 0) continue;
            for (uint32_t k = 0; k < (fr.n + kEncTile - 1) / kEncTile; k++) btiles.push_back(TileRef{ uint32_t(bt.size()), k });
            bt.push_back(Bf16Task{ frames[f].dIn, fr.signFrac, fr.exponent, fr.n });
        }
        if (!tasks.empty() || !bt.empty()) {
            size_t const bytes = tasks.size() * sizeof(EncNumTask) + tiles.size() * sizeof(TileRef)
                    + bt.size() * sizeof(Bf16Task) + btiles.size() * sizeof(TileRef) + 1024;
            if (!I.bufF.reserve(bytes)) { err = "device allocation failed"; return 70; }
            Bump b{ I.bufF.data(), 0 };
            auto* dT = reinterpret_cast<EncNumTask*>(b.take(tasks.size() * sizeof(EncNumTask)));
            auto* dTi = reinterpret_cast<TileRef*>(b.take(tiles.size() * sizeof(TileRef)));
            auto* dB = reinterpret_cast<Bf16Task*>(b.take(bt.size() * sizeof(Bf16Task)));
            auto* dBi = reinterpret_cast<TileRef*>(b.take(btiles.size() * sizeof(TileRef)));
            if (!tasks.empty()) {
                cudaMemcpyAsync(dT, tasks.data(), tasks.size() * sizeof(EncNumTask), cudaMemcpyHostToDevice, st);
                cudaMemcpyAsync(dTi, tiles.data(), tiles.size() * sizeof(TileRef), cudaMemcpyHostToDevice, st);
                launchEncNum(dT, dTi, uint32_t(tiles.size()), st);
                launches_++;
            }
            if (!bt.empty()) {
                cudaMemcpyAsync(dB, bt.data(), bt.size() * sizeof(Bf16Task), cudaMemcpyHostToDevice, st);
                cudaMemcpyAsync(dBi, btiles.data(), btiles.size() * sizeof(TileRef), cudaMemcpyHostToDevice, st);
                launchBf16(dB, dBi, uint32_t(btiles.size()), st);
                launches_++;
            }
            if (cudaStreamSynchronize(st) != cudaSuccess) { err = "device error in front end"; return 1; }
        }
    }

    endPhase();
    // ---- phase B: discovery ------------------------------------------------------
    I.jobs.clear();
    auto runFrame = [&](size_t f, bool discover, size_t* cursor, Engine& E) {
        const EncFrameSpec& F = frames[f];
        E.discover = discover;
        E.jobs = &I.jobs;
        E.jobCursor = cursor;
        E.front = &fronts[f];
        int const in = E.newStream(F.serial ? T_SERIAL : T_NUMERIC, F.w, F.n);
        E.s[in].pieces.push_back(Piece{ F.dIn, nullptr, F.n * F.w });
        int const r = F.recipe;
        if (E.s[in].bytes() < kMinStream || r == RC_STORE) { E.runSuccessor(Engine::G_STORE, in); return; }
        switch (r) {
            case RC_FSE: E.runSuccessor(Engine::G_FSE, in); break;
            case RC_TOKENIZE:
            case RC_TOKENIZE_SORTED: E.runSuccessor(Engine::G_TOKENIZE, in); break;
            case RC_BF16: E.runSuccessor(Engine::G_BF16, in); break;
            case RC_HUFFMAN: E.runSuccessor(Engine::G_HUF, in); break;
            case RC_ENTROPY: E.runSuccessor(Engine::G_ENTROPY, in); break;
            case RC_CONSTANT:
            case RC_FLATPACK:
            case RC_BITPACK: {
                // the whole input is one forced-codec job; the constant
                // graph takes serial or struct input, so numbers become
                // struct first (graph_registry.c:132)
                int const src = r == RC_CONSTANT ? E.convertFor(in, T_SERIAL | T_STRUCT) : in;
                Job* j = E.jobFor(src, r == RC_CONSTANT ? M_CONSTANT : (r == RC_FLATPACK ? M_FLATPACK : M_BITPACK), -1);
                if (j) {
                    int const g = r == RC_CONSTANT ? Engine::G_CONSTANT : (r == RC_FLATPACK ? Engine::G_FLATPACK : Engine::G_BITPACK);
                    E.graph(Engine::G_JOB, src, int(j - I.jobs.data()) | (g << 24));
                }
                break;
            }
            default: E.pipeline(r, in);
        }
    };
    // frames in parallel, each recording its jobs; then one job list in
    // frame order
    std::vector<size_t> frameJobStart(nf + 1, 0);
    {
        std::vector<std::vector<JobSeed>> seeds(nf);
        std::vector<int> errs(nf, 0);
        parallelFor(nf, [&](size_t f) {
            size_t cursor = 0;
            Engine E;
            E.seeds = &seeds[f];
            runFrame(f, true, &cursor, E);
            errs[f] = E.err;
        });
        for (size_t f = 0; f < nf; f++)
            if (errs[f]) { err = "graph not supported on the GPU path"; return errs[f]; }
        for (size_t f = 0; f < nf; f++) frameJobStart[f + 1] = frameJobStart[f] + seeds[f].size();
        I.jobs.clear();
        I.jobs.resize(frameJobStart[nf]);
        parallelFor(nf, [&](size_t f) {
            for (size_t k = 0; k < seeds[f].size(); k++) {
                Job& J = I.jobs[frameJobStart[f] + k];
                J.dsrc = seeds[f][k].dsrc;
                J.n = seeds[f][k].n;
                J.mode = seeds[f][k].mode;
                J.wide = seeds[f][k].wide;
                J.width = seeds[f][k].width;
            }
        });
        I.nbDataJobs = I.jobs.size();
    }

    endPhase();
    // ---- phase C: histograms ------------------------------------------------------
    size_t const nj = I.nbDataJobs;
    std::vector<uint32_t> hists(nj * 256);
    std::vector<HistTask> ht;
    for (size_t j = 0; j < nj; j++)
        if (!I.jobs[j].wide) ht.push_back(HistTask{ I.jobs[j].dsrc, uint32_t(I.jobs[j].n), uint32_t(j) });
    if (!ht.empty()) {
        size_t const bytes = ht.size() * sizeof(HistTask) + nj * 1024 + 256;
        if (!I.bufF.reserve(bytes)) { err = "device allocation failed"; return 70; }
        Bump b{ I.bufF.data(), 0 };
        auto* dHt = reinterpret_cast<HistTask*>(b.take(ht.size() * sizeof(HistTask)));
        auto* dH = reinterpret_cast<uint32_t*>(b.take(nj * 1024));
        cudaMemcpyAsync(dHt, ht.data(), ht.size() * sizeof(HistTask), cudaMemcpyHostToDevice, st);
        launchHist(dHt, uint32_t(ht.size()), dH, st);
        launches_++;
        cudaMemcpyAsync(hists.data(), dH, nj * 1024, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) { err = "device error in histograms"; return 1; }
    }
    // 16-bit chunks: value counts, first occurrences and maxima on the
    // device; the counts of values up to each chunk's maximum come back
    {
        std::vector<size_t> wide;
        for (size_t j = 0; j < nj; j++)
            if (I.jobs[j].wide) wide.push_back(j);
        if (!wide.empty()) {
            size_t const nw = wide.size();
            std::vector<Hist16Task> tasks(nw);
            std::vector<TileRef> tiles;
            for (size_t k = 0; k < nw; k++)
                for (uint32_t t = 0; t < (I.jobs[wide[k]].n + kEncTile - 1) / kEncTile; t++) tiles.push_back(TileRef{ uint32_t(k), t });
            size_t const bytes = nw * (2ull * 65536 * 4 + 256) + nw * sizeof(Hist16Task) + tiles.size() * sizeof(TileRef) + 1024;
            if (!I.bufW.reserve(bytes)) { err = "device allocation failed"; return 70; }
            Bump b{ I.bufW.data(), 0 };
            auto* dCount = reinterpret_cast<uint32_t*>(b.take(nw * 65536ull * 4));
            auto* dFirst = reinterpret_cast<uint32_t*>(b.take(nw * 65536ull * 4));
            auto* dMax = reinterpret_cast<uint32_t*>(b.take(nw * 4 + 4));
            auto* dTasks = reinterpret_cast<Hist16Task*>(b.take(nw * sizeof(Hist16Task)));
            auto* dTiles = reinterpret_cast<TileRef*>(b.take(tiles.size() * sizeof(TileRef) + 4));
            for (size_t k = 0; k < nw; k++) {
                const Job& J = I.jobs[wide[k]];
                tasks[k] = Hist16Task{ J.dsrc, uint32_t(J.n), dCount + k * 65536, dFirst + k * 65536, dMax + k };
            }
            cudaMemsetAsync(dCount, 0, nw * 65536ull * 4, st);
            cudaMemsetAsync(dFirst, 0xff, nw * 65536ull * 4, st);
            cudaMemsetAsync(dMax, 0, nw * 4, st);
            cudaMemcpyAsync(dTasks, tasks.data(), nw * sizeof(Hist16Task), cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(dTiles, tiles.data(), tiles.size() * sizeof(TileRef), cudaMemcpyHostToDevice, st);
            launchHist16(dTasks, dTiles, uint32_t(tiles.size()), st);
            launches_++;
            std::vector<uint32_t> mx(nw);
            cudaMemcpyAsync(mx.data(), dMax, nw * 4, cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) { err = "device error in 16-bit histograms"; return 1; }
            for (size_t k = 0; k < nw; k++) {
                Job& J = I.jobs[wide[k]];
                J.maxSym16 = mx[k];
                J.count16.resize(size_t(mx[k]) + 1);
                J.first16.resize(size_t(mx[k]) + 1);
                cudaMemcpyAsync(J.count16.data(), dCount + k * 65536, J.count16.size() * 4, cudaMemcpyDeviceToHost, st);
                cudaMemcpyAsync(J.first16.data(), dFirst + k * 65536, J.first16.size() * 4, cudaMemcpyDeviceToHost, st);
            }
            if (cudaStreamSynchronize(st) != cudaSuccess) { err = "device error in 16-bit histograms"; return 1; }
        }
    }

    endPhase();
    // ---- phase D: decisions and tables ------------------------------------------
    auto decide = [&](Job& j) {
        j.hist.n = j.n;
        j.hist.finish();
        if (j.mode == M_CONSTANT) j.codec = ent::CC_CONSTANT;
        else if (j.mode == M_FLATPACK) j.codec = ent::CC_FLATPACK;
        else if (j.mode == M_BITPACK) j.codec = ent::CC_BITPACK;
        else j.codec = ent::chooseCodec(j.hist, j.mode == M_HUF ? ent::EM_HUF : (j.mode == M_ANY ? ent::EM_ANY : ent::EM_FSE));
        switch (j.codec) {
            case ent::CC_CONSTANT: j.constVal = uint8_t(j.hist.maxSym); break;
            case ent::CC_BITPACK:
                // computeNbBits (encode_bitpack_binding.c:51-72)
                j.packBits = 1 + (j.hist.maxSym ? unsigned(31 - __builtin_clz(j.hist.maxSym)) : 0);
                j.packBytes = (j.n * j.packBits + 7) / 8;
                break;
            case ent::CC_FLATPACK: {
                j.alphabet.clear();
                std::memset(j.map, 0, 256);
                for (int s = 0; s < 256; s++)
                    if (j.hist.count[s]) {
                        j.map[s] = uint8_t(j.alphabet.size());
                        j.alphabet.push_back(uint8_t(s));
                    }
                size_t const na = j.alphabet.size();
                j.packBits = na <= 1 ? unsigned(na) : 1u + unsigned(31 - __builtin_clz(uint32_t(na - 1)));
                j.packBytes = j.n ? 1 + (j.packBits * j.n) / 8 : 0;
                break;
            }
            case ent::CC_FSE: // normalization, header and table follow on the device
                j.nbStates = j.n < 1000 ? 2 : 4;
                j.tl = ent::fseTableLog(11, j.n, j.hist.maxSym, 2);
                break;
            case ent::CC_HUF: // code lengths, codes and weights follow on the device
                j.tl = ent::fseTableLog(11, j.n, j.hist.maxSym, 1);
                j.x4 = j.n > 1000;
                break;
            default: break;
        }
    };
    // 16-bit chunks (encode_entropy_binding.c:612-681); tokenize adds the
    // Huffman-graph job of the indices, whose histogram follows from the
    // value counts
    auto decide16 = [&](size_t ji) -> bool {
        Job& J = I.jobs[ji];
        unsigned const m = J.maxSym16;
        J.card16 = 0;
        for (uint32_t c : J.count16) J.card16 += c != 0;
        J.codec = ent::chooseCodec16(J.count16.data(), m, J.n, J.card16);
        switch (J.codec) {
            case ent::CC_CONSTANT:
                J.const16[0] = uint8_t(m);
                J.const16[1] = uint8_t(m >> 8);
                return true;
            case ent::CC_BITPACK:
                J.packBits = 1 + (m ? unsigned(31 - __builtin_clz(m)) : 0);
                J.packBytes = (J.n * J.packBits + 7) / 8;
                return true;
            case ent::CC_TOK16: {
                std::vector<uint32_t> vals;
                for (unsigned v = 0; v <= m; v++)
                    if (J.count16[v]) vals.push_back(v);
                std::vector<uint32_t> order = vals;
                std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return J.first16[a] < J.first16[b]; });
                std::vector<uint8_t> rank(size_t(m) + 1, 0);
                J.alphabet16.clear();
                for (size_t k = 0; k < order.size(); k++) {
                    rank[order[k]] = uint8_t(k);
                    J.alphabet16.push_back(uint8_t(order[k]));
                    J.alphabet16.push_back(uint8_t(order[k] >> 8));
                }
                J.tokKeys.clear();
                J.tokIds.clear();
                for (uint32_t v : vals) {
                    J.tokKeys.push_back(uint16_t(v));
                    J.tokIds.push_back(rank[v]);
                }
                J.alphaBits = 1 + (m ? unsigned(31 - __builtin_clz(m)) : 0);
                J.alphaBytes = (order.size() * J.alphaBits + 7) / 8;
                Job W;
                W.n = J.n;
                W.mode = M_HUF;
                std::memset(W.hist.count, 0, sizeof(W.hist.count));
                for (size_t k = 0; k < order.size(); k++) W.hist.count[k] = J.count16[order[k]];
                decide(W);
                I.jobs.push_back(std::move(W));
                I.jobs[ji].idxJob = int(I.jobs.size() - 1);
                return true;
            }
            case ent::CC_HUF16: {
                J.code16.assign(size_t(m) + 1, 0);
                J.nbBits16.assign(size_t(m) + 1, 0);
                J.tl16 = ent::huf16Build(J.code16.data(), J.nbBits16.data(), J.count16.data(), m);
                if (J.tl16 < 0) return false;
                J.weights.resize(size_t(m) + 1);
                for (unsigned v = 0; v <= m; v++)
                    J.weights[v] = uint8_t(J.nbBits16[v] ? J.tl16 + 1 - J.nbBits16[v] : 0);
                J.x4 = J.n > 1000;
                uint64_t const maxLen = J.x4 ? J.n / 4 + 1 : J.n;
                J.streamCap = uint32_t(((8 + (maxLen * 20 + 8) / 8 + 16) + 15) & ~uint64_t(15));
                return true;
            }
            default: return true;
        }
    };
    // 16-bit chunks first (they append nested jobs), then the others on
    // host threads
    for (size_t j = 0; j < nj; j++)
        if (I.jobs[j].wide && !decide16(j)) { err = "16-bit Huffman table construction failed"; return 1; }
    parallelFor(nj, [&](size_t j) {
        if (I.jobs[j].wide) return;
        std::memcpy(I.jobs[j].hist.count, &hists[j * 256], 1024);
        decide(I.jobs[j]);
    });
    // Huffman tables on the device: every 8-bit Huffman chunk's code lengths
    // and codes (left on the device for the bitstream pass) and its weights
    // (brought back: the nested FSE graph of the weights is decided on them,
    // and the frame stores them or their FSE coding)
    {
        std::vector<size_t> hj;
        for (size_t j = 0; j < I.jobs.size(); j++)
            if (I.jobs[j].codec == ent::CC_HUF && !I.jobs[j].wide) hj.push_back(j);
        if (!hj.empty()) {
            size_t const nh = hj.size();
            size_t const tabBytes = (sizeof(ent::HufCTable) + 15) & ~size_t(15);
            size_t const upBytes = nh * sizeof(HufTableTask) + nh * 1024;
            if (!I.bufH.reserve(upBytes + nh * (tabBytes + 256) + 256) || !I.stageH.reserve(upBytes + nh * 256)) {
                err = "allocation failed";
                return 70;
            }
            uint8_t* const dBase = I.bufH.data();
            auto* dTasks = reinterpret_cast<HufTableTask*>(dBase);
            uint8_t* const dHist = dBase + nh * sizeof(HufTableTask);
            uint8_t* const dTabs = dHist + nh * 1024;
            uint8_t* const dW = dTabs + nh * tabBytes;
            auto* hTasks = reinterpret_cast<HufTableTask*>(I.stageH.p);
            uint8_t* const hHist = I.stageH.p + nh * sizeof(HufTableTask);
            uint8_t* const hW = I.stageH.p + upBytes;
            parallelFor(nh, [&](size_t k) {
                Job& J = I.jobs[hj[k]];
                std::memcpy(hHist + k * 1024, J.hist.count, 1024);
                J.dTable = dTabs + k * tabBytes;
                hTasks[k] = HufTableTask{ reinterpret_cast<const uint32_t*>(dHist + k * 1024), dTabs + k * tabBytes,
                                          dW + k * 256, J.hist.maxSym, J.tl };
            });
            cudaMemcpyAsync(dBase, I.stageH.p, upBytes, cudaMemcpyHostToDevice, st);
            launchHufTables(dTasks, uint32_t(nh), st);
            launches_++;
            cudaMemcpyAsync(hW, dW, nh * 256, cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) { err = "device error in Huffman tables"; return 1; }
            parallelFor(nh, [&](size_t k) {
                Job& J = I.jobs[hj[k]];
                J.weights.assign(hW + k * 256, hW + k * 256 + J.hist.maxSym + 1);
            });
        }
    }
    // nested weights jobs (FSE graph of Huffman weights): decided on the host
    // histogram of the weights, encoded on the device with the data jobs
    for (size_t j = 0; j < I.jobs.size(); j++) {
        Job& J = I.jobs[j];
        if (J.codec != ent::CC_HUF && J.codec != ent::CC_HUF16) continue;
        // weights stream: numeric u8; under 10 bytes it is stored, else the
        // FSE graph gets it after a numeric->serial conversion
        if (J.weights.size() < kMinStream) continue;
        Job W;
        W.hsrc = J.weights;
        W.n = J.weights.size();
        W.mode = M_FSE;
        std::memset(W.hist.count, 0, sizeof(W.hist.count));
        for (uint8_t x : W.hsrc) W.hist.count[x]++;
        J.weightsJob = int(I.jobs.size());
        I.jobs.push_back(std::move(W));
    }
    {
        // the weights jobs created above, decided on host threads
        size_t first = I.jobs.size();
        for (size_t j = 0; j < I.jobs.size(); j++)
            if (!I.jobs[j].hsrc.empty()) {
                first = j;
                break;
            }
        parallelFor(I.jobs.size() - first, [&](size_t k) {
            Job& W = I.jobs[first + k];
            if (!W.hsrc.empty()) decide(W);
        });
    }

    // the constant graph (EI_constant_typed, encode_constant_binding.c:27-30)
    // refuses input whose elements are not all equal: bytes and 2-byte
    // values by their histograms, wider elements compared on the host
    for (Job& J : I.jobs) {
        if (J.mode != M_CONSTANT) continue;
        bool constant;
        if (J.width == 2) {
            constant = J.card16 == 1;
        } else if (J.width <= 1) {
            constant = J.hist.card == 1;
        } else {
            std::vector<uint8_t> h(size_t(J.n) * J.width);
            constant = J.dsrc && cudaMemcpy(h.data(), J.dsrc, h.size(), cudaMemcpyDeviceToHost) == cudaSuccess;
            for (size_t i = 1; constant && i < J.n; i++)
                constant = std::memcmp(h.data() + i * J.width, h.data(), J.width) == 0;
        }
        if (!constant) { err = "the constant graph needs input whose elements are all equal"; return 1; }
        J.codec = ent::CC_CONSTANT;
    }
    endPhase();
    // ---- phase E: entropy bitstreams -----------------------------------------------
    {
        std::vector<FseTableTask> fseTabT;
        std::vector<FseEncTask> fseT;
        std::vector<HufEncTask> hufT;
        std::vector<PackTask> packT;
        std::vector<TileRef> packTiles;
        std::vector<Tok16Task> tok16T;
        std::vector<TileRef> tok16Tiles;
        std::vector<EncNumTask> wideNumT; // bit packing of 2-byte numbers
        std::vector<TileRef> wideNumTiles;
        std::vector<Huf16EncTask> huf16T;
        uint32_t nbSizes = 0;
        auto addWideNum = [&](const uint8_t* src, uint8_t* out, uint64_t n, unsigned bits) {
            EncNumTask t{};
            t.src = src;
            t.out = out;
            t.n = n;
            t.w = 2;
            t.mode = EOUT_BITPACK;
            t.nbBits = uint8_t(bits);
            for (uint32_t k = 0; k < (n + kEncTile - 1) / kEncTile; k++) wideNumTiles.push_back(TileRef{ uint32_t(wideNumT.size()), k });
            wideNumT.push_back(t);
        };
        // blobs computed on the host: device room from `stg`, uploaded in one copy
        struct Up {
            uint8_t* dev;
            const void* host;
            size_t bytes;
        };
        std::vector<Up> ups;
        auto layoutE = [&](Bump& b, Bump& stg, bool real) {
            nbSizes = 0;
            auto staged = [&](const void* host, size_t bytes, size_t room) -> uint8_t* {
                uint8_t* d = stg.take(room, 16);
                if (real && bytes) ups.push_back(Up{ d, host, bytes });
                return d;
            };
            for (size_t j = 0; j < I.jobs.size(); j++) {
                Job& J = I.jobs[j];
                if (J.wide) {
                    switch (J.codec) {
                        case ent::CC_BITPACK:
                            J.out = b.take(J.packBytes + 64, 16);
                            if (real) addWideNum(J.dsrc, J.out, J.n, J.packBits);
                            break;
                        case ent::CC_TOK16: {
                            size_t const na = J.tokKeys.size();
                            J.idxOut = b.take(J.n + 64, 16);
                            J.dKeys = staged(J.tokKeys.data(), 2 * J.tokKeys.size(), 2 * 256);
                            J.dIds = staged(J.tokIds.data(), J.tokIds.size(), 256);
                            I.jobs[size_t(J.idxJob)].dsrc = J.idxOut;
                            if (real) {
                                Tok16Task t{ J.dsrc, J.idxOut, reinterpret_cast<const uint16_t*>(J.dKeys), J.dIds, uint32_t(J.n),
                                             uint32_t(na) };
                                for (uint32_t k = 0; k < (J.n + kEncTile - 1) / kEncTile; k++)
                                    tok16Tiles.push_back(TileRef{ uint32_t(tok16T.size()), k });
                                tok16T.push_back(t);
                            }
                            if (ent::nextPow2Bits(uint64_t(J.maxSym16) + 1) < 16) {
                                J.alphaStaged = staged(J.alphabet16.data(), J.alphabet16.size(), 2 * na + 16);
                                J.alphaOut = b.take(J.alphaBytes + 64, 16);
                                if (real) addWideNum(J.alphaStaged, J.alphaOut, na, J.alphaBits);
                            }
                            break;
                        }
                        case ent::CC_HUF16: {
                            J.out = b.take(uint64_t(J.x4 ? 4 : 1) * J.streamCap, 16);
                            J.dTable = staged(J.code16.data(), 2 * J.code16.size(), 2 * J.code16.size() + 16);
                            J.dNbBits = staged(J.nbBits16.data(), J.nbBits16.size(), J.nbBits16.size() + 16);
                            J.sizeSlot = nbSizes;
                            nbSizes += 8;
                            if (real)
                                huf16T.push_back(Huf16EncTask{ J.dsrc, J.out, reinterpret_cast<const uint16_t*>(J.dTable), J.dNbBits,
                                                               uint32_t(J.n), J.streamCap, J.sizeSlot, J.x4 ? 1u : 0u });
                            break;
                        }
                        default: break;
                    }
                    continue;
                }
                if (!J.hsrc.empty()) J.dstaged = staged(J.hsrc.data(), J.hsrc.size(), J.hsrc.size() + 16);
                const uint8_t* src = J.hsrc.empty() ? J.dsrc : J.dstaged;
                switch (J.codec) {
                    case ent::CC_FSE: {
                        J.out = b.take(J.n + J.n / 128 + 512, 16);
                        // tables built on the device from the uploaded histogram
                        uint8_t* const table = b.take(sizeof(ent::FseCTable), 16);
                        J.dTable = table;
                        J.dNorm = b.take(2 * 256, 16);
                        J.dNcount = b.take(600, 16);
                        J.dFields = J.nbStates == 4 && J.n >= kFseLongMin
                                        ? reinterpret_cast<uint16_t*>(b.take(fseFieldBytes(uint32_t(J.n)), 16))
                                        : nullptr;
                        const uint8_t* const hist = staged(J.hist.count, 1024, 1024);
                        J.sizeSlot = nbSizes++;
                        J.ncountSlot = nbSizes++;
                        if (real) {
                            fseTabT.push_back(FseTableTask{ reinterpret_cast<const uint32_t*>(hist), J.n, table,
                                                            reinterpret_cast<int16_t*>(J.dNorm), J.dNcount,
                                                            J.hist.maxSym, J.tl, J.ncountSlot, 0 });
                            fseT.push_back(FseEncTask{ src, J.out, J.dTable, uint32_t(J.n), J.sizeSlot, J.nbStates, J.tl,
                                                       J.dFields });
                        }
                        break;
                    }
                    case ent::CC_HUF: {
                        uint32_t const seg = uint32_t((J.n + 3) / 4);
                        J.out = b.take(J.x4 ? 16 + 4ull * hufEncStreamCap(seg) : J.n + J.n / 8 + 64, 16);
                        // J.dTable: built on the device before this phase
                        J.sizeSlot = nbSizes;
                        nbSizes += 4;
                        if (real) hufT.push_back(HufEncTask{ src, J.out, J.dTable, uint32_t(J.n), J.sizeSlot, J.x4 ? 1u : 0u });
                        break;
                    }
                    case ent::CC_BITPACK:
                    case ent::CC_FLATPACK: {
                        J.out = b.take(J.packBytes + 64, 16);
                        uint8_t* map = J.codec == ent::CC_FLATPACK ? staged(J.map, 256, 256) : nullptr;
                        J.dTable = map;
                        if (real && J.n) {
                            PackTask t{ src, J.out, map, J.n, J.packBits, 0 };
                            for (uint32_t k = 0; k < (J.n + kEncTile - 1) / kEncTile; k++)
                                packTiles.push_back(TileRef{ uint32_t(packT.size()), k });
                            packT.push_back(t);
                        }
                        break;
                    }
                    default: break;
                }
            }
        };
        Bump sz, szStage;
        layoutE(sz, szStage, false);
        size_t const taskBytes = 4096 + I.jobs.size() * (sizeof(FseTableTask) + sizeof(FseEncTask) + sizeof(HufEncTask) + sizeof(PackTask)
                                                         + sizeof(Tok16Task) + 2 * sizeof(EncNumTask) + sizeof(Huf16EncTask));
        size_t tilesGuess = 0;
        for (auto& J : I.jobs) {
            if (J.codec == ent::CC_BITPACK || J.codec == ent::CC_FLATPACK) tilesGuess += (J.n + kEncTile - 1) / kEncTile;
            if (J.codec == ent::CC_TOK16) tilesGuess += 2 * ((J.n + kEncTile - 1) / kEncTile) + 1;
        }
        size_t const stageOff = (sz.used + taskBytes + tilesGuess * sizeof(TileRef) + (nbSizes + 16) * 4 + 1024 + 255)
                & ~size_t(255);
        size_t const total = stageOff + szStage.used + 256;
        if (!I.bufE.reserve(total) || !I.stage.reserve(szStage.used + 256)) { err = "allocation failed"; return 70; }
        Bump b{ I.bufE.data(), 0 };
        Bump stg{ I.bufE.data() + stageOff, 0 };
        layoutE(b, stg, true);
        if (b.used > stageOff) { err = "encode layout overflow"; return 1; }
        // longest chunks first: one lane encodes a chunk serially, so the
        // longest chains start at once and the short ones fill around them
        // (each task writes its own output and size slot)
        std::stable_sort(fseT.begin(), fseT.end(), [](const FseEncTask& a, const FseEncTask& c) { return a.n > c.n; });
        // long chunks (one lane per state) are the first nbLong of fseT
        size_t nbLong = 0;
        while (nbLong < fseT.size() && fseT[nbLong].fields) nbLong++;
        std::stable_sort(hufT.begin(), hufT.end(), [](const HufEncTask& a, const HufEncTask& c) { return a.n > c.n; });
        parallelFor(ups.size(), [&](size_t k) {
            std::memcpy(I.stage.p + (ups[k].dev - stg.base), ups[k].host, ups[k].bytes);
        });
        if (stg.used)
            cudaMemcpyAsync(stg.base, I.stage.p, stg.used, cudaMemcpyHostToDevice, st);
        auto* dFseTab = reinterpret_cast<FseTableTask*>(b.take(fseTabT.size() * sizeof(FseTableTask) + 1));
        auto* dTabErr = reinterpret_cast<uint32_t*>(b.take(16));
        auto* dFse = reinterpret_cast<FseEncTask*>(b.take(fseT.size() * sizeof(FseEncTask) + 1));
        auto* dHuf = reinterpret_cast<HufEncTask*>(b.take(hufT.size() * sizeof(HufEncTask) + 1));
        auto* dPack = reinterpret_cast<PackTask*>(b.take(packT.size() * sizeof(PackTask) + 1));
        auto* dPackTiles = reinterpret_cast<TileRef*>(b.take(packTiles.size() * sizeof(TileRef) + 1));
        auto* dSizes = reinterpret_cast<uint32_t*>(b.take((nbSizes + 1) * 4));
        auto* dTok16 = reinterpret_cast<Tok16Task*>(b.take(tok16T.size() * sizeof(Tok16Task) + 1));
        auto* dTok16Tiles = reinterpret_cast<TileRef*>(b.take(tok16Tiles.size() * sizeof(TileRef) + 1));
        auto* dWideNum = reinterpret_cast<EncNumTask*>(b.take(wideNumT.size() * sizeof(EncNumTask) + 1));
        auto* dWideNumTiles = reinterpret_cast<TileRef*>(b.take(wideNumTiles.size() * sizeof(TileRef) + 1));
        auto* dHuf16 = reinterpret_cast<Huf16EncTask*>(b.take(huf16T.size() * sizeof(Huf16EncTask) + 1));
        // uploads: the tasks (the staged blobs went up above)
        if (!fseTabT.empty())
            cudaMemcpyAsync(dFseTab, fseTabT.data(), fseTabT.size() * sizeof(FseTableTask), cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(dTabErr, 0, 4, st);
        if (!fseT.empty()) cudaMemcpyAsync(dFse, fseT.data(), fseT.size() * sizeof(FseEncTask), cudaMemcpyHostToDevice, st);
        if (!hufT.empty()) cudaMemcpyAsync(dHuf, hufT.data(), hufT.size() * sizeof(HufEncTask), cudaMemcpyHostToDevice, st);
        if (!packT.empty()) {
            cudaMemcpyAsync(dPack, packT.data(), packT.size() * sizeof(PackTask), cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(dPackTiles, packTiles.data(), packTiles.size() * sizeof(TileRef), cudaMemcpyHostToDevice, st);
        }
        if (nbSizes) cudaMemsetAsync(dSizes, 0, nbSizes * 4, st);
        // 16-bit chunks first: the tokenize indices feed their Huffman-graph
        // jobs below
        if (!tok16T.empty()) {
            cudaMemcpyAsync(dTok16, tok16T.data(), tok16T.size() * sizeof(Tok16Task), cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(dTok16Tiles, tok16Tiles.data(), tok16Tiles.size() * sizeof(TileRef), cudaMemcpyHostToDevice, st);
            launchTok16(dTok16, dTok16Tiles, uint32_t(tok16Tiles.size()), st);
            launches_++;
        }
        if (!wideNumT.empty()) {
            cudaMemcpyAsync(dWideNum, wideNumT.data(), wideNumT.size() * sizeof(EncNumTask), cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(dWideNumTiles, wideNumTiles.data(), wideNumTiles.size() * sizeof(TileRef), cudaMemcpyHostToDevice, st);
            launchEncNum(dWideNum, dWideNumTiles, uint32_t(wideNumTiles.size()), st);
            launches_++;
        }
        if (!huf16T.empty()) {
            cudaMemcpyAsync(dHuf16, huf16T.data(), huf16T.size() * sizeof(Huf16EncTask), cudaMemcpyHostToDevice, st);
            launchHuf16Enc(dHuf16, uint32_t(huf16T.size()), dSizes, st);
            launches_++;
        }
        launchFseTables(dFseTab, uint32_t(fseTabT.size()), dSizes, dTabErr, st);
        launchFseEncLong(dFse, uint32_t(nbLong), dSizes, st);
        launchFseEnc(dFse + nbLong, uint32_t(fseT.size() - nbLong), dSizes, st);
        launchHufEnc(dHuf, uint32_t(hufT.size()), dSizes, st);
        launchPack(dPack, dPackTiles, uint32_t(packTiles.size()), st);
        launches_ += (fseT.empty() ? 0 : 1) + (nbLong ? 2 : 0) + (fseT.size() > nbLong ? 1 : 0)
                     + (hufT.empty() ? 0 : 1) + (packTiles.empty() ? 0 : 1);
        std::vector<uint32_t> hs(nbSizes + 1);
        uint32_t tabErr = 0;
        if (nbSizes) cudaMemcpyAsync(hs.data(), dSizes, nbSizes * 4, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(&tabErr, dTabErr, 4, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) { err = "device error in entropy encoding"; return 1; }
        if (tabErr) { err = "FSE normalization failed"; return 1; }
        for (Job& J : I.jobs) {
            if (J.wide && J.codec == ent::CC_HUF16) {
                // the reference writes the streams into 2n + 32 bytes; each
                // stream takes 8 header bytes and fails once its whole bytes
                // reach its remaining room less 16 (encode_huffman_kernel.c:
                // 437-488, encode_entropy_binding.c:351)
                uint64_t avail = 2 * J.n + 32;
                for (int k = 0; k < (J.x4 ? 4 : 1); k++) {
                    J.sizes[k] = hs[J.sizeSlot + k];
                    J.full[k] = hs[J.sizeSlot + 4 + k];
                    if (avail < 8 || avail - 8 <= 8 || J.full[k] >= avail - 16 || 8ull + J.sizes[k] > J.streamCap) {
                        err = "16-bit Huffman stream over capacity";
                        return 1;
                    }
                    avail -= 8 + J.sizes[k];
                }
                continue;
            }
            if (J.codec == ent::CC_FSE) {
                J.ncountSize = hs[J.ncountSlot];
                J.sizes[0] = hs[J.sizeSlot];
                if (J.sizes[0] > J.n + J.n / 128 + 512) { err = "FSE bitstream over capacity"; return 1; }
            }
            if (J.codec == ent::CC_HUF) {
                for (int k = 0; k < 4; k++) J.sizes[k] = hs[J.sizeSlot + k];
                uint64_t const cap = J.x4 ? hufEncStreamCap(uint32_t((J.n + 3) / 4)) : J.n + J.n / 8 + 64;
                for (int k = 0; k < (J.x4 ? 4 : 1); k++)
                    if (J.sizes[k] > cap || (J.x4 && k < 3 && J.sizes[k] > 65535)) {
                        err = "Huffman stream over capacity";
                        return 1;
                    }
                if (J.x4) {
                    for (int k = 0; k < 3; k++) {
                        J.jump[2 * k] = uint8_t(J.sizes[k]);
                        J.jump[2 * k + 1] = uint8_t(J.sizes[k] >> 8);
                    }
                }
            }
        }
    }

    endPhase();
    // ---- phase F: replay and frame layout --------------------------------------
    struct FrameOut {
        std::vector<uint8_t> head;     // frame header + chunk header + codec headers
        std::vector<Piece> stored;     // stored streams in frame order
        size_t headerBytes = 0;        // frame header length (before the block)
        size_t total = 0;
    };
    std::vector<FrameOut> outs(nf);
    {
        // frames in parallel, each from its first job; the first failing
        // frame's error is reported
        std::vector<int> rcs(nf, 0);
        std::vector<const char*> msgs(nf, nullptr);
        parallelFor(nf, [&](size_t f) {
            size_t cursor = frameJobStart[f];
            Engine E;
            runFrame(f, false, &cursor, E);
            if (E.err) { rcs[f] = E.err; msgs[f] = "graph replay failed"; return; }
            FrameOut& O = outs[f];
            std::vector<uint8_t>& h = O.head;
            const RStream& in0 = E.s[0];
            uint32_t const magic = 0xD7B1A5C0u + 23;
            for (int b = 0; b < 4; b++) h.push_back(uint8_t(magic >> (8 * b)));
            h.push_back(uint8_t(checksums ? 3 : 0));
            h.push_back(uint8_t(1 | (typeCode(in0.type) << 4)));
            pushVarint(h, in0.bytes() + 1);
            O.headerBytes = h.size(); // the header checksum byte follows when enabled
            if (checksums) h.push_back(0);
            size_t const nd = E.nd.size();
            size_t nbStored = 0;
            for (const RStream& x : E.s) nbStored += x.store;
            pushVarint(h, nd + 1);
            pushVarint(h, nbStored);
            std::vector<uint32_t> a(nd, 0);
            pushBits(h, a, 1);
            for (size_t u = 0; u < nd; u++) a[u] = E.nd[nd - 1 - u].trid;
            pushBits(h, a, ent::nextPow2Bits(63));
            for (size_t u = 0; u < nd; u++) a[u] = E.nd[nd - 1 - u].hsz > 0;
            pushBits(h, a, 1);
            for (size_t u = 0; u < nd; u++)
                if (E.nd[nd - 1 - u].hsz) pushVarint(h, E.nd[nd - 1 - u].hsz - 1);
            for (size_t u = 0; u < nd; u++) a[u] = (E.nd[nd - 1 - u].nbOut - E.nd[nd - 1 - u].nbSO) > 0;
            pushBits(h, a, 1);
            for (size_t u = 0; u < nd; u++) {
                const RNode& x = E.nd[nd - 1 - u];
                if (x.nbOut - x.nbSO > 0) pushVarint(h, uint64_t(x.nbOut - x.nbSO - 1));
            }
            for (size_t u = 0; u < nd; u++) a[u] = 0;
            pushBits(h, a, 1);
            for (size_t u = 0; u < nd; u++) a[u] = uint32_t(E.nd[nd - 1 - u].outStart - E.nd[nd - 1 - u].in) - 1;
            pushBits(h, a, ent::nextPow2Bits(nd + nbStored));
            for (size_t i = E.s.size(); i-- > 0;)
                if (E.s[i].store) pushVarint(h, E.s[i].bytes());
            for (size_t u = 0; u < nd; u++) {
                const RNode& x = E.nd[nd - 1 - u];
                h.insert(h.end(), x.hdr, x.hdr + x.hsz);
            }
            for (size_t i = E.s.size(); i-- > 0;)
                if (E.s[i].store) {
                    uint64_t have = 0;
                    for (const Piece& p : E.s[i].pieces) {
                        O.stored.push_back(p);
                        have += p.bytes;
                    }
                    if (have != E.s[i].bytes()) { rcs[f] = 80; msgs[f] = "internal: stored stream without content"; return; }
                }
            uint64_t tot = h.size();
            for (const Piece& p : O.stored) tot += p.bytes;
            tot += checksums ? 8 : 0;
            tot += 1;
            O.total = tot;
            if (tot > caps[f]) { rcs[f] = 5; msgs[f] = "destination too small"; return; }
            sizes[f] = tot;
        });
        for (size_t f = 0; f < nf; f++)
            if (rcs[f]) { err = msgs[f]; return rcs[f]; }
    }

    endPhase();
    // ---- phase G: assembly and checksums -----------------------------------------
    {
        // host bytes go through one staging upload
        std::vector<uint8_t> stage;
        std::vector<CopyTask> copies;
        std::vector<std::pair<size_t, size_t>> hostCopies; // (stage offset, copy index)
        auto stageBytes = [&](const uint8_t* p, uint64_t n) {
            size_t const off = (stage.size() + 15) & ~size_t(15);
            stage.resize(off + n);
            if (n) std::memcpy(stage.data() + off, p, n);
            return off;
        };
        uint8_t const zero = 0;
        size_t const zeroOff = stageBytes(&zero, 1);
        for (size_t f = 0; f < nf; f++) {
            FrameOut& O = outs[f];
            uint64_t pos = 0;
            size_t const so = stageBytes(O.head.data(), O.head.size());
            copies.push_back(CopyTask{ dOut[f], nullptr, O.head.size(), 0 });
            hostCopies.push_back({ so, copies.size() - 1 });
            pos += O.head.size();
            for (const Piece& p : O.stored) {
                if (p.bytes) {
                    if (p.host) {
                        size_t const o2 = stageBytes(p.host, p.bytes);
                        copies.push_back(CopyTask{ dOut[f] + pos, nullptr, p.bytes, 0 });
                        hostCopies.push_back({ o2, copies.size() - 1 });
                    } else {
                        copies.push_back(CopyTask{ dOut[f] + pos, p.dev, p.bytes, 0 });
                    }
                }
                pos += p.bytes;
            }
            // end-of-frame marker (a zero byte) after the block checksums
            copies.push_back(CopyTask{ dOut[f] + O.total - 1, nullptr, 1, 0 });
            hostCopies.push_back({ zeroOff, copies.size() - 1 });
        }
        std::vector<TileRef> tiles;
        for (size_t i = 0; i < copies.size(); i++) {
            copies[i].tileBase = uint32_t(tiles.size());
            for (uint32_t k = 0; k < (copies[i].bytes + kTileBytes - 1) / kTileBytes; k++) tiles.push_back(TileRef{ uint32_t(i), k });
        }
        // checksum tasks: frame header (low 8 bits), block (content checksum
        // included, so it runs after the content checksum is in place)
        std::vector<HashTask> blockHash;
        std::vector<TileRef> blockBlocks;
        std::vector<PutTask> put1, put2;
        uint64_t nbBlocks = 0;
        if (checksums) {
            for (size_t f = 0; f < nf; f++) {
                FrameOut& O = outs[f];
                uint64_t const blockStart = O.headerBytes + 1;
                uint64_t const blockLen = O.total - 1 - 4 - blockStart;
                HashTask hh{};
                hh.data = dOut[f];
                hh.len = O.headerBytes;
                hh.aligned8 = (reinterpret_cast<uintptr_t>(dOut[f]) & 7) == 0;
                blockHash.push_back(hh);
                HashTask bh{};
                bh.data = dOut[f] + blockStart;
                bh.len = blockLen;
                bh.aligned8 = (reinterpret_cast<uintptr_t>(bh.data) & 7) == 0;
                bh.nbBlocks = blockLen > 240 ? uint32_t((blockLen - 1) / kHashBlock) : 0;
                blockHash.push_back(bh);
                nbBlocks += bh.nbBlocks;
            }
        }
        size_t const bytes = stage.size() + copies.size() * sizeof(CopyTask) + tiles.size() * sizeof(TileRef)
                + blockHash.size() * (sizeof(HashTask) + 8) + nbBlocks * (64 + sizeof(TileRef))
                + 3 * nf * sizeof(PutTask) + 4096;
        if (!I.bufF.reserve(bytes)) { err = "device allocation failed"; return 70; }
        Bump b{ I.bufF.data(), 0 };
        uint8_t* dStage = b.take(stage.size() + 16, 16);
        for (auto& hc : hostCopies) copies[hc.second].src = dStage + hc.first;
        auto* dCopies = reinterpret_cast<CopyTask*>(b.take(copies.size() * sizeof(CopyTask) + 1));
        auto* dTiles = reinterpret_cast<TileRef*>(b.take(tiles.size() * sizeof(TileRef) + 1));
        auto* dHT = reinterpret_cast<HashTask*>(b.take(blockHash.size() * sizeof(HashTask) + 1));
        auto* dHOut = reinterpret_cast<uint64_t*>(b.take(blockHash.size() * 8 + 8));
        auto* dSums = reinterpret_cast<uint64_t*>(b.take(nbBlocks * 64 + 64));
        auto* dBB = reinterpret_cast<TileRef*>(b.take(nbBlocks * sizeof(TileRef) + 8));
        auto* dPut1 = reinterpret_cast<PutTask*>(b.take(nf * sizeof(PutTask) + 1));
        auto* dPut2 = reinterpret_cast<PutTask*>(b.take(2 * nf * sizeof(PutTask) + 1));
        if (checksums) {
            uint64_t bb = 0;
            for (size_t i = 0; i < blockHash.size(); i++) {
                blockHash[i].hashOut = dHOut + i;
                blockHash[i].blockSums = dSums + 8 * bb;
                for (uint32_t k = 0; k < blockHash[i].nbBlocks; k++) blockBlocks.push_back(TileRef{ uint32_t(i), k });
                bb += blockHash[i].nbBlocks;
            }
            for (size_t f = 0; f < nf; f++) {
                FrameOut& O = outs[f];
                put1.push_back(PutTask{ dOut[f] + O.total - 1 - 8, contentHash[f].hashOut, 4 });
                put2.push_back(PutTask{ dOut[f] + O.headerBytes, dHOut + 2 * f, 1 });
                put2.push_back(PutTask{ dOut[f] + O.total - 1 - 4, dHOut + 2 * f + 1, 4 });
            }
        }
        cudaMemcpyAsync(dStage, stage.data(), stage.size(), cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(dCopies, copies.data(), copies.size() * sizeof(CopyTask), cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(dTiles, tiles.data(), tiles.size() * sizeof(TileRef), cudaMemcpyHostToDevice, st);
        if (checksums) {
            cudaMemcpyAsync(dHT, blockHash.data(), blockHash.size() * sizeof(HashTask), cudaMemcpyHostToDevice, st);
            if (!blockBlocks.empty())
                cudaMemcpyAsync(dBB, blockBlocks.data(), blockBlocks.size() * sizeof(TileRef), cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(dPut1, put1.data(), put1.size() * sizeof(PutTask), cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(dPut2, put2.data(), put2.size() * sizeof(PutTask), cudaMemcpyHostToDevice, st);
        }
        launchCopy(dCopies, dTiles, uint32_t(tiles.size()), st);
        launches_++;
        if (checksums) {
            if (I.hashPending) cudaStreamWaitEvent(st, I.hashDone, 0); // the content checksums go in now
            launchPut(dPut1, uint32_t(put1.size()), st);
            launchHash(dHT, uint32_t(blockHash.size()), dBB, uint32_t(blockBlocks.size()), nullptr, st);
            launchPut(dPut2, uint32_t(put2.size()), st);
            launches_ += 3 + (blockBlocks.empty() ? 0 : 1);
        }
        if (cudaStreamSynchronize(st) != cudaSuccess) { err = "device error in frame assembly"; return 1; }
        I.hashPending = false;
    }
    endPhase();
    return 0;
}

} // namespace ozl
